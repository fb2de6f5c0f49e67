"""GB300-native batched backward-Euler Newton step of GradPower.jl.

Host-side mirror of the reference's problem setup and of its
`BatchedLayout` / `GpuBatchedLayout` / `integrate_batched!` /
`integrate_gpu_cudss!` / `integrate_gpu_schur_cudss!` entry points, over the
C-ABI library `libgradpower_gb300.so` built from `csrc/`.
"""
from . import model, synthetic  # noqa: F401
