"""Build libgradpower_gb300.so for sm_103a, in-tree (gradpower.jl_gb300/_build/).

Seven translation units compiled in parallel with nvcc, then linked; no
cmake, no torch extension machinery.  Safe to call repeatedly: sources newer
than the library trigger a rebuild.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgradpower_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["gp_api.cu", "gp_kernels.cu", "gp_dag.cu", "gp_solve.cu", "gp_adjoint.cu", "gp_init.cu",
           "gp_symbolic.cpp", "gp_cluster_plan.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _deps():
    files = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    files.append(os.path.join(INCLUDE, "gradpower_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
    cmds = []
    objs = []
    for s in SOURCES:
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        src = os.path.join(SRC, s)
        if s.endswith(".cu"):
            cmd = [NVCC, *ARCH, "-lineinfo", *common, "-c", src, "-o", obj]
        else:
            cmd = [NVCC, *common, "-x", "c++", "-c", src, "-o", obj]
        cmds.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for err in ex.map(run, cmds):
            if verbose and err:
                print(err)
    link = [NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
    run(link)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
