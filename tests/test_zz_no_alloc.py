"""gp_residual_static (residual with file-scope device scratch, no
allocation) against gp_residual, called through the C ABI.

The file name sorts last so that the entry point is also exercised after
every other test has created and destroyed layouts on the device.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import synthetic_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _p(a):
    return C.c_void_p(a.ctypes.data)


def test_static_scratch_residual_matches_gp_residual(G):
    lib = G.library()
    c, w = synthetic_case("planar2k", 2)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        rng = np.random.default_rng(11)
        z = gbl.z
        zold = np.ascontiguousarray(z + 1e-3 * rng.normal(size=z.shape))
        gbl.z = z + 1e-3 * rng.normal(size=z.shape)
        ref = np.empty((c.M, gbl.n_sys))
        none = G.LY.GpFault()
        assert lib.gp_residual(gbl._h, _p(zold), C.c_double(w.dt), 0, C.addressof(none), None, _p(ref)) == 0
        for _ in range(2):
            f = np.full((c.M, gbl.n_sys), np.nan)
            assert lib.gp_residual_static(gbl._h, _p(zold), C.c_double(w.dt), _p(f)) == 0
            assert np.array_equal(f, ref)
    finally:
        gbl.close()


def test_static_scratch_rejects_oversize_layout(G):
    lib = G.library()
    # 64 scenarios of the 2000-bus grid need about 31 MB of scratch
    c, w = synthetic_case("planar2k", 64)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        zold = np.ascontiguousarray(gbl.z)
        f = np.zeros((c.M, gbl.n_sys))
        rc = lib.gp_residual_static(gbl._h, _p(zold), C.c_double(w.dt), _p(f))
        assert rc == -1
        buf = C.create_string_buffer(512)
        lib.gp_last_error(buf, 512)
        assert b"scratch" in buf.value
    finally:
        gbl.close()
