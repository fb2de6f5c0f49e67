"""The reciprocal the FP64 factorisations take of each pivot, on the GPU,
against the correctly rounded 1/x (numpy's IEEE division on the host).

The factorisations replace the division by the hardware's approximate
reciprocal refined by two Newton-Raphson steps; the bound here is one ulp
of 1/x over normal inputs across the exponent range, and the division's
exact result for the inputs that take it (zero, subnormal, very large,
infinite, NaN).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu.library()


def _recip(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    r = np.full_like(x, 7.0)
    assert lib.gp_recip_check(x.size, C.c_void_p(x.ctypes.data), C.c_void_p(r.ctypes.data)) == 0
    return r


def test_reciprocal_within_one_ulp_of_division(lib):
    rng = np.random.default_rng(5)
    n = 1 << 20
    # magnitudes log-uniform over the normal range whose reciprocals stay
    # normal, both signs; then the pivot magnitudes of the grids, densely
    mag = np.exp2(rng.uniform(-1021.5, 1020.5, size=n))
    piv = np.exp2(rng.uniform(-12.0, 14.0, size=n))
    x = np.concatenate([mag, piv]) * rng.choice([-1.0, 1.0], size=2 * n)
    # mantissas of all ones and exact powers of two
    x = np.concatenate([x, np.nextafter(np.exp2(np.arange(-1000, 1000, 7.0)), 0.0),
                        np.exp2(np.arange(-1021, 1021, 3.0))])
    r = _recip(lib, x)
    with np.errstate(all="ignore"):
        e = 1.0 / x
    ulp = np.abs(r - e) / np.spacing(np.abs(e))
    assert np.all(np.isfinite(r))
    assert ulp.max() <= 1.0, x[np.argmax(ulp)]
    # nearly always the correctly rounded value itself
    assert np.mean(r == e) > 0.99


def test_reciprocal_special_inputs_take_the_division(lib):
    tiny = np.finfo(np.float64).tiny
    x = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, tiny * 0.5, tiny, -tiny,
                  np.exp2(1021.0), np.exp2(1022.0), -np.exp2(1023.0), np.finfo(np.float64).max, 1.0, -1.0])
    r = _recip(lib, x)
    with np.errstate(all="ignore"):
        e = 1.0 / x
    same = (r == e) & (np.signbit(r) == np.signbit(e))
    assert np.all(same | (np.isnan(r) & np.isnan(e))), list(zip(x, r, e))
