"""The pivot helpers of the coarsest dense inverse on their own.

The U D U^T factorisation of each diagonal tile forms 1/d and 1/sqrt(d) of its pivots from a
single-precision seed refined by two Newton-Raphson steps (csrc/k_linalg.cu recip_newton,
rsqrt_newton); outside (1e-30, 1e30) they fall back to the plain quotient. The coarse-solve
parity tests cover them only through the whole inverse, so they are bounded here against the
correctly rounded FP64 results over pivots spanning the whole double range.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# two Newton steps from a 22-bit seed leave ~2^-85 of truncation error: what remains is the
# rounding of the last steps, a few units in the last place
ULP_BOUND = 4.0 * 2.0 ** -52


def _pivots():
    rng = np.random.default_rng(5)
    mant = rng.uniform(1.0, 10.0, 4000)
    expo = rng.integers(-300, 300, 4000)
    d = mant * 10.0 ** expo.astype(float)
    edges = [1e-30, 1e30, np.nextafter(1e-30, 1.0), np.nextafter(1e30, 0.0), np.nextafter(1e-30, 0.0),
             np.nextafter(1e30, np.inf), 1.0, 2.0, 3.0, 0.5, 1e-300, 1e300, 5e-324, 1.7976931348623157e308,
             np.finfo(np.float32).tiny, np.finfo(np.float32).max, 1e-38, 3.4e38]
    return np.concatenate([d, np.asarray(edges, dtype=float), rng.uniform(1e-3, 1e3, 2000)])


def test_pivot_reciprocals_bounded(gpu):
    from voxelfem_gb300 import _capi

    lib = _capi.load()
    d = _pivots()
    r = np.empty_like(d)
    s = np.empty_like(d)
    _capi.check(lib.vfem_debug_pivot_reciprocals(d.ctypes.data, d.size, r.ctypes.data, s.ctypes.data))
    want_r = 1.0 / d
    want_s = 1.0 / np.sqrt(d)
    fin = np.isfinite(want_r) & (want_r != 0)
    err_r = np.abs(r[fin] - want_r[fin]) / np.abs(want_r[fin])
    fin_s = np.isfinite(want_s) & (want_s != 0)
    err_s = np.abs(s[fin_s] - want_s[fin_s]) / np.abs(want_s[fin_s])
    assert err_r.max() <= ULP_BOUND, (err_r.max(), d[fin][np.argmax(err_r)])
    assert err_s.max() <= ULP_BOUND, (err_s.max(), d[fin_s][np.argmax(err_s)])
    # inside the Newton range the results are within one unit of the correctly rounded value
    inside = (d > 1e-30) & (d < 1e30)
    assert np.max(np.abs(r[inside] - want_r[inside]) / np.spacing(want_r[inside])) <= 2.0
    # the guard edges take the plain quotient: exact there
    outside = ~inside & fin
    np.testing.assert_array_equal(r[outside], want_r[outside])


def test_pivot_reciprocals_special_values(gpu):
    from voxelfem_gb300 import _capi

    lib = _capi.load()
    d = np.array([0.0, -0.0, np.inf, -1.0, np.nan])
    r = np.empty_like(d)
    s = np.empty_like(d)
    _capi.check(lib.vfem_debug_pivot_reciprocals(d.ctypes.data, d.size, r.ctypes.data, s.ctypes.data))
    with np.errstate(divide="ignore", invalid="ignore"):
        np.testing.assert_array_equal(r, 1.0 / d)
        np.testing.assert_array_equal(s, 1.0 / np.sqrt(d))
