"""Argument errors at the C ABI, checked without a GPU: each entry point validates its
arguments before touching the device, returns the status code and leaves the reference's
error text in vfem_last_error()."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from voxelfem_gb300 import _capi
    return _capi.load()  # loading needs no GPU


def _i64(v):
    return (C.c_int64 * len(v))(*v)


def _d(v):
    return (C.c_double * len(v))(*v)


def test_version(lib):
    assert lib.vfem_version() == 1


def test_grid_create_rejects_empty_axis(lib):
    out = C.c_void_p()
    rc = lib.vfem_grid_create(_i64([0, 4, 4]), _d([0, 0, 0]), _d([1, 1, 1]), C.byref(out))
    assert rc == 1
    assert lib.vfem_last_error() == b"invalid elementsPerDimension"
    assert out.value is None


def test_null_arguments(lib):
    assert lib.vfem_grid_create(_i64([4, 4, 4]), _d([0, 0, 0]), _d([1, 1, 1]), None) == 1
    assert lib.vfem_last_error() == b"null out"
    n = C.c_int64()
    assert lib.vfem_grid_dims(None, _i64([0, 0, 0]), C.byref(n), C.byref(n)) == 1
    assert lib.vfem_last_error() == b"null grid"


def test_upsample_rejects_thin_grid_with_reference_text(lib):
    # TopologyOptimizationFilter.hh:442
    a = np.zeros(16)
    b = np.zeros(64)
    rc = lib.vfem_upsample_filter(_i64([1, 4, 4]), 2, a.ctypes.data, b.ctypes.data)
    assert rc == 1
    assert lib.vfem_last_error() == b"Interpolation can only be applied to a 2^d grid or larger"
