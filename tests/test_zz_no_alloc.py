"""The allocation-free density filter (vfem_smoothing_filter_noalloc) against the
allocating entry point (vfem_smoothing_filter), through the C ABI.

Callers that cannot allocate device memory (code capturing the filter into its own
CUDA graph, code under a fixed memory budget) use the allocation-free variant; it
must give the same densities. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_filter_matches_allocating_filter(gpu):
    import torch

    from voxelfem_gb300 import _capi

    lib = _capi.load()
    dims = (23, 17, 11)
    dims_c = (C.c_int64 * 3)(*dims)
    n = int(np.prod(dims))
    rng = np.random.default_rng(12)
    stream = torch.cuda.current_stream()
    # two calls in a row per configuration, each against the allocating entry point
    for radius, ftype in [(2, 1), (2, 1), (1, 0), (6, 1)]:
        x = torch.from_numpy(rng.uniform(0.0, 1.0, n)).cuda()
        ref = torch.empty_like(x)
        out = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        _capi.check(lib.vfem_smoothing_filter(dims_c, radius, ftype, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(ref.data_ptr())))
        _capi.check(lib.vfem_smoothing_filter_noalloc(dims_c, radius, ftype, C.c_void_p(x.data_ptr()),
                                                      C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream)))
        torch.cuda.synchronize()
        err = float((out - ref).abs().max() / ref.abs().max())
        assert err < 1e-14, (radius, ftype, err)


def test_noalloc_filter_rejects_what_it_cannot_serve(gpu):
    import torch

    from voxelfem_gb300 import _capi

    lib = _capi.load()
    dims = (4, 4, 4)
    dims_c = (C.c_int64 * 3)(*dims)
    x = torch.zeros(64, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    rc = lib.vfem_smoothing_filter_noalloc(dims_c, 7, 1, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None)
    assert rc == 1 and b"exceeds the maximum" in lib.vfem_last_error()
    host = np.zeros(64)
    rc = lib.vfem_smoothing_filter_noalloc(dims_c, 1, 1, C.c_void_p(host.ctypes.data), C.c_void_p(y.data_ptr()), None)
    assert rc == 1 and b"device pointers" in lib.vfem_last_error()
