"""The allocation-free density filter (vfem_smoothing_filter_noalloc) through the C ABI.

Some callers cannot allocate device memory: code under a fixed device-memory budget, a host
application that owns every device allocation, or an OC bisection loop that cannot afford the
device synchronisation of cudaMalloc. They use the allocation-free variant, whose tap table
lives in a fixed array inside the library. It must give the same densities as the allocating
entry point (vfem_smoothing_filter) and as the CPU oracle's filter, call after call, although
every call rebuilds the shared table. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the allocating path sums the tap weights sequentially, the allocation-free one in a fixed
# warp order: the two normalisations differ by a few units in the last place
TOL = 1e-14


def _run(lib, dims, radius, ftype, x, stream):
    import torch

    from voxelfem_gb300 import _capi

    dims_c = (C.c_int64 * 3)(*dims)
    ref = torch.empty_like(x)
    out = torch.full_like(x, float("nan"))
    torch.cuda.synchronize()
    _capi.check(lib.vfem_smoothing_filter(dims_c, radius, ftype, C.c_void_p(x.data_ptr()),
                                          C.c_void_p(ref.data_ptr())))
    _capi.check(lib.vfem_smoothing_filter_noalloc(dims_c, radius, ftype, C.c_void_p(x.data_ptr()),
                                                  C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    return out.cpu().numpy(), ref.cpu().numpy()


def test_noalloc_filter_matches_allocating_filter_and_oracle(gpu, oracle):
    import torch

    from voxelfem_gb300 import _capi

    lib = _capi.load()
    rng = np.random.default_rng(12)
    stream = torch.cuda.current_stream()
    # two calls in a row per configuration (the second reuses the table the first left),
    # radii that shrink and grow between calls, and a grid one voxel thick
    cases = [((23, 17, 11), 2, 1), ((23, 17, 11), 2, 1), ((23, 17, 11), 1, 0), ((23, 17, 11), 6, 1),
             ((23, 17, 11), 3, 1), ((9, 7, 1), 2, 1), ((9, 7, 1), 2, 1)]
    for dims, radius, ftype in cases:
        n = int(np.prod(dims))
        xh = rng.uniform(0.0, 1.0, n)
        x = torch.from_numpy(xh).cuda()
        out, ref = _run(lib, dims, radius, ftype, x, stream)
        want = oracle.smoothing_filter(xh, dims, radius, ftype)
        err_ref = float(np.max(np.abs(out - ref)) / np.max(np.abs(ref)))
        err_oracle = float(np.max(np.abs(out - want)) / np.max(np.abs(want)))
        assert err_ref < TOL, (dims, radius, ftype, err_ref)
        assert err_oracle < TOL, (dims, radius, ftype, err_oracle)


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
