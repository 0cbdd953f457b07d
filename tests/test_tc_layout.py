"""Host side of the tensor-core outer matvec, without a GPU: the integer form of K0 and its
bf16 B tiles (vfem_tc_fit_k0), the base-128 digit split of the fixed-point operand,
and the operand addressing of the MMA descriptors (a digit table read in place, the second
K chunk one node row after the first), checked by contracting one element tile on the CPU."""
import ctypes as C

import numpy as np
import pytest

from voxelfem_gb300 import _capi

TY, TZ, NPY, NPZ = 8, 16, 9, 17


def fit(K0):
    lib = _capi.load()
    sc, ok = C.c_double(), C.c_int()
    tiles = np.zeros(2048, dtype=np.uint16)
    K0 = np.ascontiguousarray(K0, dtype=np.float64)
    _capi.check(lib.vfem_tc_fit_k0(K0.ctypes.data_as(C.c_void_p), C.byref(sc), tiles.ctypes.data_as(C.c_void_p),
                                   C.byref(ok)))
    vals = (tiles.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    return bool(ok.value), sc.value, vals


def k0(nu, h=(1.0, 1.0, 1.0)):
    from oracle import pyoracle as po
    ne = (2, 2, 2)
    s = po.Sim(ne, [[0.0, 0.0, 0.0], [2 * h[0], 2 * h[1], 2 * h[2]]])
    s.setMaterial(1.0, nu)
    return np.array(s.K0()).reshape(24, 24)


def digits(F):
    """A signed top digit F >> 49 and seven unsigned 7-bit fields of the two's complement F."""
    return [F >> 49] + [(F >> (7 * (7 - i))) & 127 for i in range(1, 8)]


def test_integer_form_of_k0():
    K = k0(0.3)
    ok, c, tiles = fit(K)
    assert ok
    C_ = np.rint(K / c)
    assert np.max(np.abs(K - c * C_)) <= 1e-13 * np.max(np.abs(K))
    assert np.max(np.abs(C_).sum(1)) * 16383 < 2 ** 24  # FP32 accumulators stay exact
    assert not fit(k0(0.33))[0]                         # accumulator bound exceeded
    assert not fit(k0(0.3, (1.0, 1.5, 1.0)))[0]         # stretched voxels


def test_digit_split():
    rng = np.random.default_rng(0)
    for F in list(rng.integers(-2 ** 55, 2 ** 55, 2000)) + [2 ** 55, -2 ** 55, 0, 1, -1]:
        F = int(F)
        D = digits(F)
        assert -64 <= D[0] <= 64 and all(0 <= d <= 127 for d in D[1:])
        assert sum(d * 128 ** (7 - i) for i, d in enumerate(D)) == F
        P = [128 * D[2 * a] + D[2 * a + 1] for a in range(4)]
        assert -8192 <= P[0] <= 8319 and all(0 <= p <= 16383 for p in P[1:])
        assert sum(p * 2 ** (14 * (3 - a)) for a, p in enumerate(P)) == F


def test_descriptor_addressing_contracts_elements():
    """A (digit table rows through start + 144 g + 16 r + 16 s) times B (tiles through
    q 1024 + 512 s + 128 g + 16 r) equals C u_e for every element of a tile."""
    K = k0(0.3)
    ok, c, tiles = fit(K)
    C_ = np.rint(K / c)
    rng = np.random.default_rng(1)
    # one digit pair per node component: table rows (z-major, y fastest), 8 values per row
    planes = [rng.integers(-8192, 16384, (NPZ * NPY, 3)).astype(np.float64) for _ in range(2)]
    tabs = []
    for P in planes:
        t = np.zeros(NPZ * NPY * 8)
        hi = np.floor_divide(P + 64, 128)  # any split with P = 128 hi + lo works for this check
        lo = P - 128 * hi
        t.reshape(-1, 8)[:, 0:3] = 128 * hi
        t.reshape(-1, 8)[:, 3:6] = lo
        tabs.append(t)
    acc = np.zeros((128, 32))
    for q in range(4):
        dx, dz = q >> 1, q & 1
        A = np.zeros((128, 16))
        for i in range(128):
            g, r = i // 8, i % 8
            for k in range(16):
                s, v = k // 8, k % 8
                A[i, k] = tabs[dx][dz * NPY * 8 + g * NPY * 8 + r * 8 + s * 8 + v]
        B = np.zeros((16, 32))
        for n in range(32):
            for k in range(16):
                s, v = k // 8, k % 8
                B[k, n] = tiles[q * 512 + s * 256 + (n // 8) * 64 + (n % 8) * 8 + v]
        acc += A @ B
    for i in range(128):
        ey, ez = i % 8, i // 8
        ue = np.zeros(24)
        for l in range(8):
            ldx, ldy, ldz = l >> 2 & 1, l >> 1 & 1, l & 1
            ue[3 * l:3 * l + 3] = planes[ldx][(ez + ldz) * NPY + (ey + ldy)]
        np.testing.assert_array_equal(acc[i, :24], C_ @ ue)
        assert np.all(acc[i, 24:] == 0)
