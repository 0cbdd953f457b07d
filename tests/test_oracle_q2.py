"""Triquadratic oracle checks that need no GPU: the 81 x 81 element stiffness (symmetry, rigid
modes, quadrature exactness), the element-loop applyK (symmetry, linear fields), the Q2
transfers (restriction = prolongation^T, quadratic reproduction) and the smoother's fixed
point."""
import numpy as np
import pytest

from oracle import pyoracle as po


def test_q2_k0_structure():
    K = po.q2_k0(1.0, 0.3, (1.0, 0.5, 2.0))
    assert np.abs(K - K.T).max() < 1e-15 * np.abs(K).max()
    ev = np.linalg.eigvalsh(K)
    assert np.all(ev[:6] < 1e-12 * ev[-1]) and ev[6] > 1e-6 * ev[-1]  # exactly six rigid modes
    # 3 Gauss points per axis integrate the degree-4 integrand exactly
    K4 = po.q2_k0(1.0, 0.3, (1.0, 0.5, 2.0), npts=4)
    assert np.abs(K - K4).max() < 1e-14 * np.abs(K).max()
    # translations and infinitesimal rotations are in the kernel
    xs = np.array([[a * 0.5 * 1.0, b * 0.5 * 0.5, c * 0.5 * 2.0] for a in range(3) for b in range(3) for c in range(3)])
    for d in range(3):
        t = np.zeros((27, 3))
        t[:, d] = 1
        assert np.abs(K @ t.ravel()).max() < 1e-13
    rot = np.zeros((27, 3))
    rot[:, 0], rot[:, 1] = -xs[:, 1], xs[:, 0]
    assert np.abs(K @ rot.ravel()).max() < 1e-13


def _field(ne, f):
    nn = [2 * v + 1 for v in ne]
    I, J, K = np.meshgrid(*[np.arange(n) for n in nn], indexing="ij")
    x = np.stack([I.ravel() * 0.5, J.ravel() * 0.5, K.ravel() * 0.5], axis=1)
    return f(x)


def test_q2_apply_k_linear_fields_and_symmetry():
    ne = (3, 2, 4)
    K0 = po.q2_k0(1.0, 0.3)
    Y = np.ones(int(np.prod(ne)))
    # a linear displacement field produces no force at interior nodes
    lin = _field(ne, lambda x: np.stack([0.3 * x[:, 0] + 0.1 * x[:, 1], -0.2 * x[:, 2], 0.5 * x[:, 0]], axis=1))
    f = po.q2_apply_k(ne, K0, Y, lin)
    nn = [2 * v + 1 for v in ne]
    F = f
    I, J, Kk = np.meshgrid(*[np.arange(n) for n in nn], indexing="ij")
    interior = ((I > 0) & (I < nn[0] - 1) & (J > 0) & (J < nn[1] - 1) & (Kk > 0) & (Kk < nn[2] - 1)).ravel()
    assert np.abs(F[interior]).max() < 1e-12
    rng = np.random.default_rng(0)
    Y = rng.uniform(0.1, 1.0, int(np.prod(ne)))
    u, v = rng.standard_normal((2, po.q2_num_nodes(ne), 3))
    Ku, Kv = po.q2_apply_k(ne, K0, Y, u), po.q2_apply_k(ne, K0, Y, v)
    assert abs(np.sum(v * Ku) - np.sum(u * Kv)) < 1e-12 * np.abs(np.sum(v * Ku))


def test_q2_transfers():
    ne = (4, 2, 6)
    nec = [v // 2 for v in ne]
    rng = np.random.default_rng(1)
    f = rng.standard_normal((po.q2_num_nodes(ne), 3))
    c = rng.standard_normal((po.q2_num_nodes(nec), 3))
    assert abs(np.sum(po.q2_restrict(ne, f) * c) - np.sum(f * po.q2_interp(ne, c))) < 1e-12 * np.sqrt(np.sum(f * f))
    # quadratic fields on the coarse grid are reproduced exactly
    quad = lambda x: np.stack([x[:, 0] ** 2 - x[:, 1] * x[:, 2], x[:, 2] ** 2 + x[:, 0], x[:, 1] * x[:, 0]], axis=1)
    fine = po.q2_interp(ne, _field(nec, lambda x: quad(2 * x)))
    assert np.abs(fine - _field(ne, quad)).max() < 1e-12


def test_q2_smoother_fixed_point():
    ne = (2, 2, 2)
    K0 = po.q2_k0(1.0, 0.3)
    Y = np.random.default_rng(2).uniform(0.2, 1.0, 8)
    nn = po.q2_num_nodes(ne)
    dm = np.zeros(nn, dtype=np.uint8)
    dm[:25] = 7  # x = 0 face clamped
    dm[30] = 2   # one partially constrained node
    # dense K on the free DOFs, solve, and check one sweep leaves the solution unchanged
    Kd = np.zeros((3 * nn, 3 * nn))
    for t in range(3 * nn):
        e = np.zeros(3 * nn)
        e[t] = 1.0
        Kd[:, t] = po.q2_apply_k(ne, K0, Y, e.reshape(3, nn).T).T.ravel()
    fixed = np.array([(dm[n] >> c) & 1 for c in range(3) for n in range(nn)], dtype=bool)
    b = np.random.default_rng(3).standard_normal(3 * nn)
    b[fixed] = 0
    x = np.zeros(3 * nn)
    free = ~fixed
    x[free] = np.linalg.solve(Kd[np.ix_(free, free)], b[free])
    X = x.reshape(3, nn).T.copy(order="F")
    B = b.reshape(3, nn).T.copy(order="F")
    for fwd in (True, False):
        Xs = po.q2_smooth(ne, K0, Y, dm, X, B, fwd)
        assert np.abs(Xs - X).max() < 1e-10 * np.abs(X).max()
