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


# ---- the triquadratic multigrid hierarchy (MultigridSolver<double, 2, 2, 2>) ----
def _q2_problem(ne, seed=0):
    K0 = po.q2_k0(1.0, 0.3)
    rng = np.random.default_rng(seed)
    Y = 1e-9 + rng.uniform(0.1, 1.0, int(np.prod(ne))) ** 3 * (1.0 - 1e-9)
    nn = [2 * v + 1 for v in ne]
    I, J, _ = np.meshgrid(*[np.arange(n) for n in nn], indexing="ij")
    bits = np.zeros(I.size, dtype=np.uint8)
    bits[(I == 0).ravel()] = 7                                # x = 0 face clamped
    bits[((I == nn[0] - 1) & (J == 0)).ravel()] |= 2          # roller line at x = max, y = 0
    return K0, Y, bits


def _assemble(ne, Kes):
    nn = [2 * v + 1 for v in ne]
    N = int(np.prod(nn))
    A = np.zeros((3 * N, 3 * N))
    e = 0
    for i in range(ne[0]):
        for j in range(ne[1]):
            for k in range(ne[2]):
                nodes = [((2 * i + l // 9) * nn[1] + 2 * j + (l // 3) % 3) * nn[2] + 2 * k + l % 3 for l in range(27)]
                # SoA DOF c * N + n against the element's node-major 3 l + c
                dofs = np.array([c * N + nodes[l] for l in range(27) for c in range(3)])
                A[np.ix_(dofs, dofs)] += Kes[e]
                e += 1
    return A


def _prolongation(ne_fine):
    nc = po.q2_num_nodes([v // 2 for v in ne_fine])
    cols = []
    for t in range(3 * nc):
        c = np.zeros(3 * nc)
        c[t] = 1.0
        cols.append(np.asfortranarray(po.q2_interp(ne_fine, c.reshape(3, nc).T)).T.ravel())
    return np.array(cols).T


def test_q2mg_galerkin_operators():
    ne = (4, 4, 4)
    K0, Y, bits = _q2_problem(ne)
    mg = po.Q2Multigrid(ne, K0, Y, bits, 2)
    Kprev = _assemble(ne, [Y[e] * K0 for e in range(Y.size)])
    Kc = mg.coarsened_k0()
    assert np.abs(Kc - np.transpose(Kc, (0, 2, 1))).max() < 1e-14 * np.abs(Kc).max()
    for l in (1, 2):
        nef = mg.level_ne(l - 1)
        P = _prolongation(nef)
        Kl = _assemble(mg.level_ne(l), mg.element_matrices(l))
        ref = P.T @ Kprev @ P
        assert np.abs(Kl - ref).max() < 1e-12 * np.abs(ref).max(), l
        Kprev = Kl


def test_q2mg_dirichlet_coarsening():
    ne = (8, 4, 4)
    K0, Y, bits = _q2_problem(ne)
    mg = po.Q2Multigrid(ne, K0, Y, bits, 2)
    for l in (1, 2):
        ncl = [2 * v + 1 for v in mg.level_ne(l)]
        I, J, _ = np.meshgrid(*[np.arange(n) for n in ncl], indexing="ij")
        expect = np.zeros(I.size, dtype=np.uint8)
        expect[(I == 0).ravel()] = 7
        expect[((I == ncl[0] - 1) & (J == 0)).ravel()] |= 2
        np.testing.assert_array_equal(mg.dirichlet_bits(l), expect)


def test_q2mg_pcg_matches_dense_solve_and_symmetric_vcycle():
    ne = (4, 4, 4)
    K0, Y, bits = _q2_problem(ne, seed=3)
    mg = po.Q2Multigrid(ne, K0, Y, bits, 2)
    nn = po.q2_num_nodes(ne)
    rng = np.random.default_rng(4)
    b = rng.standard_normal((nn, 3))
    m = np.stack([(bits >> c) & 1 for c in range(3)], axis=1).astype(bool)
    b[m] = 0.0
    x, it, rr = mg.pcg(b, 200, 1e-10, 2)
    assert rr <= 1e-10 and 0 < it < 60
    A = _assemble(ne, [Y[e] * K0 for e in range(Y.size)])
    free = ~m.T.ravel()
    ref = np.zeros(3 * nn)
    ref[free] = np.linalg.solve(A[np.ix_(free, free)], b.T.ravel()[free])
    assert np.abs(x.T.ravel() - ref).max() < 1e-8 * np.abs(ref).max()
    u, v = rng.standard_normal((2, nn, 3))
    u[m] = 0.0
    v[m] = 0.0
    Mu, Mv = mg.vcycle(u, 2), mg.vcycle(v, 2)
    assert abs(np.sum(v * Mu) - np.sum(u * Mv)) < 1e-10 * abs(np.sum(v * Mu))
