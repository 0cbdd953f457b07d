"""CPU checks of the 2D restatement (oracle/oracle2d.py) against first principles: the element
matrix against exact symbolic integration of the plane-stress energy, rigid-body modes, the
Galerkin identity of the coarse operators, restriction = interpolation transpose, multigrid-
preconditioned CG convergence, the smoothing filter's normalisation and the adjoint gradient
against finite differences."""
import numpy as np
import pytest

from oracle import oracle2d as o2


def test_k0_symbolic():
    sympy = pytest.importorskip("sympy")
    x, y = sympy.symbols("x y")
    E, nu, hx, hy = sympy.Rational(1), sympy.Rational(3, 10), sympy.Rational(2), sympy.Rational(1, 2)
    lam = E * nu / ((1 + nu) * (1 - nu))
    mu = E / (2 * (1 + nu))
    N = [(1 - x / hx) * (1 - y / hy), (1 - x / hx) * (y / hy), (x / hx) * (1 - y / hy), (x / hx) * (y / hy)]
    grads = [(sympy.diff(n, x), sympy.diff(n, y)) for n in N]
    K = sympy.zeros(8, 8)
    for a in range(4):
        for c in range(2):
            for b in range(4):
                for d in range(2):
                    ga, gb = grads[a], grads[b]
                    dot = ga[0] * gb[0] + ga[1] * gb[1]
                    integrand = lam * ga[c] * gb[d] + mu * ((dot if c == d else 0) + ga[d] * gb[c])
                    K[2 * a + c, 2 * b + d] = sympy.integrate(sympy.integrate(integrand, (x, 0, hx)), (y, 0, hy))
    ref = np.array(K.evalf(20), dtype=float)
    got = o2.k0_2d(1.0, 0.3, (2.0, 0.5))
    assert np.max(np.abs(got - ref)) < 1e-14 * np.max(np.abs(ref))


def test_k0_rigid_modes():
    K = o2.k0_2d(2.0, 0.25, (1.0, 1.0))
    assert np.allclose(K, K.T, atol=0)
    X = np.array([[0, 0], [0, 1], [1, 0], [1, 1]], dtype=float)
    tx = np.tile([1.0, 0.0], 4)
    ty = np.tile([0.0, 1.0], 4)
    rot = np.stack([-X[:, 1], X[:, 0]], axis=1).ravel()
    for m in (tx, ty, rot):
        assert np.max(np.abs(K @ m)) < 1e-14
    assert np.linalg.matrix_rank(K, tol=1e-10) == 5


def cantilever(ne=(16, 8), seed=0):
    rng = np.random.default_rng(seed)
    s = o2.Sim2(ne, (0, 0), (2, 1))
    s.setMaterial(1.0, 0.3)
    s.setDensities(rng.uniform(0.2, 1.0, s.NE))
    s.addDirichletCondition([0, 0], [-1e-9, -1e-9], [1e-9, 1 + 1e-9])
    f = np.zeros(2 * s.NN)
    f[s.NN + s.node(ne[0], 0)] = -1.0
    s.force = f
    return s, rng


def test_galerkin_and_transfer_transpose():
    s, rng = cantilever()
    mg = o2.MG2(s, 2)
    for l in range(2):
        c = mg.sims[l + 1]
        v, w = rng.standard_normal(2 * c.NN), rng.standard_normal(2 * c.NN)
        Pv = mg.interpolate(l, v, None, False)
        Pw = mg.interpolate(l, w, None, False)
        lhs = Pw @ mg.applyK(l, Pv)
        assert abs(lhs - w @ mg.applyK(l + 1, v)) < 1e-12 * abs(lhs)
        fv = rng.standard_normal(2 * mg.sims[l].NN)
        assert abs(mg.restrict(l, fv) @ v - fv @ Pv) < 1e-12 * np.abs(fv).sum()


def test_pcg_converges():
    s, _ = cantilever((32, 16))
    mg = o2.MG2(s, 2)
    f = s.buildLoadVector()
    u = mg.pcg(np.zeros(2 * s.NN), f, 100, 1e-10, 1, 1, False)
    r = f - s.applyK(u)
    o2.MG2.zeroDirichlet(s, r)
    assert np.linalg.norm(r) < 1e-9 * np.linalg.norm(f)
    assert mg.lastIterations < 40


def test_smoothing_filter_normalised():
    x = np.full(7 * 5, 0.37)
    for r, t in ((1, 0), (2, 1), (4, 1)):
        assert np.allclose(o2.smoothing_filter_2d(x, (7, 5), r, t), 0.37, atol=1e-15)


def test_compliance_gradient_fd():
    s, rng = cantilever((8, 4), seed=2)
    s.grav = np.array([0.0, -0.5])
    mg = o2.MG2(s, 1)

    def compliance(rho):
        s.setDensities(rho)
        mg.valid = False
        f = s.buildLoadVector()
        u = mg.pcg(np.zeros(2 * s.NN), f, 200, 1e-13, 1, 2, False)
        return 0.5 * f @ u, u

    rho = s.rho.copy()
    c0, u = compliance(rho)
    g = s.complianceGradient(u)
    for e in (0, 7, 19):
        d = np.zeros_like(rho)
        d[e] = 1e-6
        fd = (compliance(rho + d)[0] - compliance(rho - d)[0]) / 2e-6
        assert abs(fd - g[e]) < 1e-6 * max(abs(g[e]), 1e-3)


def test_langelaar_2d_gradient_fd():
    from oracle import filters as of
    rng = np.random.default_rng(3)
    shape = (6, 5)
    x = rng.uniform(0.2, 0.9, shape)
    g = rng.standard_normal(shape)
    L = of.Langelaar(shape, ndim=2)
    L.apply(x)
    grad = L.backprop(g, x)[:, :, 0]

    def J(xx):
        return float(np.sum(g * of.Langelaar(shape, ndim=2).apply(xx)[:, :, 0]))

    for idx in [(0, 0), (3, 2), (5, 4), (2, 1)]:
        d = np.zeros(shape)
        d[idx] = 1e-6
        fd = (J(x + d) - J(x - d)) / 2e-6
        assert abs(fd - grad[idx]) < 1e-6 * max(1.0, abs(grad[idx]))
