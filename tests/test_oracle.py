"""Checks of the CPU oracle itself (no GPU): it is pinned against independent
derivations and known-answer properties, because the reference ships no tests
or golden vectors and cannot be compiled here (parity unpinned)."""
import json
import os

import numpy as np
import pytest

from voxelfem_gb300 import workloads as wl

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def small_sim(oracle, ne=(8, 4, 4), rho_lo=0.3, seed=0):
    s = oracle.Sim(ne)
    wl.setup_cantilever(s, ne, rho_lo, seed)
    return s


def test_k0_matches_exact_symbolic_integration(oracle):
    with open(os.path.join(GOLDEN, "k0_exact_nu0.3.json")) as f:
        K_exact = np.array(json.load(f)["K0"])
    s = oracle.Sim((2, 2, 2))
    s.setMaterial(1.0, 0.3)
    assert rel(s.K0(), K_exact) < 1e-14


def test_k0_properties(oracle):
    s = oracle.Sim((2, 2, 2), bbox=[[0, 0, 0], [2.0, 3.0, 1.0]])  # stretched voxels
    s.setMaterial(2.5, 0.3)
    K = s.K0()
    assert np.abs(K - K.T).max() == 0.0
    ev = np.linalg.eigvalsh(K)
    assert np.all(ev > -1e-13 * ev.max())
    assert np.sum(ev < 1e-12 * ev.max()) == 6  # rigid-body modes
    # rigid translations and an infinitesimal rotation are in the null space
    pos = np.array([[(l >> 2) & 1, (l >> 1) & 1, l & 1] for l in range(8)], float) * [1.0, 1.5, 0.5]
    for c in range(3):
        t = np.zeros(24)
        t[c::3] = 1.0
        assert np.abs(K @ t).max() < 1e-13
    rot = np.zeros((8, 3))
    rot[:, 0], rot[:, 1] = -pos[:, 1], pos[:, 0]
    assert np.abs(K @ rot.ravel()).max() < 1e-12


def test_gauss_two_point_is_exact(oracle):
    """Three-point Gauss (numpy restatement) equals the oracle's two-point K0."""
    s = oracle.Sim((1, 1, 1))
    s.setMaterial(1.0, 0.3)
    nu, E = 0.3, 1.0
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    pts = [0.5 - np.sqrt(0.15), 0.5, 0.5 + np.sqrt(0.15)]
    wts = [5 / 18, 8 / 18, 5 / 18]
    K = np.zeros((24, 24))
    for a, xa in enumerate(pts):
        for b, xb in enumerate(pts):
            for c, xc in enumerate(pts):
                x = (xa, xb, xc)
                G = np.zeros((8, 3))
                for l in range(8):
                    bits = [(l >> 2) & 1, (l >> 1) & 1, l & 1]
                    for d in range(3):
                        v = 1.0
                        for e in range(3):
                            v *= (1 if bits[e] else -1) if e == d else (x[e] if bits[e] else 1 - x[e])
                        G[l, d] = v
                B = np.zeros((6, 24))
                for l in range(8):
                    B[0, 3 * l], B[1, 3 * l + 1], B[2, 3 * l + 2] = G[l]
                    B[3, 3 * l + 1], B[3, 3 * l + 2] = G[l, 2], G[l, 1]
                    B[4, 3 * l], B[4, 3 * l + 2] = G[l, 2], G[l, 0]
                    B[5, 3 * l], B[5, 3 * l + 1] = G[l, 1], G[l, 0]
                D = np.zeros((6, 6))
                D[:3, :3] = lam
                D[np.arange(3), np.arange(3)] += 2 * mu
                D[3:, 3:] = np.eye(3) * mu
                K += wts[a] * wts[b] * wts[c] * B.T @ D @ B
    assert rel(s.K0(), K) < 1e-14


def test_applyk_linear_field_and_symmetry(oracle):
    s = small_sim(oracle, (6, 4, 5))
    nn = s.nn
    # rigid translation: K t = 0 for any densities
    t = np.zeros((nn, 3))
    t[:, 1] = 1.0
    assert np.abs(s.applyK(t)).max() < 1e-14
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal((nn, 3)), rng.standard_normal((nn, 3))
    assert abs(np.sum(u * s.applyK(v)) - np.sum(v * s.applyK(u))) < 1e-11 * np.abs(u).sum()


def explicit(op, n_in, n_out):
    M = np.zeros((n_out, n_in))
    for j in range(n_in):
        e = np.zeros(n_in)
        e[j] = 1.0
        M[:, j] = op(e.reshape(-1, 3, order="F")).ravel(order="F")
    return M


def test_galerkin_identity(oracle):
    """Coarse operators equal P^T K P with P the trilinear prolongation (MultigridSolver.hh:712-819)."""
    ne = (4, 4, 4)
    s = small_sim(oracle, ne)
    mg = oracle.MG(s, 2)
    mg.updateStiffnessMatrices()
    n0, n1, n2 = (mg.levelNodes(l) for l in range(3))
    K0 = explicit(lambda u: mg.applyK(0, u), 3 * n0, 3 * n0)
    P0 = explicit(lambda c: mg.interpolate(0, c, None, accumulate=False), 3 * n1, 3 * n0)
    K1 = explicit(lambda u: mg.applyK(1, u), 3 * n1, 3 * n1)
    assert rel(K1, P0.T @ K0 @ P0) < 1e-12
    P1 = explicit(lambda c: mg.interpolate(1, c, None, accumulate=False), 3 * n2, 3 * n1)
    K2 = explicit(lambda u: mg.applyK(2, u), 3 * n2, 3 * n2)
    assert rel(K2, P1.T @ K1 @ P1) < 1e-12
    # restriction is the transpose of prolongation
    R0 = explicit(lambda f: mg.restrict(0, f), 3 * n0, 3 * n1)
    assert rel(R0, P0.T) < 1e-15


def test_color_disjointness():
    """No two nodes of one colour (x%2, y%2, z%2) share an element."""
    nn = (5, 4, 6)
    for col in range(8):
        o = [(col >> 2) & 1, (col >> 1) & 1, col & 1]
        nodes = [(i, j, k) for i in range(o[0], nn[0], 2) for j in range(o[1], nn[1], 2) for k in range(o[2], nn[2], 2)]
        seen = set()
        for (i, j, k) in nodes:
            for a in range(2):
                for b in range(2):
                    for c in range(2):
                        e = (i - a, j - b, k - c)
                        if min(e) < 0 or e[0] >= nn[0] - 1 or e[1] >= nn[1] - 1 or e[2] >= nn[2] - 1:
                            continue
                        assert e not in seen
                        seen.add(e)


def test_vcycle_preconditioner_is_symmetric(oracle):
    s = small_sim(oracle, (8, 4, 4))
    mg = oracle.MG(s, 2)
    nn = s.nn
    rng = np.random.default_rng(3)
    dm = s.dirichletMask()
    b1, b2 = rng.standard_normal((nn, 3)), rng.standard_normal((nn, 3))
    for b in (b1, b2):
        for c in range(3):
            b[(dm >> c) & 1 == 1, c] = 0
    z = np.zeros((nn, 3))
    m1 = mg.solve(z, b1, 1, 2, zeroDirichlet=True)
    m2 = mg.solve(z, b2, 1, 2, zeroDirichlet=True)
    assert abs(np.sum(b1 * m2) - np.sum(b2 * m1)) < 1e-10 * abs(np.sum(b1 * m1))


def test_pcg_true_residual_and_compliance(oracle):
    s = small_sim(oracle, (16, 8, 8))
    mg = oracle.MG(s, 3)
    b = s.buildLoadVector()
    x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-10, None, 1, 2, False)
    r = b - s.applyK(x)
    dm = s.dirichletMask()
    for c in range(3):
        r[(dm >> c) & 1 == 1, c] = 0
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.5e-10
    # compliance 1/2 f.u = 1/2 u.K u at equilibrium
    assert abs(0.5 * np.sum(b * x) - 0.5 * np.sum(x * s.applyK(x))) < 1e-8 * abs(np.sum(b * x))


def test_compliance_gradient_central_differences(oracle):
    ne = (6, 4, 4)
    s = small_sim(oracle, ne)
    mg = oracle.MG(s, 1)
    rho = wl.densities(ne, 0.3, 0)
    b = s.buildLoadVector()

    def compliance(r):
        s.setDensities(r)
        x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 400, 1e-13, None, 1, 2, False)
        return 0.5 * np.sum(b * x), x

    c0, x0 = compliance(rho)
    g = s.complianceGradient(x0)
    h = 1e-6
    for e in np.random.default_rng(5).choice(rho.size, 12, replace=False):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        fd = (compliance(rp)[0] - compliance(rm)[0]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-5 * abs(g[e]) + 1e-12


@pytest.mark.parametrize("radius,ftype,count", [(1, 0, 27), (2, 1, 93), (1, 1, 27)])
def test_smoothing_filter_weights_and_adjointness(oracle, radius, ftype, count):
    offs = [(a, b, c) for a in range(-radius, radius + 1) for b in range(-radius, radius + 1)
            for c in range(-radius, radius + 1)]
    w = [(radius + 1.0 - np.sqrt(a * a + b * b + c * c)) if ftype == 1 else 1.0 for a, b, c in offs]
    w = [v for v in w if v > 0]
    assert len(w) == count
    if (radius, ftype) == (2, 1):
        assert abs(sum(w) - 83.77852) < 1e-5
    dims = (7, 5, 4)
    rng = np.random.default_rng(2)
    x, y = rng.standard_normal(int(np.prod(dims))), rng.standard_normal(int(np.prod(dims)))
    Sx = oracle.smoothing_filter(x, dims, radius, ftype)
    Sy = oracle.smoothing_filter(y, dims, radius, ftype)
    assert abs(np.dot(y, Sx) - np.dot(x, Sy)) < 1e-12 * np.abs(x).sum()
    const = oracle.smoothing_filter(np.full(x.size, 0.7), dims, radius, ftype)
    assert np.abs(const - 0.7).max() < 1e-15


def test_projection_derivative(oracle):
    x = np.linspace(0.01, 0.99, 50)
    beta = 4.0
    h = 1e-6
    fd = (oracle.projection_apply(x + h, beta) - oracle.projection_apply(x - h, beta)) / (2 * h)
    g = oracle.projection_backprop(np.ones_like(x), x, beta)
    assert np.abs(fd - g).max() < 1e-7
    y = oracle.projection_apply(np.array([0.0, 0.5, 1.0]), beta)
    assert abs(y[0]) < 1e-15 and abs(y[1] - 0.5) < 1e-15 and abs(y[2] - 1.0) < 1e-15


def test_oc_step_meets_volume_constraint(oracle):
    ne = (8, 4, 4)
    s = oracle.Sim(ne)
    wl.setup_mbb(s, ne)
    mg = oracle.MG(s, 1)
    top = oracle.TOP(mg, [("smoothing", 1, 1), ("projection", 1.0)], 0.3)
    top.setSolver(cgIter=200, tol=1e-10)
    top.setVars(np.full(s.numElements, 0.3))
    for _ in range(3):
        top.ocStep()
        assert abs(top.evaluateConstraints()[0]) <= 1e-6
    assert np.all(top.designVars() >= 0) and np.all(top.designVars() <= 1)


def test_oracle_matches_committed_fixture(oracle):
    """Regression anchor: the oracle reproduces its committed outputs on the small cantilever."""
    d = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    ne = (8, 4, 4)
    s = small_sim(oracle, ne)
    mg = oracle.MG(s, 2)
    assert rel(s.applyK(d["u"]), d["Ku"]) < 1e-13
    mg.updateStiffnessMatrices()
    for l in range(mg.numLevels - 1):
        assert rel(mg.smooth(l, d["smooth_u%d" % l], d["smooth_b%d" % l], True), d["smooth_out%d" % l]) < 1e-12
    b = s.buildLoadVector()
    assert rel(b, d["b"]) == 0
    x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-10, None, 1, 2, False)
    assert mg.lastIterations == int(d["iterations"])
    assert rel(x, d["x"]) < 1e-10


def test_masked_layers_semantics(oracle):
    ne = (4, 6, 4)
    s = small_sim(oracle, ne)
    s.setFabricationMaskHeightByLayer(3)
    Y = s.youngModuli().reshape(ne)
    assert np.all(Y[:, 3:, :] == 0) and np.all(Y[:, :3, :] > 0)
    u = np.random.default_rng(1).standard_normal((s.nn, 3))
    Ku = s.applyK(u).reshape(ne[0] + 1, ne[1] + 1, ne[2] + 1, 3, order="F")
    # nodes above the first detached layer (y >= 4) are not visited and read back as zero
    assert np.all(Ku[:, 4:, :, :] == 0)


def test_oracle_layer_by_layer_warm_starts():
    """The oracle's sequential layer-by-layer restatement: warm-started heights converge to the
    zero-guess compliances with fewer iterations; N=1 equals the scaled previous solution."""
    from oracle import pyoracle as po
    ne = (8, 8, 4)
    rho = np.random.default_rng(3).uniform(0.3, 1.0, int(np.prod(ne)))

    def make():
        s = po.Sim(ne)
        s.setMaterial(1.0, 0.3)
        s.setParams(E0=1.0, Emin=1e-9, gamma=3.0)
        s.setGravity([0.0, -1.0, 0.0])
        s.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [float(ne[0]), 0.0, float(ne[2])], "xyz")
        s.setDensities(rho)
        return s, po.MG(s, 2)

    res = {}
    for method in ("zero", "N=3", "fd"):
        s, m = make()
        res[method] = po.layer_by_layer(s, m, method, True, 2, 500, 1e-10, 1, 2, False)
    lz, cz, iz, gz, _ = res["zero"]
    for method in ("N=3", "fd"):
        l, c, i, g, _ = res[method]
        np.testing.assert_array_equal(l, lz)
        assert np.max(np.abs(c - cz) / np.abs(cz)) < 1e-8
        assert np.max(np.abs(g - gz)) / np.max(np.abs(gz)) < 1e-6
    assert res["N=3"][2].sum() < iz.sum()


def test_oracle_mma_reaches_analytic_optimum():
    """The numpy restatement of the reference's MMA (and GCMMA) solves a box-constrained quadratic
    with a volume constraint to its analytic optimum."""
    from oracle import mma as omma
    n = 300
    t = np.random.default_rng(0).uniform(0.1, 0.9, n)
    f = lambda x: np.array([np.sum((x - t) ** 2), np.mean(x) / 0.4 - 1.0])
    df = lambda x: np.vstack([2 * (x - t), np.full(n, 1.0 / (0.4 * n))])
    lo, hi = 0.0, 10.0
    for _ in range(200):
        lam = 0.5 * (lo + hi)
        lo, hi = (lam, hi) if np.clip(t - lam, 0, 1).mean() > 0.4 else (lo, lam)
    fs = f(np.clip(t - lam, 0, 1))[0]
    for gc in (False, True):
        o = omma.MMA(n, 1, np.zeros(n), np.ones(n), f, df)
        o.enableGCMMA(gc)
        o.setInitialVar(np.full(n, 0.5))
        for _ in range(15):
            o.step()
        x = o.getOptimalVar()
        assert abs(f(x)[0] - fs) < 1e-5 * fs and f(x)[1] < 1e-6


def test_oracle_filters_adjoint():
    """The oracle's upsample and vertex-to-cell restatements are adjoint to their backprops;
    upsampling reproduces trilinear fields exactly."""
    from oracle import filters as of
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 1, (3, 4, 3))
    for F in (1, 2, 3):
        y = of.upsample(x, F)
        g = rng.standard_normal(y.shape)
        assert abs(np.sum(y * g) - np.sum(x * of.upsample_backprop(g, x.shape, F))) < 1e-12
    i, j, k = np.meshgrid(np.arange(3), np.arange(4), np.arange(3), indexing="ij")
    lin = 0.3 * i - 0.2 * j + 0.7 * k + 0.1 * i * j * k
    fi, fj, fk = np.meshgrid(np.arange(5) / 2, np.arange(7) / 2, np.arange(5) / 2, indexing="ij")
    assert np.max(np.abs(of.upsample(lin, 2) - (0.3 * fi - 0.2 * fj + 0.7 * fk + 0.1 * fi * fj * fk))) < 1e-14
    v = rng.uniform(0, 1, (4, 5, 3))
    c = of.vertex_to_cell(v)
    g = rng.standard_normal(c.shape)
    assert abs(np.sum(c * g) - np.sum(v * of.vertex_to_cell_backprop(g))) < 1e-12
