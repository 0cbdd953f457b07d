"""Triquadratic voxels on the GPU against the oracle: K0 (1e-14), applyK FP64 (1e-12) and FP32
(1e-5), the 27-colour Gauss-Seidel sweep FP64 (1e-11) and FP32 (1e-5), restriction and
prolongation (1e-13)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def make(ne, seed=0, clamp=True):
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    g = pv.TensorProductSimulator([2, 2, 2], bbox, ne)
    g.ETensor = (1.0, 0.3)
    g.E_0, g.E_min, g.gamma = 1.0, 1e-9, 3.0
    rho = np.random.default_rng(seed).uniform(0.1, 1.0, int(np.prod(ne)))
    g.setDensities(rho)
    Y = 1e-9 + rho ** 3 * (1.0 - 1e-9)
    if clamp:
        g.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, float(ne[1]), float(ne[2])], "xyz")
        g.addDirichletCondition([0.0, 0.0, 0.0], [float(ne[0]), 0.0, 0.0], [float(ne[0]), 0.0, float(ne[2])], "y")
    m = g.getDirichletMask()
    bits = (m[:, 0] * 1 + m[:, 1] * 2 + m[:, 2] * 4).astype(np.uint8)
    return g, Y, bits


@pytest.mark.parametrize("ne", [(2, 2, 2), (3, 2, 5), (8, 4, 6)])
def test_q2_k0_and_apply_k(gpu, oracle, ne):
    g, Y, bits = make(ne)
    K0 = g.fullDensityElementStiffnessMatrix()
    assert rel(K0, po.q2_k0(1.0, 0.3)) < 1e-14
    u = np.random.default_rng(1).standard_normal((g.numNodes(), 3))
    ref = po.q2_apply_k(ne, K0, Y, u)
    assert rel(g.applyK(u), ref) < 1e-12
    assert rel(g.applyK(u, precision="df"), ref) < 1e-12
    assert rel(g.applyK(u, precision="fp32"), ref) < 1e-5
    z = g.applyK(u, zeroDirichlet=True)
    ref[g.getDirichletMask()] = 0
    assert rel(z, ref) < 1e-12


@pytest.mark.parametrize("ne", [(2, 2, 2), (3, 2, 5), (8, 4, 6)])
def test_q2_gauss_seidel(gpu, oracle, ne):
    g, Y, bits = make(ne, seed=2)
    K0 = g.fullDensityElementStiffnessMatrix()
    rng = np.random.default_rng(3)
    u = rng.standard_normal((g.numNodes(), 3))
    b = rng.standard_normal((g.numNodes(), 3))
    for fwd in (True, False):
        ref = po.q2_smooth(ne, K0, Y, bits, u, b, fwd)
        assert rel(g.smoothingMulticoloredGS(u, b, fwd), ref) < 1e-11, fwd
        assert rel(g.smoothingMulticoloredGS(u, b, fwd, precision="fp32"), ref) < 1e-4, fwd


def test_q2_transfers(gpu, oracle):
    ne = (4, 2, 6)
    nec = [v // 2 for v in ne]
    rng = np.random.default_rng(4)
    f = rng.standard_normal((po.q2_num_nodes(ne), 3))
    c = rng.standard_normal((po.q2_num_nodes(nec), 3))
    assert rel(pv.q2_restriction(ne, f), po.q2_restrict(ne, f)) < 1e-13
    assert rel(pv.q2_interpolation(ne, c), po.q2_interp(ne, c)) < 1e-13
    assert rel(pv.q2_interpolation(ne, c, f, accumulate=True), po.q2_interp(ne, c, f, True)) < 1e-13


def test_q2_factory(gpu):
    g = pv.TensorProductSimulator([2, 2, 2], [[0, 0, 0], [2, 2, 2]], [2, 2, 2])
    assert g.numNodes() == 125 and g.numElements() == 8
    with pytest.raises(RuntimeError):
        g.multigridSolver(0)


@pytest.mark.parametrize("coarsenings,matvec,hierarchy", [(1, "df", "q2"), (2, "df", "q2"), (2, "fp64", "q2"),
                                                          (1, "df", "p"), (2, "df", "p"), (2, "fp64", "p")])
def test_q2_pcg_matches_dense_solve(gpu, oracle, coarsenings, matvec, hierarchy):
    """The PCG solution equals a dense direct solve of the oracle's Q2 operator on the free DOFs,
    with either preconditioner hierarchy."""
    ne = (8, 4, 4)
    g, Y, bits = make(ne, seed=5)
    K0 = g.fullDensityElementStiffnessMatrix()
    nn = g.numNodes()
    f = np.zeros((nn, 3))
    nnd = [2 * v + 1 for v in ne]
    tip = [(nnd[0] - 1) * nnd[1] * nnd[2] + j * nnd[2] + nnd[2] // 2 for j in range(nnd[1])]
    f[tip, 1] = -1.0 / len(tip)
    # dense oracle operator
    Kd = np.zeros((3 * nn, 3 * nn))
    for t in range(3 * nn):
        e = np.zeros(3 * nn)
        e[t] = 1.0
        Kd[:, t] = po.q2_apply_k(ne, K0, Y, e.reshape(3, nn).T).T.ravel()
    fixed = np.array([(bits[n] >> c) & 1 for c in range(3) for n in range(nn)], dtype=bool)
    bvec = f.T.ravel().copy()
    bvec[fixed] = 0
    xs = np.zeros(3 * nn)
    xs[~fixed] = np.linalg.solve(Kd[np.ix_(~fixed, ~fixed)], bvec[~fixed])
    xref = xs.reshape(3, nn).T
    mg = g.multigridSolver(coarsenings)
    mg.setHierarchy(hierarchy)
    mg.setOuterMatvec(matvec)
    x = mg.preconditionedConjugateGradient(np.zeros((nn, 3)), f, 200, 1e-11, None, 1, 2, False)
    assert mg.lastStats.relres <= 1e-11
    assert rel(x, xref) < 1e-8
    assert mg.lastStats.iterations < 60
    c, cref = np.sum(f * x), np.sum(f * xref)
    assert abs(c - cref) / abs(cref) < 1e-9


@pytest.mark.parametrize("ne", [(2, 2, 2), (3, 2, 5), (8, 4, 6), (16, 8, 12)])
def test_q2_fp32_line_sweep_matches_colour_launches(gpu, monkeypatch, ne):
    """The FP32 sweep's line form (one launch per (a, b) class, its three colours on whole
    z-lines) gives the same iterate, bit for bit, as 27 colour launches."""
    g, Y, bits = make(ne, seed=6)
    rng = np.random.default_rng(7)
    u = rng.standard_normal((g.numNodes(), 3))
    b = rng.standard_normal((g.numNodes(), 3))
    for fwd in (True, False):
        monkeypatch.setenv("VFEM_Q2_GS_FORM", "colours")
        ref = g.smoothingMulticoloredGS(u, b, fwd, precision="fp32")
        monkeypatch.setenv("VFEM_Q2_GS_FORM", "lines")
        np.testing.assert_array_equal(g.smoothingMulticoloredGS(u, b, fwd, precision="fp32"), ref)
