"""The reference's triquadratic multigrid hierarchy (MultigridSolver<double, 2, 2, 2>) on the GPU
against the oracle's restatement: coarsened supports bit-exact, level element matrices (level 1
from the coarsened full-density matrices, Galerkin below: FP64 1e-13, FP32 1e-6), per-level
Gauss-Seidel sweeps and residuals, the coarsest direct solve, one V-cycle, and the FP64 PCG
(same iteration count as the oracle, u and compliance to 1e-8), with the mixed-precision solve's
compliance within 1e-8 of the FP64 GPU solve."""
import numpy as np
import pytest

from oracle import pyoracle as po
from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def cantilever(ne, seed=0):
    """x = 0 face clamped, roller line (y) at x = max, y = 0; rho ~ U[0.01, 1]; E_min 1e-9."""
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    g = pv.TensorProductSimulator([2, 2, 2], bbox, ne)
    g.ETensor = (1.0, 0.3)
    g.E_0, g.E_min, g.gamma = 1.0, 1e-9, 3.0
    rho = np.random.default_rng(seed).uniform(0.01, 1.0, int(np.prod(ne)))
    g.setDensities(rho)
    Y = 1e-9 + rho ** 3 * (1.0 - 1e-9)
    g.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, float(ne[1]), float(ne[2])], "xyz")
    g.addDirichletCondition([0.0, 0.0, 0.0], [float(ne[0]), 0.0, 0.0], [float(ne[0]), 0.0, float(ne[2])], "y")
    m = g.getDirichletMask()
    bits = (m[:, 0] * 1 + m[:, 1] * 2 + m[:, 2] * 4).astype(np.uint8)
    return g, Y, bits


def tip_load(ne):
    nn = [2 * v + 1 for v in ne]
    f = np.zeros((int(np.prod(nn)), 3))
    tip = [(nn[0] - 1) * nn[1] * nn[2] + j * nn[2] + nn[2] // 2 for j in range(nn[1])]
    f[tip, 1] = -1.0 / len(tip)
    return f


CASES = [((8, 4, 4), 2), ((8, 8, 4), 2), ((16, 8, 8), 3)]


@pytest.mark.parametrize("ne,L", CASES)
def test_q2_hierarchy_levels(gpu, oracle, ne, L):
    g, Y, bits = cantilever(ne)
    K0 = g.fullDensityElementStiffnessMatrix()
    ref = po.Q2Multigrid(ne, K0, Y, bits, L)
    mg = g.multigridSolver(L)
    for l in range(1, L + 1):
        bm = ref.dirichlet_bits(l)
        np.testing.assert_array_equal(mg.levelDirichletMask(l), np.stack([(bm >> c) & 1 for c in range(3)], 1).astype(bool))
        Ke = ref.element_matrices(l)
        assert rel(mg.levelElementMatrices(l, "fp64"), Ke) < 1e-13, l
        assert rel(mg.levelElementMatrices(l, "mixed"), Ke) < 1e-6, l


@pytest.mark.parametrize("ne,L", CASES)
def test_q2_hierarchy_smoother_residual_coarse(gpu, oracle, ne, L):
    g, Y, bits = cantilever(ne, seed=1)
    K0 = g.fullDensityElementStiffnessMatrix()
    ref = po.Q2Multigrid(ne, K0, Y, bits, L)
    mg = g.multigridSolver(L)
    rng = np.random.default_rng(2)
    for l in range(L):
        nn = ref.num_nodes(l)
        u, b = rng.standard_normal((2, nn, 3))
        for fwd in (True, False):
            assert rel(mg.smoothing(l, u, b, fwd), ref.smooth(l, u, b, fwd)) < 1e-11, (l, fwd)
            assert rel(mg.smoothing(l, u, b, fwd, precision="mixed"), ref.smooth(l, u, b, fwd)) < 1e-4, (l, fwd)
        assert rel(mg.computeResidual(l, u, b), ref.residual(l, u, b)) < 1e-12, l
        assert rel(mg.computeResidual(l, u, b, precision="mixed"), ref.residual(l, u, b)) < 1e-5, l
    b = rng.standard_normal((ref.num_nodes(L), 3))
    assert rel(mg.coarseSolve(b), ref.coarse_solve(b)) < 1e-10


@pytest.mark.parametrize("ne,L", CASES)
def test_q2_hierarchy_vcycle(gpu, oracle, ne, L):
    g, Y, bits = cantilever(ne, seed=3)
    K0 = g.fullDensityElementStiffnessMatrix()
    ref = po.Q2Multigrid(ne, K0, Y, bits, L)
    mg = g.multigridSolver(L)
    r = np.random.default_rng(4).standard_normal((g.numNodes(), 3))
    r[g.getDirichletMask()] = 0.0
    for sweeps in (1, 2):
        want = ref.vcycle(r, sweeps)
        assert rel(mg.applyPreconditionerInv(r, sweeps), want) < 1e-10, sweeps
        assert rel(mg.applyPreconditionerInv(r, sweeps, precision="mixed"), want) < 1e-4, sweeps


@pytest.mark.parametrize("ne,L", CASES)
def test_q2_hierarchy_pcg(gpu, oracle, ne, L):
    """The plain method (FP64 V-cycle and matvec) takes the oracle's iterations and matches its
    solution; the mixed solve's compliance is within 1e-8 of the FP64 GPU solve."""
    g, Y, bits = cantilever(ne, seed=5)
    K0 = g.fullDensityElementStiffnessMatrix()
    ref = po.Q2Multigrid(ne, K0, Y, bits, L)
    f = tip_load(ne)
    f[g.getDirichletMask()] = 0.0
    xref, itref, rrref = ref.pcg(f, 300, 1e-8, 2)
    mg = g.multigridSolver(L)
    mg.setPrecision("fp64")
    x = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 300, 1e-8, None, 1, 2, False)
    assert mg.lastStats.iterations == itref
    assert rel(x, xref) < 1e-8
    c64 = float(np.sum(f * x))
    assert abs(c64 - np.sum(f * xref)) < 1e-8 * abs(c64)
    mg.setPrecision("mixed")
    xm = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 300, 1e-8, None, 1, 2, False)
    assert mg.lastStats.relres <= 1e-8
    assert mg.lastStats.iterations <= itref + 1
    assert abs(np.sum(f * xm) - c64) < 1e-8 * abs(c64)


def test_q2_hierarchy_rebuilds_after_density_change(gpu):
    ne, L = (8, 4, 4), 2
    g, _, _ = cantilever(ne)
    mg = g.multigridSolver(L)
    K1a = mg.levelElementMatrices(1)
    rho = np.random.default_rng(9).uniform(0.01, 1.0, g.numElements())
    g.setDensities(rho)
    K1b = mg.levelElementMatrices(1)
    assert rel(K1a, K1b) > 1e-3
    g2 = pv.TensorProductSimulator([2, 2, 2], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    with pytest.raises(RuntimeError):
        g2.multigridSolver(3).levelElementMatrices(1)  # 4 elements along y cannot be halved 3 times
