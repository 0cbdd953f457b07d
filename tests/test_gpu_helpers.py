"""Simulator helpers of the reference's Python module (VoxelFEM.cc:76-154): mesh export, field
sampling, BC indicator field, assembled K, coarser and intermediate (partial-build)
simulators. The intermediate shape's solve reproduces the masked full-grid solve of the same
build height."""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def make(ne=(8, 4, 4), rho_lo=0.3):
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    wl.setup_cantilever(sim, ne, rho_lo, 0)
    return sim


def test_mesh_and_sampling(gpu):
    sim = make()
    V, F = sim.getMesh()
    assert V.shape == (sim.numNodes(), 3) and F.shape == (sim.numElements(), 8)
    e = sim.elementNodes(0)
    np.testing.assert_array_equal(F[0], e[[0, 1, 3, 2, 4, 5, 7, 6]])
    np.testing.assert_allclose(V[e[7]], [1.0, 1.0, 1.0])
    u = np.stack([V[:, 0] * 0.5 - V[:, 1], V[:, 2] + 1.0, V[:, 0] * V[:, 1] * V[:, 2]], axis=1)
    p = np.array([[0.3, 0.7, 1.2], [7.9, 3.5, 0.1], [-1.0, 2.0, 9.0]])
    q = np.clip(p, 0, [8, 4, 4])
    exact = np.stack([q[:, 0] * 0.5 - q[:, 1], q[:, 2] + 1.0, q[:, 0] * q[:, 1] * q[:, 2]], axis=1)
    np.testing.assert_allclose(sim.sampleNodalField(u, p), exact, rtol=0, atol=1e-12)
    bc = sim.getBCIndicatorField()
    assert bc[0] == 7 and bc.max() == 8 * 2  # fixed x = 0 face (7); -y force on the loaded edge (8 x 2)


def test_assembled_k(gpu):
    sim = make()
    K = sim.getK()
    u = np.random.default_rng(0).standard_normal((sim.numNodes(), 3))
    Ku = (K @ u.reshape(-1)).reshape(-1, 3)
    ref = sim.applyK(u)
    assert np.max(np.abs(Ku - ref)) < 1e-12 * np.max(np.abs(ref))


def test_downsample_transfers(gpu):
    sim = make((8, 8, 4))
    c = sim.downsample(1)
    np.testing.assert_array_equal(c.NbElementsPerDimension, [4, 4, 2])
    assert c.ETensor == sim.ETensor and c.E_min == sim.E_min
    rho = np.random.default_rng(1).uniform(0.1, 1, sim.numElements())
    sim.downsampleDensityFieldTo(rho, c)
    rc = c.getDensities()
    assert abs(rc.mean() - rho.mean()) < 1e-14
    g = np.random.default_rng(2).standard_normal(c.numElements())
    gf = sim.upsampleDensityGradientFrom(c, g)
    assert abs(np.dot(gf, rho) - np.dot(g, rc)) < 1e-12 * abs(np.dot(g, rc))  # adjoint of the averaging
    sim.setDensitiesFromCoarseGrid(2, rc)
    np.testing.assert_allclose(sim.getDensities().reshape(8, 8, 4)[::2, ::2, ::2].ravel(), rc, rtol=0, atol=0)


def test_intermediate_shape_matches_masked_solve(gpu):
    ne = (8, 8, 4)
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    wl.setup_layer_by_layer(sim, ne, 0.3, 0)
    part = sim.getIntermediateFabricationShape(0.5)
    np.testing.assert_array_equal(part.NbElementsPerDimension, [8, 4, 4])
    np.testing.assert_array_equal(part.getDensities(), sim.getDensities().reshape(ne)[:, :4, :].ravel())
    fp = part.buildLoadVector()
    up = part.multigridSolver(2).preconditionedConjugateGradient(np.zeros_like(fp), fp, 200, 1e-11, None, 1, 2, False)
    mg = sim.multigridSolver(2)
    mg.setFabricationMaskHeightByLayer(4)
    f = sim.buildLoadVector()
    u = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 200, 1e-11, None, 1, 2, False)
    ut = sim.transferVFieldToIntermediateFabricationShape(part, u)
    assert ut.shape == up.shape
    assert np.max(np.abs(ut - up)) < 1e-8 * np.max(np.abs(up))
    acc = np.zeros(sim.numElements())
    sim.accumElementScalarFieldFromIntermediateFabricationShape(part, np.ones(part.numElements()), acc)
    assert acc.sum() == part.numElements()


def test_reference_script_idioms(gpu):
    """The idioms of the reference's Python drivers: ETensor as an object with setIsotropic, and a
    problem subclass obtained through getClassName (python/LayerByLayerOptimization.py:55-93)."""
    import numpy as np
    from voxelfem_gb300 import pyVoxelFEM
    tps = pyVoxelFEM.TensorProductSimulator([1, 1], [[0, 0], [2, 1]], [16, 8])
    e = tps.ETensor
    e.setIsotropic(1, 0.3)
    tps.ETensor = e
    assert tps.ETensor == (1.0, 0.3)
    tps.addDirichletCondition([0, 0], [0, 0], [0, 1], "xy")
    f = np.zeros((tps.numNodes(), 2))
    f[16 * 9, 1] = -1.0
    tps.setNodalForces(f)
    base = eval(pyVoxelFEM.getClassName(tps, "TopologyOptimizationProblem"))

    class Weighted(base):
        def evaluateObjective(self):
            return 2.0 * super().evaluateObjective()

    obj = pyVoxelFEM.MultigridComplianceObjective(tps.multigridSolver(2))
    top = Weighted(tps, obj, [pyVoxelFEM.TotalVolumeConstraint(0.5)], [pyVoxelFEM.ProjectionFilter(1.0)])
    top.setVars(np.full(top.numVars(), 0.5))
    assert abs(top.evaluateObjective() - 2.0 * base.evaluateObjective(top)) < 1e-15 * abs(top.evaluateObjective())
