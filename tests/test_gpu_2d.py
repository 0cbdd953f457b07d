"""The 2D (bilinear quadrilateral) path on the GPU against the numpy restatement
(oracle/oracle2d.py): simulator operators and sensitivities, every multigrid building block,
V-cycles and full multigrid, the PCG solve (iteration counts equal, solutions to 1e-9),
fabrication masks, the 2D smoothing filter and the topology-optimisation problem with OC steps."""
import json

import numpy as np
import pytest

from oracle import oracle2d as o2
from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def soa(u):
    """(nn, 2) field -> the oracle's flat SoA vector."""
    return np.asarray(u).T.ravel().copy()


def field(v, nn):
    return np.asarray(v).reshape(2, nn).T


def make_pair(ne=(16, 8), bbox=((0.0, 0.0), (2.0, 1.0)), nu=0.3, seed=0, cantilever=True, law=0):
    rng = np.random.default_rng(seed)
    tps = pv.TensorProductSimulator([1, 1], [list(bbox[0]), list(bbox[1])], list(ne))
    sim = o2.Sim2(ne, bbox[0], bbox[1])
    tps.ETensor = (1.0, nu)
    sim.setMaterial(1.0, nu)
    tps.interpolationLaw = law
    sim.law = law
    rho = rng.uniform(0.1, 1.0, sim.NE)
    tps.setDensities(rho)
    sim.setDensities(rho)
    if cantilever:
        mn, mx = [-1e-9, -1e-9], [1e-9, bbox[1][1] + 1e-9]
        tps.addDirichletCondition([0, 0], mn, mx, "xy")
        sim.addDirichletCondition([0, 0], mn, mx, "xy")
        # a partially fixed node row (roller) on the right edge, bottom
        mn2, mx2 = [bbox[1][0] - 1e-9, -1e-9], [bbox[1][0] + 1e-9, 1e-9]
        tps.addDirichletCondition([0, 0], mn2, mx2, "y")
        sim.addDirichletCondition([0, 0], mn2, mx2, "y")
    f = np.zeros((sim.NN, 2))
    f[sim.node(ne[0] // 2, ne[1]), 1] = -1.0
    tps.setNodalForces(f)
    sim.force = soa(f)
    return tps, sim, rng


def test_k0_and_apply(gpu):
    tps, sim, rng = make_pair()
    assert rel(tps.fullDensityElementStiffnessMatrix(), sim.K0) < 1e-15
    np.testing.assert_array_equal(tps.getDirichletMask()[:, 0], (sim.dmask & 1) == 1)
    u = rng.standard_normal((sim.NN, 2))
    assert rel(soa(tps.applyK(u)), sim.applyK(soa(u))) < 1e-13
    assert rel(tps.getYoungModulusScaleFactor(), sim.Y) < 1e-15
    assert rel(tps.complianceGradient(u), sim.complianceGradient(soa(u))) < 1e-13
    assert rel(tps.elementEnergyDensity(u), sim.elementEnergyDensity(soa(u))) < 1e-13
    lam = rng.standard_normal((sim.NN, 2))
    assert rel(tps.adjointSensitivity(lam, u, 0.7, 1.3), sim.adjointSensitivity(soa(lam), soa(u), 0.7, 1.3)) < 1e-13


@pytest.mark.parametrize("law", [0, 1])
def test_gravity_load_and_gradient(gpu, law):
    tps, sim, rng = make_pair(seed=3, law=law)
    tps.gravity = [0.3, -1.0]
    sim.grav = np.array([0.3, -1.0])
    assert rel(soa(tps.buildLoadVector()), sim.buildLoadVector()) < 1e-14
    u = rng.standard_normal((sim.NN, 2))
    assert rel(tps.complianceGradient(u), sim.complianceGradient(soa(u))) < 1e-13


def test_masked_operators(gpu):
    tps, sim, rng = make_pair(ne=(12, 10), seed=4)
    tps.gravity = [0.0, -1.0]
    sim.grav = np.array([0.0, -1.0])
    tps.setFabricationMaskHeightByLayer(6)
    sim.setFabricationMaskHeightByLayer(6)
    assert rel(tps.getYoungModulusScaleFactor(), sim.Y) < 1e-15
    u = rng.standard_normal((sim.NN, 2))
    assert rel(soa(tps.applyK(u)), sim.applyK(soa(u))) < 1e-13
    assert rel(soa(tps.buildLoadVector()), sim.buildLoadVector()) < 1e-14
    assert rel(tps.complianceGradient(u), sim.complianceGradient(soa(u))) < 1e-13


@pytest.mark.parametrize("mask", [None, 5])
def test_multigrid_blocks(gpu, mask):
    tps, sim, rng = make_pair(ne=(16, 16), seed=5)
    mg = tps.multigridSolver(2)
    omg = o2.MG2(sim, 2)
    if mask is not None:
        mg.setFabricationMaskHeightByLayer(mask)
        omg.setFabricationMaskHeightByLayer(mask)
    for l in range(3):
        s = omg.sims[l]
        np.testing.assert_array_equal(mg.getSimulator(l).getDirichletMask()[:, 1], (s.dmask >> 1 & 1) == 1)
        u = rng.standard_normal((s.NN, 2))
        b = rng.standard_normal((s.NN, 2))
        assert rel(soa(mg.applyK(l, u))[np.tile(s.nJ < s.nondetNodes(), 2)],
                   omg.applyK(l, soa(u))[np.tile(s.nJ < s.nondetNodes(), 2)]) < 1e-12
        h = np.tile(s.nJ < min(s.nondetNodes() + o2.MARGIN, s.nn[1]), 2)
        assert rel(soa(mg.computeResidual(l, u, b))[h], omg.computeResidual(l, soa(u), soa(b))[h]) < 1e-12
        if l < 2:
            for fwd in (True, False):
                got = soa(mg.smoothingMulticoloredGS(l, u, b, fwd))
                ref = omg.smooth(l, soa(u), soa(b), fwd)
                assert rel(got, ref) < 1e-11, (l, fwd)
            c = omg.sims[l + 1]
            rows_c = np.tile(c.nJ <= c.nondetNodes(), 2) if c.nondetNodes() < c.nn[1] else slice(None)
            assert rel(soa(mg.restriction(l, u))[rows_c], omg.restrict(l, soa(u))[rows_c]) < 1e-14
            uc = rng.standard_normal((c.NN, 2))
            assert rel(soa(mg.interpolation(l, uc)), omg.interpolate(l, soa(uc), None, False)) < 1e-14
            fine = rng.standard_normal((s.NN, 2))
            rows_f = np.tile(s.nJ < s.nondetNodes(), 2)
            assert rel(soa(mg.interpolation(l, uc, fine, True))[rows_f],
                       omg.interpolate(l, soa(uc), soa(fine), True)[rows_f]) < 1e-14
    b = rng.standard_normal((omg.sims[2].NN, 2))
    assert rel(soa(mg.coarseSolve(b)), omg.coarseSolve(soa(b))) < 1e-10


@pytest.mark.parametrize("fmg", [False, True])
def test_mg_solve(gpu, fmg):
    tps, sim, rng = make_pair(ne=(32, 16), seed=6)
    mg = tps.multigridSolver(2)
    omg = o2.MG2(sim, 2)
    f = tps.buildLoadVector()
    u0 = np.zeros_like(f)
    got = soa(mg.solve(u0, f, 3, 2, False, False, None, fmg))
    ref = omg.solve(soa(u0), soa(f), 3, 2, False, fmg)
    assert rel(got, ref) < 1e-10


@pytest.mark.parametrize("fmg,sweeps,graphs", [(False, 1, True), (True, 2, True), (False, 1, False)])
def test_pcg(gpu, fmg, sweeps, graphs):
    tps, sim, rng = make_pair(ne=(64, 32), seed=7)
    mg = tps.multigridSolver(3)
    mg.setUseGraphs(graphs)
    omg = o2.MG2(sim, 3)
    f = tps.buildLoadVector()
    x = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 200, 1e-9, None, 1, sweeps, fmg)
    xo = omg.pcg(np.zeros(2 * sim.NN), soa(f), 200, 1e-9, 1, sweeps, fmg)
    assert mg.lastStats.iterations == omg.lastIterations
    assert rel(soa(x), xo) < 1e-9
    r = soa(f) - sim.applyK(soa(x))
    o2.MG2.zeroDirichlet(sim, r)
    assert np.linalg.norm(r) < 1e-8 * np.linalg.norm(soa(f))


def test_pcg_callback_and_mask(gpu):
    tps, sim, rng = make_pair(ne=(32, 32), seed=8, cantilever=False)
    mn, mx = [-1e-9, -1e-9], [2 + 1e-9, 1e-9]
    tps.addDirichletCondition([0, 0], mn, mx, "xy")
    sim.addDirichletCondition([0, 0], mn, mx, "xy")
    tps.setNodalForces(np.zeros((sim.NN, 2)))
    sim.force = np.zeros(2 * sim.NN)
    tps.gravity = [0, -1]
    sim.grav = np.array([0.0, -1.0])
    mg = tps.multigridSolver(2)
    omg = o2.MG2(sim, 2)
    mg.setFabricationMaskHeightByLayer(13)
    omg.setFabricationMaskHeightByLayer(13)
    f = tps.buildLoadVector()
    assert rel(soa(f), sim.buildLoadVector()) < 1e-14
    seen = []
    live_n = sim.nJ < sim.nondetNodes()
    x = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 100, 1e-8,
                                           lambda it, xx, rr: seen.append(np.linalg.norm(rr[live_n])), 1, 1, False)
    ro = []
    xo = omg.pcg(np.zeros(2 * sim.NN), soa(f), 100, 1e-8, 1, 1, False, it_callback=lambda it, r: ro.append(r))
    assert len(seen) == len(ro) == omg.lastIterations
    live = np.tile(sim.nJ < sim.nondetNodes(), 2)
    assert rel(soa(x)[live], xo[live]) < 1e-9
    np.testing.assert_allclose(seen[:5], ro[:5], rtol=1e-8)


def test_direct_solve_zero_levels(gpu):
    tps, sim, rng = make_pair(ne=(8, 4), seed=9)
    f = tps.buildLoadVector()
    x = tps.solve(f)
    r = soa(f) - sim.applyK(soa(x))
    o2.MG2.zeroDirichlet(sim, r)
    assert np.linalg.norm(r) < 1e-10 * np.linalg.norm(soa(f))


@pytest.mark.parametrize("radius,ftype", [(1, 0), (2, 1), (3, 1)])
def test_smoothing_filter_2d(gpu, radius, ftype):
    rng = np.random.default_rng(radius)
    dims = (13, 7)
    x = rng.uniform(0, 1, dims[0] * dims[1])
    sf = pv.SmoothingFilter(radius, pv.SmoothingFilter.Type(ftype))
    sf.setInputDimensions(dims)
    assert rel(sf.apply(x), o2.smoothing_filter_2d(x, dims, radius, ftype)) < 1e-14


def test_topopt_oc(gpu):
    tps, sim, rng = make_pair(ne=(48, 24), seed=10)
    tps.setUniformDensities(1.0)
    sim.setDensities(np.ones(sim.NE))
    obj = pv.MultigridComplianceObjective(tps.multigridSolver(2))
    obj.tol = 1e-10
    sf = pv.SmoothingFilter(2, pv.SmoothingFilter.Type.Linear)
    pf = pv.ProjectionFilter(2.0)
    top = pv.TopologyOptimizationProblem(tps, obj, [pv.TotalVolumeConstraint(0.4)], [sf, pf])
    otop = o2.TOP2(o2.MG2(sim, 2), [("smooth", 2, 1), ("proj", 2.0)], 0.4, tol=1e-10)
    x0 = np.full(top.numVars(), pf.invert(0.4))
    top.setVars(x0)
    otop.setVars(x0)
    assert rel(top.evaluateObjective(), otop.evaluateObjective()) < 1e-9
    assert rel(top.evaluateObjectiveGradient(), otop.evaluateObjectiveGradient()) < 1e-8
    assert abs(top.evaluateConstraints()[0] - otop.evaluateConstraints()) < 1e-12
    assert rel(top.evaluateConstraintsJacobian(), otop.evaluateConstraintsJacobian()) < 1e-13
    oc = pv.OCOptimizer(top)
    for _ in range(3):
        oc.step()
        otop.ocStep()
        assert rel(top.getVars(), otop.vars[0]) < 1e-6
        assert rel(top.evaluateObjective(), otop.evaluateObjective()) < 1e-6


def test_bc_file_2d(gpu, tmp_path):
    spec = {"regions": [
        {"type": "dirichlet", "value": [0, 0, 0], "box%": {"minCorner": [-0.0001, -0.0001, 0], "maxCorner": [0.0001, 1.0001, 0]}},
        {"type": "force", "value": [0, -1, 0], "box%": {"minCorner": [0.9999, -0.0001, 0], "maxCorner": [1.0001, 0.0001, 0]}},
    ]}
    path = tmp_path / "cantilever.bc"
    path.write_text(json.dumps(spec))
    tps = pv.TensorProductSimulator([1, 1], [[0, 0], [2, 1]], [16, 8])
    tps.applyDisplacementsAndLoadsFromFile(str(path))
    m = tps.getDirichletMask()
    nn = tps.NbNodesPerDimension
    assert m[: nn[1]].all() and not m[nn[1]:].any()
    f = tps.buildLoadVector()
    assert f[16 * nn[1] + 0, 1] == -1.0 and np.count_nonzero(f) == 1
    V, F = tps.getMesh()
    assert V.shape == (tps.numNodes(), 3) and F.shape == (tps.numElements(), 4)


def lbl_pair(ne=(32, 16), seed=11):
    rng = np.random.default_rng(seed)
    bbox = ((0.0, 0.0), (2.0, 1.0))
    tps = pv.TensorProductSimulator([1, 1], [list(bbox[0]), list(bbox[1])], list(ne))
    sim = o2.Sim2(ne, bbox[0], bbox[1])
    tps.ETensor = (1.0, 0.3)
    sim.setMaterial(1.0, 0.3)
    rho = rng.uniform(0.3, 1.0, sim.NE)
    tps.setDensities(rho)
    sim.setDensities(rho)
    mn, mx = [-1e-9, -1e-9], [bbox[1][0] + 1e-9, 1e-9]
    tps.addDirichletCondition([0, 0], mn, mx, "xy")
    sim.addDirichletCondition([0, 0], mn, mx, "xy")
    tps.gravity = [0.0, -1.0]
    sim.grav = np.array([0.0, -1.0])
    return tps, sim


@pytest.mark.parametrize("method,slots,inc", [("zero", 4, 1), ("fd", 1, 1), ("N=3", 1, 1), ("N=2", 2, 3),
                                              ("constant", 1, 2)])
def test_layer_by_layer_2d(gpu, method, slots, inc):
    tps, sim = lbl_pair()
    mg = tps.multigridSolver(2)
    lbl = pv.LayerByLayerEvaluator(tps)
    lbl.selectInitMethod(method)
    lbl.run(mg, True, inc, 200, 1e-8, None, 1, 1, False, slots=slots)
    omg = o2.MG2(sim, 2)
    layers, comps, iters, grad, _ = o2.layer_by_layer(sim, omg, method, True, inc, 200, 1e-8, 1, 1, False)
    np.testing.assert_array_equal(lbl.layers, layers)
    same_path = slots == 1 or method == "zero"
    assert rel(lbl.compliances, comps) < (1e-9 if same_path else 1e-6)
    if same_path:
        np.testing.assert_array_equal(lbl.iterations, iters)
    n = len(layers)
    assert rel(lbl.gradient(), grad / n) < 1e-6
    assert abs(lbl.objective() - 0.5 * comps.sum() / n) < 1e-7 * abs(lbl.objective())


@pytest.mark.parametrize("fmg,sweeps", [(False, 1), (True, 2)])
def test_pcg_mixed_2d(gpu, fmg, sweeps):
    tps, sim, rng = make_pair(ne=(64, 32), seed=13)
    mg = tps.multigridSolver(3)
    mg.setPrecision("mixed")
    omg = o2.MG2(sim, 3)
    f = tps.buildLoadVector()
    x = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 200, 1e-10, None, 1, sweeps, fmg)
    xo = omg.pcg(np.zeros(2 * sim.NN), soa(f), 200, 1e-10, 1, sweeps, fmg)
    r = soa(f) - sim.applyK(soa(x))
    o2.MG2.zeroDirichlet(sim, r)
    assert np.linalg.norm(r) < 1e-9 * np.linalg.norm(soa(f))
    assert rel(soa(x), xo) < 1e-8
    assert abs(mg.lastStats.iterations - omg.lastIterations) <= 2


def test_lbl_and_problem_mixed_2d(gpu):
    tps, sim = lbl_pair(seed=14)
    mg = tps.multigridSolver(2)
    mg.setPrecision("mixed")
    lbl = pv.LayerByLayerEvaluator(tps)
    lbl.selectInitMethod("N=3")
    lbl.run(mg, True, 2, 200, 1e-9, None, 1, 1, False)
    layers, comps, iters, grad, _ = o2.layer_by_layer(sim, o2.MG2(sim, 2), "N=3", True, 2, 200, 1e-9, 1, 1, False)
    np.testing.assert_array_equal(lbl.layers, layers)
    assert rel(lbl.compliances, comps) < 1e-7
    assert rel(lbl.gradient(), grad / len(layers)) < 1e-6
    # the problem's solve follows the solver's precision
    tps2, sim2, _ = make_pair(ne=(32, 16), seed=15)
    mg2 = tps2.multigridSolver(2)
    mg2.setPrecision("mixed")
    obj = pv.MultigridComplianceObjective(mg2)
    obj.tol = 1e-10
    top = pv.TopologyOptimizationProblem(tps2, obj, [pv.TotalVolumeConstraint(0.5)], [pv.ProjectionFilter(1.0)])
    otop = o2.TOP2(o2.MG2(sim2, 2), [("proj", 1.0)], 0.5, tol=1e-10)
    x0 = np.full(top.numVars(), 0.6)
    top.setVars(x0)
    otop.setVars(x0)
    assert rel(top.evaluateObjective(), otop.evaluateObjective()) < 1e-8
    assert rel(top.evaluateObjectiveGradient(), otop.evaluateObjectiveGradient()) < 1e-7


def test_helpers_2d(gpu):
    tps, sim, rng = make_pair(ne=(8, 6), seed=16)
    u = rng.standard_normal((sim.NN, 2))
    K = tps.getK()
    Ku = (K @ u.reshape(-1)).reshape(-1, 2)
    assert rel(soa(Ku), sim.applyK(soa(u))) < 1e-13
    # bilinear sampling reproduces nodal values at nodes and linear fields everywhere
    P = np.array([tps.nodePosition(n) for n in (0, 7, sim.NN - 1)])
    np.testing.assert_allclose(tps.sampleNodalField(u, P), u[[0, 7, sim.NN - 1]], atol=1e-14)
    V, F = tps.getMesh()
    lin = V[:, 0] * 0.7 - V[:, 1] * 0.2
    q = rng.uniform([0, 0], [2, 1], (5, 2))
    np.testing.assert_allclose(tps.sampleNodalField(lin[:, None], q)[:, 0], q[:, 0] * 0.7 - q[:, 1] * 0.2, atol=1e-14)
    # downsampling: densities averaged 2 x 2, gradients spread back
    c = tps.downsample(1)
    np.testing.assert_array_equal(c.NbElementsPerDimension, (4, 3))
    rho = rng.uniform(0, 1, sim.NE)
    tps.downsampleDensityFieldTo(rho, c)
    np.testing.assert_allclose(c.getDensities(), rho.reshape(4, 2, 3, 2).mean(axis=(1, 3)).ravel(), atol=1e-15)
    gc = rng.standard_normal(c.numElements())
    gf = tps.upsampleDensityGradientFrom(c, gc)
    assert abs(gf.sum() - gc.sum()) < 1e-12
    # symmetry conditions pin the normal component on the chosen face
    s2 = pv.TensorProductSimulator([1, 1], [[0, 0], [2, 1]], [8, 6])
    s2.applySymmetryConditions([1, 0], [False, False])
    m = s2.getDirichletMask()
    x0 = np.arange(s2.numNodes()) < 7
    assert m[x0, 0].all() and not m[x0, 1].any() and not m[~x0].any()


def test_intermediate_shape_2d(gpu):
    tps, sim = lbl_pair(ne=(16, 8), seed=17)
    rho = tps.getDensities()
    it = tps.getIntermediateFabricationShape(0.5)
    np.testing.assert_array_equal(it.NbElementsPerDimension, (16, 4))
    np.testing.assert_allclose(it.getDensities(), rho.reshape(16, 8)[:, :4].ravel())
    assert it.getDirichletMask()[np.arange(it.numNodes()) % 5 == 0].all()
    # its compliance equals the masked full grid's at the same height
    mgi = it.multigridSolver(1)
    fi = it.buildLoadVector()
    ui = mgi.preconditionedConjugateGradient(np.zeros_like(fi), fi, 200, 1e-12, None, 1, 2, False)
    mg = tps.multigridSolver(1)
    mg.setFabricationMaskHeightByLayer(4)
    f = tps.buildLoadVector()
    u = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 200, 1e-12, None, 1, 2, False)
    live = (np.arange(tps.numNodes()) % 9) <= 4
    assert abs(np.sum(fi * ui) - np.sum((f * u)[live])) < 1e-9 * abs(np.sum(fi * ui))


def test_autograd_compliance_2d(gpu):
    torch = pytest.importorskip("torch")
    from voxelfem_gb300 import autograd as vag
    tps, sim, rng = make_pair(ne=(8, 4), seed=18)
    tps.gravity = [0.0, -0.4]
    rho0 = rng.uniform(0.3, 1.0, sim.NE)
    mg = tps.multigridSolver(1)
    solver = vag.SolverContext(tps, mg, cgIter=400, tol=1e-13)
    rho = torch.tensor(rho0, dtype=torch.float64, requires_grad=True)
    C = vag.compliance(rho, solver)
    C.backward()
    g = rho.grad.numpy()

    def comp(r):
        return float(vag.compliance(torch.tensor(r, dtype=torch.float64), solver))

    for e in (0, 13, 31):
        d = np.zeros_like(rho0)
        d[e] = 1e-6
        fd = (comp(rho0 + d) - comp(rho0 - d)) / 2e-6
        assert abs(fd - g[e]) < 1e-5 * max(abs(g[e]), 1e-3)
