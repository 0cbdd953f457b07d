"""GPU parity: the CUDA library (through its C ABI, via voxelfem_gb300.pyVoxelFEM)
against the CPU oracle on the same seeded inputs.

Tolerances: single operators (applyK, residual, one smoothing sweep, transfers,
coarse solve, sensitivities, filters) agree to 1e-12 relative (FP64; only the
summation order differs); the FP64 MG-PCG follows the same iterations and its
displacements and compliance agree to 1e-8 relative; sensitivities to 1e-6.
"""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make_pair(oracle, ne, rho_lo=0.3, seed=0, levels=None, mask_layer=None, bbox=None):
    if bbox is None:
        bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    g = pv.TensorProductSimulator([1, 1, 1], bbox, ne)
    o = oracle.Sim(ne, bbox)
    wl.setup_cantilever(g, ne, rho_lo, seed)
    wl.setup_cantilever(o, ne, rho_lo, seed)
    if mask_layer is not None:
        g.setFabricationMaskHeightByLayer(mask_layer)
        o.setFabricationMaskHeightByLayer(mask_layer)
    if levels is None:
        return g, o
    gm = g.multigridSolver(levels)
    om = oracle.MG(o, levels)
    if mask_layer is not None:
        gm.setFabricationMaskHeightByLayer(mask_layer)
        om.setFabricationMaskHeightByLayer(mask_layer)
    return g, o, gm, om


@pytest.mark.parametrize("ne", [(4, 2, 2), (6, 5, 3), (16, 8, 8)])
def test_applyk_fine(gpu, oracle, ne):
    g, o = make_pair(oracle, ne)
    assert g.k0IsCube()  # unit-cube voxels: the fine FP32 kernels hold K0 as 10 class values
    np.testing.assert_array_equal(g.fullDensityElementStiffnessMatrix().shape, (24, 24))
    assert rel(g.fullDensityElementStiffnessMatrix(), o.K0()) < 1e-14
    assert rel(g.getYoungModulusScaleFactor(), o.youngModuli()) < 1e-15
    u = np.random.default_rng(1).standard_normal((g.numNodes(), 3))
    assert rel(g.applyK(u), o.applyK(u)) < 1e-12


def test_dirichlet_and_load(gpu, oracle):
    ne = (8, 4, 6)
    g, o = make_pair(oracle, ne)
    gm = g.getDirichletMask()
    om = o.dirichletMask()
    bits = gm[:, 0] * 1 + gm[:, 1] * 2 + gm[:, 2] * 4
    np.testing.assert_array_equal(bits.astype(np.uint8), om)
    np.testing.assert_array_equal(g.buildLoadVector(), o.buildLoadVector())


@pytest.fixture(params=["rows", "planes"])
def stencil_layout(request, monkeypatch):
    """Assembled coarse stencils as node-contiguous rows (small levels) or colour-ordered
    planes (large levels): force one layout on every level of the solver under test."""
    monkeypatch.setenv("VFEM_STENCIL_ROWS_MAX_NODES", "1000000000" if request.param == "rows" else "0")
    return request.param


def test_level_operators(gpu, oracle, stencil_layout):
    ne = (16, 8, 8)
    g, o, gm, om = make_pair(oracle, ne, levels=3)
    om.updateStiffnessMatrices()
    gm.updateStiffnessMatrices()
    rng = np.random.default_rng(2)
    for l in range(gm.numLevels):
        assert np.array_equal(gm.getSimulator(l).NbElementsPerDimension, om.levelElems(l))
        if l > 0:
            m = gm.getSimulator(l).getDirichletMask()
            bits = (m[:, 0] * 1 + m[:, 1] * 2 + m[:, 2] * 4).astype(np.uint8)
            np.testing.assert_array_equal(bits, om.levelDirichletMask(l))
        nn = om.levelNodes(l)
        u = rng.standard_normal((nn, 3))
        b = rng.standard_normal((nn, 3))
        assert rel(gm.applyK(l, u), om.applyK(l, u)) < 1e-12, l
        assert rel(gm.computeResidual(l, u, b), om.computeResidual(l, u, b)) < 1e-12, l
        if l < gm.numLevels - 1:
            for fwd in (True, False):
                assert rel(gm.smoothingMulticoloredGS(l, u, b, fwd), om.smooth(l, u, b, fwd)) < 1e-11, (l, fwd)
            assert rel(gm.restriction(l, u), om.restrict(l, u)) < 1e-13
            c = rng.standard_normal((om.levelNodes(l + 1), 3))
            assert rel(gm.interpolation(l, c, u, accumulate=True), om.interpolate(l, c, u, True)) < 1e-13
            assert rel(gm.interpolation(l, c, None, accumulate=False), om.interpolate(l, c, None, False)) < 1e-13
    nc = om.levelNodes(gm.numLevels - 1)
    bc = rng.standard_normal((nc, 3))
    assert rel(gm.coarseSolve(bc), om.coarseSolve(bc)) < 1e-10


@pytest.mark.parametrize("ne,levels", [((16, 8, 8), 2), ((32, 16, 16), 3)])
def test_pcg_fp64(gpu, oracle, stencil_layout, ne, levels):
    g, o, gm, om = make_pair(oracle, ne, levels=levels)
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    xg = gm.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    xo = om.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    assert gm.lastStats.iterations == om.lastIterations
    assert gm.lastStats.relres <= 1e-8
    assert rel(xg, xo) < 1e-8
    cg, co = 0.5 * np.sum(b * xg), 0.5 * np.sum(b * xo)
    assert abs(cg - co) / abs(co) < 1e-8
    # sensitivities and element energy at the solution
    assert rel(g.complianceGradient(xg), o.complianceGradient(xo)) < 1e-6
    assert rel(g.complianceGradient(xo), o.complianceGradient(xo)) < 1e-12
    assert rel(g.elementEnergyDensity(xo), o.elementEnergyDensity(xo)) < 1e-12


def test_pcg_fmg_and_multiple_cycles(gpu, oracle):
    ne = (16, 8, 8)
    g, o, gm, om = make_pair(oracle, ne, levels=2)
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    xg = gm.preconditionedConjugateGradient(x0, b, 50, 1e-9, None, 2, 1, True)
    xo = om.preconditionedConjugateGradient(x0, b, 50, 1e-9, None, 2, 1, True)
    assert gm.lastStats.iterations == om.lastIterations
    assert rel(xg, xo) < 1e-8


def test_mg_solve_vcycles(gpu, oracle):
    ne = (16, 8, 8)
    g, o, gm, om = make_pair(oracle, ne, levels=2)
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    assert rel(gm.solve(x0, b, 3, 2), om.solve(x0, b, 3, 2)) < 1e-10
    assert rel(gm.solve(x0, b, 2, 1, fullMultigrid=True), om.solve(x0, b, 2, 1, fullMultigrid=True)) < 1e-10


@pytest.mark.parametrize("levels", [2, 3])
def test_masked_layers(gpu, oracle, stencil_layout, levels):
    ne = (16, 16, 8)
    g, o, gm, om = make_pair(oracle, ne, levels=levels, mask_layer=9)
    assert rel(g.getYoungModulusScaleFactor(), o.youngModuli()) < 1e-15
    u = np.random.default_rng(3).standard_normal((g.numNodes(), 3))
    assert rel(g.applyK(u), o.applyK(u)) < 1e-12
    b = g.buildLoadVector()
    xg = gm.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-8, None, 1, 2, False)
    xo = om.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-8, None, 1, 2, False)
    assert gm.lastStats.iterations == om.lastIterations
    assert rel(xg, xo) < 1e-8


def test_pcg_mixed_precision(gpu, oracle, stencil_layout):
    """Mixed precision (FP32 V-cycle inside FP64 CG) at 32x16x16 for each outer matvec: relative
    residual 1e-8, a true FP64 residual below 2e-8 and a compliance within 1e-8 of the FP64 GPU
    solve of the same system (and of the oracle's)."""
    ne = (32, 16, 16)
    g, o, gm, om = make_pair(oracle, ne, levels=3)
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    xo = om.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    gm.setPrecision("fp64")
    x64 = gm.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    c64 = 0.5 * np.sum(b * x64)
    co = 0.5 * np.sum(b * xo)
    for matvec, kind in (("df", "tensor"), ("df-simt", "df-simt"), ("fp64", "fp64")):
        gm.setPrecision("mixed", matvec)
        assert gm.outerMatvecKind() == kind
        xg = gm.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
        assert gm.lastStats.relres <= 1e-8
        # true residual of the mixed solution, evaluated in FP64
        r = b - g.applyK(xg)
        r[g.getDirichletMask()] = 0
        assert np.linalg.norm(r) / np.linalg.norm(b) < 2e-8
        cg = 0.5 * np.sum(b * xg)
        assert abs(cg - c64) / abs(c64) < 1e-8, (matvec, abs(cg - c64) / abs(c64))
        assert abs(cg - co) / abs(co) < 1e-8, (matvec, abs(cg - co) / abs(co))
    gm.setPrecision("fp64")


C1_NE = (64, 32, 32)


def test_c1_plain_method_against_oracle(gpu, oracle):
    """The plain method at its CPU-runnable size: the 64x32x32 cantilever, rho U[0.3, 1] seed 0,
    E0 = 1, Emin = 1e-9, nu = 0.3, p = 3, 3 coarsenings, one V-cycle with 2 + 2 sweeps per CG
    iteration, tol 1e-8, zero guess, FP64 throughout. The GPU takes the oracle's iteration count;
    displacements and compliance agree to 1e-8 and sensitivities to 1e-6. The mixed form of the
    same solve lands within 1e-8 of the FP64 GPU compliance."""
    g, o, gm, om = make_pair(oracle, C1_NE, rho_lo=0.3, seed=0, levels=3)
    assert gm.numLevels == 4
    b = g.buildLoadVector()
    np.testing.assert_array_equal(b, o.buildLoadVector())
    x0 = np.zeros_like(b)
    xg = gm.preconditionedConjugateGradient(x0, b, 200, 1e-8, None, 1, 2, False)
    xo = om.preconditionedConjugateGradient(x0, b, 200, 1e-8, None, 1, 2, False)
    assert gm.lastStats.iterations == om.lastIterations
    assert gm.lastStats.relres <= 1e-8
    assert rel(xg, xo) < 1e-8
    cg, co = 0.5 * np.sum(b * xg), 0.5 * np.sum(b * xo)
    assert abs(cg - co) / abs(co) < 1e-8
    assert rel(g.complianceGradient(xg), o.complianceGradient(xo)) < 1e-6
    gm.setPrecision("mixed")
    xm = gm.preconditionedConjugateGradient(x0, b, 200, 1e-8, None, 1, 2, False)
    assert gm.lastStats.relres <= 1e-8
    cm = 0.5 * np.sum(b * xm)
    assert abs(cm - cg) / abs(cg) < 1e-8, abs(cm - cg) / abs(cg)
    assert rel(g.complianceGradient(xm), o.complianceGradient(xo)) < 1e-6
    gm.setPrecision("fp64")


def test_pcg_mixed_precision_stretched_voxels(gpu, oracle):
    """Unequal element edges: K0 lacks the cube structure and the fine FP32 / double-float
    kernels read the full 24 x 24 table."""
    ne = (16, 8, 8)
    bbox = [[0.0, 0.0, 0.0], [16.0, 4.0, 12.0]]
    g, o, gm, om = make_pair(oracle, ne, levels=3, bbox=bbox)
    assert not g.k0IsCube()
    assert rel(g.fullDensityElementStiffnessMatrix(), o.K0()) < 1e-14
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    xo = om.preconditionedConjugateGradient(x0, b, 200, 1e-8, None, 1, 2, False)
    gm.setPrecision("mixed", "df")
    xg = gm.preconditionedConjugateGradient(x0, b, 200, 1e-8, None, 1, 2, False)
    r = b - g.applyK(xg)
    r[g.getDirichletMask()] = 0
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2e-8
    cg, co = 0.5 * np.sum(b * xg), 0.5 * np.sum(b * xo)
    assert abs(cg - co) / abs(co) < 1e-6
    gm.setPrecision("fp64")
    xg = gm.preconditionedConjugateGradient(x0, b, 200, 1e-8, None, 1, 2, False)
    assert gm.lastStats.iterations == om.lastIterations
    assert rel(xg, xo) < 1e-8


@pytest.mark.parametrize("radius,ftype", [(1, 0), (2, 1), (3, 1)])
def test_filters(gpu, oracle, radius, ftype):
    dims = (10, 7, 5)
    x = np.random.default_rng(4).uniform(0, 1, int(np.prod(dims)))
    sf = pv.SmoothingFilter(radius, ftype)
    sf.setInputDimensions(dims)
    assert rel(sf.apply(x), oracle.smoothing_filter(x, dims, radius, ftype)) < 1e-14
    pf = pv.ProjectionFilter(3.0)
    assert rel(pf.apply(x), oracle.projection_apply(x, 3.0)) < 1e-14
    g = np.random.default_rng(5).standard_normal(x.size)
    assert rel(pf.backprop(g, x), oracle.projection_backprop(g, x, 3.0)) < 1e-14


def test_topopt_oc(gpu, oracle):
    ne = (16, 8, 8)
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    g = pv.TensorProductSimulator([1, 1, 1], bbox, ne)
    o = oracle.Sim(ne)
    wl.setup_mbb(g, ne)
    wl.setup_mbb(o, ne)
    gm = g.multigridSolver(2)
    om = oracle.MG(o, 2)
    obj = pv.MultigridComplianceObjective(gm)
    obj.tol = 1e-10
    obj.cgIter = 200
    top = pv.TopologyOptimizationProblem(g, obj, [pv.TotalVolumeConstraint(0.3)],
                                         [pv.SmoothingFilter(2, pv.SmoothingFilter.Type.Linear), pv.ProjectionFilter(1.0)])
    otop = oracle.TOP(om, [("smoothing", 2, 1), ("projection", 1.0)], 0.3)
    otop.setSolver(cgIter=200, tol=1e-10)
    x = np.full(g.numElements(), 0.3)
    top.setVars(x)
    otop.setVars(x)
    assert abs(top.evaluateObjective() - otop.evaluateObjective()) / abs(otop.evaluateObjective()) < 1e-8
    assert rel(top.evaluateObjectiveGradient(), otop.evaluateObjectiveGradient()) < 1e-6
    assert abs(top.evaluateConstraints()[0] - otop.evaluateConstraints()[0]) < 1e-12
    assert rel(top.evaluateConstraintsJacobian(), otop.evaluateConstraintsJacobian()) < 1e-12
    oc = pv.OCOptimizer(top)
    for _ in range(3):
        oc.step()
        otop.ocStep()
        assert rel(top.getVars(), otop.designVars()) < 1e-6
    assert abs(top.evaluateConstraints()[0]) < 1e-6


def _c2_golden():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cantilever_256x128x128_oracle.json")
    with open(path) as f:
        return json.load(f)


def test_full_size_fp64_and_mixed_against_oracle_golden(gpu):
    """256x128x128 (12.8M DOF): the FP64 GPU solve takes the oracle's iterations and agrees on compliance to
    1e-8; the mixed solve reaches 1e-8 and agrees to 1e-8; size-independent properties of applyK hold."""
    gold = _c2_golden()
    ne = (256, 128, 128)
    g = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [256.0, 128.0, 128.0]], ne)
    wl.setup_cantilever(g, ne, 0.01, 0)
    mg = g.multigridSolver(5)
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    x = mg.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    assert mg.lastStats.iterations == gold["iterations"]
    c = 0.5 * np.sum(b * x)
    assert abs(c - gold["compliance"]) / abs(gold["compliance"]) < 1e-8
    mg.setPrecision("mixed")
    xm = mg.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    assert mg.lastStats.relres <= 1e-8
    cm = 0.5 * np.sum(b * xm)
    assert abs(cm - gold["compliance"]) / abs(gold["compliance"]) < 1e-8
    # applyK at full size: rigid translation in the null space, symmetry
    t = np.zeros_like(b)
    t[:, 0] = 1.0
    assert np.abs(g.applyK(t)).max() < 1e-12
    rng = np.random.default_rng(11)
    u, v = rng.standard_normal(b.shape), rng.standard_normal(b.shape)
    assert abs(np.sum(u * g.applyK(v)) - np.sum(v * g.applyK(u))) < 1e-12 * np.sum(np.abs(u * g.applyK(u)))


@pytest.mark.parametrize("ne,levels", [((32, 16, 16), 3), ((64, 32, 32), 3)])
def test_pcg_mixed_bf16_stencils(gpu, oracle, ne, levels):
    """Smoothing-level stencils stored in bf16 (applied in FP32): the mixed solve still reaches
    relative residual 1e-8, a true FP64 residual below 2e-8 and a compliance within 1e-8 of the
    FP64 GPU solve, within one iteration of the FP32-stencil solve."""
    g, o, gm, om = make_pair(oracle, ne, levels=levels)
    b = g.buildLoadVector()
    x0 = np.zeros_like(b)
    gm.setPrecision("fp64")
    c64 = 0.5 * np.sum(b * gm.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False))
    gm.setPrecision("mixed")
    gm.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    its32 = gm.lastStats.iterations
    gm.setStencilStorage("bf16")
    x = gm.preconditionedConjugateGradient(x0, b, 100, 1e-8, None, 1, 2, False)
    assert gm.lastStats.relres <= 1e-8
    assert gm.lastStats.iterations <= its32 + 1, (gm.lastStats.iterations, its32)
    r = b - g.applyK(x)
    r[g.getDirichletMask()] = 0
    assert np.linalg.norm(r) / np.linalg.norm(b) < 2e-8
    cm = 0.5 * np.sum(b * x)
    assert abs(cm - c64) / abs(c64) < 1e-8
    gm.setStencilStorage("fp32")
