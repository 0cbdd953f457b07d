"""Layer-by-layer evaluation (LayerByLayerEvaluator) against the oracle. Zero guesses: per-height
oracle solves and the concurrent-slot schedule against one-at-a-time: per-height compliance to
1e-8, the same PCG iteration counts, the averaged gradient to 1e-6 (FP64), bit-identical
compliances for any slot count (the gradient sum differs only in its summation order), and
mixed precision within 1e-6 of FP64. Warm starts ("N=3", "fd", "constant"): one chain follows
the oracle's sequential restatement with the same iteration count at every height; several
chains converge to the same compliances; zeroInit=False restarts from the full-design solution."""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu

NE = (16, 16, 8)
LEVELS = 3  # numLevels: two coarsenings
INC = 3
TOL = 1e-10


def _configure(sim, rho):
    if hasattr(sim, "ETensor"):
        sim.ETensor = (1.0, 0.3)
        sim.E_0 = 1.0
        sim.E_min = 1e-9
        sim.gamma = 3.0
        sim.gravity = [0.0, -1.0, 0.0]
    else:
        sim.setMaterial(1.0, 0.3)
        sim.setParams(E0=1.0, Emin=1e-9, gamma=3.0)
        sim.setGravity([0.0, -1.0, 0.0])
    # base plate fixed (build direction y)
    sim.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [float(NE[0]), 0.0, float(NE[2])], "xyz")
    sim.setDensities(rho)


def _gpu_sim():
    rho = np.random.default_rng(3).uniform(0.3, 1.0, int(np.prod(NE)))
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in NE]], NE)
    _configure(sim, rho)
    return sim, rho


def _oracle_lbl(oracle, rho, layers):
    comp, its, grad = [], [], np.zeros(rho.size)
    for lay in layers:
        o = oracle.Sim(NE)
        _configure(o, rho)
        o.setFabricationMaskHeightByLayer(int(lay))
        om = oracle.MG(o, LEVELS - 1)
        om.setFabricationMaskHeightByLayer(int(lay))
        f = o.buildLoadVector()
        u = om.preconditionedConjugateGradient(np.zeros_like(f), f, 500, TOL, None, 1, 2, False)
        comp.append(float(np.sum(f * u)))
        its.append(om.lastIterations)
        grad += o.complianceGradient(u)
    return np.array(comp), np.array(its), grad


def test_lbl_matches_oracle_and_slot_schedules_agree(gpu, oracle):
    sim, rho = _gpu_sim()
    mg = sim.multigridSolver(LEVELS - 1)
    runs = {}
    for slots in (1, 3):
        ev = pv.LayerByLayerEvaluator(sim)
        ev.selectInitMethod("zero")
        ev.run(mg, True, INC, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=slots)
        runs[slots] = ev
    ev1, ev3 = runs[1], runs[3]
    np.testing.assert_array_equal(ev1.layers, [16, 13, 10, 7, 4, 1])
    np.testing.assert_array_equal(ev1.compliances, ev3.compliances)
    np.testing.assert_array_equal(ev1.iterations, ev3.iterations)
    g1, g3 = ev1.gradient(), ev3.gradient()
    assert np.max(np.abs(g1 - g3)) <= 1e-13 * np.max(np.abs(g1))

    comp, its, grad = _oracle_lbl(oracle, rho, ev1.layers)
    assert np.max(np.abs(ev1.compliances - comp) / np.abs(comp)) < 1e-8
    np.testing.assert_array_equal(ev1.iterations, its)
    assert abs(ev1.objective() - 0.5 * comp.sum() / len(comp)) / abs(ev1.objective()) < 1e-8
    g = grad / len(comp)
    assert np.max(np.abs(ev1.gradient() - g)) / np.max(np.abs(g)) < 1e-6
    # the source simulator is untouched
    assert sim.getFabricationMaskHeight() >= NE[1]


def test_lbl_mixed_precision(gpu, oracle):
    sim, rho = _gpu_sim()
    mg = sim.multigridSolver(LEVELS - 1)
    ev64 = pv.LayerByLayerEvaluator(sim)
    ev64.selectInitMethod("zero")
    ev64.run(mg, True, INC, 500, TOL, mgSmoothingIterations=2, slots=4)
    mg.setPrecision("mixed")
    evm = pv.LayerByLayerEvaluator(sim)
    evm.selectInitMethod("zero")
    evm.run(mg, True, INC, 500, TOL, mgSmoothingIterations=2, slots=4)
    assert np.max(np.abs(evm.compliances - ev64.compliances) / np.abs(ev64.compliances)) < 1e-6
    assert np.max(np.abs(evm.gradient() - ev64.gradient())) / np.max(np.abs(ev64.gradient())) < 1e-5


def test_graphs_survive_mask_changes(gpu, oracle):
    """Captured solve graphs read the fabrication mask from device memory: solving at several
    mask heights with one solver reproduces fresh oracle solves at each height."""
    sim, rho = _gpu_sim()
    mg = sim.multigridSolver(LEVELS - 1)
    for lay in (16, 9, 5, 12):
        mg.setFabricationMaskHeightByLayer(lay)
        f = sim.buildLoadVector()
        u = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 500, TOL, None, 1, 2, False)
        o = oracle.Sim(NE)
        _configure(o, rho)
        o.setFabricationMaskHeightByLayer(lay)
        om = oracle.MG(o, LEVELS - 1)
        om.setFabricationMaskHeightByLayer(lay)
        fo = o.buildLoadVector()
        np.testing.assert_allclose(f, fo, rtol=0, atol=1e-14)
        uo = om.preconditionedConjugateGradient(np.zeros_like(fo), fo, 500, TOL, None, 1, 2, False)
        assert mg.lastStats.iterations == om.lastIterations, lay
        assert np.max(np.abs(u - uo)) / np.max(np.abs(uo)) < 1e-8, lay


@pytest.mark.parametrize("method", ["N=3", "fd", "constant", "N=1"])
def test_lbl_warm_start_matches_sequential_oracle(gpu, oracle, method):
    sim, rho = _gpu_sim()
    mg = sim.multigridSolver(LEVELS - 1)
    ev = pv.LayerByLayerEvaluator(sim)
    ev.selectInitMethod(method)
    ev.run(mg, True, INC, 500, TOL, mgIterations=1, mgSmoothingIterations=2)
    o = oracle.Sim(NE)
    _configure(o, rho)
    om = oracle.MG(o, LEVELS - 1)
    lay, comp, its, grad, _ = oracle.layer_by_layer(o, om, method, True, INC, 500, TOL, 1, 2, False)
    np.testing.assert_array_equal(ev.layers, lay)
    np.testing.assert_array_equal(ev.iterations, its)
    assert np.max(np.abs(ev.compliances - comp) / np.abs(comp)) < 1e-8
    g = grad / len(comp)
    assert np.max(np.abs(ev.gradient() - g)) / np.max(np.abs(g)) < 1e-6
    if method == "N=3":
        # warm starts save iterations against zero guesses
        ez = pv.LayerByLayerEvaluator(sim)
        ez.selectInitMethod("zero")
        ez.run(mg, True, INC, 500, TOL, mgIterations=1, mgSmoothingIterations=2)
        assert ev.iterations.sum() < ez.iterations.sum()


def test_lbl_warm_chains_and_restart(gpu, oracle):
    sim, rho = _gpu_sim()
    mg = sim.multigridSolver(LEVELS - 1)
    ev1 = pv.LayerByLayerEvaluator(sim)
    ev1.run(mg, True, INC, 500, TOL, mgSmoothingIterations=2, slots=1)
    ev3 = pv.LayerByLayerEvaluator(sim)
    ev3.run(mg, True, INC, 500, TOL, mgSmoothingIterations=2, slots=3)
    assert np.max(np.abs(ev3.compliances - ev1.compliances) / np.abs(ev1.compliances)) < 1e-8
    # a chain head starts from zero: with 3 chains of 2 heights, heights 0, 2, 4 match the
    # zero-guess iteration counts of a single chain's first height pattern
    assert ev3.iterations[0] == ev1.iterations[0]
    # restart from the previous run's full-design solution
    ev1.run(mg, False, INC, 500, TOL, mgSmoothingIterations=2, slots=1)
    assert ev1.iterations[0] == 0
    assert np.max(np.abs(ev3.compliances - ev1.compliances) / np.abs(ev1.compliances)) < 1e-8


def test_autotuner_and_tuned_run(gpu, tmp_path, monkeypatch):
    """The autotuner times slot counts and fine-sweep forms (which leave the results unchanged)
    and caches the fastest; a tuned run reads the cache and reproduces the plain run."""
    from voxelfem_gb300 import autotune

    sim, rho = _gpu_sim()
    mg = sim.multigridSolver(LEVELS - 1)
    mg.setPrecision("mixed")
    path = str(tmp_path / "cache.json")
    entry = autotune.tune_layer_by_layer(sim, mg, "zero", tol=TOL, sample_increment=3,
                                         candidates={"slots": (1, 3), "sweepForm": ("lines", "colours", "planes"),
                                                     "mgSmoothingIterations": (2,)}, path=path)
    assert len(entry["candidates"]) == 6
    assert all(c["max_rel_diff"] == 0.0 for c in entry["candidates"])
    monkeypatch.setattr(autotune, "CACHE", path)
    assert autotune.lookup(sim, mg, "zero")["sweepForm"] == entry["sweepForm"]
    plain = pv.LayerByLayerEvaluator(sim)
    plain.selectInitMethod("zero")
    plain.run(mg, True, INC, 500, TOL, mgSmoothingIterations=2)
    tuned = pv.LayerByLayerEvaluator(sim)
    tuned.selectInitMethod("zero")
    tuned.run(mg, True, INC, 500, TOL, mgSmoothingIterations="tuned", tuned=True)
    np.testing.assert_array_equal(tuned.compliances, plain.compliances)
    np.testing.assert_array_equal(tuned.iterations, plain.iterations)
