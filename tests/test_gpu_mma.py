"""The device Method of Moving Asymptotes against the oracle's numpy restatement of the
reference (oracle/mma.py): iterates agree to 1e-9 over 12 steps (MMA and GCMMA) on a
box-constrained quadratic with a volume constraint, and on a compliance-minimisation problem
driven by the GPU solver; both reach the analytic optimum of the quadratic."""
import numpy as np
import pytest

from oracle import mma as omma
from voxelfem_gb300 import pyOptimizer

pytestmark = pytest.mark.gpu


def quad_problem(n, seed=0):
    t = np.random.default_rng(seed).uniform(0.1, 0.9, n)

    def f(x):
        return np.array([np.sum((x - t) ** 2), np.mean(x) / 0.4 - 1.0])

    def df(x):
        return np.vstack([2 * (x - t), np.full(n, 1.0 / (0.4 * n))])

    return t, f, df


@pytest.mark.parametrize("gcmma", [False, True])
@pytest.mark.parametrize("n", [7, 3000])
def test_mma_matches_oracle(gpu, gcmma, n):
    t, f, df = quad_problem(n)
    g = pyOptimizer.MMA(n, 1, np.zeros(n), np.ones(n), f, df)
    o = omma.MMA(n, 1, np.zeros(n), np.ones(n), f, df)
    g.enableGCMMA(gcmma)
    o.enableGCMMA(gcmma)
    x0 = np.full(n, 0.5)
    g.setInitialVar(x0)
    o.setInitialVar(x0)
    for k in range(12):
        g.step()
        o.step()
        xg, xo = g.getOptimalVar(), o.getOptimalVar()
        assert np.max(np.abs(xg - xo)) < 1e-9, k
    # analytic optimum: x = clip(t - lambda, 0, 1) with mean(x) = 0.4
    lo, hi = 0.0, 10.0
    for _ in range(200):
        lam = 0.5 * (lo + hi)
        if np.clip(t - lam, 0, 1).mean() > 0.4:
            lo = lam
        else:
            hi = lam
    xs = np.clip(t - lam, 0, 1)
    assert abs(f(xg)[0] - f(xs)[0]) < 1e-5 * f(xs)[0]
    assert f(xg)[1] < 1e-6


def test_mma_errors(gpu):
    n = 5
    t, f, df = quad_problem(n)
    g = pyOptimizer.MMA(n, 1, np.zeros(n), np.ones(n), f, df)
    with pytest.raises(RuntimeError):
        g.step()  # no initial value
    bad = pyOptimizer.MMA(n, 1, np.zeros(n), np.ones(n), lambda x: np.zeros(1), df)
    bad.setInitialVar(np.full(n, 0.5))
    with pytest.raises(RuntimeError):
        bad.step()


def test_mma_compliance_problem(gpu, oracle):
    """Minimum compliance with a volume constraint on a small cantilever, the solve on the GPU:
    the device optimiser follows the oracle's MMA on the same callbacks."""
    from voxelfem_gb300 import pyVoxelFEM as pv
    from voxelfem_gb300 import workloads as wl

    ne = (16, 8, 8)
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    wl.setup_cantilever(sim, ne, 0.5, 0)
    mg = sim.multigridSolver(2)
    f = sim.buildLoadVector()
    n = sim.numElements()

    def fun(x):
        sim.setDensities(x)
        u = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 200, 1e-10, None, 1, 2, False)
        return np.array([np.sum(f * u), np.mean(x) / 0.3 - 1.0])

    def grad(x):
        sim.setDensities(x)
        u = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 200, 1e-10, None, 1, 2, False)
        return np.vstack([2.0 * sim.complianceGradient(u), np.full(n, 1.0 / (0.3 * n))])

    g = pyOptimizer.MMA(n, 1, np.full(n, 1e-3), np.ones(n), fun, grad)
    o = omma.MMA(n, 1, np.full(n, 1e-3), np.ones(n), fun, grad)
    x0 = np.full(n, 0.3)
    g.setInitialVar(x0)
    o.setInitialVar(x0)
    c0 = fun(x0)[0]
    for k in range(4):
        g.step()
        o.step()
        assert np.max(np.abs(g.getOptimalVar() - o.getOptimalVar())) < 1e-7, k
    assert fun(g.getOptimalVar())[0] < c0
