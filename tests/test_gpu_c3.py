"""Full-size topology optimisation through the differentiable solve: the 3D MBB beam at
192x96x96 voxels (5.45M DOF), volume fraction 0.3 from uniform 0.3, SmoothingFilter(2, Linear)
then ProjectionFilter(1), 50 OC iterations whose gradients come from ComplianceVolume (GPU
forward solve, adjoint backward).

At iterations 0 and 50:
- the gradient is compared with the oracle's sensitivity: an FP64 CPU solve to 1e-12, the
  compliance gradient, then the filter chain's transpose (1e-6 relative);
- a central finite difference with step 1e-6 is taken along a random +-1 direction on 64
  random elements (FP64 solves to 1e-13, warm-started from the base solution). A single-element
  difference at this size changes the compliance by ~1e-11 relative, below the solve noise, so
  the 64 elements are probed jointly.

Along the way the OC bisection meets the volume constraint to 1e-6 and the compliance
decreases."""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

NE = (192, 96, 96)
LEVELS = 4  # optMGLevel([192, 96, 96], 3)
VOLFRAC = 0.3


def oc_update(x, dJ, dV, chain, m=0.2, p=0.5, ctol=1e-6):
    """OptimalityCriterion::step (OptimalityCriterion.hh:51-138) on host vectors; the constraint
    is 1 - mean(filtered x) / V*, its gradient -dV / V*."""
    dc = -dV / VOLFRAC

    def stepped(lam):
        with np.errstate(all="ignore"):
            r = x * np.power(dJ / (dc * lam), p)
            r = np.minimum(np.maximum(np.minimum(np.maximum(r, x - m), x + m), 0.0), 1.0)
        return np.where(np.isfinite(r), r, x)

    def viol(lam):
        chain.setDesignVars(stepped(lam))
        return 1.0 - float(np.mean(chain.physicalVars())) / VOLFRAC

    lo, hi = 1e-3, 1e3
    while viol(lo) > 0:
        lo /= 2
    while viol(hi) < 0:
        hi *= 2
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        v = viol(mid)
        if abs(v) <= ctol:
            break
        if v > 0:
            hi = mid
        else:
            lo = mid
    return stepped(mid), v


def test_c3_topology_optimisation_full_size(gpu, oracle):
    import torch
    from voxelfem_gb300 import autograd as vag

    bbox = [[0.0, 0.0, 0.0], [float(v) for v in NE]]
    sim = pv.TensorProductSimulator([1, 1, 1], bbox, NE)
    x, _ = wl.setup_mbb(sim, NE, VOLFRAC)
    mg = sim.multigridSolver(LEVELS)
    mg.setPrecision("mixed")
    solver = vag.SolverContext(sim, mg, cgIter=500, tol=1e-10)
    chain = pv.FilterChain([pv.SmoothingFilter(2, pv.SmoothingFilter.Type.Linear), pv.ProjectionFilter(1.0)], NE)
    # the plain FP64 solver for the finite differences
    mg64 = sim.multigridSolver(LEVELS)
    o = oracle.Sim(NE)
    wl.setup_mbb(o, NE, VOLFRAC)
    omg = oracle.MG(o, LEVELS)
    rng = np.random.default_rng(3)
    comps = []

    def check(xd):
        xt = torch.tensor(xd, dtype=torch.float64, requires_grad=True)
        C, V = vag.ComplianceVolume.apply(xt, solver, chain, "self")
        C.backward()
        g = xt.grad.numpy().copy()
        # the oracle's sensitivity at the same design
        chain.setDesignVars(xd)
        rho = chain.physicalVars()
        o.setDensities(rho)
        f = o.buildLoadVector()
        uo = omg.preconditionedConjugateGradient(np.zeros_like(f), f, 500, 1e-12, None, 1, 2, False)
        gref = chain.backprop(o.complianceGradient(uo))
        assert float(np.max(np.abs(g - gref)) / np.max(np.abs(gref))) < 1e-6
        # directional finite difference over 64 random elements, FP64 solves warm-started
        idx = rng.choice(xd.size, 64, replace=False)
        v = np.zeros_like(xd)
        v[idx] = rng.choice([-1.0, 1.0], 64)
        sim.setDensities(rho)
        fb = sim.buildLoadVector()
        ub = mg64.preconditionedConjugateGradient(np.zeros_like(fb), fb, 500, 1e-13, None, 1, 2, False)
        h = 1e-6
        vals = []
        for s in (+1, -1):
            chain.setDesignVars(xd + s * h * v)
            sim.setDensities(chain.physicalVars())
            fs = sim.buildLoadVector()
            us = mg64.preconditionedConjugateGradient(ub, fs, 500, 1e-13, None, 1, 2, False)
            vals.append(0.5 * float(np.sum(fs * us)))
        solver.invalidate()  # the FD solves changed the simulator's densities
        fd = (vals[0] - vals[1]) / (2 * h)
        gv = float(np.dot(g, v))
        print("oracle rel %.2e, directional FD rel %.2e" % (float(np.max(np.abs(g - gref)) / np.max(np.abs(gref))),
                                                           abs(fd - gv) / abs(gv)))
        assert abs(fd - gv) < 1e-3 * abs(gv), (fd, gv)
        return float(C.detach()), g, V

    C0, g, V = check(x)
    comps.append(C0)
    xt = x.copy()
    for it in range(50):
        xtt = torch.tensor(xt, dtype=torch.float64, requires_grad=True)
        C, V = vag.ComplianceVolume.apply(xtt, solver, chain, "self")
        (C + 0.0 * V).backward()
        dJ = xtt.grad.numpy().copy()
        dV = chain.backprop(np.full(xt.size, 1.0 / xt.size))
        xt, viol = oc_update(xt, dJ, dV, chain)
        assert abs(viol) <= 1e-6
        comps.append(float(C.detach()))
    C50, g50, _ = check(xt)
    assert comps[-1] < 0.5 * comps[0]
    assert C50 <= comps[-1] * (1 + 1e-6)
