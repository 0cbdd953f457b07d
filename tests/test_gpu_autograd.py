"""Differentiable solve: torch.autograd wrappers against central finite differences and the
oracle's compliance gradient (tolerances: 1e-5 relative vs finite differences, 1e-6 vs the
oracle gradient, as the FP64 solves converge to 1e-12)."""
import numpy as np
import pytest
import torch

from voxelfem_gb300 import autograd as vag
from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

NE = (8, 4, 4)
GRAV = [0.0, -0.3, 0.1]


def _setup(oracle, rho_lo=0.3):
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in NE]]
    sim = pv.TensorProductSimulator([1, 1, 1], bbox, NE)
    rho, _ = wl.setup_cantilever(sim, NE, rho_lo, 0)
    sim.gravity = GRAV
    mg = sim.multigridSolver(2)
    o = oracle.Sim(NE)
    wl.setup_cantilever(o, NE, rho_lo, 0)
    o.setGravity(GRAV)
    return sim, mg, o, rho


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_compliance_adjoint_gradient_vs_fd_and_oracle(gpu, oracle):
    sim, mg, o, rho0 = _setup(oracle)
    solver = vag.SolverContext(sim, mg, cgIter=400, tol=1e-13)
    rho = torch.tensor(rho0, dtype=torch.float64, requires_grad=True)
    C = vag.compliance(rho, solver)
    C.backward()
    g = rho.grad.numpy()

    # the oracle's hand-written compliance gradient at its own FP64 solution
    o.setDensities(rho0)
    omg = oracle.MG(o, 2)
    f = o.buildLoadVector()
    uo = omg.preconditionedConjugateGradient(np.zeros_like(f), f, 400, 1e-13, None, 1, 2, False)
    go = o.complianceGradient(uo)
    assert _rel(g, go) < 1e-6
    c = float(C.detach())
    assert abs(c - 0.5 * float(np.sum(f * uo))) / abs(c) < 1e-8

    # central differences on a few elements
    rng = np.random.default_rng(5)
    h = 1e-6
    for e in rng.choice(rho0.size, 10, replace=False):
        vals = []
        for s in (+1, -1):
            r = rho0.copy()
            r[e] += s * h
            vals.append(float(vag.compliance(torch.tensor(r), solver)))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-5 * np.max(np.abs(g)), (e, fd, g[e])


def test_displacement_solve_generic_objective_vs_fd(gpu, oracle):
    """A non-compliance objective J = sum(w * u): the backward is a genuine adjoint solve."""
    sim, mg, o, rho0 = _setup(oracle)
    solver = vag.SolverContext(sim, mg, cgIter=400, tol=1e-13)
    w = torch.tensor(np.random.default_rng(7).standard_normal((sim.numNodes(), 3)))
    rho = torch.tensor(rho0, dtype=torch.float64, requires_grad=True)
    J = (w * vag.DisplacementSolve.apply(rho, solver)).sum()
    J.backward()
    g = rho.grad.numpy()
    h = 1e-6
    for e in np.random.default_rng(9).choice(rho0.size, 8, replace=False):
        vals = []
        for s in (+1, -1):
            r = rho0.copy()
            r[e] += s * h
            vals.append(float((w * vag.DisplacementSolve.apply(torch.tensor(r), solver)).sum()))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-5 * np.max(np.abs(g)), (e, fd, g[e])


@pytest.mark.parametrize("adjoint", ["solve", "self"])
def test_compliance_volume_through_filter_chain(gpu, oracle, adjoint):
    sim, mg, o, rho0 = _setup(oracle)
    solver = vag.SolverContext(sim, mg, cgIter=400, tol=1e-13)
    chain = pv.FilterChain([pv.SmoothingFilter(1, pv.SmoothingFilter.Type.Linear), pv.ProjectionFilter(2.0)], NE)
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    x = torch.tensor(rho0, dtype=torch.float64, device=dev, requires_grad=True)
    C, V = vag.ComplianceVolume.apply(x, solver, chain, adjoint)
    (C + 3.0 * V).backward()
    g = x.grad.cpu().numpy()

    # reference gradient: oracle compliance gradient at the filtered densities, chain transpose
    chain.setDesignVars(rho0)
    rho_phys = chain.physicalVars()
    o.setDensities(rho_phys)
    omg = oracle.MG(o, 2)
    f = o.buildLoadVector()
    uo = omg.preconditionedConjugateGradient(np.zeros_like(f), f, 400, 1e-13, None, 1, 2, False)
    gref = chain.backprop(o.complianceGradient(uo) + 3.0 / rho0.size)
    assert _rel(g, gref) < 1e-6
    assert abs(float(V.detach()) - np.mean(rho_phys)) < 1e-14

    h = 1e-6
    for e in np.random.default_rng(11).choice(rho0.size, 6, replace=False):
        vals = []
        for s in (+1, -1):
            xx = rho0.copy()
            xx[e] += s * h
            Cp, Vp = vag.ComplianceVolume.apply(torch.tensor(xx), solver, chain, adjoint)
            vals.append(float(Cp) + 3.0 * float(Vp))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-5 * np.max(np.abs(g)), (e, fd, g[e])
