"""torch.autograd wrappers of the solve-and-sensitivity path.

The reference computes the compliance gradient by hand (TopologyOptimizationObjective.hh:41-47,
TensorProductSimulator.hh:973-1005) and backpropagates it through the filter chain
(TopologyOptimizationFilter.hh:90-187). Here the same quantities are exposed as differentiable
torch functions whose backward passes run on the device:

* ``DisplacementSolve``: u(rho) = K(rho)^-1 f(rho). Backward solves the adjoint system
  K lam = dJ/du with the same multigrid-preconditioned CG (K is symmetric) and applies the fused
  per-element kernel lam^T (df/drho_e - dK_e/drho_e u_e) (``vfem_grid_adjoint_sensitivity``).
* ``LoadVector``: f(rho) (nodal forces plus self-weight); backward lam^T df/drho.
* ``ComplianceVolume``: design variables -> (compliance, volume fraction) through the filter
  chain, the solve and the constraint, in one Function whose backward runs the adjoint solve
  (``adjoint="solve"``) or uses the self-adjointness of compliance (``adjoint="self"``,
  lam = u / 2, the reference's shortcut), then the filter chain's transpose.

Tensors cross into the library as host float64 arrays; the solves and kernels run on the GPU.
"""
import numpy as np
import torch

from . import pyVoxelFEM as pv


def _np(t):
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


class SolverContext:
    """A simulator, its multigrid solver and the PCG settings of the reference's
    MultigridComplianceObjective (TopologyOptimizationObjective.hh:98-104)."""

    def __init__(self, sim, mg, cgIter=200, tol=1e-10, mgIterations=1, mgSmoothingIterations=2,
                 fullMultigrid=False):
        self.sim = sim
        self.mg = mg
        self.cgIter = int(cgIter)
        self.tol = float(tol)
        self.mgIterations = int(mgIterations)
        self.mgSmoothingIterations = int(mgSmoothingIterations)
        self.fullMultigrid = bool(fullMultigrid)
        self._rho = None

    def set_densities(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        if self._rho is None or not np.array_equal(self._rho, rho):
            self.sim.setDensities(rho)
            self._rho = rho.copy()

    def solve(self, b):
        x0 = np.zeros_like(b)
        return self.mg.preconditionedConjugateGradient(x0, b, self.cgIter, self.tol, None, self.mgIterations,
                                                       self.mgSmoothingIterations, self.fullMultigrid)


class DisplacementSolve(torch.autograd.Function):
    """u = K(rho)^-1 f(rho) on the solver's grid; rho are the physical densities (ne,)."""

    @staticmethod
    def forward(ctx, rho, solver):
        r = _np(rho)
        solver.set_densities(r)
        f = solver.sim.buildLoadVector()
        u = solver.solve(f)
        ctx.solver, ctx.rho, ctx.u = solver, r, u
        return torch.from_numpy(u).to(rho.device)

    @staticmethod
    def backward(ctx, grad_u):
        solver = ctx.solver
        solver.set_densities(ctx.rho)
        g = _np(grad_u).reshape(ctx.u.shape).copy()
        g[solver.sim.getDirichletMask()] = 0.0  # constrained components do not depend on rho
        lam = solver.solve(g)  # adjoint system on the same symmetric operator
        grad = solver.sim.adjointSensitivity(lam, ctx.u, 1.0, 1.0)
        return torch.from_numpy(grad).to(grad_u.device), None


class LoadVector(torch.autograd.Function):
    """f(rho): nodal forces plus the self-weight load (TensorProductSimulator.hh:1269-1288)."""

    @staticmethod
    def forward(ctx, rho, solver):
        r = _np(rho)
        solver.set_densities(r)
        ctx.solver, ctx.rho = solver, r
        return torch.from_numpy(solver.sim.buildLoadVector()).to(rho.device)

    @staticmethod
    def backward(ctx, grad_f):
        solver = ctx.solver
        solver.set_densities(ctx.rho)
        g = _np(grad_f).reshape(-1, getattr(solver.sim, "_nc", 3))
        zero = np.zeros_like(g)
        grad = solver.sim.adjointSensitivity(g, zero, 1.0, 0.0)
        return torch.from_numpy(grad).to(grad_f.device), None


def compliance(rho, solver):
    """C(rho) = 1/2 f(rho) . u(rho), differentiable through an adjoint solve."""
    u = DisplacementSolve.apply(rho, solver)
    f = LoadVector.apply(rho, solver)
    return 0.5 * (f * u).sum()


class ComplianceVolume(torch.autograd.Function):
    """(x design variables) -> (compliance, mean physical density) through the filter chain.

    backward: dC/drho by the adjoint method, lam solving K lam = f / 2 (``adjoint="solve"``) or
    lam = u / 2 (``adjoint="self"``); dV/drho = 1 / ne; both through the filter chain's
    transpose.
    """

    @staticmethod
    def forward(ctx, x, solver, chain, adjoint="solve"):
        if adjoint not in ("solve", "self"):
            raise ValueError("adjoint must be 'solve' or 'self'")
        chain.setDesignVars(_np(x))
        rho = chain.physicalVars()
        solver.set_densities(rho)
        f = solver.sim.buildLoadVector()
        u = solver.solve(f)
        ctx.solver, ctx.chain, ctx.rho, ctx.xd, ctx.u, ctx.f = solver, chain, rho, _np(x), u, f
        ctx.adjoint = adjoint
        dev = x.device
        return (torch.tensor(0.5 * float(np.sum(f * u)), dtype=torch.float64, device=dev),
                torch.tensor(float(np.mean(rho)), dtype=torch.float64, device=dev))

    @staticmethod
    def backward(ctx, gC, gV):
        solver, chain = ctx.solver, ctx.chain
        solver.set_densities(ctx.rho)
        sim = solver.sim
        if ctx.adjoint == "solve":
            b = 0.5 * ctx.f
            b[sim.getDirichletMask()] = 0.0
            lam = solver.solve(b)
            dC = sim.adjointSensitivity(lam, ctx.u, 1.0, 1.0) + sim.adjointSensitivity(ctx.u, ctx.u, 0.5, 0.0)
        else:
            dC = sim.complianceGradient(ctx.u)
        g = float(gC) * dC + float(gV) / ctx.rho.size
        chain.setDesignVars(ctx.xd)
        gx = chain.backprop(g)
        return torch.from_numpy(gx).to(gC.device), None, None, None


__all__ = ["SolverContext", "DisplacementSolve", "LoadVector", "compliance", "ComplianceVolume", "pv"]
