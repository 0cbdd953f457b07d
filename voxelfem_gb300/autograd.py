"""torch.autograd wrappers of the solve-and-sensitivity path.

The reference computes the compliance gradient by hand (TopologyOptimizationObjective.hh:41-47,
TensorProductSimulator.hh:973-1005) and backpropagates it through the filter chain
(TopologyOptimizationFilter.hh:90-187). Here the same quantities are exposed as differentiable
torch functions whose forward and backward passes run on the device:

* ``DisplacementSolve``: u(rho) = K(rho)^-1 f(rho). Backward solves the adjoint system
  K lam = dJ/du with the same multigrid-preconditioned CG (K is symmetric) and applies the fused
  per-element kernel lam^T (df/drho_e - dK_e/drho_e u_e) (``vfem_grid_adjoint_sensitivity``).
* ``LoadVector``: f(rho) (nodal forces plus self-weight); backward lam^T df/drho.
* ``ComplianceVolume``: design variables -> (compliance, volume fraction) through the filter
  chain, the solve and the constraint, in one Function whose backward runs the adjoint solve
  (``adjoint="solve"``) or uses the self-adjointness of compliance (``adjoint="self"``,
  lam = u / 2, the reference's shortcut), then the filter chain's transpose.

Tensors stay on the GPU: CUDA float64 tensors cross the C ABI as device pointers (a nodal
field is a contiguous (components, numNodes) tensor, the (numNodes, components) column-major
layout of the library), so the densities, loads, displacements, adjoints and the filter chain's
intermediate values never visit the host. Inputs on the CPU are moved to the GPU, and results
are returned on the input's device. Before each library call the current torch stream is
synchronised, because the library runs on its own streams.
"""
import ctypes as C

import numpy as np
import torch

from . import _capi
from . import pyVoxelFEM as pv

_DEV = torch.device("cuda")


def _np(t):
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


def _dev(t):
    return t.detach().to(_DEV, torch.float64).contiguous()


def _lib():
    return _capi.load()


def _sync():
    torch.cuda.current_stream().synchronize()


def _p(t):
    return C.c_void_p(t.data_ptr())


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
        self.nc = getattr(sim, "_nc", 3)
        self.nn, self.ne = sim.numNodes(), sim.numElements()
        two = self.nc == 2
        L = _lib()
        self._set_rho = L.vfem_grid2_set_densities if two else L.vfem_grid_set_densities
        self._load = L.vfem_grid2_build_load if two else L.vfem_grid_build_load
        self._adjoint = L.vfem_grid2_adjoint_sensitivity if two else L.vfem_grid_adjoint_sensitivity
        self._pcg = L.vfem_mg2_pcg if two else L.vfem_mg_pcg
        self._rho = None
        self._rho_t = None
        self._dmask = None
        self.lastStats = None

    def invalidate(self):
        """Forget the cached densities (after the simulator's densities were set elsewhere)."""
        self._rho = None
        self._rho_t = None

    # ---- host arrays (numpy) ----
    def set_densities(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        if self._rho is None or not np.array_equal(self._rho, rho):
            self.sim.setDensities(rho)
            self._rho = rho.copy()
            self._rho_t = None

    def solve(self, b):
        x0 = np.zeros_like(b)
        return self.mg.preconditionedConjugateGradient(x0, b, self.cgIter, self.tol, None, self.mgIterations,
                                                       self.mgSmoothingIterations, self.fullMultigrid)

    # ---- device tensors ----
    def set_densities_dev(self, rho):
        """rho: CUDA float64 (ne,)."""
        if self._rho_t is None or not torch.equal(self._rho_t, rho):
            _sync()
            _capi.check(self._set_rho(self.sim._h, _p(rho)))
            self._rho_t = rho.clone()
            self._rho = None

    def load_dev(self):
        f = torch.empty(self.nc, self.nn, dtype=torch.float64, device=_DEV)
        # the caching allocator may hand out a block that kernels queued on torch's stream
        # still read; the library writes f on its own stream
        _sync()
        _capi.check(self._load(self.sim._h, _p(f)))
        return f

    def solve_dev(self, b):
        """K^-1 b for a (nc, nn) CUDA tensor, from a zero initial guess."""
        x = torch.zeros_like(b)
        stats = _capi.PcgStats()
        _sync()
        _capi.check(self._pcg(self.mg._h, _p(x), _p(b), self.cgIter, self.tol, self.mgIterations,
                              self.mgSmoothingIterations, int(self.fullMultigrid), 0, _capi.PCG_CALLBACK(), None,
                              C.byref(stats)))
        self.lastStats = stats
        return x

    def adjoint_dev(self, lam, u, wF, wK):
        """lam^T (wF df/drho - wK dK/drho u) per element, (ne,) CUDA tensor."""
        out = torch.empty(self.ne, dtype=torch.float64, device=_DEV)
        _sync()
        _capi.check(self._adjoint(self.sim._h, _p(lam), _p(u), float(wF), float(wK), _p(out)))
        return out

    def dirichlet_mask_dev(self):
        if self._dmask is None:
            m = self.sim.getDirichletMask()  # (nn, nc) bool
            self._dmask = torch.from_numpy(np.ascontiguousarray(m.T)).to(_DEV)
        return self._dmask


# ---- the filter chain on device tensors ----
def _dims(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))


def _filter_apply_dev(flt, x):
    """One filter of a FilterChain applied to a CUDA tensor (the same library kernels as
    Filter.apply, on device pointers)."""
    L = _lib()
    _sync()
    if isinstance(flt, pv.SmoothingFilter):
        out = torch.empty_like(x)
        d = _dims(flt._dims)
        fn = L.vfem_smoothing_filter2 if d.size == 2 else L.vfem_smoothing_filter
        _capi.check(fn(d.ctypes.data_as(_capi._i64), flt.radius, int(flt.type), _p(x), _p(out)))
        return out
    if isinstance(flt, pv.ProjectionFilter):
        out = torch.empty_like(x)
        _capi.check(L.vfem_projection_apply(x.numel(), float(flt.beta), _p(x), _p(out)))
        return out
    if isinstance(flt, pv.UpsampleFilter):
        out = torch.empty(int(np.prod(flt._out)), dtype=torch.float64, device=_DEV)
        d = _dims(flt._in)
        fn = L.vfem_upsample_filter2 if d.size == 2 else L.vfem_upsample_filter
        _capi.check(fn(d.ctypes.data_as(_capi._i64), flt.factor, _p(x), _p(out)))
        return out
    if isinstance(flt, pv.VertexToCellFilter):
        out = torch.empty(int(np.prod(flt._out)), dtype=torch.float64, device=_DEV)
        d = _dims(flt._in)
        fn = L.vfem_vertex_to_cell_filter2 if d.size == 2 else L.vfem_vertex_to_cell_filter
        _capi.check(fn(d.ctypes.data_as(_capi._i64), _p(x), _p(out)))
        return out
    if isinstance(flt, pv.LangelaarFilter):
        out = torch.empty_like(x)
        _capi.check(L.vfem_langelaar_apply(flt._h, _p(x), _p(out)))
        return out
    return torch.from_numpy(np.ascontiguousarray(flt.apply(x.cpu().numpy()))).to(_DEV)


def _filter_backprop_dev(flt, g, v):
    """The filter's transpose applied to g (v: the filter's input at the last forward pass)."""
    L = _lib()
    _sync()
    if isinstance(flt, pv.SmoothingFilter):
        return _filter_apply_dev(flt, g)  # symmetric under the reflecting boundary
    if isinstance(flt, pv.ProjectionFilter):
        out = torch.empty_like(g)
        _capi.check(L.vfem_projection_backprop(g.numel(), float(flt.beta), _p(g), _p(v), _p(out)))
        return out
    if isinstance(flt, pv.UpsampleFilter):
        out = torch.empty(int(np.prod(flt._in)), dtype=torch.float64, device=_DEV)
        d = _dims(flt._in)
        fn = L.vfem_upsample_filter2_backprop if d.size == 2 else L.vfem_upsample_filter_backprop
        _capi.check(fn(d.ctypes.data_as(_capi._i64), flt.factor, _p(g), _p(out)))
        return out
    if isinstance(flt, pv.VertexToCellFilter):
        out = torch.empty(int(np.prod(flt._in)), dtype=torch.float64, device=_DEV)
        d = _dims(flt._in)
        fn = L.vfem_vertex_to_cell_filter2_backprop if d.size == 2 else L.vfem_vertex_to_cell_filter_backprop
        _capi.check(fn(d.ctypes.data_as(_capi._i64), _p(g), _p(out)))
        return out
    if isinstance(flt, pv.LangelaarFilter):
        out = torch.empty_like(g)
        _capi.check(L.vfem_langelaar_backprop(flt._h, _p(g), _p(v), _p(out)))
        return out
    return torch.from_numpy(np.ascontiguousarray(flt.backprop(g.cpu().numpy(), v.cpu().numpy()))).to(_DEV)


def chain_forward_dev(chain, x):
    """FilterChain.setDesignVars on a CUDA tensor; returns every intermediate field."""
    vs = [x]
    for flt in chain.filters:
        vs.append(_filter_apply_dev(flt, vs[-1]))
    return vs


def chain_backprop_dev(chain, g, vs):
    """FilterChain.backprop (TopologyOptimizationFilter.hh:162-175) with the intermediates of
    chain_forward_dev."""
    for i in range(len(chain.filters) - 1, -1, -1):
        g = _filter_backprop_dev(chain.filters[i], g, vs[i])
    return g


class DisplacementSolve(torch.autograd.Function):
    """u = K(rho)^-1 f(rho) on the solver's grid; rho are the physical densities (ne,); u is
    returned as (numNodes, components)."""

    @staticmethod
    def forward(ctx, rho, solver):
        r = _dev(rho)
        solver.set_densities_dev(r)
        u = solver.solve_dev(solver.load_dev())
        ctx.solver, ctx.rho, ctx.u = solver, r, u
        return u.t().to(rho.device)

    @staticmethod
    def backward(ctx, grad_u):
        solver = ctx.solver
        solver.set_densities_dev(ctx.rho)
        g = _dev(grad_u.t())
        g[solver.dirichlet_mask_dev()] = 0.0  # constrained components do not depend on rho
        lam = solver.solve_dev(g)  # adjoint system on the same symmetric operator
        grad = solver.adjoint_dev(lam, ctx.u, 1.0, 1.0)
        return grad.to(grad_u.device), None


class LoadVector(torch.autograd.Function):
    """f(rho): nodal forces plus the self-weight load (TensorProductSimulator.hh:1269-1288)."""

    @staticmethod
    def forward(ctx, rho, solver):
        r = _dev(rho)
        solver.set_densities_dev(r)
        ctx.solver, ctx.rho = solver, r
        return solver.load_dev().t().to(rho.device)

    @staticmethod
    def backward(ctx, grad_f):
        solver = ctx.solver
        solver.set_densities_dev(ctx.rho)
        g = _dev(grad_f.t())
        grad = solver.adjoint_dev(g, torch.zeros_like(g), 1.0, 0.0)
        return grad.to(grad_f.device), None


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
        vs = chain_forward_dev(chain, _dev(x))
        rho = vs[-1]
        solver.set_densities_dev(rho)
        f = solver.load_dev()
        u = solver.solve_dev(f)
        ctx.solver, ctx.chain, ctx.vs, ctx.u, ctx.f = solver, chain, vs, u, f
        ctx.adjoint = adjoint
        dev = x.device
        return 0.5 * torch.dot(f.flatten(), u.flatten()).to(dev), rho.mean().to(dev)

    @staticmethod
    def backward(ctx, gC, gV):
        solver, chain = ctx.solver, ctx.chain
        rho = ctx.vs[-1]
        solver.set_densities_dev(rho)
        if ctx.adjoint == "solve":
            b = 0.5 * ctx.f
            b[solver.dirichlet_mask_dev()] = 0.0
            lam = solver.solve_dev(b)
            dC = solver.adjoint_dev(lam, ctx.u, 1.0, 1.0) + solver.adjoint_dev(ctx.u, ctx.u, 0.5, 0.0)
        else:
            dC = solver.adjoint_dev(ctx.u, ctx.u, 1.0, 0.5)
        g = gC.to(_DEV, torch.float64) * dC + gV.to(_DEV, torch.float64) / rho.numel()
        gx = chain_backprop_dev(chain, g.contiguous(), ctx.vs)
        return gx.to(gC.device), None, None, None


__all__ = ["SolverContext", "DisplacementSolve", "LoadVector", "compliance", "ComplianceVolume",
           "chain_forward_dev", "chain_backprop_dev", "pv"]
