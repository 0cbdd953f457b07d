"""ctypes front end of the CPU oracle (test infrastructure only).

Imported by tests/, ``__graft_entry__.smoke`` and the CPU-baseline leg of
``bench.py``; never by the ``voxelfem_gb300`` package. Nodal fields are numpy
arrays of shape (numNodes, 3) stored column-major (SoA), exactly the layout of
the reference's ``VField`` (TensorProductSimulator.hh:180).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

_d = C.POINTER(C.c_double)
_l = C.POINTER(C.c_long)
_u8 = C.POINTER(C.c_uint8)
_i = C.POINTER(C.c_int)
CB = C.CFUNCTYPE(None, C.c_long, C.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        sigs = {
            "ovf_last_error": (C.c_char_p, []),
            "ovf_num_threads": (C.c_int, []),
            "ovf_set_num_threads": (None, [C.c_int]),
            "ovf_sim_create": (C.c_void_p, [_l, _d, _d]),
            "ovf_sim_destroy": (None, [C.c_void_p]),
            "ovf_sim_set_material": (None, [C.c_void_p, C.c_double, C.c_double]),
            "ovf_sim_set_params": (None, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
            "ovf_sim_set_densities": (C.c_int, [C.c_void_p, _d]),
            "ovf_sim_get_Y": (None, [C.c_void_p, _d]),
            "ovf_sim_get_K0": (None, [C.c_void_p, _d]),
            "ovf_sim_add_dirichlet": (C.c_int, [C.c_void_p, _d, _d, _d, C.c_int]),
            "ovf_sim_set_forces": (None, [C.c_void_p, _d]),
            "ovf_sim_set_gravity": (None, [C.c_void_p, _d]),
            "ovf_sim_get_dirichlet_mask": (None, [C.c_void_p, _u8]),
            "ovf_sim_set_mask_layer": (C.c_int, [C.c_void_p, C.c_long]),
            "ovf_sim_apply_k": (None, [C.c_void_p, _d, _d]),
            "ovf_sim_build_load": (None, [C.c_void_p, _d]),
            "ovf_sim_compliance_gradient": (None, [C.c_void_p, _d, _d]),
            "ovf_sim_element_energy": (None, [C.c_void_p, _d, _d]),
            "ovf_mg_create": (C.c_void_p, [C.c_void_p, C.c_int]),
            "ovf_mg_destroy": (None, [C.c_void_p]),
            "ovf_mg_set_symmetric": (None, [C.c_void_p, C.c_int]),
            "ovf_mg_num_levels": (C.c_int, [C.c_void_p]),
            "ovf_mg_level_dims": (None, [C.c_void_p, C.c_int, _l]),
            "ovf_mg_set_mask_layer": (C.c_int, [C.c_void_p, C.c_long]),
            "ovf_mg_level_dirichlet_mask": (None, [C.c_void_p, C.c_int, _u8]),
            "ovf_mg_update_stiffness": (C.c_int, [C.c_void_p]),
            "ovf_mg_apply_k": (C.c_int, [C.c_void_p, C.c_int, _d, _d]),
            "ovf_mg_residual": (C.c_int, [C.c_void_p, C.c_int, _d, _d, _d]),
            "ovf_mg_smooth": (C.c_int, [C.c_void_p, C.c_int, _d, _d, C.c_int]),
            "ovf_mg_restrict": (C.c_int, [C.c_void_p, C.c_int, _d, _d]),
            "ovf_mg_interpolate": (C.c_int, [C.c_void_p, C.c_int, _d, _d, C.c_int]),
            "ovf_mg_coarse_solve": (C.c_int, [C.c_void_p, _d, _d]),
            "ovf_mg_solve": (C.c_int, [C.c_void_p, _d, _d, C.c_long, C.c_long, C.c_int, C.c_int, _d]),
            "ovf_mg_pcg": (C.c_int, [C.c_void_p, _d, _d, C.c_long, C.c_double, C.c_long, C.c_long, C.c_int,
                                     C.c_int, _l, _d, CB]),
            "ovf_smoothing_filter": (None, [_l, C.c_int, C.c_int, _d, _d]),
            "ovf_projection_apply": (None, [C.c_long, C.c_double, _d, _d]),
            "ovf_projection_backprop": (None, [C.c_long, C.c_double, _d, _d, _d]),
            "ovf_top_create": (C.c_void_p, [C.c_void_p, C.c_int, _i, _i, _i, _d, C.c_double]),
            "ovf_top_destroy": (None, [C.c_void_p]),
            "ovf_top_set_solver": (None, [C.c_void_p, C.c_long, C.c_double, C.c_long, C.c_long, C.c_int, C.c_int]),
            "ovf_top_set_vars": (C.c_int, [C.c_void_p, _d]),
            "ovf_top_objective": (C.c_double, [C.c_void_p]),
            "ovf_top_gradient": (C.c_int, [C.c_void_p, _d]),
            "ovf_top_constraint": (C.c_double, [C.c_void_p]),
            "ovf_top_jacobian": (C.c_int, [C.c_void_p, _d]),
            "ovf_top_get_u": (None, [C.c_void_p, _d]),
            "ovf_top_get_physical": (None, [C.c_void_p, _d]),
            "ovf_top_get_design": (None, [C.c_void_p, _d]),
            "ovf_top_last_iters": (C.c_long, [C.c_void_p]),
            "ovf_top_oc_step": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, _l]),
            "ovf_q2_k0": (None, [C.c_double, C.c_double, _d, C.c_int, _d]),
            "ovf_q2_apply_k": (None, [_l, _d, _d, _d, _d]),
            "ovf_q2_smooth": (None, [_l, _d, _d, _u8, _d, _d, C.c_int]),
            "ovf_q2_interp": (None, [_l, _d, _d, C.c_int]),
            "ovf_q2_restrict": (None, [_l, _d, _d]),
            "ovf_q2mg_create": (C.c_void_p, [_l, _d, _d, _u8, C.c_int]),
            "ovf_q2mg_destroy": (None, [C.c_void_p]),
            "ovf_q2mg_level_dims": (None, [C.c_void_p, C.c_int, _l]),
            "ovf_q2mg_level_dirichlet": (None, [C.c_void_p, C.c_int, _u8]),
            "ovf_q2mg_level_ke": (None, [C.c_void_p, C.c_int, _d]),
            "ovf_q2mg_coarsened_k0": (None, [C.c_void_p, _d]),
            "ovf_q2mg_smooth": (C.c_int, [C.c_void_p, C.c_int, _d, _d, C.c_int]),
            "ovf_q2mg_residual": (C.c_int, [C.c_void_p, C.c_int, _d, _d, _d]),
            "ovf_q2mg_coarse_solve": (C.c_int, [C.c_void_p, _d, _d]),
            "ovf_q2mg_vcycle": (C.c_int, [C.c_void_p, _d, _d, C.c_long]),
            "ovf_q2mg_pcg": (C.c_int, [C.c_void_p, _d, _d, C.c_long, C.c_double, C.c_long, _l, _d]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().ovf_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(_d)


def vfield(a, nn):
    """(nn, 3) float64 column-major copy of ``a``."""
    a = np.asarray(a, dtype=np.float64).reshape(nn, 3)
    return np.asfortranarray(a)


def set_num_threads(n):
    lib().ovf_set_num_threads(int(n))


def num_threads():
    return lib().ovf_num_threads()


def cmask_bits(mask):
    return sum(1 << "xyz".index(ch) for ch in mask)


class Sim:
    """Oracle TensorProductSimulator for Q1 hexahedra."""

    def __init__(self, elems, bbox=None):
        self.ne = tuple(int(v) for v in elems)
        if bbox is None:
            bbox = [[0.0, 0.0, 0.0], [float(v) for v in self.ne]]
        self.bbox = np.asarray(bbox, dtype=np.float64)
        ne = (C.c_long * 3)(*self.ne)
        self.h = lib().ovf_sim_create(ne, _dp(np.ascontiguousarray(self.bbox[0])), _dp(np.ascontiguousarray(self.bbox[1])))
        self.nn = (self.ne[0] + 1) * (self.ne[1] + 1) * (self.ne[2] + 1)
        self.numElements = self.ne[0] * self.ne[1] * self.ne[2]

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ovf_sim_destroy(self.h)
            self.h = None

    def setMaterial(self, E, nu):
        lib().ovf_sim_set_material(self.h, E, nu)

    def setParams(self, E0=1.0, Emin=1e-4, gamma=3.0, q=3.0, law=0):
        lib().ovf_sim_set_params(self.h, E0, Emin, gamma, q, law)

    def setDensities(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        assert rho.size == self.numElements
        _check(lib().ovf_sim_set_densities(self.h, _dp(rho)))

    def youngModuli(self):
        out = np.empty(self.numElements)
        lib().ovf_sim_get_Y(self.h, _dp(out))
        return out

    def K0(self):
        out = np.empty(576)
        lib().ovf_sim_get_K0(self.h, _dp(out))
        return out.reshape(24, 24)

    def addDirichletCondition(self, u, minCorner, maxCorner, componentMask="xyz"):
        u = np.ascontiguousarray(u, dtype=np.float64)
        mn = np.ascontiguousarray(minCorner, dtype=np.float64)
        mx = np.ascontiguousarray(maxCorner, dtype=np.float64)
        _check(lib().ovf_sim_add_dirichlet(self.h, _dp(u), _dp(mn), _dp(mx), cmask_bits(componentMask)))

    def setForces(self, f):
        f = vfield(f, self.nn)
        lib().ovf_sim_set_forces(self.h, _dp(f))

    setNodalForces = setForces

    def setGravity(self, g):
        g = np.ascontiguousarray(g, dtype=np.float64)
        lib().ovf_sim_set_gravity(self.h, _dp(g))

    def dirichletMask(self):
        out = np.empty(self.nn, dtype=np.uint8)
        lib().ovf_sim_get_dirichlet_mask(self.h, out.ctypes.data_as(_u8))
        return out

    def setFabricationMaskHeightByLayer(self, l):
        _check(lib().ovf_sim_set_mask_layer(self.h, int(l)))

    def applyK(self, u):
        u = vfield(u, self.nn)
        out = np.asfortranarray(np.empty((self.nn, 3)))
        lib().ovf_sim_apply_k(self.h, _dp(u), _dp(out))
        return out

    def buildLoadVector(self):
        out = np.asfortranarray(np.empty((self.nn, 3)))
        lib().ovf_sim_build_load(self.h, _dp(out))
        return out

    def complianceGradient(self, u):
        u = vfield(u, self.nn)
        out = np.empty(self.numElements)
        lib().ovf_sim_compliance_gradient(self.h, _dp(u), _dp(out))
        return out

    def elementEnergyDensity(self, u):
        u = vfield(u, self.nn)
        out = np.empty(self.numElements)
        lib().ovf_sim_element_energy(self.h, _dp(u), _dp(out))
        return out


class MG:
    """Oracle MultigridSolver (keeps its fine Sim alive)."""

    def __init__(self, sim, levels):
        self.sim = sim
        h = lib().ovf_mg_create(sim.h, int(levels))
        if not h:
            raise RuntimeError(lib().ovf_last_error().decode())
        self.h = h
        self.numLevels = lib().ovf_mg_num_levels(h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ovf_mg_destroy(self.h)
            self.h = None

    def levelElems(self, l):
        ne = (C.c_long * 3)()
        lib().ovf_mg_level_dims(self.h, l, ne)
        return tuple(ne)

    def levelNodes(self, l):
        ne = self.levelElems(l)
        return (ne[0] + 1) * (ne[1] + 1) * (ne[2] + 1)

    def setSymmetricGaussSeidel(self, sym):
        lib().ovf_mg_set_symmetric(self.h, int(bool(sym)))

    def setFabricationMaskHeightByLayer(self, l):
        _check(lib().ovf_mg_set_mask_layer(self.h, int(l)))

    def levelDirichletMask(self, l):
        out = np.empty(self.levelNodes(l), dtype=np.uint8)
        lib().ovf_mg_level_dirichlet_mask(self.h, l, out.ctypes.data_as(_u8))
        return out

    def updateStiffnessMatrices(self):
        _check(lib().ovf_mg_update_stiffness(self.h))

    def applyK(self, l, u):
        nn = self.levelNodes(l)
        u = vfield(u, nn)
        out = np.asfortranarray(np.zeros((nn, 3)))
        _check(lib().ovf_mg_apply_k(self.h, l, _dp(u), _dp(out)))
        return out

    def computeResidual(self, l, u, b):
        nn = self.levelNodes(l)
        u, b = vfield(u, nn), vfield(b, nn)
        out = np.asfortranarray(np.zeros((nn, 3)))
        _check(lib().ovf_mg_residual(self.h, l, _dp(u), _dp(b), _dp(out)))
        return out

    def smooth(self, l, u, b, forward=True):
        nn = self.levelNodes(l)
        u, b = vfield(u, nn).copy(order="F"), vfield(b, nn)
        _check(lib().ovf_mg_smooth(self.h, l, _dp(u), _dp(b), int(bool(forward))))
        return u

    def restrict(self, l, fine):
        fine = vfield(fine, self.levelNodes(l))
        out = np.asfortranarray(np.zeros((self.levelNodes(l + 1), 3)))
        _check(lib().ovf_mg_restrict(self.h, l, _dp(fine), _dp(out)))
        return out

    def interpolate(self, l, coarse, fine=None, accumulate=True):
        coarse = vfield(coarse, self.levelNodes(l + 1))
        nn = self.levelNodes(l)
        out = np.asfortranarray(np.zeros((nn, 3))) if fine is None else vfield(fine, nn).copy(order="F")
        _check(lib().ovf_mg_interpolate(self.h, l, _dp(coarse), _dp(out), int(bool(accumulate))))
        return out

    def coarseSolve(self, b):
        nn = self.levelNodes(self.numLevels - 1)
        b = vfield(b, nn)
        out = np.asfortranarray(np.zeros((nn, 3)))
        _check(lib().ovf_mg_coarse_solve(self.h, _dp(b), _dp(out)))
        return out

    def solve(self, u, f, numSteps, numSmoothingSteps, zeroDirichlet=False, fullMultigrid=False):
        nn = self.sim.nn
        u, f = vfield(u, nn), vfield(f, nn)
        out = np.asfortranarray(np.zeros((nn, 3)))
        _check(lib().ovf_mg_solve(self.h, _dp(u), _dp(f), numSteps, numSmoothingSteps, int(zeroDirichlet),
                                  int(fullMultigrid), _dp(out)))
        return out

    def preconditionedConjugateGradient(self, u, b, maxIter, tol, it_callback=None, mgIterations=1,
                                        mgSmoothingIterations=1, fullMultigrid=False,
                                        dirichletAlreadySatisfied=False):
        nn = self.sim.nn
        x = vfield(u, nn).copy(order="F")
        b = vfield(b, nn)
        iters = C.c_long(0)
        rel = C.c_double(0)
        cb = CB(it_callback) if it_callback else CB()
        _check(lib().ovf_mg_pcg(self.h, _dp(x), _dp(b), int(maxIter), float(tol), int(mgIterations),
                                int(mgSmoothingIterations), int(fullMultigrid), int(dirichletAlreadySatisfied),
                                C.byref(iters), C.byref(rel), cb))
        self.lastIterations = iters.value
        self.lastRelativeResidual = rel.value
        return x


def smoothing_filter(x, dims, radius, ftype):
    dims_c = (C.c_long * 3)(*dims)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lib().ovf_smoothing_filter(dims_c, int(radius), int(ftype), _dp(x), _dp(out))
    return out


def projection_apply(x, beta):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lib().ovf_projection_apply(x.size, float(beta), _dp(x), _dp(out))
    return out


def projection_backprop(g, vars_, beta):
    g = np.ascontiguousarray(g, dtype=np.float64)
    vars_ = np.ascontiguousarray(vars_, dtype=np.float64)
    out = np.empty_like(g)
    lib().ovf_projection_backprop(g.size, float(beta), _dp(g), _dp(vars_), _dp(out))
    return out


class TOP:
    """Oracle TopologyOptimizationProblem with an MG compliance objective.

    ``filters`` is a list of ("smoothing", radius, type) / ("projection", beta).
    """

    def __init__(self, mg, filters, volfrac):
        self.mg = mg
        kinds, radii, types, betas = [], [], [], []
        for f in filters:
            if f[0] == "smoothing":
                kinds.append(0); radii.append(int(f[1])); types.append(int(f[2])); betas.append(0.0)
            else:
                kinds.append(1); radii.append(0); types.append(0); betas.append(float(f[1]))
        n = len(kinds)
        arr_i = C.c_int * max(n, 1)
        arr_d = C.c_double * max(n, 1)
        self.h = lib().ovf_top_create(mg.h, n, arr_i(*kinds), arr_i(*radii), arr_i(*types), arr_d(*betas),
                                      float(volfrac))
        self.ne = mg.sim.numElements

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ovf_top_destroy(self.h)
            self.h = None

    def setSolver(self, cgIter=100, tol=1e-5, mgIterations=1, mgSmoothingIterations=2, fullMultigrid=True,
                  zeroInit=False):
        lib().ovf_top_set_solver(self.h, cgIter, tol, mgIterations, mgSmoothingIterations, int(fullMultigrid),
                                 int(zeroInit))

    def setVars(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check(lib().ovf_top_set_vars(self.h, _dp(x)))

    def evaluateObjective(self):
        return lib().ovf_top_objective(self.h)

    def evaluateObjectiveGradient(self):
        out = np.empty(self.ne)
        _check(lib().ovf_top_gradient(self.h, _dp(out)))
        return out

    def evaluateConstraints(self):
        return np.array([lib().ovf_top_constraint(self.h)])

    def evaluateConstraintsJacobian(self):
        out = np.empty(self.ne)
        _check(lib().ovf_top_jacobian(self.h, _dp(out)))
        return out.reshape(1, -1)

    def u(self):
        out = np.asfortranarray(np.empty((self.mg.sim.nn, 3)))
        lib().ovf_top_get_u(self.h, _dp(out))
        return out

    def designVars(self):
        out = np.empty(self.ne)
        lib().ovf_top_get_design(self.h, _dp(out))
        return out

    def physicalVars(self):
        out = np.empty(self.ne)
        lib().ovf_top_get_physical(self.h, _dp(out))
        return out

    def lastIterations(self):
        return lib().ovf_top_last_iters(self.h)

    def ocStep(self, m=0.2, p=0.5, ctol=1e-6):
        probes = C.c_long(0)
        _check(lib().ovf_top_oc_step(self.h, m, p, ctol, C.byref(probes)))
        return probes.value


# ---- triquadratic voxels ----
def q2_num_nodes(ne):
    return int(np.prod([2 * int(v) + 1 for v in ne]))


def q2_k0(E=1.0, nu=0.3, h=(1.0, 1.0, 1.0), npts=3):
    """81 x 81 triquadratic element stiffness with npts Gauss points per axis."""
    out = np.empty(6561)
    lib().ovf_q2_k0(float(E), float(nu), _dp(np.ascontiguousarray(h, dtype=np.float64)), int(npts), _dp(out))
    return out.reshape(81, 81)


def _ne(ne):
    return (C.c_long * 3)(*[int(v) for v in ne])


def q2_apply_k(ne, K0, Y, u):
    nn = q2_num_nodes(ne)
    u = vfield(u, nn)
    out = np.zeros((nn, 3), order="F")
    lib().ovf_q2_apply_k(_ne(ne), _dp(np.ascontiguousarray(K0, dtype=np.float64)),
                         _dp(np.ascontiguousarray(Y, dtype=np.float64)), _dp(u), _dp(out))
    return out


def q2_smooth(ne, K0, Y, dmask_bits, u, b, forward=True):
    nn = q2_num_nodes(ne)
    x = vfield(u, nn).copy(order="F")
    b = vfield(b, nn)
    m = np.ascontiguousarray(dmask_bits, dtype=np.uint8)
    lib().ovf_q2_smooth(_ne(ne), _dp(np.ascontiguousarray(K0, dtype=np.float64)),
                        _dp(np.ascontiguousarray(Y, dtype=np.float64)), m.ctypes.data_as(_u8), _dp(x), _dp(b),
                        int(bool(forward)))
    return x


def q2_interp(ne_fine, coarse, fine=None, accumulate=False):
    nf = q2_num_nodes(ne_fine)
    nc = q2_num_nodes([int(v) // 2 for v in ne_fine])
    c = vfield(coarse, nc)
    out = np.zeros((nf, 3), order="F") if fine is None else vfield(fine, nf).copy(order="F")
    lib().ovf_q2_interp(_ne(ne_fine), _dp(c), _dp(out), int(bool(accumulate)))
    return out


def q2_restrict(ne_fine, fine):
    nf = q2_num_nodes(ne_fine)
    nc = q2_num_nodes([int(v) // 2 for v in ne_fine])
    f = vfield(fine, nf)
    out = np.zeros((nc, 3), order="F")
    lib().ovf_q2_restrict(_ne(ne_fine), _dp(f), _dp(out))
    return out


class Q2Multigrid:
    """The reference's triquadratic hierarchy (MultigridSolver<double, 2, 2, 2>): halved Q2 meshes,
    level-1 operator from the 8 coarsened full-density element matrices, Galerkin element
    matrices below, dense Cholesky on the coarsest free DOFs."""

    def __init__(self, ne, K0, Y, dmask_bits, coarsenings):
        self.ne = [int(v) for v in ne]
        self.coarsenings = int(coarsenings)
        m = np.ascontiguousarray(dmask_bits, dtype=np.uint8)
        self.h = lib().ovf_q2mg_create(_ne(ne), _dp(np.ascontiguousarray(K0, dtype=np.float64)),
                                       _dp(np.ascontiguousarray(Y, dtype=np.float64)), m.ctypes.data_as(_u8),
                                       int(coarsenings))
        if not self.h:
            raise RuntimeError(lib().ovf_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().ovf_q2mg_destroy(self.h)
            self.h = None

    def level_ne(self, l):
        out = (C.c_long * 3)()
        lib().ovf_q2mg_level_dims(self.h, int(l), out)
        return [int(v) for v in out]

    def num_nodes(self, l):
        return q2_num_nodes(self.level_ne(l))

    def dirichlet_bits(self, l):
        out = np.empty(self.num_nodes(l), dtype=np.uint8)
        lib().ovf_q2mg_level_dirichlet(self.h, int(l), out.ctypes.data_as(_u8))
        return out

    def element_matrices(self, l):
        ne = self.level_ne(l)
        out = np.empty(int(np.prod(ne)) * 6561)
        lib().ovf_q2mg_level_ke(self.h, int(l), _dp(out))
        return out.reshape(-1, 81, 81)

    def coarsened_k0(self):
        out = np.empty(8 * 6561)
        lib().ovf_q2mg_coarsened_k0(self.h, _dp(out))
        return out.reshape(8, 81, 81)

    def smooth(self, l, u, b, forward=True):
        nn = self.num_nodes(l)
        x = vfield(u, nn).copy(order="F")
        _check(lib().ovf_q2mg_smooth(self.h, int(l), _dp(x), _dp(vfield(b, nn)), int(bool(forward))))
        return x

    def residual(self, l, u, b):
        nn = self.num_nodes(l)
        out = np.zeros((nn, 3), order="F")
        _check(lib().ovf_q2mg_residual(self.h, int(l), _dp(vfield(u, nn)), _dp(vfield(b, nn)), _dp(out)))
        return out

    def coarse_solve(self, b):
        nn = self.num_nodes(self.coarsenings)
        out = np.zeros((nn, 3), order="F")
        _check(lib().ovf_q2mg_coarse_solve(self.h, _dp(vfield(b, nn)), _dp(out)))
        return out

    def vcycle(self, b, sweeps):
        nn = self.num_nodes(0)
        out = np.zeros((nn, 3), order="F")
        _check(lib().ovf_q2mg_vcycle(self.h, _dp(vfield(b, nn)), _dp(out), int(sweeps)))
        return out

    def pcg(self, b, maxIter=500, tol=1e-8, sweeps=2, x0=None):
        nn = self.num_nodes(0)
        x = np.zeros((nn, 3), order="F") if x0 is None else vfield(x0, nn).copy(order="F")
        it = C.c_long(0)
        rr = C.c_double(0.0)
        _check(lib().ovf_q2mg_pcg(self.h, _dp(x), _dp(vfield(b, nn)), int(maxIter), float(tol), int(sweeps),
                                  C.byref(it), C.byref(rr)))
        return x, it.value, rr.value



def _lbl_init(method):
    if method == "zero":
        return "zero", 0
    if method == "constant":
        return "fd", 1
    if method == "fd":
        return "fd", 2
    if isinstance(method, str) and method.startswith("N="):
        return "subspace", int(method[2:])
    raise RuntimeError("Unrecognized method " + str(method))


def layer_by_layer(sim, mg, method="N=3", zero_init=True, layer_increment=1, max_iter=500, tol=1e-8,
                   mg_iterations=1, mg_smoothing_iterations=1, fmg=False, u_full=None):
    """Restatement of LayerByLayerEvaluator::run (LayerByLayer.hh:223-296) with its initial-guess
    generators (LayerByLayer.hh:55-209): heights ny, ny - inc, ..., each solved from a guess built
    from the previous heights' solutions (newest first, at most N kept; pushed after every height
    but the last). "fd": 0, u(0) or 2 u(0) - u(1); "constant": u(0); "N=<s>": the Galerkin
    projection onto the last s solutions, A_ij = u_i . K u_j, b_i = u_i . f for the NEW mask
    (formed directly: the reference maintains the same quantities by recurrences,
    LayerByLayer.hh:162-204), c = JacobiSVD(A).solve(b), i.e. the minimum-norm least-squares
    solution with singular values <= s eps sigma_max dropped. Guesses are zero on detached nodes.
    Returns (layers, compliances f.u over nondetached nodes, PCG iterations, gradient sum,
    full-design solution)."""
    kind, nmax = _lbl_init(method)
    ne = sim.ne
    ny = ne[1]
    nn1 = (ne[1] + 1, ne[2] + 1)
    jrow = (np.arange(sim.nn) // nn1[1]) % nn1[0]
    hist = []
    layers, comps, iters = [], [], []
    grad = np.zeros(sim.numElements)
    l = ny
    while l > 0:
        sim.setFabricationMaskHeightByLayer(l)
        mg.setFabricationMaskHeightByLayer(l)
        live = jrow <= l  # nondetached node rows
        f = sim.buildLoadVector()
        s = len(hist)
        if not zero_init and l == ny and u_full is not None:
            g = u_full.copy()
        elif kind == "zero" or s == 0:
            g = np.zeros((sim.nn, 3))
        elif kind == "fd":
            g = hist[0].copy() if s == 1 else 2.0 * hist[0] - hist[1]
        else:
            Ku = [sim.applyK(u) for u in hist]
            A = np.array([[float(np.sum((hist[i] * Ku[j])[live])) for j in range(s)] for i in range(s)])
            A = 0.5 * (A + A.T)
            b = np.array([float(np.sum((hist[i] * f)[live])) for i in range(s)])
            c = np.linalg.lstsq(A, b, rcond=s * np.finfo(np.float64).eps)[0]
            g = sum(c[i] * hist[i] for i in range(s))
        g[~live] = 0.0
        u = mg.preconditionedConjugateGradient(g, f, max_iter, tol, None, mg_iterations, mg_smoothing_iterations, fmg)
        layers.append(l)
        comps.append(float(np.sum((f * u)[live])))
        iters.append(mg.lastIterations)
        grad += sim.complianceGradient(u)
        if l == ny:
            u_full = u.copy()
        if l >= layer_increment and nmax > 0:
            hist.insert(0, u.copy())
            del hist[nmax:]
        l -= min(layer_increment, l)
    return np.array(layers), np.array(comps), np.array(iters), grad, u_full
