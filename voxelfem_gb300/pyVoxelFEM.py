"""Drop-in counterpart of VoxelFEM's pybind11 module ``pyVoxelFEM`` for the solve path.

Names, arguments, defaults, return shapes and error behaviour follow
python_bindings/VoxelFEM.cc (pyVoxelFEM) so that reference scripts run
unchanged on the GB300 library. Every numerical operation runs in the CUDA
library through the C ABI of include/vfem.h; nodal fields are float64 arrays of
shape (numNodes, 3) and element fields flat (numElements,) arrays in row-major
grid order, as the reference's Eigen type casters produce.

Scope: 3D trilinear voxels in double precision ([1, 1, 1], NumberType.DOUBLE).
Multigrid solvers additionally expose a mixed-precision mode
(``setPrecision("mixed")``: FP32 V-cycle inside FP64 CG) that the reference
does not have.
"""
import ctypes as C
import enum
import json
import os

import numpy as np

from . import _capi
from ._capi import check, ptr


class NumberType(enum.IntEnum):
    DOUBLE = 0
    FLOAT = 1


class InterpolationLaw(enum.IntEnum):
    SIMP = 0
    RAMP = 1


SIMP = InterpolationLaw.SIMP
RAMP = InterpolationLaw.RAMP


def _lib():
    return _capi.load()


def _as_vfield(u, nn, nc=3):
    a = np.asarray(u, dtype=np.float64)
    if a.shape != (nn, nc):
        if a.size == nc * nn and a.ndim == 1:
            a = a.reshape(nn, nc)
        else:
            raise RuntimeError("Invalid input size")
    return np.asfortranarray(a)


def _new_vfield(nn, nc=3):
    return np.zeros((nn, nc), order="F")


def _as_elems(x, ne):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
    if a.size != ne:
        raise RuntimeError("Invalid input size")
    return a


def _cmask(mask, dim=3):
    bits = 0
    for ch in mask:
        if ch not in "xyz":
            raise RuntimeError("Invalid component mask " + mask)
        bits |= 1 << "xyz".index(ch)
    return bits & ((1 << dim) - 1)


def _arr3(v):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))
    return a


class ElasticityTensor:
    """The isotropic elasticity tensor held by a simulator's ``ETensor`` property: it unpacks and
    compares as the pair (young, poisson), and ``setIsotropic(E, nu)`` is the method the
    reference's scripts call on MeshFEM's tensor (``e = tps.ETensor; e.setIsotropic(1, nu);
    tps.ETensor = e``)."""

    def __init__(self, young=1.0, poisson=0.0):
        self.young, self.poisson = float(young), float(poisson)

    def setIsotropic(self, young, poisson):
        self.young, self.poisson = float(young), float(poisson)

    def __iter__(self):
        return iter((self.young, self.poisson))

    def __getitem__(self, i):
        return (self.young, self.poisson)[i]

    def __len__(self):
        return 2

    def __eq__(self, other):
        try:
            return tuple(self) == tuple(other)
        except TypeError:
            return NotImplemented

    def __repr__(self):
        return "ElasticityTensor(young=%g, poisson=%g)" % (self.young, self.poisson)


def TensorProductSimulator(degreesPerDimension, domainBBox, elementsPerDimension, numberType=NumberType.DOUBLE):
    """Factory of pyVoxelFEM.TensorProductSimulator (VoxelFEM.cc:423-430)."""
    degs = [int(d) for d in degreesPerDimension]
    if int(numberType) != int(NumberType.DOUBLE) or degs not in ([1, 1], [1, 1, 1], [2, 2, 2]):
        raise RuntimeError("No template instantiation matching degreesPerDimension/number type!")
    if degs == [2, 2, 2]:
        return TensorProductSimulator_3D_Q2(domainBBox, elementsPerDimension)
    if degs == [1, 1]:
        return TensorProductSimulator_2D(domainBBox, elementsPerDimension)
    return TensorProductSimulator_3D(domainBBox, elementsPerDimension)


class TensorProductSimulator_3D:
    """TensorProductSimulator<double, 1, 1, 1> (TensorProductSimulator.hh:166-623)."""

    _nc = 3

    def __init__(self, domainBBox, elementsPerDimension):
        bb = [np.asarray(domainBBox[0], dtype=np.float64).reshape(3), np.asarray(domainBBox[1], dtype=np.float64).reshape(3)]
        ne = np.ascontiguousarray(np.asarray(elementsPerDimension, dtype=np.int64).reshape(3))
        h = C.c_void_p()
        check(_lib().vfem_grid_create(ne.ctypes.data_as(_capi._i64), _capi.dptr(np.ascontiguousarray(bb[0])),
                                      _capi.dptr(np.ascontiguousarray(bb[1])), C.byref(h)))
        self._h = h
        self._bbox = (bb[0].copy(), bb[1].copy())
        self._ne = tuple(int(v) for v in ne)
        self._nn = (self._ne[0] + 1) * (self._ne[1] + 1) * (self._ne[2] + 1)
        self._nel = self._ne[0] * self._ne[1] * self._ne[2]
        self._forces = np.zeros((self._nn, 3), order="F")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_grid_destroy(h)
            self._h = None

    # --- sizes / geometry ---
    def numNodes(self):
        return self._nn

    def numElements(self):
        return self._nel

    @property
    def gridShape(self):
        return np.array(self._ne)

    @property
    def NbElementsPerDimension(self):
        return np.array(self._ne)

    @property
    def NbNodesPerDimension(self):
        return np.array([n + 1 for n in self._ne])

    @property
    def domain(self):
        return (self._bbox[0].copy(), self._bbox[1].copy())

    bbox = domain

    @property
    def dx(self):
        return (self._bbox[1] - self._bbox[0]) / np.array(self._ne)

    @property
    def elementVolume(self):
        return float(np.prod(self.dx))

    def nodePosition(self, ni):
        nn = self.NbNodesPerDimension
        i, rem = divmod(int(ni), nn[1] * nn[2])
        j, k = divmod(rem, nn[2])
        return self._bbox[0] + np.array([i, j, k]) * self.dx

    def elementNodes(self, ei):
        ne = self._ne
        i, rem = divmod(int(ei), ne[1] * ne[2])
        j, k = divmod(rem, ne[2])
        nn = self.NbNodesPerDimension
        return np.array([((i + (l >> 2 & 1)) * nn[1] + j + (l >> 1 & 1)) * nn[2] + k + (l & 1) for l in range(8)])

    def elemNodeGlobalIndex(self, ei, n):
        return int(self.elementNodes(ei)[int(n)])

    def elementIndexForGridCell(self, cellIdxs):
        i, j, k = (int(v) for v in cellIdxs)
        return (i * self._ne[1] + j) * self._ne[2] + k

    # --- material ---
    def readMaterial(self, materialPath):
        with open(materialPath) as f:
            mat = json.load(f)
        if mat.get("type", "isotropic_material") not in ("isotropic_material", "isotropic"):
            raise RuntimeError("Only isotropic materials are supported")
        self.ETensor = (float(mat["young"]), float(mat["poisson"]))

    @property
    def ETensor(self):
        E, nu = C.c_double(), C.c_double()
        check(_lib().vfem_grid_get_etensor(self._h, C.byref(E), C.byref(nu)))
        return ElasticityTensor(E.value, nu.value)

    @ETensor.setter
    def ETensor(self, value):
        E, nu = value
        check(_lib().vfem_grid_set_etensor(self._h, float(E), float(nu)))

    def _params(self):
        v = [C.c_double() for _ in range(4)]
        law = C.c_int()
        check(_lib().vfem_grid_get_material_params(self._h, *[C.byref(x) for x in v], C.byref(law)))
        return [x.value for x in v] + [law.value]

    def _set_param(self, idx, value):
        p = self._params()
        p[idx] = value
        check(_lib().vfem_grid_set_material_params(self._h, p[0], p[1], p[2], p[3], int(p[4])))

    E_0 = property(lambda self: self._params()[0], lambda self, v: self._set_param(0, float(v)))
    E_min = property(lambda self: self._params()[1], lambda self, v: self._set_param(1, float(v)))
    gamma = property(lambda self: self._params()[2], lambda self, v: self._set_param(2, float(v)))
    q = property(lambda self: self._params()[3], lambda self, v: self._set_param(3, float(v)))
    interpolationLaw = property(lambda self: InterpolationLaw(self._params()[4]),
                                lambda self, v: self._set_param(4, int(v)))

    @property
    def gravity(self):
        g = np.zeros(3)
        check(_lib().vfem_grid_get_gravity(self._h, _capi.dptr(g)))
        return g

    @gravity.setter
    def gravity(self, g):
        check(_lib().vfem_grid_set_gravity(self._h, _capi.dptr(_arr3(g))))

    def fullDensityElementStiffnessMatrix(self):
        K = np.empty(576)
        check(_lib().vfem_grid_get_k0(self._h, _capi.dptr(K)))
        return K.reshape(24, 24)

    def k0IsCube(self):
        """Whether K0 has the cube structure the fast fine-level kernels use (diagnostic)."""
        v = C.c_int32()
        check(_lib().vfem_grid_k0_is_cube(self._h, C.byref(v)))
        return bool(v.value)

    def elementStiffnessMatrix(self, ei):
        return self.elementYoungModulusScaleFactor(ei) * self.fullDensityElementStiffnessMatrix()

    def clearCachedElementStiffness(self):
        """No per-element stiffness cache exists here (elements are scaled copies of K0)."""

    # --- mesh, sampling and BC fields (TensorProductSimulator.hh:689-712, 746-778, 1161-1179) ---
    def mesh(self):
        return self

    def getMesh(self):
        """(V, F): node positions (nn, 3) and hexahedra (ne, 8) in Gmsh node order."""
        nn = self.NbNodesPerDimension
        I, J, K = np.meshgrid(np.arange(nn[0]), np.arange(nn[1]), np.arange(nn[2]), indexing="ij")
        V = self._bbox[0] + np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1) * self.dx
        ne = self._ne
        i, j, k = np.meshgrid(np.arange(ne[0]), np.arange(ne[1]), np.arange(ne[2]), indexing="ij")
        base = (i.ravel() * nn[1] + j.ravel()) * nn[2] + k.ravel()
        off = [(l >> 2 & 1) * nn[1] * nn[2] + (l >> 1 & 1) * nn[2] + (l & 1) for l in range(8)]
        order = [0, 1, 3, 2, 4, 5, 7, 6]  # pairs (0,1), (3,2), (4,5), (7,6)
        F = np.stack([base + off[l] for l in order], axis=1)
        return V, F

    def sampleNodalField(self, u, p):
        """Trilinear interpolation of the nodal field u (nn x c) at the rows of p, each point
        clamped into the domain first."""
        u = np.asarray(u, dtype=np.float64).reshape(self._nn, -1)
        p = np.clip(np.atleast_2d(np.asarray(p, dtype=np.float64)), self._bbox[0], self._bbox[1])
        t = (p - self._bbox[0]) / self.dx
        e = np.minimum(np.floor(t).astype(np.int64), np.array(self._ne) - 1)
        x = t - e
        nn = self.NbNodesPerDimension
        out = np.zeros((p.shape[0], u.shape[1]))
        for l in range(8):
            b = [(l >> 2) & 1, (l >> 1) & 1, l & 1]
            w = np.prod([x[:, d] if b[d] else 1.0 - x[:, d] for d in range(3)], axis=0)
            n = ((e[:, 0] + b[0]) * nn[1] + e[:, 1] + b[1]) * nn[2] + e[:, 2] + b[2]
            out += w[:, None] * u[n]
        return out

    def getBCIndicatorField(self):
        """Per node: Dirichlet component bits + 8 x force component bits."""
        d = self.getDirichletMask()
        f = self.getForceMask()
        return (d[:, 0] * 1 + d[:, 1] * 2 + d[:, 2] * 4 + 8 * (f[:, 0] * 1 + f[:, 1] * 2 + f[:, 2] * 4)).astype(np.float64)

    def getK(self):
        """The assembled stiffness matrix (3 nn x 3 nn, DOF 3 n + c) as a scipy CSC matrix."""
        import scipy.sparse as sp
        K0 = self.fullDensityElementStiffnessMatrix()
        Y = self.getYoungModulusScaleFactor()
        ne = self._ne
        nn = self.NbNodesPerDimension
        i, j, k = np.meshgrid(np.arange(ne[0]), np.arange(ne[1]), np.arange(ne[2]), indexing="ij")
        base = (i.ravel() * nn[1] + j.ravel()) * nn[2] + k.ravel()
        nodes = np.stack([base + (l >> 2 & 1) * nn[1] * nn[2] + (l >> 1 & 1) * nn[2] + (l & 1) for l in range(8)], 1)
        dofs = (3 * nodes[:, :, None] + np.arange(3)[None, None, :]).reshape(-1, 24)
        rows = np.repeat(dofs, 24, axis=1).ravel()
        cols = np.tile(dofs, (1, 24)).ravel()
        vals = (Y[:, None] * K0.ravel()[None, :]).ravel()
        return sp.csc_matrix((vals, (rows, cols)), shape=(3 * self._nn, 3 * self._nn))

    def solveWithImposedLoads(self):
        return self.solve(self.buildLoadVector())

    # --- coarser and intermediate simulators (TensorProductSimulator.hh:793-803, 1852-1992, 1994-2035) ---
    def _copy_material(self, other):
        other.ETensor = self.ETensor
        other.E_min = self.E_min
        other.E_0 = self.E_0
        other.gamma = self.gamma

    def downsample(self, downsamplingLevels):
        """A coarser simulator (elements / 2^levels, same domain and material), no BCs applied."""
        f = 2 ** int(downsamplingLevels)
        ne = np.array(self._ne)
        if (ne % f).any():
            raise RuntimeError("Grid size must be divisible by 2^downsamplingLevels")
        c = TensorProductSimulator_3D([self._bbox[0], self._bbox[1]], ne // f)
        self._copy_material(c)
        return c

    def _factor(self, coarse):
        f = self._ne[0] // coarse._ne[0]
        if any(f * coarse._ne[d] != self._ne[d] for d in range(3)):
            raise RuntimeError("Invalid downsampled simulator")
        return f

    def downsampleDensityFieldTo(self, densities, coarseTPS):
        f = self._factor(coarseTPS)
        rho = np.asarray(densities, dtype=np.float64).reshape(-1)
        if rho.size != self._nel:
            raise RuntimeError("Invalid input densities size (%d vs %d)" % (rho.size, self._nel))
        a = rho.reshape(self._ne)
        c = a.reshape(self._ne[0] // f, f, self._ne[1] // f, f, self._ne[2] // f, f).sum(axis=(1, 3, 5)) / f ** 3
        coarseTPS.setDensities(c.ravel())

    def upsampleDensityGradientFrom(self, coarseTPS, g_coarse):
        f = self._factor(coarseTPS)
        g = np.asarray(g_coarse, dtype=np.float64).reshape(-1)
        if g.size != coarseTPS._nel:
            raise RuntimeError("Invalid coarse gradient size")
        gc = g.reshape(coarseTPS._ne)
        return (np.repeat(np.repeat(np.repeat(gc, f, 0), f, 1), f, 2) / f ** 3).ravel()

    def setDensitiesFromCoarseGrid(self, upscalingFactor, rho):
        f = int(upscalingFactor)
        rho = np.asarray(rho, dtype=np.float64).reshape(-1)
        if self._nel != f ** 3 * rho.size:
            raise RuntimeError("Incorrect rho size")
        rc = rho.reshape(tuple(v // f for v in self._ne))
        self.setDensities(np.repeat(np.repeat(np.repeat(rc, f, 0), f, 1), f, 2).ravel())

    def getIntermediateFabricationShape(self, yfrac, validateBoundaryConditions=True, law=None):
        """The partial build up to height fraction yfrac along y: same material, the densities of
        the lower layers, self-weight gravity and the build plate (y = min) fixed."""
        if yfrac < 0 or yfrac > 1:
            raise RuntimeError("hfrac is out of bounds")
        full = self._ne[1]
        h = int(round(yfrac * full))
        if abs(yfrac * full - h) > 1e-10:
            raise RuntimeError("hfrac chops off a noninteger number of element layers")
        lo, hi = self._bbox[0].copy(), self._bbox[1].copy()
        hi[1] = lo[1] + yfrac * (self._bbox[1][1] - lo[1])
        ne = np.array(self._ne)
        ne[1] = h
        r = TensorProductSimulator_3D([lo, hi], ne)
        if law is not None:
            r.interpolationLaw = law
        r.ETensor = self.ETensor
        self.transferDensitiesToIntermediateFabricationShape(r)
        r.E_min, r.E_0, r.gamma = self.E_min, self.E_0, self.gamma
        g = self.gravity
        if not np.any(g):
            if validateBoundaryConditions:
                raise RuntimeError("Original simulator has unexpected boundary conditions for layer-by-layer simulation")
            g = np.array([0.0, -1.0, 0.0])
        r.gravity = g
        if validateBoundaryConditions:
            bad = RuntimeError("Original simulator has unexpected boundary conditions for layer-by-layer simulation")
            if self.getForceMask().any():
                raise bad
            m = self.getDirichletMask()
            nn = self.NbNodesPerDimension
            jrow = (np.arange(self._nn) // nn[2]) % nn[1]
            if not m[jrow == 0].all() or m[jrow != 0].any():
                raise bad
        r.addDirichletCondition([0.0, 0.0, 0.0], [lo[0], lo[1], lo[2]], [hi[0], lo[1], hi[2]], "xyz")
        return r

    def _check_intermediate(self, itps):
        if itps._ne[0] != self._ne[0] or itps._ne[2] != self._ne[2] or itps._ne[1] > self._ne[1]:
            raise RuntimeError("Intermediate shape is of unexpected size")

    def transferDensitiesToIntermediateFabricationShape(self, intermediateTPS):
        rho = self.getDensities().reshape(self._ne)
        intermediateTPS.setDensities(rho[:, :intermediateTPS._ne[1], :].ravel())

    def transferVFieldToIntermediateFabricationShape(self, intermediateTPS, u):
        self._check_intermediate(intermediateTPS)
        nn = self.NbNodesPerDimension
        u = np.asarray(u, dtype=np.float64).reshape(nn[0], nn[1], nn[2], -1)
        ny = intermediateTPS._ne[1] + 1
        return np.asfortranarray(u[:, :ny, :, :].reshape(-1, u.shape[-1]))

    def accumElementScalarFieldFromIntermediateFabricationShape(self, intermediateTPS, rho_in, rho_accum):
        """rho_accum (this grid's elements, modified in place) += rho_in on the partial build's cells."""
        acc = rho_accum.reshape(self._ne)
        acc[:, :intermediateTPS._ne[1], :] += np.asarray(rho_in, dtype=np.float64).reshape(intermediateTPS._ne)

    # --- densities ---
    def getDensities(self):
        out = np.empty(self._nel)
        check(_lib().vfem_grid_get_densities(self._h, ptr(out)))
        return out

    def setDensities(self, rho):
        if np.asarray(rho).size != self._nel:
            raise RuntimeError("Incorrect rho size")
        a = _as_elems(rho, self._nel)
        check(_lib().vfem_grid_set_densities(self._h, ptr(a)))

    def setUniformDensities(self, density):
        check(_lib().vfem_grid_set_uniform_densities(self._h, float(density)))

    def setDensity(self, ei, value):
        if value > 1.0 or value < 0:
            raise RuntimeError("Density value (%g) has to be in between 0 and 1" % value)
        rho = self.getDensities()
        rho[int(ei)] = value
        self.setDensities(rho)

    def elementDensity(self, ei):
        return float(self.getDensities()[int(ei)])

    def getYoungModulusScaleFactor(self):
        out = np.empty(self._nel)
        check(_lib().vfem_grid_get_young_moduli(self._h, ptr(out)))
        return out

    def elementYoungModulusScaleFactor(self, ei):
        return float(self.getYoungModulusScaleFactor()[int(ei)])

    # --- boundary conditions ---
    def addDirichletCondition(self, u, minCorner, maxCorner, componentMask="xyz"):
        check(_lib().vfem_grid_add_dirichlet(self._h, _capi.dptr(_arr3(u)), _capi.dptr(_arr3(minCorner)),
                                             _capi.dptr(_arr3(maxCorner)), _cmask(componentMask)))

    def applySymmetryConditions(self, symmetry_axes, minMaxFace=(False, False, False)):
        ax = (C.c_int * 3)(*[int(bool(v)) for v in symmetry_axes])
        mf = (C.c_int * 3)(*[int(bool(v)) for v in minMaxFace])
        check(_lib().vfem_grid_apply_symmetry(self._h, ax, mf))

    def setNodalForces(self, forces):
        """Dense nodal force boundary condition (BCBuilder::setForce for every node)."""
        f = _as_vfield(forces, self._nn)
        self._forces = f.copy(order="F")
        check(_lib().vfem_grid_set_nodal_forces(self._h, ptr(f)))

    def applyDisplacementsAndLoadsFromFile(self, bcPath):
        apply_bc_file(self, bcPath)

    def getDirichletMask(self):
        m = np.zeros(self._nn, dtype=np.uint8)
        check(_lib().vfem_grid_get_dirichlet_mask(self._h, m.ctypes.data_as(_capi._u8)))
        return np.stack([(m >> c) & 1 for c in range(3)], axis=1).astype(bool)

    def getForceMask(self):
        return self._forces != 0

    def getDirichletVarsAndValues(self):
        m = self.getDirichletMask()
        nodes, comps = np.nonzero(m)
        return (list(3 * nodes + comps), [0.0] * len(nodes))

    # --- layer-by-layer fabrication mask ---
    def setFabricationMaskHeightByLayer(self, l):
        check(_lib().vfem_grid_set_mask_layer(self._h, int(l)))

    def getFabricationMaskHeight(self):
        h = C.c_double()
        check(_lib().vfem_grid_get_mask_height(self._h, C.byref(h)))
        return h.value

    # --- physics ---
    def applyK(self, u):
        u = _as_vfield(u, self._nn)
        out = _new_vfield(self._nn)
        check(_lib().vfem_grid_apply_k(self._h, ptr(u), ptr(out)))
        return out

    def buildLoadVector(self):
        out = _new_vfield(self._nn)
        check(_lib().vfem_grid_build_load(self._h, ptr(out)))
        return out

    def complianceGradient(self, u):
        u = _as_vfield(u, self._nn)
        out = np.empty(self._nel)
        check(_lib().vfem_grid_compliance_gradient(self._h, ptr(u), ptr(out)))
        return out

    def adjointSensitivity(self, lam, u, loadWeight=1.0, stiffnessWeight=1.0):
        """lam^T (loadWeight df/drho - stiffnessWeight dK/drho u) per element (fused kernel)."""
        lam = _as_vfield(lam, self._nn)
        u = _as_vfield(u, self._nn)
        out = np.empty(self._nel)
        check(_lib().vfem_grid_adjoint_sensitivity(self._h, ptr(lam), ptr(u), float(loadWeight),
                                                   float(stiffnessWeight), ptr(out)))
        return out

    def elementEnergyDensity(self, u):
        u = _as_vfield(u, self._nn)
        out = np.empty(self._nel)
        check(_lib().vfem_grid_element_energy(self._h, ptr(u), ptr(out)))
        return out

    def solve(self, f):
        """Direct solve (TensorProductSimulator::solve) through a zero-coarsening hierarchy."""
        mg = self.multigridSolver(0)
        return mg.preconditionedConjugateGradient(np.zeros((self._nn, 3)), f, 1, 0.0)

    def multigridSolver(self, numCoarseningLevels):
        return MultigridSolver(self, int(numCoarseningLevels))


def apply_bc_file(tps, path):
    """Minimal reader of the reference's `.bc` JSON regions ("box%" or "box"; types
    "dirichlet[x|y|z...]" and "force"; forces split equally over the region's nodes,
    TensorProductSimulator.hh:600-652). A 2D simulator reads the first two entries of each
    vector (the reference's 2D files carry a third, zero coordinate)."""
    with open(path) as f:
        spec = json.load(f)
    dim = tps._nc
    lo, hi = tps.domain
    size = hi - lo
    nn = tps.NbNodesPerDimension
    dx = tps.dx
    grids = np.meshgrid(*[np.arange(nn[d]) for d in range(dim)], indexing="ij")
    pos = np.stack([lo[d] + grids[d].ravel() * dx[d] for d in range(dim)], axis=1)
    forces = np.zeros((tps.numNodes(), dim))
    have_force = False
    vec = lambda v: np.asarray(v, dtype=float).reshape(-1)[:dim]
    for reg in spec["regions"]:
        if "box%" in reg:
            b = reg["box%"]
            mn = lo + vec(b["minCorner"]) * size
            mx = lo + vec(b["maxCorner"]) * size
        elif "box" in reg:
            mn = vec(reg["box"]["minCorner"])
            mx = vec(reg["box"]["maxCorner"])
        else:
            raise RuntimeError("Unsupported boundary condition region")
        typ = reg["type"]
        val = vec(reg["value"])
        inside = np.all((pos >= mn) & (pos <= mx), axis=1)
        if typ.startswith("dirichlet"):
            comps = typ[len("dirichlet"):] or "xyz"
            if not inside.any():
                raise RuntimeError("Dirichlet region unmatched")
            tps.addDirichletCondition(val, mn, mx, comps)
        elif typ == "force":
            idx = np.nonzero(inside)[0]
            if idx.size == 0:
                raise RuntimeError("Force constraint region unmatched")
            forces[idx] = val / idx.size
            have_force = True
        else:
            raise RuntimeError('Illegal constraint type, only "dirichlet" and "force" accepted')
    if have_force:
        tps.setNodalForces(forces)


class _LevelSimulator:
    """Read-only view of a coarse level (MultigridSolver::getSimulator(l), l > 0)."""

    def __init__(self, mg, l):
        self._mg, self._l = mg, l
        ne = np.zeros(3, dtype=np.int64)
        check(_lib().vfem_mg_level_dims(mg._h, l, ne.ctypes.data_as(_capi._i64)))
        self._ne = tuple(int(v) for v in ne)

    def numNodes(self):
        return int(np.prod([n + 1 for n in self._ne]))

    def numElements(self):
        return int(np.prod(self._ne))

    @property
    def NbElementsPerDimension(self):
        return np.array(self._ne)

    gridShape = NbElementsPerDimension

    @property
    def NbNodesPerDimension(self):
        return np.array([n + 1 for n in self._ne])

    def getDirichletMask(self):
        m = np.zeros(self.numNodes(), dtype=np.uint8)
        check(_lib().vfem_mg_level_dirichlet_mask(self._mg._h, self._l, m.ctypes.data_as(_capi._u8)))
        return np.stack([(m >> c) & 1 for c in range(3)], axis=1).astype(bool)


class MultigridSolver:
    """MultigridSolver<double, 1, 1, 1> (MultigridSolver.hh); created by tps.multigridSolver(levels).
    Constructed on a 2D simulator it is a MultigridSolver2D."""

    def __new__(cls, tps=None, numCoarseningLevels=0):
        if cls is MultigridSolver and isinstance(tps, TensorProductSimulator_2D):
            return MultigridSolver2D(tps, numCoarseningLevels)
        return super().__new__(cls)

    def __init__(self, tps, numCoarseningLevels):
        h = C.c_void_p()
        check(_lib().vfem_mg_create(tps._h, int(numCoarseningLevels), C.byref(h)))
        self._h = h
        self._tps = tps  # keeps the fine simulator alive (MultigridSolver.hh:1164)
        n = C.c_int()
        check(_lib().vfem_mg_num_levels(h, C.byref(n)))
        self.numLevels = n.value
        self._prec = "fp64"
        self.lastStats = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_mg_destroy(h)
            self._h = None

    def _nn(self, l):
        return self.getSimulator(l).numNodes()

    def getSimulator(self, l):
        if l == 0:
            return self._tps
        if l < 0 or l >= self.numLevels:
            raise IndexError("level out of range")
        return _LevelSimulator(self, l)

    def setPrecision(self, precision="fp64", outerMatvec="df"):
        """'fp64' (the reference's method) or 'mixed' (FP32 V-cycle in FP64 CG); the outer
        matvec of the mixed mode is 'df' (FP64-class without FP64 arithmetic: tensor cores for
        cube voxels with a rational Poisson ratio, else double-float), 'df-simt' (double-float
        on the FP32 units) or 'fp64'."""
        p = {"fp64": 0, "mixed": 1}[precision]
        m = {"fp64": 0, "df": 1, "df-simt": 2}[outerMatvec]
        check(_lib().vfem_mg_set_precision(self._h, p, m))
        self._prec = precision

    SWEEP_FORMS = {"colours": 0, "lines": 1, "planes": 2, "staged": 3}

    def setSweepForm(self, form):
        """Form of the FP32 fine Gauss-Seidel sweep of the mixed V-cycle: 'lines' (default),
        'staged', 'colours' or 'planes'; every form gives identical iterates."""
        check(_lib().vfem_mg_set_sweep_form(self._h, self.SWEEP_FORMS[form]))

    def setStencilStorage(self, kind="fp32"):
        """Mixed precision: 'bf16' stores the smoothing levels' assembled stencils in bf16 (half
        the bytes a colour pass streams), 'fp32' (default) in FP32; both are applied in FP32."""
        check(_lib().vfem_mg_set_stencil_bf16(self._h, {"fp32": 0, "bf16": 1}[kind]))

    def stiffnessRebuilds(self):
        """(full, band): hierarchy rebuilds run in full and as band-partial updates after a
        fabrication-mask change (diagnostic)."""
        full, band = C.c_int64(), C.c_int64()
        check(_lib().vfem_mg_stiffness_rebuilds(self._h, C.byref(full), C.byref(band)))
        return full.value, band.value

    def outerMatvecKind(self):
        """'fp64', 'df-simt' or 'tensor': the outer matvec the mixed solve uses now."""
        k = C.c_int()
        check(_lib().vfem_mg_outer_matvec_kind(self._h, C.byref(k)))
        return {0: "fp64", 1: "df-simt", 2: "tensor"}[k.value]

    def outerApply(self, u, rhs=None):
        """K u (rhs - K u when rhs is given), constrained components zeroed, through the outer
        matvec of the mixed solve (diagnostic)."""
        nn = self._nn(0)
        u = _as_vfield(u, nn)
        out = _new_vfield(nn)
        r = None if rhs is None else _as_vfield(rhs, nn)
        check(_lib().vfem_mg_outer_apply(self._h, ptr(u), None if r is None else ptr(r), ptr(out)))
        return out

    def setDeviceLoop(self, on):
        """Run a solve as one device-resident graph loop (default) or one graph per iteration."""
        check(_lib().vfem_mg_set_device_loop(self._h, int(bool(on))))

    def setUseGraphs(self, use):
        check(_lib().vfem_mg_set_use_graphs(self._h, int(bool(use))))

    def setSymmetricGaussSeidel(self, symmetric):
        check(_lib().vfem_mg_set_symmetric_gs(self._h, int(bool(symmetric))))

    def setFabricationMaskHeightByLayer(self, h):
        check(_lib().vfem_mg_set_mask_layer(self._h, int(h)))

    def updateStiffnessMatrices(self):
        check(_lib().vfem_mg_update_stiffness(self._h))

    def applyK(self, l, u):
        nn = self._nn(l)
        u = _as_vfield(u, nn)
        out = _new_vfield(nn)
        check(_lib().vfem_mg_apply_k(self._h, int(l), ptr(u), ptr(out)))
        return out

    def computeResidual(self, l, u, b):
        nn = self._nn(l)
        u, b = _as_vfield(u, nn), _as_vfield(b, nn)
        out = _new_vfield(nn)
        check(_lib().vfem_mg_residual(self._h, int(l), ptr(u), ptr(b), ptr(out)))
        return out

    def zeroOutDirichletComponents(self, l, u):
        u = _as_vfield(u, self._nn(l)).copy(order="F")
        check(_lib().vfem_mg_zero_dirichlet(self._h, int(l), ptr(u)))
        return u

    def smoothingMulticoloredGS(self, l, u, b, forwardSweep=True):
        nn = self._nn(l)
        u = _as_vfield(u, nn).copy(order="F")
        b = _as_vfield(b, nn)
        check(_lib().vfem_mg_smooth(self._h, int(l), ptr(u), ptr(b), int(bool(forwardSweep))))
        return u

    def restriction(self, l, fine):
        fine = _as_vfield(fine, self._nn(l))
        out = _new_vfield(self._nn(l + 1))
        check(_lib().vfem_mg_restrict(self._h, int(l), ptr(fine), ptr(out)))
        return out

    def interpolation(self, l, coarse, fine=None, accumulate=False):
        coarse = _as_vfield(coarse, self._nn(l + 1))
        out = _new_vfield(self._nn(l)) if fine is None else _as_vfield(fine, self._nn(l)).copy(order="F")
        check(_lib().vfem_mg_interpolate(self._h, int(l), ptr(coarse), ptr(out), int(bool(accumulate))))
        return out

    def coarseSolve(self, b):
        nn = self._nn(self.numLevels - 1)
        b = _as_vfield(b, nn)
        out = _new_vfield(nn)
        check(_lib().vfem_mg_coarse_solve(self._h, ptr(b), ptr(out)))
        return out

    def solve(self, u, f, numSteps, numSmoothingSteps, stiffnessUpdated=False, zeroDirichlet=False,
              it_callback=None, fullMultigrid=False):
        nn = self._nn(0)
        u, f = _as_vfield(u, nn), _as_vfield(f, nn)
        if it_callback is None:
            out = _new_vfield(nn)
            check(_lib().vfem_mg_solve(self._h, ptr(u), ptr(f), int(numSteps), int(numSmoothingSteps),
                                       int(bool(zeroDirichlet)), int(bool(fullMultigrid)), ptr(out)))
            return out
        # per-step callbacks: one cycle at a time (FMG only on the first step)
        x = u
        for i in range(int(numSteps)):
            out = _new_vfield(nn)
            check(_lib().vfem_mg_solve(self._h, ptr(x), ptr(f), 1, int(numSmoothingSteps), int(bool(zeroDirichlet)),
                                       int(bool(fullMultigrid) and i == 0), ptr(out)))
            it_callback(i, out)
            x = out
        return x

    def preconditionedConjugateGradient(self, u, b, maxIter, tol, it_callback=None, mgIterations=1,
                                        mgSmoothingIterations=1, fullMultigrid=False):
        nn = self._nn(0)
        x = _as_vfield(u, nn).copy(order="F")
        b = _as_vfield(b, nn)
        stats = _capi.PcgStats()
        cb = _capi.PCG_CALLBACK()
        if it_callback is not None:
            def _cb(user, it, rnorm, xdev, rdev):
                xa = _device_to_host(xdev, nn)
                ra = _device_to_host(rdev, nn)
                it_callback(int(it), xa, ra)
                return 0
            cb = _capi.PCG_CALLBACK(_cb)
        check(_lib().vfem_mg_pcg(self._h, ptr(x), ptr(b), int(maxIter), float(tol), int(mgIterations),
                                 int(mgSmoothingIterations), int(bool(fullMultigrid)), 0, cb, None, C.byref(stats)))
        self.lastStats = stats
        return x


_cudart = None


def _device_to_host(dev_ptr, nn, nc=3):
    """Copy a device FP64 (nn, nc) field to a new host array (used by per-iteration callbacks)."""
    global _cudart
    if _cudart is None:
        import ctypes.util
        name = ctypes.util.find_library("cudart") or "libcudart.so"
        try:
            _cudart = C.CDLL(name)
        except OSError:
            import glob
            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
            _cudart = C.CDLL(cands[0])
    out = np.empty((nn, nc), order="F")
    rc = _cudart.cudaMemcpy(C.c_void_p(out.ctypes.data), C.c_void_p(dev_ptr), C.c_size_t(out.nbytes), 4)
    if rc != 0:
        raise RuntimeError("cudaMemcpy failed in callback")
    return out


# ---------------------------------------------------------------------------
# Topology optimisation layer
# ---------------------------------------------------------------------------
class Filter:
    def apply(self, x):
        raise NotImplementedError


class SmoothingFilter(Filter):
    """SmoothingFilter(radius=1, type=Const) (TopologyOptimizationFilter.hh:285-400)."""

    class Type(enum.IntEnum):
        Const = 0
        Linear = 1

    def __init__(self, radius=1, type=None):
        self.radius = int(radius)
        self.type = SmoothingFilter.Type.Const if type is None else SmoothingFilter.Type(int(type))
        self._dims = None

    def setInputDimensions(self, gridDims):
        self._dims = tuple(int(v) for v in gridDims)

    setOutputDimensions = setInputDimensions

    @property
    def inputDimensions(self):
        return np.array(self._dims)

    outputDimensions = inputDimensions

    def apply(self, x):
        if self._dims is None:
            raise RuntimeError("Filter grid dimensions not set. Initialize a TopologyOptimizationProblem object "
                               "with this filter before using it.")
        a = _as_elems(x, int(np.prod(self._dims)))
        out = np.empty_like(a)
        dims = np.array(self._dims, dtype=np.int64)
        fn = _lib().vfem_smoothing_filter2 if len(self._dims) == 2 else _lib().vfem_smoothing_filter
        check(fn(dims.ctypes.data_as(_capi._i64), self.radius, int(self.type), ptr(a), ptr(out)))
        return out

    backprop = lambda self, g, vars_=None: self.apply(g)


class ProjectionFilter(Filter):
    """ProjectionFilter(beta) (TopologyOptimizationFilter.hh:189-245)."""

    def __init__(self, beta=1.0):
        if beta <= 0:
            raise RuntimeError("Beta parameter has to be positive (received beta = %g)" % beta)
        self._beta = float(beta)
        self._dims = None

    @property
    def beta(self):
        return self._beta

    @beta.setter
    def beta(self, b):
        if b <= 0:
            raise RuntimeError("Beta parameter has to be positive (received beta = %g)" % b)
        self._beta = float(b)

    def setInputDimensions(self, gridDims):
        self._dims = tuple(int(v) for v in gridDims)

    setOutputDimensions = setInputDimensions

    @property
    def inputDimensions(self):
        return np.array(self._dims)

    outputDimensions = inputDimensions

    def apply(self, x):
        a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
        out = np.empty_like(a)
        check(_lib().vfem_projection_apply(a.size, self._beta, ptr(a), ptr(out)))
        return out

    def backprop(self, g, vars_):
        g = np.ascontiguousarray(np.asarray(g, dtype=np.float64).reshape(-1))
        v = np.ascontiguousarray(np.asarray(vars_, dtype=np.float64).reshape(-1))
        out = np.empty_like(g)
        check(_lib().vfem_projection_backprop(g.size, self._beta, ptr(g), ptr(v), ptr(out)))
        return out

    def invert(self, filteredValue):
        if filteredValue > 1.0 or filteredValue < 0.0:
            raise RuntimeError("ProjectionFilter::invert domain error: target density for inversion is outside [0, 1].")
        return np.arctanh((2 * filteredValue - 1) * np.tanh(0.5 * self._beta)) / self._beta + 0.5


class _ReshapingFilter(Filter):
    """Dimension bookkeeping of the filters that change the grid size."""

    def _set(self, inDims, outDims):
        self._in = tuple(int(v) for v in inDims)
        self._out = tuple(int(v) for v in outDims)

    @property
    def inputDimensions(self):
        return np.array(self._in)

    @property
    def outputDimensions(self):
        return np.array(self._out)

    def _need(self):
        if getattr(self, "_in", None) is None:
            raise RuntimeError("Filter grid dimensions not set. Initialize a TopologyOptimizationProblem object "
                               "with this filter before using it.")


class UpsampleFilter(_ReshapingFilter):
    """UpsampleFilter(factor=2) (TopologyOptimizationFilter.hh:402-505): trilinear upsampling of a
    node-valued grid from s to (s - 1) * factor + 1 values per axis."""

    def __init__(self, factor=2):
        self.factor = int(factor)
        self._in = None

    def setInputDimensions(self, gridDims):
        d = np.asarray(gridDims, dtype=np.int64)
        if (d < 2).any():
            raise RuntimeError("Interpolation can only be applied to a 2^d grid or larger")
        self._set(d, (d - 1) * self.factor + 1)

    def setOutputDimensions(self, gridDims):
        d = np.asarray(gridDims, dtype=np.int64)
        if (d < 2).any():
            raise RuntimeError("Interpolation can only be applied to a 2^d grid or larger")
        i = (d - 1) // self.factor + 1
        if ((i - 1) * self.factor + 1 != d).any():
            raise RuntimeError("Output size is not divisible by factor")
        self._set(i, d)

    def apply(self, x):
        self._need()
        a = _as_elems(x, int(np.prod(self._in)))
        out = np.empty(int(np.prod(self._out)))
        dims = np.array(self._in, dtype=np.int64)
        fn = _lib().vfem_upsample_filter2 if len(self._in) == 2 else _lib().vfem_upsample_filter
        check(fn(dims.ctypes.data_as(_capi._i64), self.factor, ptr(a), ptr(out)))
        return out

    def backprop(self, g, vars_=None):
        self._need()
        a = _as_elems(g, int(np.prod(self._out)))
        out = np.empty(int(np.prod(self._in)))
        dims = np.array(self._in, dtype=np.int64)
        fn = _lib().vfem_upsample_filter2_backprop if len(self._in) == 2 else _lib().vfem_upsample_filter_backprop
        check(fn(dims.ctypes.data_as(_capi._i64), self.factor, ptr(a), ptr(out)))
        return out


class VertexToCellFilter(_ReshapingFilter):
    """VertexToCellFilter (TopologyOptimizationFilter.hh:507-575): cell value = mean of its
    corner values (vertex grid s -> cell grid s - 1)."""

    def __init__(self):
        self._in = None

    def setInputDimensions(self, gridDims):
        d = np.asarray(gridDims, dtype=np.int64)
        if (d < 2).any():
            raise RuntimeError("Input grid must be 2^d or larger.")
        self._set(d, d - 1)

    def setOutputDimensions(self, gridDims):
        d = np.asarray(gridDims, dtype=np.int64)
        self._set(d + 1, d)

    def apply(self, x):
        self._need()
        a = _as_elems(x, int(np.prod(self._in)))
        out = np.empty(int(np.prod(self._out)))
        dims = np.array(self._in, dtype=np.int64)
        fn = _lib().vfem_vertex_to_cell_filter2 if len(self._in) == 2 else _lib().vfem_vertex_to_cell_filter
        check(fn(dims.ctypes.data_as(_capi._i64), ptr(a), ptr(out)))
        return out

    def backprop(self, g, vars_=None):
        self._need()
        a = _as_elems(g, int(np.prod(self._out)))
        out = np.empty(int(np.prod(self._in)))
        dims = np.array(self._in, dtype=np.int64)
        fn = (_lib().vfem_vertex_to_cell_filter2_backprop if len(self._in) == 2
              else _lib().vfem_vertex_to_cell_filter_backprop)
        check(fn(dims.ctypes.data_as(_capi._i64), ptr(a), ptr(out)))
        return out


class LangelaarFilter(_ReshapingFilter):
    """LangelaarFilter (TopologyOptimizationFilter.hh:577-709): the additive-manufacturing
    overhang filter along the build direction y. Stateful like the reference's: its previous
    output enters the own-voxel term of each supporting region, and backprop uses the smax and
    filtered values of the last apply."""

    def __init__(self):
        self._in = None
        self._h = None

    def setInputDimensions(self, gridDims):
        self._set(gridDims, gridDims)
        self._release()
        h = C.c_void_p()
        dims = np.array(self._in, dtype=np.int64)
        fn = _lib().vfem_langelaar2_create if len(self._in) == 2 else _lib().vfem_langelaar_create
        check(fn(dims.ctypes.data_as(_capi._i64), C.byref(h)))
        self._h = h

    setOutputDimensions = setInputDimensions

    def _release(self):
        if getattr(self, "_h", None) is not None and _capi._lib is not None:
            _capi._lib.vfem_langelaar_destroy(self._h)
        self._h = None

    def __del__(self):
        self._release()

    def apply(self, x):
        self._need()
        a = _as_elems(x, int(np.prod(self._in)))
        out = np.empty_like(a)
        check(_lib().vfem_langelaar_apply(self._h, ptr(a), ptr(out)))
        return out

    def backprop(self, g, vars_):
        self._need()
        a = _as_elems(g, int(np.prod(self._in)))
        v = _as_elems(vars_, int(np.prod(self._in)))
        out = np.empty_like(a)
        check(_lib().vfem_langelaar_backprop(self._h, ptr(a), ptr(v), ptr(out)))
        return out


class FilterChain:
    """FilterChain (TopologyOptimizationFilter.hh:90-187), host-side composition of device filters.
    The chain produces a density grid of outGridDimensions; dimension-changing filters
    (UpsampleFilter, VertexToCellFilter) are sized backwards from it, like the reference."""

    def __init__(self, filters, outGridDimensions):
        self.filters = list(filters)
        dims = tuple(int(v) for v in outGridDimensions)
        self._out = dims
        for f in reversed(self.filters):
            f.setOutputDimensions(dims)
            dims = tuple(int(v) for v in f.inputDimensions)
        self._dims = dims
        self._vars = None

    def numVars(self):
        return int(np.prod(self._dims))

    def numPhysicalVars(self):
        return int(np.prod(self._out))

    def gridDims(self):
        return np.array(self._dims)

    def physicalGridDims(self):
        return np.array(self._out)

    def setDesignVars(self, xDesign):
        v = [_as_elems(xDesign, self.numVars())]
        for f in self.filters:
            v.append(f.apply(v[-1]))
        self._vars = v

    def designVars(self):
        return self._vars[0].copy()

    def physicalVars(self):
        return self._vars[-1].copy()

    def backprop(self, g):
        g = _as_elems(g, self.numPhysicalVars())
        for i in range(len(self.filters) - 1, -1, -1):
            g = self.filters[i].backprop(g, self._vars[i])
        return g


class TotalVolumeConstraint:
    """TotalVolumeConstraint(volumeFraction) (TopologyOptimizationConstraint.hh:24-40)."""

    def __init__(self, volumeFraction):
        self.volumeFraction = float(volumeFraction)

    def evaluate(self, x):
        return 1.0 - np.mean(x) / self.volumeFraction


class MultigridComplianceObjective:
    """MultigridComplianceObjective(mg) (TopologyOptimizationObjective.hh:71-105)."""

    def __init__(self, mg_solver):
        self.mg = mg_solver
        self.cgIter = 100
        self.tol = 1e-5
        self.mgIterations = 1
        self.mgSmoothingIterations = 2
        self.fullMultigrid = True
        self.zeroInit = False
        self.residual_cb = None
        tps = mg_solver.getSimulator(0)
        self._f = tps.buildLoadVector()
        self._problem = None
        # the reference solves once at construction (updateCache of the current densities)
        self._u = mg_solver.preconditionedConjugateGradient(np.zeros_like(self._f), self._f, self.cgIter, self.tol,
                                                            None, self.mgIterations, self.mgSmoothingIterations,
                                                            self.fullMultigrid)

    def u(self):
        if self._problem is not None:
            return self._problem._get_u()
        return self._u

    def f(self):
        return self._f

    def compliance(self):
        return 0.5 * float(np.sum(self.f() * self.u()))

    def gradient(self):
        return self.mg.getSimulator(0).complianceGradient(self.u())


def ComplianceObjective(simulator):
    """ComplianceObjective(sim): direct solve; served by a zero-coarsening MG objective."""
    return MultigridComplianceObjective(simulator.multigridSolver(0))


class TopologyOptimizationProblem:
    """TopologyOptimizationProblem(simulator, objective, constraints, filters) (TopologyOptimizationProblem.hh)."""

    def __init__(self, simulator, objective, constraints, filters):
        if len(constraints) != 1 or not isinstance(constraints[0], TotalVolumeConstraint):
            raise RuntimeError("Applicable only for a topology optimization with a single (volume) constraint")
        self._sim = simulator
        self._objective = objective
        self.constraints = list(constraints)
        self.filters = list(filters)
        self.filterChain = FilterChain(self.filters, simulator.NbElementsPerDimension)
        kinds, radii, types, betas = [], [], [], []
        for f in self.filters:
            if isinstance(f, SmoothingFilter):
                kinds.append(0); radii.append(f.radius); types.append(int(f.type)); betas.append(0.0)
            elif isinstance(f, ProjectionFilter):
                kinds.append(1); radii.append(0); types.append(0); betas.append(f.beta)
            else:
                raise RuntimeError("Unsupported filter type " + type(f).__name__)
        n = max(len(kinds), 1)
        h = C.c_void_p()
        create = _lib().vfem_problem2_create if simulator._nc == 2 else _lib().vfem_problem_create
        check(create(objective.mg._h, len(kinds), (C.c_int * n)(*kinds), (C.c_int * n)(*radii), (C.c_int * n)(*types),
                     (C.c_double * n)(*betas), self.constraints[0].volumeFraction, C.byref(h)))
        self._h = h
        objective._problem = self
        self._ne = simulator.numElements()
        self._varsSet = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_problem_destroy(h)
            self._h = None

    @property
    def objective(self):
        return self._objective

    def _sync_solver(self):
        o = self._objective
        check(_lib().vfem_problem_set_solver(self._h, int(o.cgIter), float(o.tol), int(o.mgIterations),
                                             int(o.mgSmoothingIterations), int(bool(o.fullMultigrid)),
                                             int(bool(o.zeroInit))))

    def numVars(self):
        return self._ne

    def getVars(self):
        out = np.empty(self._ne)
        check(_lib().vfem_problem_get_vars(self._h, ptr(out)))
        return out

    def setVars(self, x, forceUpdate=False):
        self._sync_solver()
        a = _as_elems(x, self._ne)
        check(_lib().vfem_problem_set_vars(self._h, ptr(a)))
        self.filterChain.setDesignVars(a)
        self._varsSet = True
        return True

    def _get_u(self):
        nn = self._sim.numNodes()
        out = _new_vfield(nn, self._sim._nc)
        check(_lib().vfem_problem_get_u(self._h, ptr(out)))
        return out

    def evaluateObjective(self):
        v = C.c_double()
        check(_lib().vfem_problem_objective(self._h, C.byref(v)))
        return v.value

    def evaluateObjectiveGradient(self):
        out = np.empty(self._ne)
        check(_lib().vfem_problem_gradient(self._h, ptr(out)))
        return out

    def evaluateConstraints(self):
        v = C.c_double()
        check(_lib().vfem_problem_constraint(self._h, C.byref(v)))
        return np.array([v.value])

    def evaluateConstraintsJacobian(self):
        out = np.empty(self._ne)
        check(_lib().vfem_problem_jacobian(self._h, ptr(out)))
        return out.reshape(1, -1)

    def getDensities(self):
        return self._sim.getDensities()

    def lastSolveStats(self):
        s = _capi.PcgStats()
        check(_lib().vfem_problem_last_solve(self._h, C.byref(s)))
        return s


class OCOptimizer:
    """OCOptimizer(problem).step(m=0.2, p=0.5, ctol=1e-6, inplace=True) (OptimalityCriterion.hh:51-138)."""

    def __init__(self, problem):
        self.problem = problem
        self.lastProbes = 0

    def step(self, m=0.2, p=0.5, ctol=1e-6, inplace=True, objectiveGradient=None):
        """One OC step. ``objectiveGradient`` (optional, not in the reference): a gradient of the
        objective with respect to the design variables computed elsewhere (a numpy array, or a
        CUDA float64 tensor passed as a device pointer), used instead of
        evaluateObjectiveGradient."""
        probes = C.c_int64()
        self.problem._sync_solver()
        if objectiveGradient is None:
            check(_lib().vfem_problem_oc_step(self.problem._h, float(m), float(p), float(ctol), C.byref(probes)))
        else:
            g = objectiveGradient
            if hasattr(g, "data_ptr"):
                if g.numel() != self.problem.numVars() or not g.is_contiguous():
                    raise RuntimeError("Invalid input size")
                import torch
                torch.cuda.current_stream().synchronize()
                gp = C.c_void_p(g.data_ptr())
            else:
                g = np.ascontiguousarray(g, dtype=np.float64)
                if g.size != self.problem.numVars():
                    raise RuntimeError("Invalid input size")
                gp = g.ctypes.data_as(C.c_void_p)
            check(_lib().vfem_problem_oc_step_with_gradient(self.problem._h, float(m), float(p), float(ctol), gp,
                                                            C.byref(probes)))
        self.lastProbes = probes.value
        self.problem.filterChain.setDesignVars(self.problem.getVars())


class TensorProductSimulator_3D_Q2:
    """TensorProductSimulator<double, 2, 2, 2>: triquadratic voxels (27 nodes per element).

    Provides the element stiffness (81 x 81), SIMP moduli, zero-displacement supports, ``applyK``
    and the 27-colour block Gauss-Seidel sweep of the reference's generic multigrid smoother
    (``smoothingMulticoloredGS``), in FP64 or FP32 (``precision="fp32"``). Nodal fields are
    (numNodes, 3) with node (I, J, K) at index (I * NY + J) * NZ + K, NY = 2 ny + 1.
    """

    def __init__(self, domainBBox, elementsPerDimension):
        bb = [np.asarray(domainBBox[0], dtype=np.float64).reshape(3), np.asarray(domainBBox[1], dtype=np.float64).reshape(3)]
        ne = np.ascontiguousarray(np.asarray(elementsPerDimension, dtype=np.int64).reshape(3))
        h = C.c_void_p()
        check(_lib().vfem_q2_create(ne.ctypes.data_as(_capi._i64), _capi.dptr(np.ascontiguousarray(bb[0])),
                                    _capi.dptr(np.ascontiguousarray(bb[1])), C.byref(h)))
        self._h = h
        self._ne = tuple(int(v) for v in ne)
        self._nn = (2 * self._ne[0] + 1) * (2 * self._ne[1] + 1) * (2 * self._ne[2] + 1)
        self._nel = self._ne[0] * self._ne[1] * self._ne[2]
        self._E = (1.0, 0.0)
        self._params = [1.0, 1e-4, 3.0, 3.0, 0]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_q2_destroy(h)
            self._h = None

    def numNodes(self):
        return self._nn

    def numElements(self):
        return self._nel

    @property
    def NbElementsPerDimension(self):
        return np.array(self._ne)

    @property
    def NbNodesPerDimension(self):
        return np.array([2 * v + 1 for v in self._ne])

    @property
    def ETensor(self):
        return ElasticityTensor(*self._E)

    @ETensor.setter
    def ETensor(self, value):
        E, nu = value
        check(_lib().vfem_q2_set_etensor(self._h, float(E), float(nu)))
        self._E = (float(E), float(nu))

    def _set_param(self, idx, value):
        self._params[idx] = value
        p = self._params
        check(_lib().vfem_q2_set_material_params(self._h, float(p[0]), float(p[1]), float(p[2]), float(p[3]),
                                                 int(p[4])))

    E_0 = property(lambda self: self._params[0], lambda self, v: self._set_param(0, float(v)))
    E_min = property(lambda self: self._params[1], lambda self, v: self._set_param(1, float(v)))
    gamma = property(lambda self: self._params[2], lambda self, v: self._set_param(2, float(v)))
    q = property(lambda self: self._params[3], lambda self, v: self._set_param(3, float(v)))

    def fullDensityElementStiffnessMatrix(self):
        K = np.empty(6561)
        check(_lib().vfem_q2_get_k0(self._h, _capi.dptr(K)))
        return K.reshape(81, 81)

    def setDensities(self, rho):
        a = _as_elems(rho, self._nel)
        if np.any(a > 1.0) or np.any(a < 0.0):
            raise RuntimeError("Density value has to be in between 0 and 1")
        check(_lib().vfem_q2_set_densities(self._h, ptr(a)))

    def addDirichletCondition(self, u, minCorner, maxCorner, componentMask="xyz"):
        """Supports on the nodes inside the box (TensorProductSimulator::addDirichletCondition).
        Triquadratic grids take homogeneous supports only: u must be zero."""
        if np.any(_arr3(u) != 0.0):
            raise RuntimeError("triquadratic grids support zero prescribed displacements only")
        check(_lib().vfem_q2_add_dirichlet(self._h, _capi.dptr(_arr3(minCorner)), _capi.dptr(_arr3(maxCorner)),
                                           _cmask(componentMask)))

    def getDirichletMask(self):
        m = np.empty(self._nn, dtype=np.uint8)
        check(_lib().vfem_q2_get_dirichlet_mask(self._h, m.ctypes.data_as(C.c_void_p)))
        return np.stack([(m >> c) & 1 for c in range(3)], axis=1).astype(bool)

    def applyK(self, u, precision="fp64", zeroDirichlet=False):
        u = _as_vfield(u, self._nn)
        out = _new_vfield(self._nn)
        p = {"fp64": 0, "fp32": 1, "df": 2}[precision]
        check(_lib().vfem_q2_apply_k(self._h, ptr(u), ptr(out), p, int(bool(zeroDirichlet))))
        return out

    def smoothingMulticoloredGS(self, u, b, forwardSweep=True, precision="fp64"):
        x = _as_vfield(u, self._nn).copy(order="F")
        b = _as_vfield(b, self._nn)
        p = {"fp64": 0, "fp32": 1}[precision]
        check(_lib().vfem_q2_smooth(self._h, ptr(x), ptr(b), int(bool(forwardSweep)), p))
        return x

    def multigridSolver(self, numCoarseningLevels):
        """MultigridSolver(self, numCoarseningLevels) for this grid (MultigridSolver<double, 2, 2, 2>):
        FP64 outer PCG, preconditioned by the reference's hierarchy of halved Q2 meshes (default)
        or by a p-multigrid step onto the trilinear mesh (``setHierarchy("p")``)."""
        return _Q2MultigridSolver(self, int(numCoarseningLevels))


_Q2_PREC = {"fp64": 0, "mixed": 1}


class _Q2MultigridSolver:
    def __init__(self, tps, numCoarseningLevels):
        if numCoarseningLevels < 1:
            raise RuntimeError("the triquadratic solver needs at least one coarsening")
        self.tps = tps
        self.coarsenings = numCoarseningLevels
        self.lastStats = None

    def setOuterMatvec(self, outerMatvec="df"):
        """CG matvec in 'df' (double-float) or 'fp64'."""
        check(_lib().vfem_q2_set_outer_matvec(self.tps._h, {"fp64": 0, "df": 1}[outerMatvec]))

    def setHierarchy(self, hierarchy="q2"):
        """Preconditioner hierarchy: 'q2' (the reference's halved Q2 meshes, default) or 'p'
        (Q2 smoothing around a trilinear V-cycle on the same mesh; mixed precision only)."""
        check(_lib().vfem_q2_set_hierarchy(self.tps._h, {"q2": 0, "p": 1}[hierarchy]))

    def setPrecision(self, precision="mixed"):
        """'fp64' (the reference's method: FP64 V-cycle and CG matvec) or 'mixed' (default: FP32
        V-cycle, double-float CG matvec)."""
        check(_lib().vfem_q2_set_precision(self.tps._h, _Q2_PREC[precision]))

    # ---- per-level access to the Q2 hierarchy (MultigridSolver.hh) ----
    def numNodes(self, l):
        n = C.c_int64()
        check(_lib().vfem_q2_mg_num_nodes(self.tps._h, self.coarsenings, int(l), C.byref(n)))
        return n.value

    def levelDirichletMask(self, l):
        m = np.empty(self.numNodes(l), dtype=np.uint8)
        check(_lib().vfem_q2_mg_level_dirichlet(self.tps._h, self.coarsenings, int(l), m.ctypes.data_as(C.c_void_p)))
        return np.stack([(m >> c) & 1 for c in range(3)], axis=1).astype(bool)

    def levelElementMatrices(self, l, precision="fp64"):
        ne = [v >> int(l) for v in self.tps._ne]
        out = np.empty(int(np.prod(ne)) * 6561)
        check(_lib().vfem_q2_mg_level_ke(self.tps._h, self.coarsenings, int(l), _Q2_PREC[precision], _capi.dptr(out)))
        return out.reshape(-1, 81, 81)

    def smoothing(self, l, u, b, forwardSweep=True, precision="fp64"):
        nn = self.numNodes(l)
        x = _as_vfield(u, nn).copy(order="F")
        b = _as_vfield(b, nn)
        check(_lib().vfem_q2_mg_smooth(self.tps._h, self.coarsenings, int(l), ptr(x), ptr(b), int(bool(forwardSweep)),
                                       _Q2_PREC[precision]))
        return x

    def computeResidual(self, l, u, b, precision="fp64"):
        nn = self.numNodes(l)
        out = _new_vfield(nn)
        u, b = _as_vfield(u, nn), _as_vfield(b, nn)  # held: ptr() keeps no reference
        check(_lib().vfem_q2_mg_residual(self.tps._h, self.coarsenings, int(l), ptr(u), ptr(b), ptr(out),
                                         _Q2_PREC[precision]))
        return out

    def coarseSolve(self, b, precision="fp64"):
        nn = self.numNodes(self.coarsenings)
        out = _new_vfield(nn)
        b = _as_vfield(b, nn)
        check(_lib().vfem_q2_mg_coarse_solve(self.tps._h, self.coarsenings, ptr(b), ptr(out), _Q2_PREC[precision]))
        return out

    def applyPreconditionerInv(self, r, mgSmoothingIterations=1, precision="fp64"):
        """One V-cycle from zero on K x = r (MultigridSolver.hh:576-580)."""
        nn = self.tps.numNodes()
        out = _new_vfield(nn)
        r = _as_vfield(r, nn)
        check(_lib().vfem_q2_mg_vcycle(self.tps._h, self.coarsenings, ptr(r), ptr(out),
                                       int(mgSmoothingIterations), _Q2_PREC[precision]))
        return out

    def preconditionedConjugateGradient(self, u, b, maxIter, tol, it_callback=None, mgIterations=1,
                                        mgSmoothingIterations=1, fullMultigrid=False):
        if it_callback is not None or mgIterations != 1 or fullMultigrid:
            raise RuntimeError("triquadratic solves support one cycle per iteration without callbacks")
        nn = self.tps.numNodes()
        x = _as_vfield(u, nn).copy(order="F")
        b = _as_vfield(b, nn)
        stats = _capi.PcgStats()
        check(_lib().vfem_q2_pcg(self.tps._h, self.coarsenings, ptr(x), ptr(b), int(maxIter), float(tol),
                                 int(mgSmoothingIterations), C.byref(stats)))
        self.lastStats = stats
        return x


def q2_restriction(elementsPerDimensionFine, fine):
    """Q2 restriction P^T from a grid with the given elements per axis to its 2x coarsening."""
    ne = np.ascontiguousarray(np.asarray(elementsPerDimensionFine, dtype=np.int64).reshape(3))
    nf = int(np.prod(2 * ne + 1))
    nc = int(np.prod(ne + 1))
    fine = _as_vfield(fine, nf)
    out = _new_vfield(nc)
    check(_lib().vfem_q2_restrict(ne.ctypes.data_as(C.c_void_p), ptr(fine), ptr(out)))
    return out


def q2_interpolation(elementsPerDimensionFine, coarse, fine=None, accumulate=False):
    """Q2 prolongation P (coarse quadratic interpolant at the fine nodes)."""
    ne = np.ascontiguousarray(np.asarray(elementsPerDimensionFine, dtype=np.int64).reshape(3))
    nf = int(np.prod(2 * ne + 1))
    nc = int(np.prod(ne + 1))
    coarse = _as_vfield(coarse, nc)
    out = _new_vfield(nf) if fine is None else _as_vfield(fine, nf).copy(order="F")
    check(_lib().vfem_q2_interpolate(ne.ctypes.data_as(C.c_void_p), ptr(coarse), ptr(out), int(bool(accumulate))))
    return out


class LayerByLayerEvaluator:
    """LayerByLayerEvaluator(lblSim) (LayerByLayer.hh:223-296): compliance of every partial build
    height, averaged, with its gradient.

    ``run(solver, zeroInit, layerIncrement, maxIter, tol, ...)`` visits the heights
    ny, ny - layerIncrement, ..., > 0 like the reference. ``selectInitMethod`` chooses the
    initial guesses as the reference does: ``"N=3"`` (default; Galerkin projection onto the last
    3 solutions), ``"N=<k>"``, ``"fd"``, ``"constant"`` or ``"zero"``. Warm-started heights form
    chains: ``slots`` (default 1, the reference's sequential algorithm) contiguous runs of
    heights solved concurrently, each in order. With ``"zero"`` every height is independent
    and the solves run ``slots`` (default 8) at a time. ``solver`` supplies the number of
    coarsening levels and the precision.
    """

    def __init__(self, lblSim):
        self.sim = lblSim
        self.layers = np.zeros(0, dtype=np.int64)
        self.compliances = np.zeros(0)
        self.iterations = np.zeros(0, dtype=np.int64)
        self._grad = np.zeros(lblSim.numElements())
        self.initMethod = "N=3"
        self._h = None
        self._key = None

    def __del__(self):
        self._release()

    def _release(self):
        if getattr(self, "_h", None) is not None:
            try:
                if self.sim._nc == 2:
                    _lib().vfem_lbl2_destroy(self._h)
                else:
                    _lib().vfem_lbl_destroy(self._h)
            except Exception:
                pass
            self._h = None

    def _handle(self, coarsenings, slots, precision):
        key = (coarsenings, slots, precision)
        if self._h is None or self._key != key:
            self._release()
            h = C.c_void_p()
            if self.sim._nc == 2:
                check(_lib().vfem_lbl2_create(self.sim._h, coarsenings, slots, precision, C.byref(h)))
            else:
                check(_lib().vfem_lbl_create(self.sim._h, coarsenings, slots, precision, C.byref(h)))
            self._h, self._key = h, key
        return self._h

    def selectInitMethod(self, method):
        self._init_kind(method)
        self.initMethod = method

    @staticmethod
    def _init_kind(method):
        fixed = {"zero": (0, 0), "constant": (1, 1), "fd": (2, 2)}
        if method in fixed:
            return fixed[method]
        if isinstance(method, str) and method.startswith("N="):
            try:
                n = int(method[2:])
            except ValueError:
                n = -1
            if 1 <= n <= 8:
                return 3, n
        raise RuntimeError("Unrecognized method " + str(method))

    def run(self, solver, zeroInit=True, layerIncrement=1, maxIter=500, tol=1e-8, it_callback=None,
            mgIterations=1, mgSmoothingIterations=1, fmg=False, verbose=False, lblCallback=None, slots=None,
            sweepForm=None, tuned=False):
        """``slots`` and ``sweepForm`` (the fine sweep's launch form, MultigridSolver.setSweepForm)
        shape the execution only. ``tuned=True`` takes both from the autotuner's cache entry for
        this grid, solver and initial-guess method (voxelfem_gb300.autotune), when there is one;
        ``mgSmoothingIterations="tuned"`` also takes the tuned smoothing sweep count."""
        if tuned or mgSmoothingIterations == "tuned":
            from . import autotune
            best = autotune.lookup(self.sim, solver, self.initMethod)
            if best is not None:
                if tuned:
                    slots = best["slots"] if slots is None else slots
                    sweepForm = best["sweepForm"] if sweepForm is None else sweepForm
                if mgSmoothingIterations == "tuned":
                    mgSmoothingIterations = best["mgSmoothingIterations"]
            if mgSmoothingIterations == "tuned":
                mgSmoothingIterations = 1
        if it_callback is not None:
            raise RuntimeError("per-iteration callbacks are not available for device-resident solves")
        ny = int(self.sim.NbElementsPerDimension[1])
        inc = int(layerIncrement)
        if inc < 1:
            raise RuntimeError("layerIncrement must be positive")
        layers = []
        l = ny
        while l > 0:
            layers.append(l)
            l -= min(inc, l)
        self.layers = np.array(layers, dtype=np.int64)
        n = len(layers)
        self.compliances = np.zeros(n)
        self.iterations = np.zeros(n, dtype=np.int64)
        self._grad = np.zeros(self.sim.numElements())
        precision = 1 if getattr(solver, "_prec", "fp64") == "mixed" else 0
        kind, hist = self._init_kind(self.initMethod)
        if slots is None:
            slots = 8 if kind == 0 else 1
        h = self._handle(int(solver.numLevels - 1), int(slots), precision)
        two = self.sim._nc == 2
        check((_lib().vfem_lbl2_set_init if two else _lib().vfem_lbl_set_init)(h, kind, hist))
        if not two:
            check(_lib().vfem_lbl_set_sweep_form(h, MultigridSolver.SWEEP_FORMS[sweepForm or "lines"]))
        run = _lib().vfem_lbl2_run if two else _lib().vfem_lbl_run
        check(run(h, ptr(self.layers), n, int(maxIter), float(tol), int(mgIterations), int(mgSmoothingIterations),
                  int(bool(fmg)), int(bool(zeroInit)), ptr(self.compliances), ptr(self.iterations), ptr(self._grad)))
        for t, lay in enumerate(layers):
            if verbose:
                print("Layer %d: %g" % (lay, self.compliances[t]))
            if lblCallback is not None:
                lblCallback(lay, self.compliances[t], None, None)

    def objective(self):
        return 0.5 * float(np.sum(self.compliances)) / max(len(self.compliances), 1)

    def gradient(self):
        return self._grad / max(len(self.compliances), 1)


# ---------------------------------------------------------------------------
# 2D: bilinear quadrilaterals (TensorProductSimulator<double, 1, 1>, registered by
# VoxelFEM.cc:413-414 beside the 3D instantiation)
# ---------------------------------------------------------------------------
def _arr2(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1)[:2])


class TensorProductSimulator_2D:
    """TensorProductSimulator<double, 1, 1>: nodal fields (numNodes, 2), node (i, j) -> i * ny1 + j,
    plane-stress isotropic material (MeshFEM ElasticityTensor<Real, 2>::setIsotropic)."""

    _nc = 2

    def __init__(self, domainBBox, elementsPerDimension):
        bb = [np.asarray(domainBBox[0], dtype=np.float64).reshape(2), np.asarray(domainBBox[1], dtype=np.float64).reshape(2)]
        ne = np.ascontiguousarray(np.asarray(elementsPerDimension, dtype=np.int64).reshape(2))
        h = C.c_void_p()
        check(_lib().vfem_grid2_create(ne.ctypes.data_as(_capi._i64), _capi.dptr(np.ascontiguousarray(bb[0])),
                                       _capi.dptr(np.ascontiguousarray(bb[1])), C.byref(h)))
        self._h = h
        self._bbox = (bb[0].copy(), bb[1].copy())
        self._ne = tuple(int(v) for v in ne)
        self._nn = (self._ne[0] + 1) * (self._ne[1] + 1)
        self._nel = self._ne[0] * self._ne[1]
        self._forces = np.zeros((self._nn, 2), order="F")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_grid2_destroy(h)
            self._h = None

    # --- sizes / geometry ---
    def numNodes(self):
        return self._nn

    def numElements(self):
        return self._nel

    @property
    def gridShape(self):
        return np.array(self._ne)

    NbElementsPerDimension = gridShape

    @property
    def NbNodesPerDimension(self):
        return np.array([n + 1 for n in self._ne])

    @property
    def domain(self):
        return (self._bbox[0].copy(), self._bbox[1].copy())

    bbox = domain

    @property
    def dx(self):
        return (self._bbox[1] - self._bbox[0]) / np.array(self._ne)

    @property
    def elementVolume(self):
        return float(np.prod(self.dx))

    def nodePosition(self, ni):
        i, j = divmod(int(ni), self._ne[1] + 1)
        return self._bbox[0] + np.array([i, j]) * self.dx

    def elementNodes(self, ei):
        i, j = divmod(int(ei), self._ne[1])
        ny1 = self._ne[1] + 1
        return np.array([(i + (l >> 1)) * ny1 + j + (l & 1) for l in range(4)])

    def elemNodeGlobalIndex(self, ei, n):
        return int(self.elementNodes(ei)[int(n)])

    def elementIndexForGridCell(self, cellIdxs):
        i, j = (int(v) for v in cellIdxs)
        return i * self._ne[1] + j

    # --- material ---
    def readMaterial(self, materialPath):
        with open(materialPath) as f:
            mat = json.load(f)
        if mat.get("type", "isotropic_material") not in ("isotropic_material", "isotropic"):
            raise RuntimeError("Only isotropic materials are supported")
        self.ETensor = (float(mat["young"]), float(mat["poisson"]))

    @property
    def ETensor(self):
        E, nu = C.c_double(), C.c_double()
        check(_lib().vfem_grid2_get_etensor(self._h, C.byref(E), C.byref(nu)))
        return ElasticityTensor(E.value, nu.value)

    @ETensor.setter
    def ETensor(self, value):
        E, nu = value
        check(_lib().vfem_grid2_set_etensor(self._h, float(E), float(nu)))

    def _params(self):
        v = [C.c_double() for _ in range(4)]
        law = C.c_int()
        check(_lib().vfem_grid2_get_material_params(self._h, *[C.byref(x) for x in v], C.byref(law)))
        return [x.value for x in v] + [law.value]

    def _set_param(self, idx, value):
        p = self._params()
        p[idx] = value
        check(_lib().vfem_grid2_set_material_params(self._h, p[0], p[1], p[2], p[3], int(p[4])))

    E_0 = property(lambda self: self._params()[0], lambda self, v: self._set_param(0, float(v)))
    E_min = property(lambda self: self._params()[1], lambda self, v: self._set_param(1, float(v)))
    gamma = property(lambda self: self._params()[2], lambda self, v: self._set_param(2, float(v)))
    q = property(lambda self: self._params()[3], lambda self, v: self._set_param(3, float(v)))
    interpolationLaw = property(lambda self: InterpolationLaw(self._params()[4]),
                                lambda self, v: self._set_param(4, int(v)))

    @property
    def gravity(self):
        g = np.zeros(2)
        check(_lib().vfem_grid2_get_gravity(self._h, _capi.dptr(g)))
        return g

    @gravity.setter
    def gravity(self, g):
        check(_lib().vfem_grid2_set_gravity(self._h, _capi.dptr(_arr2(g))))

    def fullDensityElementStiffnessMatrix(self):
        K = np.empty(64)
        check(_lib().vfem_grid2_get_k0(self._h, _capi.dptr(K)))
        return K.reshape(8, 8)

    def elementStiffnessMatrix(self, ei):
        return self.elementYoungModulusScaleFactor(ei) * self.fullDensityElementStiffnessMatrix()

    def clearCachedElementStiffness(self):
        """No per-element stiffness cache exists here (elements are scaled copies of K0)."""

    # --- mesh, sampling and BC fields (TensorProductSimulator.hh:689-712, 746-778, 1161-1179) ---
    def mesh(self):
        return self

    def getMesh(self):
        """(V, F): node positions (nn, 3) with z = 0 and quadrilaterals (ne, 4) in Gmsh order."""
        nn = self.NbNodesPerDimension
        I, J = np.meshgrid(np.arange(nn[0]), np.arange(nn[1]), indexing="ij")
        V = np.zeros((self._nn, 3))
        V[:, :2] = self._bbox[0] + np.stack([I.ravel(), J.ravel()], axis=1) * self.dx
        i, j = np.meshgrid(np.arange(self._ne[0]), np.arange(self._ne[1]), indexing="ij")
        base = i.ravel() * nn[1] + j.ravel()
        off = [(l >> 1) * nn[1] + (l & 1) for l in range(4)]
        F = np.stack([base + off[l] for l in (0, 1, 3, 2)], axis=1)
        return V, F

    def sampleNodalField(self, u, p):
        """Bilinear interpolation of the nodal field u (nn x c) at the rows of p (clamped into the domain)."""
        u = np.asarray(u, dtype=np.float64).reshape(self._nn, -1)
        p = np.atleast_2d(np.asarray(p, dtype=np.float64))[:, :2]
        p = np.clip(p, self._bbox[0], self._bbox[1])
        t = (p - self._bbox[0]) / self.dx
        e = np.minimum(np.floor(t).astype(np.int64), np.array(self._ne) - 1)
        x = t - e
        ny1 = self._ne[1] + 1
        out = np.zeros((p.shape[0], u.shape[1]))
        for l in range(4):
            b = [l >> 1, l & 1]
            w = np.prod([x[:, d] if b[d] else 1.0 - x[:, d] for d in range(2)], axis=0)
            out += w[:, None] * u[(e[:, 0] + b[0]) * ny1 + e[:, 1] + b[1]]
        return out

    def getBCIndicatorField(self):
        d = self.getDirichletMask()
        f = self.getForceMask()
        return (d[:, 0] * 1 + d[:, 1] * 2 + 8 * (f[:, 0] * 1 + f[:, 1] * 2)).astype(np.float64)

    def getK(self):
        """The assembled stiffness matrix (2 nn x 2 nn, DOF 2 n + c) as a scipy CSC matrix."""
        import scipy.sparse as sp
        K0 = self.fullDensityElementStiffnessMatrix()
        Y = self.getYoungModulusScaleFactor()
        i, j = np.meshgrid(np.arange(self._ne[0]), np.arange(self._ne[1]), indexing="ij")
        base = i.ravel() * (self._ne[1] + 1) + j.ravel()
        nodes = np.stack([base + (l >> 1) * (self._ne[1] + 1) + (l & 1) for l in range(4)], 1)
        dofs = (2 * nodes[:, :, None] + np.arange(2)[None, None, :]).reshape(-1, 8)
        rows = np.repeat(dofs, 8, axis=1).ravel()
        cols = np.tile(dofs, (1, 8)).ravel()
        vals = (Y[:, None] * K0.ravel()[None, :]).ravel()
        return sp.csc_matrix((vals, (rows, cols)), shape=(2 * self._nn, 2 * self._nn))

    def solveWithImposedLoads(self):
        return self.solve(self.buildLoadVector())

    # --- coarser and intermediate simulators ---
    def _copy_material(self, other):
        other.ETensor = self.ETensor
        other.E_min = self.E_min
        other.E_0 = self.E_0
        other.gamma = self.gamma

    def downsample(self, downsamplingLevels):
        f = 2 ** int(downsamplingLevels)
        ne = np.array(self._ne)
        if (ne % f).any():
            raise RuntimeError("Grid size must be divisible by 2^downsamplingLevels")
        c = TensorProductSimulator_2D([self._bbox[0], self._bbox[1]], ne // f)
        self._copy_material(c)
        return c

    def _factor(self, coarse):
        f = self._ne[0] // coarse._ne[0]
        if any(f * coarse._ne[d] != self._ne[d] for d in range(2)):
            raise RuntimeError("Invalid downsampled simulator")
        return f

    def downsampleDensityFieldTo(self, densities, coarseTPS):
        f = self._factor(coarseTPS)
        rho = np.asarray(densities, dtype=np.float64).reshape(-1)
        if rho.size != self._nel:
            raise RuntimeError("Invalid input densities size (%d vs %d)" % (rho.size, self._nel))
        c = rho.reshape(self._ne[0] // f, f, self._ne[1] // f, f).sum(axis=(1, 3)) / f ** 2
        coarseTPS.setDensities(c.ravel())

    def upsampleDensityGradientFrom(self, coarseTPS, g_coarse):
        f = self._factor(coarseTPS)
        g = np.asarray(g_coarse, dtype=np.float64).reshape(coarseTPS._ne)
        return (np.repeat(np.repeat(g, f, 0), f, 1) / f ** 2).ravel()

    def setDensitiesFromCoarseGrid(self, upscalingFactor, rho):
        f = int(upscalingFactor)
        rho = np.asarray(rho, dtype=np.float64).reshape(-1)
        if self._nel != f ** 2 * rho.size:
            raise RuntimeError("Incorrect rho size")
        rc = rho.reshape(tuple(v // f for v in self._ne))
        self.setDensities(np.repeat(np.repeat(rc, f, 0), f, 1).ravel())

    def getIntermediateFabricationShape(self, yfrac, validateBoundaryConditions=True, law=None):
        if yfrac < 0 or yfrac > 1:
            raise RuntimeError("hfrac is out of bounds")
        full = self._ne[1]
        h = int(round(yfrac * full))
        if abs(yfrac * full - h) > 1e-10:
            raise RuntimeError("hfrac chops off a noninteger number of element layers")
        lo, hi = self._bbox[0].copy(), self._bbox[1].copy()
        hi[1] = lo[1] + yfrac * (self._bbox[1][1] - lo[1])
        r = TensorProductSimulator_2D([lo, hi], [self._ne[0], h])
        if law is not None:
            r.interpolationLaw = law
        r.ETensor = self.ETensor
        self.transferDensitiesToIntermediateFabricationShape(r)
        r.E_min, r.E_0, r.gamma = self.E_min, self.E_0, self.gamma
        g = self.gravity
        bad = RuntimeError("Original simulator has unexpected boundary conditions for layer-by-layer simulation")
        if not np.any(g):
            if validateBoundaryConditions:
                raise bad
            g = np.array([0.0, -1.0])
        r.gravity = g
        if validateBoundaryConditions:
            if self.getForceMask().any():
                raise bad
            m = self.getDirichletMask()
            jrow = np.arange(self._nn) % (self._ne[1] + 1)
            if not m[jrow == 0].all() or m[jrow != 0].any():
                raise bad
        r.addDirichletCondition([0.0, 0.0], [lo[0], lo[1]], [hi[0], lo[1]], "xy")
        return r

    def _check_intermediate(self, itps):
        if itps._ne[0] != self._ne[0] or itps._ne[1] > self._ne[1]:
            raise RuntimeError("Intermediate shape is of unexpected size")

    def transferDensitiesToIntermediateFabricationShape(self, intermediateTPS):
        rho = self.getDensities().reshape(self._ne)
        intermediateTPS.setDensities(rho[:, :intermediateTPS._ne[1]].ravel())

    def transferVFieldToIntermediateFabricationShape(self, intermediateTPS, u):
        self._check_intermediate(intermediateTPS)
        u = np.asarray(u, dtype=np.float64).reshape(self._ne[0] + 1, self._ne[1] + 1, -1)
        return np.asfortranarray(u[:, :intermediateTPS._ne[1] + 1, :].reshape(-1, u.shape[-1]))

    def accumElementScalarFieldFromIntermediateFabricationShape(self, intermediateTPS, rho_in, rho_accum):
        acc = rho_accum.reshape(self._ne)
        acc[:, :intermediateTPS._ne[1]] += np.asarray(rho_in, dtype=np.float64).reshape(intermediateTPS._ne)

    # --- densities ---
    def getDensities(self):
        out = np.empty(self._nel)
        check(_lib().vfem_grid2_get_densities(self._h, ptr(out)))
        return out

    def setDensities(self, rho):
        if np.asarray(rho).size != self._nel:
            raise RuntimeError("Incorrect rho size")
        rho = _as_elems(rho, self._nel)  # held: ptr() keeps no reference
        check(_lib().vfem_grid2_set_densities(self._h, ptr(rho)))

    def setUniformDensities(self, density):
        check(_lib().vfem_grid2_set_uniform_densities(self._h, float(density)))

    def setDensity(self, ei, value):
        if value > 1.0 or value < 0:
            raise RuntimeError("Density value (%g) has to be in between 0 and 1" % value)
        rho = self.getDensities()
        rho[int(ei)] = value
        self.setDensities(rho)

    def elementDensity(self, ei):
        return float(self.getDensities()[int(ei)])

    def getYoungModulusScaleFactor(self):
        out = np.empty(self._nel)
        check(_lib().vfem_grid2_get_young_moduli(self._h, ptr(out)))
        return out

    def elementYoungModulusScaleFactor(self, ei):
        return float(self.getYoungModulusScaleFactor()[int(ei)])

    # --- boundary conditions ---
    def addDirichletCondition(self, u, minCorner, maxCorner, componentMask="xyz"):
        check(_lib().vfem_grid2_add_dirichlet(self._h, _capi.dptr(_arr2(u)), _capi.dptr(_arr2(minCorner)),
                                              _capi.dptr(_arr2(maxCorner)), _cmask(componentMask, 2)))

    def applySymmetryConditions(self, symmetry_axes, minMaxFace=(False, False)):
        ax = (C.c_int * 2)(*[int(bool(v)) for v in list(symmetry_axes)[:2]])
        mf = (C.c_int * 2)(*[int(bool(v)) for v in list(minMaxFace)[:2]])
        check(_lib().vfem_grid2_apply_symmetry(self._h, ax, mf))

    def setNodalForces(self, forces):
        f = _as_vfield(forces, self._nn, 2)
        self._forces = f.copy(order="F")
        check(_lib().vfem_grid2_set_nodal_forces(self._h, ptr(f)))

    def applyDisplacementsAndLoadsFromFile(self, bcPath):
        apply_bc_file(self, bcPath)

    def getDirichletMask(self):
        m = np.zeros(self._nn, dtype=np.uint8)
        check(_lib().vfem_grid2_get_dirichlet_mask(self._h, m.ctypes.data_as(_capi._u8)))
        return np.stack([(m >> c) & 1 for c in range(2)], axis=1).astype(bool)

    def getForceMask(self):
        return self._forces != 0

    def getDirichletVarsAndValues(self):
        m = self.getDirichletMask()
        vals = np.zeros((self._nn, 2), order="F")
        check(_lib().vfem_grid2_get_dirichlet_values(self._h, ptr(vals)))
        nodes, comps = np.nonzero(m)
        return (list(2 * nodes + comps), list(vals[nodes, comps]))

    # --- layer-by-layer fabrication mask ---
    def setFabricationMaskHeightByLayer(self, l):
        check(_lib().vfem_grid2_set_mask_layer(self._h, int(l)))

    def getFabricationMaskHeight(self):
        h = C.c_double()
        check(_lib().vfem_grid2_get_mask_height(self._h, C.byref(h)))
        return h.value

    # --- physics ---
    def applyK(self, u):
        u = _as_vfield(u, self._nn, 2)
        out = _new_vfield(self._nn, 2)
        check(_lib().vfem_grid2_apply_k(self._h, ptr(u), ptr(out)))
        return out

    def buildLoadVector(self):
        out = _new_vfield(self._nn, 2)
        check(_lib().vfem_grid2_build_load(self._h, ptr(out)))
        return out

    def complianceGradient(self, u):
        u = _as_vfield(u, self._nn, 2)
        out = np.empty(self._nel)
        check(_lib().vfem_grid2_compliance_gradient(self._h, ptr(u), ptr(out)))
        return out

    def adjointSensitivity(self, lam, u, loadWeight=1.0, stiffnessWeight=1.0):
        lam = _as_vfield(lam, self._nn, 2)
        u = _as_vfield(u, self._nn, 2)
        out = np.empty(self._nel)
        check(_lib().vfem_grid2_adjoint_sensitivity(self._h, ptr(lam), ptr(u), float(loadWeight),
                                                    float(stiffnessWeight), ptr(out)))
        return out

    def elementEnergyDensity(self, u):
        u = _as_vfield(u, self._nn, 2)
        out = np.empty(self._nel)
        check(_lib().vfem_grid2_element_energy(self._h, ptr(u), ptr(out)))
        return out

    def solve(self, f):
        """Direct solve (TensorProductSimulator::solve) through a zero-coarsening hierarchy."""
        mg = self.multigridSolver(0)
        return mg.preconditionedConjugateGradient(np.zeros((self._nn, 2)), f, 1, 0.0)

    def multigridSolver(self, numCoarseningLevels):
        return MultigridSolver2D(self, int(numCoarseningLevels))


class _LevelSimulator2D:
    """Read-only view of a coarse 2D level (MultigridSolver::getSimulator(l), l > 0)."""

    _nc = 2

    def __init__(self, mg, l):
        self._mg, self._l = mg, l
        ne = np.zeros(2, dtype=np.int64)
        check(_lib().vfem_mg2_level_dims(mg._h, l, ne.ctypes.data_as(_capi._i64)))
        self._ne = tuple(int(v) for v in ne)

    def numNodes(self):
        return (self._ne[0] + 1) * (self._ne[1] + 1)

    def numElements(self):
        return self._ne[0] * self._ne[1]

    @property
    def NbElementsPerDimension(self):
        return np.array(self._ne)

    gridShape = NbElementsPerDimension

    @property
    def NbNodesPerDimension(self):
        return np.array([n + 1 for n in self._ne])

    def getDirichletMask(self):
        m = np.zeros(self.numNodes(), dtype=np.uint8)
        check(_lib().vfem_mg2_level_dirichlet_mask(self._mg._h, self._l, m.ctypes.data_as(_capi._u8)))
        return np.stack([(m >> c) & 1 for c in range(2)], axis=1).astype(bool)


class MultigridSolver2D:
    """MultigridSolver<double, 1, 1> (MultigridSolver.hh) over a TensorProductSimulator_2D."""

    def __init__(self, tps, numCoarseningLevels):
        h = C.c_void_p()
        check(_lib().vfem_mg2_create(tps._h, int(numCoarseningLevels), C.byref(h)))
        self._h = h
        self._tps = tps
        n = C.c_int()
        check(_lib().vfem_mg2_num_levels(h, C.byref(n)))
        self.numLevels = n.value
        self.lastStats = None
        self._prec = "fp64"

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_mg2_destroy(h)
            self._h = None

    def _nn(self, l):
        return self.getSimulator(l).numNodes()

    def getSimulator(self, l):
        if l == 0:
            return self._tps
        if l < 0 or l >= self.numLevels:
            raise IndexError("level out of range")
        return _LevelSimulator2D(self, l)

    def setPrecision(self, precision="fp64", outerMatvec="df"):
        """'fp64' (the reference's method) or 'mixed': the PCG preconditioner's V-cycle in FP32
        inside FP64 CG, whose matvec is 'df' (default: double-float on the FP32 units, FP64-class
        accuracy) or 'fp64'."""
        p = {"fp64": 0, "mixed": 1}[precision]
        m = {"fp64": 0, "df": 1}[outerMatvec]
        check(_lib().vfem_mg2_set_precision(self._h, p))
        check(_lib().vfem_mg2_set_outer_matvec(self._h, m))
        self._prec = precision

    def setUseGraphs(self, use):
        check(_lib().vfem_mg2_set_use_graphs(self._h, int(bool(use))))

    def setSymmetricGaussSeidel(self, symmetric):
        check(_lib().vfem_mg2_set_symmetric_gs(self._h, int(bool(symmetric))))

    def setFabricationMaskHeightByLayer(self, h):
        check(_lib().vfem_mg2_set_mask_layer(self._h, int(h)))

    def updateStiffnessMatrices(self):
        check(_lib().vfem_mg2_update_stiffness(self._h))

    def applyK(self, l, u):
        nn = self._nn(l)
        u = _as_vfield(u, nn, 2)
        out = _new_vfield(nn, 2)
        check(_lib().vfem_mg2_apply_k(self._h, int(l), ptr(u), ptr(out)))
        return out

    def computeResidual(self, l, u, b):
        nn = self._nn(l)
        u, b = _as_vfield(u, nn, 2), _as_vfield(b, nn, 2)
        out = _new_vfield(nn, 2)
        check(_lib().vfem_mg2_residual(self._h, int(l), ptr(u), ptr(b), ptr(out)))
        return out

    def zeroOutDirichletComponents(self, l, u):
        u = _as_vfield(u, self._nn(l), 2).copy(order="F")
        check(_lib().vfem_mg2_zero_dirichlet(self._h, int(l), ptr(u)))
        return u

    def smoothingMulticoloredGS(self, l, u, b, forwardSweep=True):
        nn = self._nn(l)
        u = _as_vfield(u, nn, 2).copy(order="F")
        b = _as_vfield(b, nn, 2)
        check(_lib().vfem_mg2_smooth(self._h, int(l), ptr(u), ptr(b), int(bool(forwardSweep))))
        return u

    def restriction(self, l, fine):
        fine = _as_vfield(fine, self._nn(l), 2)
        out = _new_vfield(self._nn(l + 1), 2)
        check(_lib().vfem_mg2_restrict(self._h, int(l), ptr(fine), ptr(out)))
        return out

    def interpolation(self, l, coarse, fine=None, accumulate=False):
        coarse = _as_vfield(coarse, self._nn(l + 1), 2)
        out = _new_vfield(self._nn(l), 2) if fine is None else _as_vfield(fine, self._nn(l), 2).copy(order="F")
        check(_lib().vfem_mg2_interpolate(self._h, int(l), ptr(coarse), ptr(out), int(bool(accumulate))))
        return out

    def coarseSolve(self, b):
        nn = self._nn(self.numLevels - 1)
        b = _as_vfield(b, nn, 2)
        out = _new_vfield(nn, 2)
        check(_lib().vfem_mg2_coarse_solve(self._h, ptr(b), ptr(out)))
        return out

    def solve(self, u, f, numSteps, numSmoothingSteps, stiffnessUpdated=False, zeroDirichlet=False,
              it_callback=None, fullMultigrid=False):
        nn = self._nn(0)
        u, f = _as_vfield(u, nn, 2), _as_vfield(f, nn, 2)
        if it_callback is None:
            out = _new_vfield(nn, 2)
            check(_lib().vfem_mg2_solve(self._h, ptr(u), ptr(f), int(numSteps), int(numSmoothingSteps),
                                        int(bool(zeroDirichlet)), int(bool(fullMultigrid)), ptr(out)))
            return out
        x = u
        for i in range(int(numSteps)):
            out = _new_vfield(nn, 2)
            check(_lib().vfem_mg2_solve(self._h, ptr(x), ptr(f), 1, int(numSmoothingSteps), int(bool(zeroDirichlet)),
                                        int(bool(fullMultigrid) and i == 0), ptr(out)))
            it_callback(i, out)
            x = out
        return x

    def preconditionedConjugateGradient(self, u, b, maxIter, tol, it_callback=None, mgIterations=1,
                                        mgSmoothingIterations=1, fullMultigrid=False):
        nn = self._nn(0)
        x = _as_vfield(u, nn, 2).copy(order="F")
        b = _as_vfield(b, nn, 2)
        stats = _capi.PcgStats()
        cb = _capi.PCG_CALLBACK()
        if it_callback is not None:
            def _cb(user, it, rnorm, xdev, rdev):
                it_callback(int(it), _device_to_host(xdev, nn, 2), _device_to_host(rdev, nn, 2))
                return 0
            cb = _capi.PCG_CALLBACK(_cb)
        check(_lib().vfem_mg2_pcg(self._h, ptr(x), ptr(b), int(maxIter), float(tol), int(mgIterations),
                                  int(mgSmoothingIterations), int(bool(fullMultigrid)), 0, cb, None, C.byref(stats)))
        self.lastStats = stats
        return x

    def timeKernel(self, kernel, reps=20):
        """Average device milliseconds of one launch (0 applyK, 1 GS sweep, 2 V-cycle, 3 PCG iteration)."""
        ms = C.c_double()
        check(_lib().vfem_mg2_time_kernel(self._h, int(kernel), int(reps), C.byref(ms)))
        return ms.value


def getClassName(simulator, name):
    """pyVoxelFEM.getClassName (VoxelFEM.cc:250-254): the name under which the class `name` for
    this simulator's instantiation is reachable, for scripts that subclass it via eval."""
    if not hasattr(detail, name):
        raise RuntimeError("Unknown class " + name)
    return "pyVoxelFEM.detail." + name


class _Detail:
    """The module's ``detail`` namespace (VoxelFEM.cc:405): the instantiated classes by name."""

    TopologyOptimizationProblem = TopologyOptimizationProblem
    MultigridComplianceObjective = MultigridComplianceObjective
    OCOptimizer = OCOptimizer
    LayerByLayerEvaluator = LayerByLayerEvaluator
    MultigridSolver = MultigridSolver
    MultigridSolver2D = MultigridSolver2D
    TensorProductSimulator_2D = TensorProductSimulator_2D
    TensorProductSimulator_3D = TensorProductSimulator_3D
    TensorProductSimulator_3D_Q2 = TensorProductSimulator_3D_Q2


detail = _Detail
