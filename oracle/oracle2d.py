"""Numpy restatement of VoxelFEM's solve-and-sensitivity path for bilinear quadrilaterals
(``TensorProductSimulator<double, 1, 1>``), the oracle of the GPU 2D engine.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke`` and the CPU-baseline
leg of ``bench.py``; never by the ``voxelfem_gb300`` package.

PARITY UNPINNED: the reference cannot be compiled here (its MeshFEM submodule, Eigen, TBB and
CHOLMOD are absent) and ships no tests or golden vectors. The functions below follow the
reference source with N = 2, citing the file:line each one restates; the tests pin the
element matrix to exact symbolic integration and check symmetry, Galerkin identities and
finite-difference gradients.

Conventions (identical to the reference):
  * node (i, j) -> i * (ny + 1) + j, element (i, j) -> i * ny + j (NDVector.hh:249-265);
  * element local node l = 2 a + b for the corner (i + a, j + b); element DOF 2 l + c;
  * nodal vector fields are SoA: component c of node n at [c * NN + n] (Eigen ColMajor VField,
    TensorProductSimulator.hh:180);
  * the 2D isotropic elasticity tensor is MeshFEM's ``ElasticityTensor<Real, 2>::setIsotropic``,
    lambda = E nu / ((1 + nu)(1 - (N - 1) nu)) = E nu / (1 - nu^2) (plane stress), mu = E / (2 (1 + nu)).
"""
import numpy as np

BUILD_DIR = 1
NONE = 2147483647
MARGIN = 4  # MultigridSolver.hh:532
GP = (0.21132486540518711775, 0.78867513459481288225)


def k0_2d(E, nu, h):
    """Element stiffness (TensorProductSimulator.hh:67-80 with 2-point Gauss per axis)."""
    lam = E * nu / ((1 + nu) * (1 - nu))
    mu = E / (2 * (1 + nu))
    K = np.zeros((8, 8))
    for a in range(2):
        for b in range(2):
            xi = (GP[a], GP[b])
            grad = np.zeros((4, 2))
            for l in range(4):
                bits = ((l >> 1) & 1, l & 1)
                for d in range(2):
                    v = 1.0
                    for e in range(2):
                        if e == d:
                            v *= (1.0 if bits[e] else -1.0) / h[e]
                        else:
                            v *= xi[e] if bits[e] else 1.0 - xi[e]
                    grad[l, d] = v
            eps = np.zeros((8, 2, 2))
            for l in range(4):
                for c in range(2):
                    E_ = eps[2 * l + c]
                    E_[c, :] += 0.5 * grad[l]
                    E_[:, c] += 0.5 * grad[l]
            tr = eps[:, 0, 0] + eps[:, 1, 1]
            dd = np.einsum("ipq,jpq->ij", eps, eps)
            K += 0.25 * (lam * np.outer(tr, tr) + 2 * mu * dd)
    return K * (h[0] * h[1])


class Sim2:
    """TensorProductSimulator<double, 1, 1> state (TensorProductSimulator.hh:2055-2141)."""

    def __init__(self, ne, bmin=(0.0, 0.0), bmax=None):
        self.ne = (int(ne[0]), int(ne[1]))
        self.nn = (self.ne[0] + 1, self.ne[1] + 1)
        self.NE = self.ne[0] * self.ne[1]
        self.NN = self.nn[0] * self.nn[1]
        self.bmin = np.asarray(bmin, dtype=float)
        self.bmax = np.asarray(bmax if bmax is not None else self.ne, dtype=float)
        self.h = (self.bmax - self.bmin) / np.asarray(self.ne, dtype=float)
        self.E, self.nu = 1.0, 0.0  # ETensor(1, 0) default (TensorProductSimulator.hh:2114)
        self.E0, self.Emin, self.gamma, self.q, self.law = 1.0, 1e-4, 3.0, 3.0, 0
        self.rho = np.zeros(self.NE)
        self.Y = np.zeros(self.NE)
        self.dmask = np.zeros(self.NN, dtype=np.uint8)
        self.dval = np.zeros(2 * self.NN)
        self.force = np.zeros(2 * self.NN)
        self.grav = np.zeros(2)
        self.maskH = np.inf
        self.firstMaskedE = NONE
        self.firstDetN = NONE
        I, J = np.meshgrid(np.arange(self.ne[0]), np.arange(self.ne[1]), indexing="ij")
        self.eI, self.eJ = I.ravel(), J.ravel()
        self.en = np.stack([(self.eI + (l >> 1)) * self.nn[1] + self.eJ + (l & 1) for l in range(4)], axis=1)
        NI, NJ = np.meshgrid(np.arange(self.nn[0]), np.arange(self.nn[1]), indexing="ij")
        self.nI, self.nJ = NI.ravel(), NJ.ravel()
        self.K0 = k0_2d(self.E, self.nu, self.h)
        self.Ke = None  # per-element matrices of a coarse level

    def node(self, i, j):
        return i * self.nn[1] + j

    def nondetNodes(self):
        return min(self.firstDetN, self.nn[1])

    def setMaterial(self, E, nu):
        self.E, self.nu = float(E), float(nu)
        self.K0 = k0_2d(self.E, self.nu, self.h)

    def setParams(self, E0=1.0, Emin=1e-4, gamma=3.0, q=3.0, law=0):
        self.E0, self.Emin, self.gamma, self.q, self.law = E0, Emin, gamma, q, law

    # TensorProductSimulator.hh:2055-2060, 2088-2102
    def updateY(self):
        if self.law == 0:
            Y = self.Emin + self.rho ** self.gamma * (self.E0 - self.Emin)
        else:
            Y = self.Emin + self.rho * (self.E0 - self.Emin) / (1 + self.q * (1 - self.rho))
        if self.maskH < self.bmax[BUILD_DIR]:
            Y = np.where(self.eJ >= self.firstMaskedE, 0.0, Y)
        self.Y = Y

    def setDensities(self, rho):
        self.rho = np.asarray(rho, dtype=float).ravel().copy()
        self.updateY()

    # TensorProductSimulator.hh:290-303, 327-331
    def setMaskHeight(self, hgt, update=True):
        if hgt < 0 or hgt > self.bmax[BUILD_DIR]:
            raise RuntimeError("Fabrication height out of range")
        self.maskH = hgt
        self.firstMaskedE = int(np.ceil(hgt / self.h[BUILD_DIR] - 1e-10))
        self.firstDetN = self.firstMaskedE + 1
        if update:
            self.updateY()

    def setFabricationMaskHeightByLayer(self, l):
        self.setMaskHeight(self.h[BUILD_DIR] * l)

    # TensorProductSimulator.hh:241-252 with BCBuilder::setDirichlet :73-88
    def addDirichletCondition(self, u, mn, mx, componentMask="xyz"):
        cm = sum(1 << c for c, ch in enumerate("xy") if ch in componentMask)
        px = self.bmin[0] + self.nI * self.h[0]
        py = self.bmin[1] + self.nJ * self.h[1]
        inside = (px >= mn[0]) & (px <= mx[0]) & (py >= mn[1]) & (py <= mx[1])
        for n in np.nonzero(inside)[0]:
            for c in range(2):
                if not (cm >> c) & 1:
                    continue
                if not (self.dmask[n] >> c) & 1:
                    self.dmask[n] |= 1 << c
                    self.dval[c * self.NN + n] = u[c]
                elif abs(self.dval[c * self.NN + n] - u[c]) > 1e-10:
                    raise RuntimeError("Conflicting dirichlet displacements.")

    def elemDisp(self, u):
        u = np.asarray(u)
        return np.stack([u[c * self.NN + self.en[:, l]] for l in range(4) for c in range(2)], axis=1)

    def scatter(self, fe):
        out = np.zeros(2 * self.NN)
        for c in range(2):
            idx = self.en.ravel()
            out[c * self.NN:(c + 1) * self.NN] = np.bincount(idx, weights=fe[:, c::2].ravel(), minlength=self.NN)
        return out

    def elementMatrices(self):
        return self.Y[:, None, None] * self.K0[None] if self.Ke is None else self.Ke

    # TPSStencils.hh:189-390 (ZeroInit applyK; detached rows come out zero)
    def applyK(self, u):
        ue = self.elemDisp(u)
        if self.Ke is None:
            return self.scatter((ue @ self.K0.T) * self.Y[:, None])
        return self.scatter(np.matmul(self.Ke, ue[:, :, None])[:, :, 0])

    def diagBlocks(self):
        M = np.zeros((self.NN, 2, 2))
        for l in range(4):
            if self.Ke is None:
                blk = self.Y[:, None, None] * self.K0[None, 2 * l:2 * l + 2, 2 * l:2 * l + 2]
            else:
                blk = self.Ke[:, 2 * l:2 * l + 2, 2 * l:2 * l + 2]
            for r in range(2):
                for c in range(2):
                    M[:, r, c] += np.bincount(self.en[:, l], weights=blk[:, r, c], minlength=self.NN)
        return M

    # TensorProductSimulator.hh:1269-1288 (integrated Q1 shape function = 1/4)
    def buildLoadVector(self):
        f = self.force.copy()
        if np.any(self.grav != 0):
            keep = self.eJ < self.firstMaskedE
            w = 0.25 * self.rho * self.h[0] * self.h[1]
            fe = np.zeros((self.NE, 8))
            for l in range(4):
                for c in range(2):
                    fe[:, 2 * l + c] = np.where(keep, self.grav[c] * w, 0.0)
            f += self.scatter(fe)
        return f

    def _dY(self):
        if self.law == 0:
            return self.gamma * self.rho ** (self.gamma - 1.0) * (self.E0 - self.Emin)
        return (1 + self.q) * (self.E0 - self.Emin) / (1 + self.q * (1 - self.rho)) ** 2

    # TensorProductSimulator.hh:973-1005
    def complianceGradient(self, u):
        ue = self.elemDisp(u)
        uKu = np.einsum("ei,ij,ej->e", ue, self.K0, ue)
        g = -0.5 * self._dY() * uKu
        if np.any(self.grav != 0):
            vol = self.h[0] * self.h[1]
            g = g + 0.25 * vol * sum(self.grav[c] * ue[:, c::2].sum(axis=1) for c in range(2))
        return np.where(self.eJ >= self.firstMaskedE, 0.0, g)

    # lam^T (df/drho - dK/drho u) (TensorProductSimulator.hh:1007-1055)
    def adjointSensitivity(self, lam, u, wF=1.0, wK=1.0):
        le, ue = self.elemDisp(lam), self.elemDisp(u)
        g = -wK * self._dY() * np.einsum("ei,ij,ej->e", le, self.K0, ue)
        if np.any(self.grav != 0):
            vol = self.h[0] * self.h[1]
            g = g + wF * 0.25 * vol * sum(self.grav[c] * le[:, c::2].sum(axis=1) for c in range(2))
        return np.where(self.eJ >= self.firstMaskedE, 0.0, g)

    # TensorProductSimulator.hh:638-654
    def elementEnergyDensity(self, u):
        ue = self.elemDisp(u)
        return 0.5 * self.Y * np.einsum("ei,ij,ej->e", ue, self.K0, ue)


def _phis():
    """Interpolation from a coarse element's corners to each child's corners
    (MultigridSolver.hh:664-687): phis[child][fine_n, coarse_n]."""
    out = []
    for fx in range(2):
        for fy in range(2):
            P = np.zeros((4, 4))
            for fn in range(4):
                p = (0.5 * (fn >> 1) + 0.5 * fx, 0.5 * (fn & 1) + 0.5 * fy)
                for cn in range(4):
                    bits = (cn >> 1, cn & 1)
                    P[fn, cn] = np.prod([p[d] if bits[d] else 1 - p[d] for d in range(2)])
            out.append(P)
    return out


class MG2:
    """MultigridSolver<double, 1, 1> (MultigridSolver.hh) over a Sim2."""

    def __init__(self, fine, coarsenings):
        self.sims = [fine]
        self.symmetricGS = True
        ne = list(fine.ne)
        for _ in range(coarsenings):
            if ne[0] % 2 or ne[1] % 2:
                raise RuntimeError("Grid size currently must be divisible by 2^numCoarseningLevels")
            ne = [ne[0] // 2, ne[1] // 2]
            c = Sim2(ne, fine.bmin, fine.bmax)
            c.setMaterial(fine.E, fine.nu)
            self._coarsenDirichlet(self.sims[-1], c)
            self.sims.append(c)
        L = len(self.sims)
        self.x = [np.zeros(2 * s.NN) for s in self.sims]
        self.b = [np.zeros(2 * s.NN) for s in self.sims]
        self.r = [np.zeros(2 * s.NN) for s in self.sims]
        self.I2 = [np.kron(P, np.eye(2)) for P in _phis()]  # phi (x) Id_2, 8 x 8
        self.valid = False
        self.L = L

    # MultigridSolver.hh:58-103
    @staticmethod
    def _coarsenDirichlet(f, c):
        for fn in np.nonzero(f.dmask)[0]:
            fidx = (f.nI[fn], f.nJ[fn])
            e, pob = [0, 0], [0, 0]
            for d in range(2):
                p = f.bmin[d] + fidx[d] * f.h[d]
                fd = (p - c.bmin[d]) / c.h[d]
                ed = c.ne[d] - 1 if abs(fd - c.ne[d]) < 1e-10 else int(fd)
                e[d] = ed
                cref = (p - (c.bmin[d] + ed * c.h[d])) / c.h[d]
                pob[d] = 0 if abs(cref) < 1e-9 else (1 if abs(cref - 1.0) < 1e-9 else -1)
            for ln in range(4):
                lb = (ln >> 1, ln & 1)
                if any(pob[d] != -1 and pob[d] != lb[d] for d in range(2)):
                    continue
                cn = c.node(e[0] + lb[0], e[1] + lb[1])
                for comp in range(2):
                    if (f.dmask[fn] >> comp) & 1 and not (c.dmask[cn] >> comp) & 1:
                        c.dmask[cn] |= 1 << comp
                        c.dval[comp * c.NN + cn] = 0.0

    def setFabricationMaskHeightByLayer(self, l):
        f = self.sims[0]
        f.setMaskHeight(f.h[BUILD_DIR] * l)
        for s in self.sims[1:]:
            s.setMaskHeight(f.maskH, update=False)
        self.valid = False

    # MultigridSolver.hh:712-819 (coarsenedKe), 846-905
    def updateStiffnessMatrices(self):
        for l in range(1, self.L):
            s, f = self.sims[l], self.sims[l - 1]
            Kf = f.elementMatrices()
            Ke = np.zeros((s.NE, 8, 8))
            ci = 0
            for a in range(2):
                for b in range(2):
                    child = (2 * s.eI + a) * f.ne[1] + 2 * s.eJ + b
                    I = self.I2[ci]
                    Ke += np.matmul(np.matmul(I.T[None], Kf[child]), I[None])
                    ci += 1
            Ke[s.eJ >= s.firstMaskedE] = 0.0
            s.Ke = Ke
        self.valid = True

    def _ensure(self):
        if not self.valid:
            self.updateStiffnessMatrices()

    def applyK(self, l, u):
        if l > 0:
            self._ensure()
        return self.sims[l].applyK(u)

    @staticmethod
    def zeroDirichlet(s, u):
        for c in range(2):
            u[c * s.NN:(c + 1) * s.NN][(s.dmask >> c) & 1 == 1] = 0.0

    @staticmethod
    def enforceDirichlet(s, u, zero):
        for c in range(2):
            m = (s.dmask >> c) & 1 == 1
            u[c * s.NN:(c + 1) * s.NN][m] = 0.0 if zero else s.dval[c * s.NN:(c + 1) * s.NN][m]

    # MultigridSolver.hh:527-541
    def computeResidual(self, l, u, b, res=None):
        s = self.sims[l]
        res = np.zeros(2 * s.NN) if res is None else res
        h = min(s.nondetNodes() + MARGIN, s.nn[1])
        rows = s.nJ < h
        for c in range(2):
            res[c * s.NN:(c + 1) * s.NN][rows] = b[c * s.NN:(c + 1) * s.NN][rows]
        res -= self.applyK(l, u)
        self.zeroDirichlet(s, res)
        return res

    # smoothingMulticoloredGS + m_smoothNode (MultigridSolver.hh:348-458). Nodes of one colour
    # share no element, so each colour is one vectorised block update.
    def smooth(self, l, u, b, forward=True):
        if l > 0:
            self._ensure()
        s = self.sims[l]
        key = (id(s.Ke), s.Y.ctypes.data, float(s.Y.sum()))
        cached = getattr(self, "_diag", {}).get(l)
        if cached is None or cached[0] != key:
            self._diag = getattr(self, "_diag", {})
            self._diag[l] = (key, s.diagBlocks())
        M = self._diag[l][1]
        nyv = s.nondetNodes()
        NN = s.NN
        for ci in range(4):
            col = ci if forward else 3 - ci
            sel = np.nonzero((s.nI % 2 == (col >> 1)) & (s.nJ % 2 == (col & 1)) & (s.nJ < nyv) & (s.dmask != 3))[0]
            if sel.size == 0:
                continue
            Ku = s.applyK(u)
            bms = np.stack([b[sel] - Ku[sel], b[NN + sel] - Ku[NN + sel]], axis=1)
            Mn = M[sel]
            dm = s.dmask[sel]
            du = np.zeros_like(bms)
            full = dm == 0
            det = Mn[:, 0, 0] * Mn[:, 1, 1] - Mn[:, 0, 1] * Mn[:, 1, 0]
            du[full, 0] = ((Mn[:, 1, 1] * bms[:, 0] - Mn[:, 0, 1] * bms[:, 1]) / det)[full]
            du[full, 1] = ((Mn[:, 0, 0] * bms[:, 1] - Mn[:, 1, 0] * bms[:, 0]) / det)[full]
            part = ~full
            if part.any():
                ud = np.zeros((part.sum(), 2))
                Mp, bp, dp = Mn[part], bms[part], dm[part]
                for i in ((0, 1) if forward else (1, 0)):
                    free = ((dp >> i) & 1) == 0
                    ud[:, i] = (bp[:, i] - (Mp[:, i, 0] * ud[:, 0] + Mp[:, i, 1] * ud[:, 1])) * free / Mp[:, i, i]
                du[part] = ud
            u[sel] += du[:, 0]
            u[NN + sel] += du[:, 1]
        return u

    @staticmethod
    def _prolong1d(nc):
        """Bilinear prolongation along one axis, (2 (nc - 1) + 1) x nc (MultigridSolver.hh:163-212)."""
        nf = 2 * (nc - 1) + 1
        P = np.zeros((nf, nc))
        for f in range(nf):
            if f % 2 == 0:
                P[f, f // 2] = 1.0
            else:
                P[f, f // 2] = P[f, f // 2 + 1] = 0.5
        return P

    # MultigridSolver.hh:217-275 (full weighting = P^T over the nondetached fine rows)
    def restrict(self, l, vals):
        fs, cs = self.sims[l], self.sims[l + 1]
        cyv, fyv = cs.nondetNodes(), fs.nondetNodes()
        Px, Py = self._prolong1d(cs.nn[0]), self._prolong1d(cs.nn[1])
        res = np.zeros(2 * cs.NN)
        for c in range(2):
            F = np.asarray(vals[c * fs.NN:(c + 1) * fs.NN]).reshape(fs.nn).copy()
            F[:, fyv:] = 0.0
            C = Px.T @ F @ Py
            C[:, cyv:] = 0.0
            res[c * cs.NN:(c + 1) * cs.NN] = C.ravel()
        return res

    # MultigridSolver.hh:163-212
    def interpolate(self, l, cvals, out=None, accumulate=True):
        fs, cs = self.sims[l], self.sims[l + 1]
        out = np.zeros(2 * fs.NN) if out is None else out
        fyv = fs.nondetNodes() if accumulate else fs.nn[1]
        Px, Py = self._prolong1d(cs.nn[0]), self._prolong1d(cs.nn[1])
        for c in range(2):
            Fv = Px @ np.asarray(cvals[c * cs.NN:(c + 1) * cs.NN]).reshape(cs.nn) @ Py.T
            O = out[c * fs.NN:(c + 1) * fs.NN].reshape(fs.nn)
            if accumulate:
                O[:, :fyv] += Fv[:, :fyv]
            else:
                O[:, :fyv] = Fv[:, :fyv]
        return out

    @staticmethod
    def maskedSetZero(s, u, margin):
        h = min(s.nondetNodes() + margin, s.nn[1])
        for c in range(2):
            u[c * s.NN:(c + 1) * s.NN][s.nJ < h] = 0.0

    # TensorProductSimulator.hh:1181-1230 (dense solve of the free DOFs of the coarsest level)
    def coarseSolve(self, b):
        self._ensure()
        s = self.sims[-1]
        fixed = np.zeros(2 * s.NN, dtype=bool)
        for c in range(2):
            fixed[c::2] = ((s.dmask >> c) & 1 == 1) | (s.nJ >= s.firstDetN)
        Ke = s.elementMatrices()
        A = np.zeros((2 * s.NN, 2 * s.NN))  # node-major DOF 2 n + c
        dofs = np.stack([2 * s.en[:, l] + c for l in range(4) for c in range(2)], axis=1)
        for i in range(8):
            for j in range(8):
                np.add.at(A, (dofs[:, i], dofs[:, j]), Ke[:, i, j])
        free = np.nonzero(~fixed)[0]
        rhs = np.array([b[(d % 2) * s.NN + d // 2] for d in free])
        sol = np.linalg.solve(A[np.ix_(free, free)], rhs)
        x = np.zeros(2 * s.NN)
        for t, d in enumerate(free):
            x[(d % 2) * s.NN + d // 2] = sol[t]
        return x

    # MultigridSolver.hh:617-658
    def vcycle(self, l, sweeps, residualSystem):
        if l == self.L - 1:
            self.x[l] = self.coarseSolve(self.b[l])
            return
        s = self.sims[l]
        self.enforceDirichlet(s, self.x[l], residualSystem)
        for _ in range(sweeps):
            self.smooth(l, self.x[l], self.b[l], True)
        self.computeResidual(l, self.x[l], self.b[l], self.r[l])
        self.b[l + 1] = self.restrict(l, self.r[l])
        self.maskedSetZero(self.sims[l + 1], self.x[l + 1], MARGIN)
        self.vcycle(l + 1, sweeps, True)
        self.interpolate(l, self.x[l + 1], self.x[l], True)
        for _ in range(sweeps):
            self.smooth(l, self.x[l], self.b[l], not self.symmetricGS)

    # MultigridSolver.hh:587-609
    def fullMultigrid(self, l, sweeps, residualSystem):
        if l == self.L - 1:
            self.x[l] = self.coarseSolve(self.b[l])
            return
        self.b[l + 1] = self.restrict(l, self.b[l])
        self.fullMultigrid(l + 1, sweeps, residualSystem)
        self.interpolate(l, self.x[l + 1], self.x[l], False)
        self.vcycle(l, sweeps, residualSystem)

    # MultigridSolver.hh:547-573
    def solve(self, u0, f, numSteps, numSmoothingSteps, zeroDirichlet=False, fullMultigrid=False):
        self._ensure()
        self.x[0] = np.asarray(u0, dtype=float).copy()
        if numSteps == 0:
            return self.x[0].copy()
        self.b[0] = np.asarray(f, dtype=float).copy()
        if fullMultigrid:
            self.fullMultigrid(0, numSmoothingSteps, zeroDirichlet)
            for _ in range(1, numSteps):
                self.vcycle(0, numSmoothingSteps, zeroDirichlet)
        else:
            for _ in range(numSteps):
                self.vcycle(0, numSmoothingSteps, zeroDirichlet)
        return self.x[0].copy()

    @staticmethod
    def maskedDot(s, a, b):
        rows = s.nJ < s.nondetNodes()
        return float(sum(np.dot(a[c * s.NN:(c + 1) * s.NN][rows], b[c * s.NN:(c + 1) * s.NN][rows]) for c in range(2)))

    # MultigridSolver.hh:1047-1152
    def pcg(self, x, b, maxIter, tol, mgIterations=1, mgSmoothingIterations=1, fullMultigrid=False,
            dirichletSatisfied=False, it_callback=None):
        fs = self.sims[0]
        NN = fs.NN
        x = np.asarray(x, dtype=float).copy()
        b = np.asarray(b, dtype=float)
        if not dirichletSatisfied:
            self.enforceDirichlet(fs, x, False)
        bnorm2 = self.maskedDot(fs, b, b)
        r = self.computeResidual(0, x, b)
        rsq = self.maskedDot(fs, r, r)
        rows = np.concatenate([fs.nJ < fs.nondetNodes()] * 2)
        rMr, d, it = 0.0, None, 0
        while it < maxIter and rsq > tol * tol * bnorm2:
            it += 1
            if mgIterations > 0:
                s = self.solve(np.zeros(2 * NN), r, mgIterations, mgSmoothingIterations, True, fullMultigrid)
            else:
                s = r.copy()
            self.zeroDirichlet(fs, s)
            old, rMr = rMr, self.maskedDot(fs, r, s)
            d = s.copy() if d is None else (rMr / old) * d + s
            Ad = self.applyK(0, d)
            self.zeroDirichlet(fs, Ad)
            alpha = rMr / self.maskedDot(fs, d, Ad)
            x[rows] += alpha * d[rows]
            r[rows] -= alpha * Ad[rows]
            rsq = self.maskedDot(fs, r, r)
            if it_callback is not None:
                it_callback(it, np.sqrt(rsq))
        self.lastIterations = it
        self.lastRelres = np.sqrt(rsq / bnorm2) if bnorm2 > 0 else np.sqrt(rsq)
        return x


def _reflect(i, s):
    while i < 0 or i >= s:
        if i >= s:
            i = 2 * s - i - 1
        if i < 0:
            i = -i - 1
    return i


def smoothing_filter_2d(x, dims, radius, ftype):
    """SmoothingFilter ApplyImpl<2> (TopologyOptimizationFilter.hh:285-400); ftype 0 Const, 1 Linear."""
    nx, ny = dims
    x = np.asarray(x, dtype=float).reshape(nx, ny)
    out = np.zeros_like(x)
    W = 0.0
    for a in range(-radius, radius + 1):
        for b in range(-radius, radius + 1):
            w = (radius + 1.0 - np.sqrt(a * a + b * b)) if ftype == 1 else 1.0
            if w <= 0:
                continue
            ii = np.array([_reflect(i + a, nx) for i in range(nx)])
            jj = np.array([_reflect(j + b, ny) for j in range(ny)])
            out += w * x[np.ix_(ii, jj)]
            W += w
    return (out / W).ravel()


def projection(x, beta):
    th = np.tanh(0.5 * beta)
    return (th + np.tanh(beta * (np.asarray(x) - 0.5))) / (2 * th)


def projection_backprop(g, v, beta):
    return np.asarray(g) * (1.0 - np.tanh(beta * (np.asarray(v) - 0.5)) ** 2) / (2 * np.tanh(0.5 * beta) / beta)


class TOP2:
    """TopologyOptimizationProblem with a MultigridComplianceObjective, a filter chain and a
    total-volume constraint (TopologyOptimizationProblem.hh:41-121,
    TopologyOptimizationObjective.hh:71-105) plus the OC step (OptimalityCriterion.hh:51-138).
    filters: list of ("smooth", radius, type) or ("proj", beta)."""

    def __init__(self, mg, filters, volfrac, cgIter=100, tol=1e-5, mgIterations=1, mgSmoothingIterations=2,
                 fullMultigrid=True, zeroInit=False):
        self.mg, self.sim = mg, mg.sims[0]
        self.filters, self.volfrac = filters, volfrac
        self.cgIter, self.tol, self.mgIter, self.mgSweeps = cgIter, tol, mgIterations, mgSmoothingIterations
        self.fmg, self.zeroInit = fullMultigrid, zeroInit
        self.f = self.sim.buildLoadVector()
        self.u = np.zeros(2 * self.sim.NN)
        self.lambda_min, self.lambda_max = 1.0, 2.0

    def _apply(self, fs, x):
        if fs[0] == "smooth":
            return smoothing_filter_2d(x, self.sim.ne, fs[1], fs[2])
        return projection(x, fs[1])

    def _backprop(self, g):
        for i in range(len(self.filters) - 1, -1, -1):
            fs = self.filters[i]
            if fs[0] == "smooth":
                g = smoothing_filter_2d(g, self.sim.ne, fs[1], fs[2])
            else:
                g = projection_backprop(g, self.vars[i], fs[1])
        return g

    def setVars(self, x):
        self.vars = [np.asarray(x, dtype=float).copy()]
        for fs in self.filters:
            self.vars.append(self._apply(fs, self.vars[-1]))
        rho = self.vars[-1]
        if np.any(rho > 1.0) or np.any(rho < 0):
            raise RuntimeError("Density value out of range")
        self.sim.setDensities(rho)
        self.mg.valid = False
        if self.zeroInit:
            self.u[:] = 0.0
        self.u = self.mg.pcg(self.u, self.f, self.cgIter, self.tol, self.mgIter, self.mgSweeps, self.fmg)

    def evaluateObjective(self):
        return 0.5 * float(np.dot(self.f, self.u))

    def evaluateObjectiveGradient(self):
        return self._backprop(self.sim.complianceGradient(self.u))

    def evaluateConstraints(self):
        return 1.0 - self.vars[-1].mean() / self.volfrac

    def evaluateConstraintsJacobian(self):
        return self._backprop(np.full(self.sim.NE, -1.0 / (self.volfrac * self.sim.NE)))

    def _constraintAt(self, x):
        for fs in self.filters:
            x = self._apply(fs, x)
        return 1.0 - x.mean() / self.volfrac

    def ocStep(self, m=0.2, p=0.5, ctol=1e-6):
        dJ = self.evaluateObjectiveGradient()
        dc = self.evaluateConstraintsJacobian()
        x0 = self.vars[0].copy()

        def step(lam):
            with np.errstate(all="ignore"):
                res = x0 * np.power(dJ / (dc * lam), p)
                res = np.minimum(np.maximum(np.minimum(np.maximum(res, x0 - m), x0 + m), 0.0), 1.0)
                return np.where(np.isfinite(res), res, x0)

        lmid = 0.5 * (self.lambda_min + self.lambda_max)
        self.lambda_max = 32 * self.lambda_max - 31 * lmid
        self.lambda_min = max(32 * self.lambda_min - 31 * lmid, 0.01)
        nit = 0
        while nit < 100:
            if self._constraintAt(step(self.lambda_min)) < 0:
                break
            self.lambda_max = self.lambda_min
            self.lambda_min /= 2
            nit += 1
        if nit == 0:
            while nit < 100:
                if self._constraintAt(step(self.lambda_max)) > 0:
                    break
                self.lambda_min = self.lambda_max
                self.lambda_max *= 2
                nit += 1
        while True:
            lmid = 0.5 * (self.lambda_min + self.lambda_max)
            viol = self._constraintAt(step(lmid))
            if abs(viol) <= ctol:
                break
            if viol < 0:
                self.lambda_min = lmid
            if viol > 0:
                self.lambda_max = lmid
        self.setVars(step(lmid))


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
    """LayerByLayerEvaluator::run (LayerByLayer.hh:223-296) with its initial-guess generators
    (LayerByLayer.hh:55-209) on the 2D simulator: heights ny, ny - inc, ..., each solved from a
    guess built from the previous heights' solutions ("fd": u(0) or 2 u(0) - u(1); "constant":
    u(0); "N=<s>": Galerkin projection onto the last s solutions, A_ij = u_i . K u_j,
    b_i = u_i . f over the nondetached nodes of the new mask, minimum-norm least squares with
    singular values <= s eps sigma_max dropped). Returns (layers, compliances, PCG iterations,
    gradient sum, full-design solution)."""
    kind, nmax = _lbl_init(method)
    ny = sim.ne[1]
    hist, layers, comps, iters = [], [], [], []
    grad = np.zeros(sim.NE)
    l = ny
    while l > 0:
        mg.setFabricationMaskHeightByLayer(l)
        live = np.tile(sim.nJ <= l, 2)
        f = sim.buildLoadVector()
        s = len(hist)
        if not zero_init and l == ny and u_full is not None:
            g = u_full.copy()
        elif kind == "zero" or s == 0:
            g = np.zeros(2 * sim.NN)
        elif kind == "fd":
            g = hist[0].copy() if s == 1 else 2.0 * hist[0] - hist[1]
        else:
            Ku = [sim.applyK(u) for u in hist]
            A = np.array([[float(np.dot(hist[i][live], Ku[j][live])) for j in range(s)] for i in range(s)])
            A = 0.5 * (A + A.T)
            b = np.array([float(np.dot(hist[i][live], f[live])) for i in range(s)])
            c = np.linalg.lstsq(A, b, rcond=s * np.finfo(np.float64).eps)[0]
            g = sum(c[i] * hist[i] for i in range(s))
        g[~live] = 0.0
        u = mg.pcg(g, f, max_iter, tol, mg_iterations, mg_smoothing_iterations, fmg, dirichletSatisfied=True)
        layers.append(l)
        comps.append(float(np.dot(f[live], u[live])))
        iters.append(mg.lastIterations)
        grad += sim.complianceGradient(u)
        if l == ny:
            u_full = u.copy()
        if l >= layer_increment and nmax > 0:
            hist.insert(0, u.copy())
            del hist[nmax:]
        l -= min(layer_increment, l)
    return np.array(layers), np.array(comps), np.array(iters), grad, u_full
