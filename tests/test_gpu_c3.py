"""Full-size topology optimisation through the differentiable solve: the 3D MBB beam at
192x96x96 voxels (5.45M DOF), volume fraction 0.3 from uniform 0.3, SmoothingFilter(2, Linear)
then ProjectionFilter(1), 50 OC iterations.

Set-up: the boundary conditions come from the reference's own examples/bcs/3D/mbb_N.bc and the
material from examples/materials/B9Creator.material (their text is stored in
tests/golden/reference_bcs.json), read by applyDisplacementsAndLoadsFromFile / readMaterial; the
oracle simulator takes the same regions from the oracle's reader, and the two Dirichlet masks and
load vectors must agree bit for bit.

Loop: every iteration's gradient comes from ComplianceVolume (GPU forward solve, adjoint backward)
and drives the library's OC step on the GPU (OCOptimizer.step with that gradient), which meets the
volume constraint to 1e-6.

At iterations 0 and 50:
- the autograd gradient is compared with the oracle's sensitivity: the oracle's filters, an FP64
  CPU solve to 1e-12, the oracle's compliance gradient and the oracle's filter transposes
  (1e-6 relative); the problem's own gradient (evaluateObjectiveGradient) agrees as well;
- a central finite difference with step 1e-6 along a random +-1 direction v on 64 random
  elements: C(x + hv) - C(x - hv) from two FP64 GPU solves (to 1e-13), to 1e-5 relative. The difference is
  evaluated as 1/2 u+^T (K- - K+) u- = 1/2 sum_e (E-_e - E+_e) u+_e^T K0 u-_e, which equals
  1/2 f^T (u+ - u-) exactly for exact solves (the MBB load does not depend on the densities),
  over the few thousand elements whose densities differ. Forming it as a difference of two
  compliances instead cancels ~11 of the 16 digits at this size (a single solve's 1e-13
  residual is then ~1e-2 of the difference); that form is checked too, at its noise floor (1e-3).
"""
import json
import os

import numpy as np
import pytest

from oracle import bc_oracle
from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu

NE = (192, 96, 96)
LEVELS = 4  # optMGLevel([192, 96, 96], 3)
VOLFRAC = 0.3
E0, EMIN, GAMMA = 1.0, 1e-9, 3.0
BETA = 1.0
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_bcs.json")


def _oracle_chain(oracle, x):
    sm = oracle.smoothing_filter(x, NE, 2, 1)
    return sm, oracle.projection_apply(sm, BETA)


def _oracle_chain_transpose(oracle, g, sm):
    return oracle.smoothing_filter(oracle.projection_backprop(g, sm, BETA), NE, 2, 1)


def _element_bilinear(K0, up, um, elems):
    """u+_e^T K0 u-_e for the listed elements (flat indices), local node l = 4a + 2b + c."""
    nx, ny, nz = NE
    i, rem = np.divmod(elems, ny * nz)
    j, k = np.divmod(rem, nz)
    ue_p = np.empty((elems.size, 24))
    ue_m = np.empty((elems.size, 24))
    for l in range(8):
        a, b, c = (l >> 2) & 1, (l >> 1) & 1, l & 1
        node = ((i + a) * (ny + 1) + (j + b)) * (nz + 1) + (k + c)
        for d in range(3):
            ue_p[:, 3 * l + d] = up[node, d]
            ue_m[:, 3 * l + d] = um[node, d]
    return np.einsum("ei,ij,ej->e", ue_p, K0, ue_m)


def test_c3_topology_optimisation_full_size(gpu, oracle, tmp_path):
    import torch
    from voxelfem_gb300 import autograd as vag

    with open(GOLD) as f:
        gold = json.load(f)
    bc_path = tmp_path / "mbb_N.bc"
    bc_path.write_text(gold["bc3d"]["mbb_N.bc"])
    mat_path = tmp_path / gold["material"]["file"]
    mat_path.write_text(gold["material"]["text"])
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in NE]]

    sim = pv.TensorProductSimulator([1, 1, 1], bbox, NE)
    sim.readMaterial(str(mat_path))
    sim.E_0, sim.E_min, sim.gamma = E0, EMIN, GAMMA
    sim.applyDisplacementsAndLoadsFromFile(str(bc_path))
    x = np.full(sim.numElements(), VOLFRAC)
    sim.setDensities(x)

    o = oracle.Sim(NE)
    o.setMaterial(gold["material"]["young"], gold["material"]["poisson"])
    o.setParams(E0=E0, Emin=EMIN, gamma=GAMMA)
    text = gold["bc3d"]["mbb_N.bc"]
    bits, _, forces = bc_oracle.apply_bc_text_vectorized(text, NE, bbox)
    for typ, val, mn, mx in bc_oracle.read_regions(text, NE, bbox):
        if typ.startswith("dirichlet"):
            o.addDirichletCondition(val, mn, mx, typ[len("dirichlet"):] or "xyz")
    o.setNodalForces(forces)
    o.setDensities(x)
    np.testing.assert_array_equal(o.dirichletMask(), bits)
    m = sim.getDirichletMask()
    np.testing.assert_array_equal(m[:, 0] * 1 + m[:, 1] * 2 + m[:, 2] * 4, bits)
    np.testing.assert_array_equal(sim.buildLoadVector(), o.buildLoadVector())
    K0 = o.K0()
    assert float(np.max(np.abs(np.asarray(sim.fullDensityElementStiffnessMatrix()) - K0))) < 1e-14

    # the device-resident problem whose OC step the loop drives, with its own solver
    mg_top = sim.multigridSolver(LEVELS)
    mg_top.setPrecision("mixed")
    obj = pv.MultigridComplianceObjective(mg_top)
    obj.tol, obj.cgIter = 1e-10, 500
    filters = [pv.SmoothingFilter(2, pv.SmoothingFilter.Type.Linear), pv.ProjectionFilter(BETA)]
    top = pv.TopologyOptimizationProblem(sim, obj, [pv.TotalVolumeConstraint(VOLFRAC)], filters)
    top.setVars(x)
    oc = pv.OCOptimizer(top)
    # the differentiable solve
    mg = sim.multigridSolver(LEVELS)
    mg.setPrecision("mixed")
    solver = vag.SolverContext(sim, mg, cgIter=500, tol=1e-10)
    chain = pv.FilterChain([pv.SmoothingFilter(2, pv.SmoothingFilter.Type.Linear), pv.ProjectionFilter(BETA)], NE)
    # the plain FP64 solver for the finite differences
    mg64 = sim.multigridSolver(LEVELS)
    omg = oracle.MG(o, LEVELS)
    rng = np.random.default_rng(3)

    def autograd_gradient(xd):
        xt = torch.tensor(xd, dtype=torch.float64, requires_grad=True)
        C, V = vag.ComplianceVolume.apply(xt, solver, chain, "self")
        C.backward()
        return float(C.detach()), xt.grad.numpy().copy()

    def check(xd, g):
        # the oracle's sensitivity at the same design
        sm, rho = _oracle_chain(oracle, xd)
        chain.setDesignVars(xd)
        assert float(np.max(np.abs(chain.physicalVars() - rho))) < 1e-14
        o.setDensities(rho)
        f = o.buildLoadVector()
        uo = omg.preconditionedConjugateGradient(np.zeros_like(f), f, 500, 1e-12, None, 1, 2, False)
        gref = _oracle_chain_transpose(oracle, o.complianceGradient(uo), sm)
        err_oracle = float(np.max(np.abs(g - gref)) / np.max(np.abs(gref)))
        assert err_oracle < 1e-6, err_oracle
        # central difference along v over 64 random elements, FP64 GPU solves
        idx = rng.choice(xd.size, 64, replace=False)
        v = np.zeros_like(xd)
        v[idx] = rng.choice([-1.0, 1.0], 64)
        h = 1e-6
        sim.setDensities(rho)
        fb = sim.buildLoadVector()
        ub = mg64.preconditionedConjugateGradient(np.zeros_like(fb), fb, 500, 1e-13, None, 1, 2, False)
        us, rhos, comps = [], [], []
        for s in (+1, -1):
            _, rs = _oracle_chain(oracle, xd + s * h * v)
            sim.setDensities(rs)
            fs = sim.buildLoadVector()
            assert np.array_equal(fs, fb)  # the MBB load does not depend on the densities
            u = mg64.preconditionedConjugateGradient(ub, fs, 500, 1e-13, None, 1, 2, False)
            us.append(u)
            rhos.append(rs)
            comps.append(0.5 * float(np.sum(fs * u)))
        solver.invalidate()  # the difference solves changed the simulator's densities
        Ep = EMIN + rhos[0] ** GAMMA * (E0 - EMIN)
        Em = EMIN + rhos[1] ** GAMMA * (E0 - EMIN)
        changed = np.flatnonzero(Ep != Em)
        dC = 0.5 * float(np.sum((Em[changed] - Ep[changed]) * _element_bilinear(K0, us[0], us[1], changed)))
        fd = dC / (2 * h)
        fd_plain = (comps[0] - comps[1]) / (2 * h)
        gv = float(np.dot(g, v))
        print("oracle rel %.2e, central difference rel %.2e (as a compliance difference %.2e), %d elements moved"
              % (err_oracle, abs(fd - gv) / abs(gv), abs(fd_plain - gv) / abs(gv), changed.size))
        assert abs(fd - gv) < 1e-5 * abs(gv), (fd, gv)
        assert abs(fd_plain - gv) < 1e-3 * abs(gv), (fd_plain, gv)

    comps = []
    xk = top.getVars().copy()
    for it in range(51):
        C, g = autograd_gradient(xk)
        comps.append(C)
        if it in (0, 50):
            gp = top.evaluateObjectiveGradient()
            assert float(np.max(np.abs(gp - g)) / np.max(np.abs(g))) < 1e-6
            assert abs(top.evaluateObjective() - C) / abs(C) < 1e-8
            check(xk, g)
        if it == 50:
            break
        oc.step(objectiveGradient=g)
        solver.invalidate()
        xk = top.getVars().copy()
        assert abs(top.evaluateConstraints()[0]) <= 1e-6
    assert comps[-1] < 0.5 * comps[0]
