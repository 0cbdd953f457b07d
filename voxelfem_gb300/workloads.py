"""Seeded synthetic problem set-ups of the solve-path workloads.

* ``cantilever``: x = 0 face fully fixed; a total downward (-y) unit load split
  equally over the line of nodes at x = max, z = mid; densities i.i.d.
  uniform[rho_lo, 1] from ``numpy.random.default_rng(seed)`` in row-major
  element order; E0 = 1, Emin = 1e-9, nu = 0.3, SIMP p = 3; unit voxels.
  (64x32x32 with rho in [0.3, 1] is the CPU-runnable parity case; 256x128x128
  with rho in [0.01, 1] is the 12.8M-DOF precision case.)
* ``mbb``: the 3D MBB beam of the reference's ``mbb_N.bc`` regions (x = 0,
  z = 0 edge fixed, x = max, z = 0 edge fixed in y/z, unit -y load at the top
  centre), densities uniform.
* ``layer_by_layer``: base face y = 0 fixed, self-weight gravity (0, -1, 0).

Each builder takes the simulator class of the API it targets (the GPU
``voxelfem_gb300.pyVoxelFEM`` or the CPU oracle wrapper), so the same inputs
feed both sides of a parity check.
"""
import numpy as np


def cantilever_forces(ne):
    nx, ny, nz = ne
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    f = np.zeros((nn, 3), order="F")
    idx = np.arange(nn).reshape(nx + 1, ny + 1, nz + 1)
    line = idx[nx, :, nz // 2].ravel()
    f[line, 1] = -1.0 / line.size
    return f


def densities(ne, rho_lo, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(rho_lo, 1.0, int(np.prod(ne)))


def setup_cantilever(sim, ne, rho_lo=0.3, seed=0, set_forces=None):
    """Apply the cantilever material, densities and boundary conditions to ``sim``."""
    nx, ny, nz = ne
    sim_set_material(sim)
    sim.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, float(ny), float(nz)], "xyz")
    f = cantilever_forces(ne)
    if set_forces is None:
        sim.setNodalForces(f)
    else:
        set_forces(f)
    rho = densities(ne, rho_lo, seed)
    sim.setDensities(rho)
    return rho, f


def sim_set_material(sim):
    if hasattr(sim, "ETensor"):
        sim.ETensor = (1.0, 0.3)
        sim.E_0 = 1.0
        sim.E_min = 1e-9
        sim.gamma = 3.0
    else:  # oracle wrapper
        sim.setMaterial(1.0, 0.3)
        sim.setParams(E0=1.0, Emin=1e-9, gamma=3.0)


def mbb_regions(ne):
    """Boundary conditions of the reference's examples/bcs/3D/mbb_N.bc in absolute coordinates."""
    nx, ny, nz = (float(v) for v in ne)
    eps = 1e-4
    dir_all = ([0.0, 0.0, 0.0], [-eps * nx, -eps * ny, -eps * nz], [eps * nx, (1 + eps) * ny, eps * nz], "xyz")
    dir_yz = ([0.0, 0.0, 0.0], [(1 - eps) * nx, -eps * ny, -eps * nz], [(1 + eps) * nx, (1 + eps) * ny, eps * nz], "yz")
    force_box = ([0.4999 * nx, 0.4999 * ny, 0.9999 * nz], [0.5001 * nx, 0.5001 * ny, 1.0001 * nz])
    return [dir_all, dir_yz], force_box


def setup_mbb(sim, ne, volfrac=0.3):
    sim_set_material(sim)
    dirs, (fmn, fmx) = mbb_regions(ne)
    for u, mn, mx, mask in dirs:
        sim.addDirichletCondition(u, mn, mx, mask)
    nx, ny, nz = ne
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    pos = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1).astype(float)
    inside = np.all((pos >= np.array(fmn)) & (pos <= np.array(fmx)), axis=1)
    f = np.zeros((nn, 3), order="F")
    f[inside, 1] = -1.0 / inside.sum()
    sim.setNodalForces(f)
    rho = np.full(nx * ny * nz, volfrac)
    sim.setDensities(rho)
    return rho, f


def setup_layer_by_layer(sim, ne, rho_lo=0.1, seed=0):
    sim_set_material(sim)
    nx, ny, nz = ne
    sim.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [float(nx), 0.0, float(nz)], "xyz")
    if hasattr(sim, "gravity"):
        sim.gravity = [0.0, -1.0, 0.0]
    else:
        sim.setGravity([0.0, -1.0, 0.0])
    rho = densities(ne, rho_lo, seed)
    sim.setDensities(rho)
    return rho
