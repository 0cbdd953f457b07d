"""The first PCG iteration split around the side-stream hierarchy rebuild gives the same solve.

When the densities (or the fabrication mask) change, the mixed solve rebuilds the Galerkin
hierarchy on a side stream and runs its first iteration as three graphs joined to the rebuild's
events (level 0's down leg, the lower down legs after the level operators, the rest after the
coarsest inverse); VFEM_PEEL_FIRST=0 waits for the whole rebuild and runs every iteration in the
device-resident loop. Both must give bit-identical iterates and iteration counts, including the
edge cases of the loop condition: an already converged start (no iteration), an iteration limit
of one, and a band-partial rebuild after a mask change.
"""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

NE = (64, 32, 32)


def _solver(monkeypatch, peel, levels=4):
    monkeypatch.setenv("VFEM_PEEL_FIRST", "1" if peel else "0")
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in NE]], NE)
    wl.setup_cantilever(sim, NE, 0.01, 0)
    mg = sim.multigridSolver(levels)
    mg.setPrecision("mixed")
    return sim, mg


def _solve(sim, mg, x0, maxIter=500, tol=1e-8, sweeps=2):
    f = sim.buildLoadVector()
    x = mg.preconditionedConjugateGradient(x0, f, maxIter, tol, None, 1, sweeps, False)
    return x, mg.lastStats.iterations


@pytest.mark.parametrize("levels", [3, 4])
def test_peeled_first_iteration_is_bit_identical(gpu, monkeypatch, levels):
    runs = []
    for peel in (True, False):
        sim, mg = _solver(monkeypatch, peel, levels)
        out = []
        for seed in (1, 2):
            sim.setDensities(wl.densities(NE, 0.01, seed))
            x, it = _solve(sim, mg, np.zeros((sim.numNodes(), 3)))
            out.append((x, it))
            # a converged start (the same densities set again: the hierarchy is rebuilt): no
            # iteration, x returned as given
            sim.setDensities(wl.densities(NE, 0.01, seed))
            x2, it2 = _solve(sim, mg, x)
            out.append((x2, it2))
            # the density change forces a rebuild; one iteration only
            sim.setDensities(wl.densities(NE, 0.01, seed + 10))
            x3, it3 = _solve(sim, mg, np.zeros((sim.numNodes(), 3)), maxIter=1)
            out.append((x3, it3))
        # mask changes: band-partial rebuilds
        for h in (20, 13):
            mg.setFabricationMaskHeightByLayer(h)
            out.append(_solve(sim, mg, np.zeros((sim.numNodes(), 3))))
        runs.append(out)
    for (xa, ia), (xb, ib) in zip(*runs):
        assert ia == ib
        np.testing.assert_array_equal(xa, xb)
    its = [it for _, it in runs[0]]
    assert its[1] == 0 and its[2] == 1 and its[0] > 5
