"""Band-partial hierarchy updates after fabrication-mask changes against full rebuilds.

When only the fabrication mask moves (the layer-by-layer evaluator's height sequence), the
reference updates just the band of coarse operators that the changed element layers reach
(m_partialStiffnessMatrixUpdate, MultigridSolver.hh:907-1017) and refactors its coarsest system.
The library does the same: the level-1 stencil, the level-2+ element matrices and stencils are
rebuilt only for the rows between the old and the new masked layer, the coarsest dense inverse
in full. A solver that updates by bands must give bit-identical solves to one that rebuilds
everything, for heights that go down, up, jump and return, in FP64 and mixed precision.
"""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

NE = (32, 32, 16)
HEIGHTS = [32, 31, 27, 20, 21, 9, 1, 2, 16, 32]


def _solver(monkeypatch, band, levels, prec):
    monkeypatch.setenv("VFEM_BAND_UPDATE", "1" if band else "0")
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in NE]], NE)
    wl.setup_layer_by_layer(sim, NE, 0.1, 0)
    mg = sim.multigridSolver(levels)
    mg.setPrecision(prec)
    return sim, mg


@pytest.mark.parametrize("levels,prec", [(2, "fp64"), (3, "mixed"), (4, "mixed")])
def test_band_updates_equal_full_rebuilds(gpu, monkeypatch, levels, prec):
    sb, mb = _solver(monkeypatch, True, levels, prec)
    sf, mf = _solver(monkeypatch, False, levels, prec)
    for h in HEIGHTS:
        xs = []
        for sim, mg in ((sb, mb), (sf, mf)):
            mg.setFabricationMaskHeightByLayer(h)
            f = sim.buildLoadVector()
            xs.append((mg.preconditionedConjugateGradient(np.zeros_like(f), f, 300, 1e-10, None, 1, 2, False),
                       mg.lastStats.iterations))
        assert xs[0][1] == xs[1][1], h
        np.testing.assert_array_equal(xs[0][0], xs[1][0], err_msg="height %d" % h)
    full_b, band_b = mb.stiffnessRebuilds()
    full_f, band_f = mf.stiffnessRebuilds()
    assert full_b == 1 and band_b == len(HEIGHTS) - 1, (full_b, band_b)
    assert band_f == 0 and full_f == len(HEIGHTS)
