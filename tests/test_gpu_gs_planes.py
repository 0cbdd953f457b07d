"""The fused forms of the FP32 fine sweep against the eight colour launches of the reference's
order (MultigridSolver.hh:409-458):
- line pairs: four launches per sweep, each running two colours adjacent in the order, (x, y)
  parity fixed and z parity 0 then 1, on whole z-lines per CTA with a block barrier between;
- plane pairs: two launches per sweep, all x-even planes then all x-odd planes, one thread-block
  cluster per plane running its four (y, z) colours between cluster barriers;
- staged line pairs: the line-pair schedule with each CTA's neighbourhood tile (u of three
  planes, the lines' rows and their neighbours, and the moduli) copied to shared memory first.

All forms run the same node updates on the same operands in the same order, so mixed-precision
solves whose V-cycles use one or another give bit-identical iterates: pre- and post-smoothing
(forward and colour-reversed), odd and even plane and line counts, detached rows (layer-by-layer
masks), partially constrained nodes and non-cube voxels.
"""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _solve(monkeypatch, mode, ne, levels, bbox=None, mask_layer=None, partial=False, symmetric=True):
    monkeypatch.setenv("VFEM_GS_MODE", mode)
    if bbox is None:
        bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    g = pv.TensorProductSimulator([1, 1, 1], bbox, ne)
    wl.setup_cantilever(g, ne, 0.3, 0)
    if partial:
        # roller supports on the y = 0 face: y fixed only
        g.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [bbox[1][0], 0.0, bbox[1][2]], "y")
    if mask_layer is not None:
        g.setFabricationMaskHeightByLayer(mask_layer)
    mg = g.multigridSolver(levels)
    mg.setSymmetricGaussSeidel(symmetric)
    if mask_layer is not None:
        mg.setFabricationMaskHeightByLayer(mask_layer)
    mg.setPrecision("mixed")
    b = g.buildLoadVector()
    x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-9, None, 1, 2, False)
    return x, mg.lastStats.iterations


@pytest.mark.parametrize("ne,levels,kw", [
    ((16, 8, 8), 2, {}),
    ((36, 28, 20), 2, {}),
    ((64, 32, 32), 3, {}),
    ((24, 20, 12), 2, {"partial": True}),
    ((16, 16, 8), 2, {"mask_layer": 9}),
    ((20, 12, 12), 2, {"bbox": [[0.0, 0.0, 0.0], [20.0, 6.0, 18.0]]}),
    ((16, 8, 8), 2, {"symmetric": False}),
    ((128, 48, 40), 3, {}),
])
def test_fused_sweeps_equal_colour_sweeps(gpu, monkeypatch, ne, levels, kw):
    xa, ia = _solve(monkeypatch, "colours", ne, levels, **kw)
    for mode in ("lines", "planes", "staged"):
        xb, ib = _solve(monkeypatch, mode, ne, levels, **kw)
        assert ia == ib, mode
        np.testing.assert_array_equal(xa, xb, err_msg=mode)


@pytest.mark.parametrize("prec,kw", [("mixed", {}), ("fp64", {}), ("mixed", {"mask_layer": 11}),
                                     ("mixed", {"partial": True})])
def test_stencil_line_pairs_equal_colour_passes(gpu, monkeypatch, prec, kw):
    """Coarse plane-layout levels: colour pairs on whole z-lines (four launches per sweep)
    against eight colour launches, bit for bit (FP64 and mixed V-cycles)."""
    ne = (32, 24, 16)

    def solve(lines):
        monkeypatch.setenv("VFEM_STENCIL_LINES_MAX_NODES", "100000000" if lines else "0")
        g = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
        wl.setup_cantilever(g, ne, 0.3, 0)
        if kw.get("partial"):
            g.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [float(ne[0]), 0.0, float(ne[2])], "y")
        mg = g.multigridSolver(3)
        if "mask_layer" in kw:
            mg.setFabricationMaskHeightByLayer(kw["mask_layer"])
        mg.setPrecision(prec)
        b = g.buildLoadVector()
        x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-9, None, 1, 2, False)
        return x, mg.lastStats.iterations

    xa, ia = solve(False)
    xb, ib = solve(True)
    assert ia == ib
    np.testing.assert_array_equal(xa, xb)
