"""Layer-by-layer at full size against the oracle.

The 128^3 workload (rho U[0.1, 1] seed 0, base y = 0 fixed, self-weight gravity (0, -1, 0), every
build height 1..128, 5 coarsenings, zero guesses, tol 1e-8, 2 + 2 sweeps): the batched
mixed-precision evaluation of all 128 heights, and FP64 GPU solves at heights 1, 16, 64 and 128,
against the oracle's FP64 solves at those heights (tests/golden/lbl_128_oracle.json, made by
tests/golden/make_golden.py --lbl). Per height: f.u to 1e-8 and the oracle's iteration count.
"""
import json
import os

import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

NE = (128, 128, 128)
COARSENINGS = 5
TOL = 1e-8


def _golden():
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lbl_128_oracle.json")
    with open(path) as f:
        return {h["height"]: h for h in json.load(f)["heights"]}


def test_c4_layer_by_layer_full_size_against_oracle(gpu):
    gold = _golden()
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in NE]], NE)
    wl.setup_layer_by_layer(sim, NE, 0.1, 0)
    mg = sim.multigridSolver(COARSENINGS)
    # FP64 (the reference's method) at the sampled heights
    for h, ref in gold.items():
        mg.setFabricationMaskHeightByLayer(h)
        f = sim.buildLoadVector()
        u = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 500, TOL, None, 1, 2, False)
        fu = float(np.sum(f * u))
        assert mg.lastStats.iterations == ref["iterations"], (h, mg.lastStats.iterations, ref["iterations"])
        assert abs(fu - ref["f_dot_u"]) / abs(ref["f_dot_u"]) < 1e-8, (h, fu, ref["f_dot_u"])
    mg.setFabricationMaskHeightByLayer(NE[1])
    # every height, mixed precision, batched over concurrent solver slots
    mg.setPrecision("mixed")
    ev = pv.LayerByLayerEvaluator(sim)
    ev.selectInitMethod("zero")
    ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=8)
    np.testing.assert_array_equal(ev.layers, np.arange(NE[1], 0, -1))
    by_h = dict(zip(ev.layers.tolist(), zip(ev.compliances.tolist(), ev.iterations.tolist())))
    for h, ref in gold.items():
        c, its = by_h[h]
        assert abs(c - ref["f_dot_u"]) / abs(ref["f_dot_u"]) < 1e-8, (h, c, ref["f_dot_u"])
        assert its == ref["iterations"], (h, its, ref["iterations"])
    assert np.all(np.isfinite(ev.compliances)) and np.all(ev.compliances > 0)
