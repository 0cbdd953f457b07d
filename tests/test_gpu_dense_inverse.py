"""The coarsest dense inverse in one cooperative launch (phases separated by a bounded grid
barrier; VFEM_DENSE_PERSISTENT=1) against the default form with one launch per phase: the same tile operations in the same order,
so bit-identical inverses, for coarsest systems of one to dozens of tiles; and both against the
oracle's Cholesky solve (1e-10)."""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ne,levels", [((8, 4, 4), 2), ((32, 16, 16), 3), ((64, 32, 32), 3), ((64, 32, 32), 4)])
def test_persistent_dense_inverse_is_bit_identical(gpu, oracle, monkeypatch, ne, levels):
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    wl.setup_cantilever(sim, ne, 0.3, 0)
    mg = sim.multigridSolver(levels)
    o = oracle.Sim(ne, [[0.0, 0.0, 0.0], [float(v) for v in ne]])
    wl.setup_cantilever(o, ne, 0.3, 0)
    om = oracle.MG(o, levels)
    nc = int(np.prod([v // 2 ** levels + 1 for v in ne]))  # levels = coarsenings
    b = np.random.default_rng(1).standard_normal((nc, 3))
    out = []
    for persistent in ("1", "0", "1"):
        monkeypatch.setenv("VFEM_DENSE_PERSISTENT", persistent)
        sim.setDensities(wl.densities(ne, 0.3, 0))  # the next use rebuilds the hierarchy
        out.append(mg.coarseSolve(b))
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])
    ref = om.coarseSolve(b)
    assert np.max(np.abs(out[0] - ref)) < 1e-10 * np.max(np.abs(ref))
