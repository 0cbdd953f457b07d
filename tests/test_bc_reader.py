"""The `.bc` reader of the Python mirror (regions "box%" / "box", "dirichlet[comps]" and "force"
with the force split equally over the region's nodes, TensorProductSimulator.hh:600-652),
exercised on the host against a recording stand-in for the simulator."""
import json

import numpy as np
import pytest


class FakeSim:
    def __init__(self, ne, lo, hi):
        self._nc = len(ne)
        self.domain = (np.asarray(lo, float), np.asarray(hi, float))
        self.NbNodesPerDimension = [n + 1 for n in ne]
        self.dx = (self.domain[1] - self.domain[0]) / np.asarray(ne, float)
        self.dirichlet = []
        self.forces = None

    def numNodes(self):
        return int(np.prod(self.NbNodesPerDimension))

    def addDirichletCondition(self, val, mn, mx, comps):
        self.dirichlet.append((np.asarray(val), np.asarray(mn), np.asarray(mx), comps))

    def setNodalForces(self, f):
        self.forces = np.array(f)


@pytest.fixture(scope="module")
def reader():
    from voxelfem_gb300.pyVoxelFEM import apply_bc_file
    return apply_bc_file


def _write(tmp_path, regions):
    p = tmp_path / "case.bc"
    p.write_text(json.dumps({"regions": regions}))
    return str(p)


def test_cantilever_regions_3d(tmp_path, reader):
    sim = FakeSim([4, 2, 2], [0, 0, 0], [4, 2, 2])
    path = _write(tmp_path, [
        {"type": "dirichlet", "value": [0, 0, 0], "box%": {"minCorner": [0, 0, 0], "maxCorner": [0, 1, 1]}},
        {"type": "force", "value": [0, -1, 0], "box%": {"minCorner": [1, 0, 0.5], "maxCorner": [1, 1, 0.5]}},
    ])
    reader(sim, path)
    (val, mn, mx, comps), = sim.dirichlet
    assert comps == "xyz" and np.all(val == 0)
    assert np.allclose(mn, [0, 0, 0]) and np.allclose(mx, [0, 2, 2])
    # the x = 4, z = 1 line holds 3 nodes (y = 0, 1, 2), each with a third of the load
    f = sim.forces.reshape(5, 3, 3, 3)
    assert np.allclose(f[4, :, 1, 1], -1.0 / 3.0)
    assert np.isclose(f[..., 1].sum(), -1.0) and np.all(f[..., 0] == 0) and np.all(f[..., 2] == 0)
    assert np.count_nonzero(f) == 3


def test_absolute_box_and_component_mask(tmp_path, reader):
    sim = FakeSim([2, 2, 2], [0, 0, 0], [1, 1, 1])
    path = _write(tmp_path, [
        {"type": "dirichletyz", "value": [0, 0.5, 0], "box": {"minCorner": [0, 0, 0], "maxCorner": [0, 1, 1]}},
    ])
    reader(sim, path)
    (val, mn, mx, comps), = sim.dirichlet
    assert comps == "yz" and np.allclose(val, [0, 0.5, 0]) and np.allclose(mx, [0, 1, 1])
    assert sim.forces is None


def test_2d_reads_first_two_entries(tmp_path, reader):
    sim = FakeSim([4, 2], [0, 0], [2, 1])
    path = _write(tmp_path, [
        {"type": "dirichlet", "value": [0, 0, 0], "box%": {"minCorner": [0, 0, 0], "maxCorner": [0, 1, 0]}},
        {"type": "force", "value": [0, -2, 0], "box%": {"minCorner": [1, 0, 0], "maxCorner": [1, 0, 0]}},
    ])
    reader(sim, path)
    (val, mn, mx, comps), = sim.dirichlet
    assert val.shape == (2,) and mx.shape == (2,) and np.allclose(mx, [0, 1])
    f = sim.forces.reshape(5, 3, 2)
    assert np.allclose(f[4, 0], [0, -2]) and np.count_nonzero(f) == 1


@pytest.mark.parametrize("region, msg", [
    ({"type": "force", "value": [0, 1, 0], "box": {"minCorner": [9, 9, 9], "maxCorner": [9, 9, 9]}},
     "Force constraint region unmatched"),
    ({"type": "dirichlet", "value": [0, 0, 0], "box": {"minCorner": [9, 9, 9], "maxCorner": [9, 9, 9]}},
     "Dirichlet region unmatched"),
    ({"type": "pressure", "value": [0, 1, 0], "box": {"minCorner": [0, 0, 0], "maxCorner": [1, 1, 1]}},
     'Illegal constraint type, only "dirichlet" and "force" accepted'),
    ({"type": "force", "value": [0, 1, 0], "sphere": {}}, "Unsupported boundary condition region"),
])
def test_errors(tmp_path, reader, region, msg):
    sim = FakeSim([2, 2, 2], [0, 0, 0], [1, 1, 1])
    with pytest.raises(RuntimeError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        reader(sim, _write(tmp_path, [region]))
