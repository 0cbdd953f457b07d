"""The reference's own boundary-condition and material files, on the host.

tests/golden/reference_bcs.json holds every examples/bcs/3D/*.bc and examples/bcs/*.bc file of the
reference (their JSON text) with the Dirichlet bits, values and nodal forces that the oracle's
restatement of TensorProductSimulator.hh:600-658 gives on a few grids, plus B9Creator.material.
Checked here: the oracle reproduces the fixture, hand-derived facts about the files hold, and the
Python mirror's reader (voxelfem_gb300.pyVoxelFEM.apply_bc_file) sends the regions that yield the
same bits and forces (its Dirichlet boxes are evaluated by a stand-in with the library's closed-box
rule; the GPU test of the same fixture runs the library itself).
"""
import json
import os

import numpy as np
import pytest

from oracle import bc_oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_bcs.json")


@pytest.fixture(scope="module")
def gold():
    with open(GOLD) as f:
        return json.load(f)


def _text(gold, case):
    return gold["bc3d" if case["dim"] == 3 else "bc2d"][case["file"]]


def _dense(case):
    nn = int(np.prod([n + 1 for n in case["ne"]]))
    dim = case["dim"]
    bits = np.zeros(nn, dtype=np.uint8)
    forces = np.zeros((nn, dim))
    dval = np.zeros((nn, dim))
    for n, b, v in zip(case["dirichlet_nodes"], case["dirichlet_bits"], case["dirichlet_values"]):
        bits[n] = b
        dval[n] = v
    for n, f in zip(case["force_nodes"], case["forces"]):
        forces[n] = f
    return bits, dval, forces


def test_fixture_covers_every_reference_file(gold):
    assert len(gold["bc3d"]) == 11 and len(gold["bc2d"]) == 13
    assert {c["file"] for c in gold["cases"] if c["dim"] == 3} == set(gold["bc3d"])
    assert {c["file"] for c in gold["cases"] if c["dim"] == 2} == set(gold["bc2d"])
    assert gold["material"]["young"] == 1.0 and gold["material"]["poisson"] == 0.3


def test_oracle_reproduces_fixture(gold):
    for case in gold["cases"]:
        text = _text(gold, case)
        if "error" in case:
            with pytest.raises(RuntimeError, match=case["error"]):
                bc_oracle.apply_bc_text(text, case["ne"], case["bbox"])
            continue
        bits, dval, forces = bc_oracle.apply_bc_text(text, case["ne"], case["bbox"])
        gb, gv, gf = _dense(case)
        np.testing.assert_array_equal(bits, gb)
        np.testing.assert_array_equal(dval, gv)
        np.testing.assert_array_equal(forces, gf)


def test_vectorised_form_equals_loop_form(gold):
    for case in gold["cases"]:
        text = _text(gold, case)
        if "error" in case:
            with pytest.raises(RuntimeError, match=case["error"]):
                bc_oracle.apply_bc_text_vectorized(text, case["ne"], case["bbox"])
            continue
        a = bc_oracle.apply_bc_text(text, case["ne"], case["bbox"])
        b = bc_oracle.apply_bc_text_vectorized(text, case["ne"], case["bbox"])
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_known_answers(gold):
    cases = {(c["file"], c["dim"], tuple(c["ne"])): c for c in gold["cases"]}
    # mbb_N (3D) on 20x10x12 over [-1,3]x[0.5,1.5]x[2,4]: fixed x = min, z = min line (all
    # components) and the x = max, z = min line in y and z; the load sits on the single node at
    # the centre of the top face
    c = cases[("mbb_N.bc", 3, (20, 10, 12))]
    bits, _, forces = _dense(c)
    idx = np.arange(bits.size).reshape(21, 11, 13)
    np.testing.assert_array_equal(bits[idx[0, :, 0]], 7)
    np.testing.assert_array_equal(bits[idx[20, :, 0]], 6)
    assert np.count_nonzero(bits) == 22
    assert c["force_nodes"] == [int(idx[10, 5, 12])] and c["forces"] == [[0.0, -1.0, 0.0]]
    # forces spread equally: every region's nodes carry value / count and sum to the value
    c = cases[("cantilever_uniform.bc", 3, (20, 10, 12))]
    f = np.asarray(c["forces"])
    assert len(c["force_nodes"]) == 9 and np.allclose(f.sum(axis=0), [0, -1, 0], atol=1e-15)
    np.testing.assert_array_equal(f[:, 1], -1.0 / 9.0)
    # the 2D files' third coordinate is ignored: mbb_N (2D) on 20x10 fixes (0, 0) fully and
    # (20, 0) in y; the load is on the top-centre node
    c = cases[("mbb_N.bc", 2, (20, 10))]
    assert c["dirichlet_nodes"] == [0, 20 * 11] and c["dirichlet_bits"] == [3, 2]
    assert c["force_nodes"] == [10 * 11 + 10]
    # regions between grid lines match no node: the reference raises
    assert cases[("hump.bc", 3, (10, 10, 8))]["error"] == "Force constraint region unmatched"


class _ClosedBoxSim:
    """Stand-in simulator: evaluates Dirichlet boxes on the node positions with the library's
    closed-box rule (Grid::addDirichlet) and records the dense forces."""

    def __init__(self, ne, bbox):
        self._nc = len(ne)
        lo, hi = np.asarray(bbox[0], float), np.asarray(bbox[1], float)
        self.domain = (lo, hi)
        self.NbNodesPerDimension = [n + 1 for n in ne]
        self.dx = (hi - lo) / np.asarray(ne, float)
        self.pos = bc_oracle.node_positions(ne, bbox)
        self.bits = np.zeros(self.pos.shape[0], dtype=np.uint8)
        self.forces = np.zeros((self.pos.shape[0], self._nc))

    def numNodes(self):
        return self.pos.shape[0]

    def addDirichletCondition(self, val, mn, mx, comps):
        inside = np.all((self.pos >= np.asarray(mn)) & (self.pos <= np.asarray(mx)), axis=1)
        for ch in comps:
            c = "xyz".index(ch)
            if c < self._nc:  # a 2D grid has no z component
                self.bits[inside] |= np.uint8(1 << c)

    def setNodalForces(self, f):
        self.forces = np.array(f)


def test_mirror_reader_matches_fixture(gold, tmp_path):
    from voxelfem_gb300.pyVoxelFEM import apply_bc_file

    for case in gold["cases"]:
        path = tmp_path / case["file"]
        path.write_text(_text(gold, case))
        sim = _ClosedBoxSim(case["ne"], case["bbox"])
        if "error" in case:
            with pytest.raises(RuntimeError, match=case["error"]):
                apply_bc_file(sim, str(path))
            continue
        apply_bc_file(sim, str(path))
        gb, _, gf = _dense(case)
        np.testing.assert_array_equal(sim.bits, gb)
        np.testing.assert_array_equal(sim.forces, gf)
