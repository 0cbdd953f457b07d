"""The reference's own boundary-condition and material files through the library.

Every examples/bcs/3D/*.bc and examples/bcs/*.bc file of the reference (stored with its expected
masks and forces in tests/golden/reference_bcs.json, made by tests/golden/make_bc_golden.py from the
oracle's restatement of TensorProductSimulator.hh:600-658) is applied with
applyDisplacementsAndLoadsFromFile to a GPU simulator: the Dirichlet component masks and the nodal
load vector must equal the fixture bit for bit, and regions that match no node must raise the
reference's error. B9Creator.material read with readMaterial must give the oracle's K0.
"""
import json
import os

import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_bcs.json")


@pytest.fixture(scope="module")
def gold():
    with open(GOLD) as f:
        return json.load(f)


def test_reference_bc_files_bit_exact(gpu, gold, tmp_path):
    for case in gold["cases"]:
        dim = case["dim"]
        text = gold["bc3d" if dim == 3 else "bc2d"][case["file"]]
        path = tmp_path / ("%dd_%s" % (dim, case["file"]))
        path.write_text(text)
        sim = pv.TensorProductSimulator([1] * dim, case["bbox"], case["ne"])
        sim.gravity = [0.0] * dim
        if "error" in case:
            with pytest.raises(RuntimeError, match=case["error"]):
                sim.applyDisplacementsAndLoadsFromFile(str(path))
            continue
        sim.applyDisplacementsAndLoadsFromFile(str(path))
        nn = sim.numNodes()
        bits = np.zeros(nn, dtype=np.uint8)
        for n, b in zip(case["dirichlet_nodes"], case["dirichlet_bits"]):
            bits[n] = b
        forces = np.zeros((nn, dim))
        for n, f in zip(case["force_nodes"], case["forces"]):
            forces[n] = f
        m = sim.getDirichletMask()
        got = np.zeros(nn, dtype=np.uint8)
        for c in range(dim):
            got |= (m[:, c].astype(np.uint8) << c)
        np.testing.assert_array_equal(got, bits, err_msg=case["file"])
        np.testing.assert_array_equal(sim.buildLoadVector(), forces, err_msg=case["file"])


def test_reference_material_file(gpu, gold, oracle, tmp_path):
    mat = gold["material"]
    path = tmp_path / mat["file"]
    path.write_text(mat["text"])
    ne = (4, 3, 2)
    g = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [4.0, 3.0, 2.0]], ne)
    g.readMaterial(str(path))
    o = oracle.Sim(ne)
    o.setMaterial(mat["young"], mat["poisson"])
    k0 = np.asarray(g.fullDensityElementStiffnessMatrix())
    assert float(np.max(np.abs(k0 - o.K0())) / np.max(np.abs(o.K0()))) < 1e-14
