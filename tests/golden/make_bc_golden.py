"""Generate tests/golden/reference_bcs.json from the reference's own example data.

The reference ships boundary-condition region files (examples/bcs/3D/*.bc for 3D grids,
examples/bcs/*.bc for 2D grids) and a material file (examples/materials/B9Creator.material);
its drivers read them with applyDisplacementsAndLoadsFromFile and readMaterial
(python/LayerByLayerOptimization.py:177-185, python/CoarseningLevelBenchmark.py:77-85). They
are the only reference-held data on the solve path, so they pin the boundary-condition
semantics. The reference itself cannot be built here (its MeshFEM submodule is empty), so the
expected masks, Dirichlet values and nodal forces come from the oracle's restatement
(oracle/bc_oracle.py), on a few grids each. The fixture stores every input file's JSON text as
well: the reference tree is not available where the GPU tests run.

Run from the repository root, where the reference checkout exists:
    python tests/golden/make_bc_golden.py [reference_root]
"""
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import bc_oracle  # noqa: E402

GRIDS_3D = [((10, 10, 8), [[0.0, 0.0, 0.0], [10.0, 10.0, 8.0]]),
            ((20, 10, 12), [[-1.0, 0.5, 2.0], [3.0, 1.5, 4.0]])]
GRIDS_2D = [((20, 10), [[0.0, 0.0], [2.0, 1.0]]),
            ((32, 16), [[0.0, 0.0], [32.0, 16.0]])]


def _case(name, text, ne, bbox):
    try:
        bits, dval, forces = bc_oracle.apply_bc_text(text, ne, bbox)
    except RuntimeError as e:
        return {"file": name, "ne": list(ne), "bbox": bbox, "error": str(e)}
    nz = [int(n) for n in range(bits.size) if bits[n]]
    fz = [int(n) for n in range(forces.shape[0]) if (forces[n] != 0).any()]
    return {"file": name, "ne": list(ne), "bbox": bbox,
            "dirichlet_nodes": nz, "dirichlet_bits": [int(bits[n]) for n in nz],
            "dirichlet_values": [[float(v) for v in dval[n]] for n in nz],
            "force_nodes": fz, "forces": [[float(v) for v in forces[n]] for n in fz]}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    files3 = sorted(glob.glob(os.path.join(ref, "examples", "bcs", "3D", "*.bc")))
    files2 = sorted(glob.glob(os.path.join(ref, "examples", "bcs", "*.bc")))
    out = {"bc3d": {}, "bc2d": {}, "cases": []}
    for path in files3:
        name = os.path.basename(path)
        with open(path) as f:
            text = json.dumps(json.loads(f.read()), separators=(",", ":"))
        out["bc3d"][name] = text
        for ne, bbox in GRIDS_3D:
            out["cases"].append(dict(_case(name, text, ne, bbox), dim=3))
    for path in files2:
        name = os.path.basename(path)
        with open(path) as f:
            text = json.dumps(json.loads(f.read()), separators=(",", ":"))
        out["bc2d"][name] = text
        for ne, bbox in GRIDS_2D:
            out["cases"].append(dict(_case(name, text, ne, bbox), dim=2))
    mpath = os.path.join(ref, "examples", "materials", "B9Creator.material")
    with open(mpath) as f:
        mtext = json.dumps(json.loads(f.read()), separators=(",", ":"))
    E, nu = bc_oracle.read_material_text(mtext)
    out["material"] = {"file": "B9Creator.material", "text": mtext, "young": E, "poisson": nu}
    with open(os.path.join(HERE, "reference_bcs.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("%d 3D files, %d 2D files, %d cases" % (len(files3), len(files2), len(out["cases"])))


if __name__ == "__main__":
    main()
