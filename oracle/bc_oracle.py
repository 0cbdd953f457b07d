"""CPU restatement of the reference's boundary-condition and material file readers.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by the fixture script under tests/golden/,
never by the product path.

What it restates:

* ``TensorProductSimulator::applyDisplacementsAndLoads`` (TensorProductSimulator.hh:600-652)
  with its ``BCBuilder`` (:464-593): each region is tested against every node position
  (``nodePosition``, :349-353: minCorner + index * dx). A ``force`` region spreads its value
  equally over the nodes it contains (value / count, :629-630) and overwrites earlier forces on
  those nodes (``setForce``, :514); a ``dirichlet`` region merges its component mask into the
  node's (``setDirichlet``, :492-507): a newly constrained component takes the region's value, an
  already constrained one must agree to 1e-10 ("Conflicting dirichlet displacements."). A region
  that contains no node raises "Force constraint region unmatched" / "Dirichlet region
  unmatched" (:622, :645).
* ``applyDisplacementsAndLoadsFromFile`` (:654-658) reads the file with MeshFEM's
  ``readBoundaryConditions``. MeshFEM is not vendored with the reference (its submodule
  directory is empty), so its file format is restated from the reference's own example files
  and call sites: a JSON object whose ``regions`` list holds ``{"type", "value", "box%" |
  "box"}``; ``box%`` corners are fractions of the mesh bounding box (minCorner + fraction *
  size), ``box`` corners absolute; the type is ``force`` or ``dirichlet`` followed by the
  constrained component letters (none: all components). Vectors may carry more entries than
  the dimension (the reference's 2D files write a zero third coordinate); the first ``dim`` are
  used.
* ``readMaterial`` (TensorProductSimulator.hh:333-338 via ``Materials::Constant``): an
  ``isotropic_material`` JSON with ``young`` and ``poisson``.

Containment is the closed box (min <= p <= max in every coordinate), evaluated in double
precision on the node positions, node by node in index order.
"""
import json

import numpy as np


def node_positions(ne, bbox):
    """Node coordinates in the reference's flat order (index (i * ny1 + j) * nz1 + k)."""
    ne = [int(v) for v in ne]
    lo = np.asarray(bbox[0], dtype=float)
    hi = np.asarray(bbox[1], dtype=float)
    dx = (hi - lo) / np.asarray(ne, dtype=float)
    dim = len(ne)
    pos = []
    if dim == 3:
        for i in range(ne[0] + 1):
            for j in range(ne[1] + 1):
                for k in range(ne[2] + 1):
                    pos.append((lo[0] + i * dx[0], lo[1] + j * dx[1], lo[2] + k * dx[2]))
    else:
        for i in range(ne[0] + 1):
            for j in range(ne[1] + 1):
                pos.append((lo[0] + i * dx[0], lo[1] + j * dx[1]))
    return np.asarray(pos, dtype=float)


def _components(typ, dim):
    suffix = typ[len("dirichlet"):]
    letters = "xyz"[:dim]
    if suffix == "":
        return [True] * dim
    mask = [False] * dim
    for ch in suffix:
        if ch not in letters:
            raise RuntimeError("invalid component mask '%s'" % suffix)
        mask[letters.index(ch)] = True
    return mask


def read_regions(text, ne, bbox):
    """The regions of a .bc file as (type, value, minCorner, maxCorner) in absolute coordinates."""
    spec = json.loads(text)
    dim = len(ne)
    lo = np.asarray(bbox[0], dtype=float)
    hi = np.asarray(bbox[1], dtype=float)
    size = hi - lo
    out = []
    for reg in spec["regions"]:
        val = [float(v) for v in reg["value"]][:dim]
        if "box%" in reg:
            b = reg["box%"]
            mn = [lo[d] + float(b["minCorner"][d]) * size[d] for d in range(dim)]
            mx = [lo[d] + float(b["maxCorner"][d]) * size[d] for d in range(dim)]
        elif "box" in reg:
            b = reg["box"]
            mn = [float(b["minCorner"][d]) for d in range(dim)]
            mx = [float(b["maxCorner"][d]) for d in range(dim)]
        else:
            raise RuntimeError("unsupported region shape")
        out.append((reg["type"], val, mn, mx))
    return out


def apply_bc_text(text, ne, bbox):
    """Dirichlet component bits (bit c: component c fixed), Dirichlet values and nodal forces
    of a .bc file on the grid ``ne`` over ``bbox``."""
    dim = len(ne)
    pos = node_positions(ne, bbox)
    nn = pos.shape[0]
    comp = np.zeros((nn, dim), dtype=bool)
    dval = np.zeros((nn, dim))
    forces = np.zeros((nn, dim))
    for typ, val, mn, mx in read_regions(text, ne, bbox):
        inside = []
        for n in range(nn):
            p = pos[n]
            if all(mn[d] <= p[d] <= mx[d] for d in range(dim)):
                inside.append(n)
        if typ == "force":
            if not inside:
                raise RuntimeError("Force constraint region unmatched")
            for n in inside:
                for d in range(dim):
                    forces[n, d] = val[d] / len(inside)
        elif typ.startswith("dirichlet"):
            cm = _components(typ, dim)
            if not inside:
                raise RuntimeError("Dirichlet region unmatched")
            for n in inside:
                for d in range(dim):
                    if not cm[d]:
                        continue
                    if not comp[n, d]:
                        comp[n, d] = True
                        dval[n, d] = val[d]
                    elif abs(dval[n, d] - val[d]) > 1e-10:
                        raise RuntimeError("Conflicting dirichlet displacements.")
        else:
            raise RuntimeError('Illegal constraint type, only "dirichlet" and "force" accepted')
    bits = np.zeros(nn, dtype=np.uint8)
    for d in range(dim):
        bits |= (comp[:, d].astype(np.uint8) << d)
    return bits, dval, forces


def read_material_text(text):
    """(young, poisson) of an isotropic material file."""
    mat = json.loads(text)
    if mat.get("type", "isotropic_material") not in ("isotropic_material", "isotropic"):
        raise RuntimeError("Only isotropic materials are supported")
    return float(mat["young"]), float(mat["poisson"])


def apply_bc_text_vectorized(text, ne, bbox):
    """apply_bc_text for large grids: the same rules with the node loop vectorised (numpy);
    equal to the loop form bit for bit (the same comparisons on the same doubles)."""
    dim = len(ne)
    axes = []
    lo = np.asarray(bbox[0], dtype=float)
    hi = np.asarray(bbox[1], dtype=float)
    dx = (hi - lo) / np.asarray(ne, dtype=float)
    for d in range(dim):
        axes.append(lo[d] + np.arange(int(ne[d]) + 1) * dx[d])
    shape = tuple(int(n) + 1 for n in ne)
    nn = int(np.prod(shape))
    comp = np.zeros((nn, dim), dtype=bool)
    dval = np.zeros((nn, dim))
    forces = np.zeros((nn, dim))
    for typ, val, mn, mx in read_regions(text, ne, bbox):
        sel = [(axes[d] >= mn[d]) & (axes[d] <= mx[d]) for d in range(dim)]
        inside = np.ones(shape, dtype=bool)
        for d in range(dim):
            bshape = [1] * dim
            bshape[d] = shape[d]
            inside = inside & sel[d].reshape(bshape)
        idx = np.flatnonzero(inside.ravel())
        if typ == "force":
            if idx.size == 0:
                raise RuntimeError("Force constraint region unmatched")
            for d in range(dim):
                forces[idx, d] = val[d] / idx.size
        elif typ.startswith("dirichlet"):
            cm = _components(typ, dim)
            if idx.size == 0:
                raise RuntimeError("Dirichlet region unmatched")
            for d in range(dim):
                if not cm[d]:
                    continue
                new = idx[~comp[idx, d]]
                old = idx[comp[idx, d]]
                if old.size and np.any(np.abs(dval[old, d] - val[d]) > 1e-10):
                    raise RuntimeError("Conflicting dirichlet displacements.")
                comp[new, d] = True
                dval[new, d] = val[d]
        else:
            raise RuntimeError('Illegal constraint type, only "dirichlet" and "force" accepted')
    bits = np.zeros(nn, dtype=np.uint8)
    for d in range(dim):
        bits |= (comp[:, d].astype(np.uint8) << d)
    return bits, dval, forces
