"""numpy restatements of the reference's UpsampleFilter, VertexToCellFilter and LangelaarFilter
(TopologyOptimizationFilter.hh:402-709), the oracle of the GPU filters (test infrastructure
only). Grids are row-major 3D arrays (x slowest, z fastest); the *_2d functions and
Langelaar(shape, ndim=2) restate the N = 2 instantiations on (x, y) arrays."""
import numpy as np


def upsample(a, F):
    """UpsampleFilter::ApplyImpl (:445-470): every coarse cell's trilinear interpolant sampled at
    the fine nodes of the cell (cells visited in order; shared nodes get equal values)."""
    a = np.asarray(a, dtype=np.float64)
    out = np.zeros(tuple((s - 1) * F + 1 for s in a.shape))
    t = np.arange(F + 1) / F
    w = [1.0 - t, t]
    for i in range(a.shape[0] - 1):
        for j in range(a.shape[1] - 1):
            for k in range(a.shape[2] - 1):
                blk = np.zeros((F + 1, F + 1, F + 1))
                for c in range(8):
                    b0, b1, b2 = (c >> 2) & 1, (c >> 1) & 1, c & 1
                    blk += a[i + b0, j + b1, k + b2] * (w[b0][:, None, None] * w[b1][None, :, None] * w[b2][None, None, :])
                out[i * F:i * F + F + 1, j * F:j * F + F + 1, k * F:k * F + F + 1] = blk
    return out


def upsample_backprop(g, in_shape, F):
    """UpsampleFilter::BackpropImpl (:474-505)."""
    g = np.asarray(g, dtype=np.float64)
    out = np.zeros(in_shape)
    for c in np.ndindex(*in_shape):
        lo = [F * c[d] - (F - 1 if c[d] > 0 else 0) for d in range(3)]
        hi = [F * c[d] + 1 + (F - 1 if c[d] < in_shape[d] - 1 else 0) for d in range(3)]
        acc = 0.0
        for n in np.ndindex(*[hi[d] - lo[d] for d in range(3)]):
            f = [lo[d] + n[d] for d in range(3)]
            phi = np.prod([1.0 - abs(f[d] - F * c[d]) / F for d in range(3)])
            acc += phi * g[tuple(f)]
        out[c] = acc
    return out


def vertex_to_cell(v):
    v = np.asarray(v, dtype=np.float64)
    return 0.125 * sum(v[a:a + v.shape[0] - 1, b:b + v.shape[1] - 1, c:c + v.shape[2] - 1]
                       for a in (0, 1) for b in (0, 1) for c in (0, 1))


def vertex_to_cell_backprop(g):
    g = np.asarray(g, dtype=np.float64)
    out = np.zeros(tuple(s + 1 for s in g.shape))
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                out[a:a + g.shape[0], b:b + g.shape[1], c:c + g.shape[2]] += g
    return 0.125 * out


class Langelaar:
    """LangelaarFilter (:577-709) with NDVector::visitSupportingRegion (NDVector.hh:211-229) as
    written: below, x -/+ 1 below, two below, and the voxel itself (whose output value is the one
    left by the previous application; the output buffer starts at zero). For N = 2 the loop over
    d stops after d = 0: below and x -/+ 1 below only (shape (nx, ny), held as (nx, ny, 1))."""
    P, Q, EPS = 40.0, 40.0 - 1.58, 1e-4

    def __init__(self, shape, ndim=3):
        self.ndim = ndim
        self.shape = tuple(shape) + ((1,) if ndim == 2 else ())
        self.out = np.zeros(self.shape)

    def region(self, i, j, k):
        r = [(i, j - 1, k)]
        if i - 1 >= 0:
            r.append((i - 1, j - 1, k))
        if i + 1 < self.shape[0]:
            r.append((i + 1, j - 1, k))
        if self.ndim == 2:
            return r
        if j - 2 >= 0:
            r.append((i, j - 2, k))
        r.append((i, j, k))
        return r

    def smin(self, a, b):
        return 0.5 * (a + b - np.sqrt((a - b) ** 2 + self.EPS) + np.sqrt(self.EPS))

    def apply(self, x):
        x = np.asarray(x, dtype=np.float64).reshape(self.shape)
        out = self.out
        out[:, 0, :] = x[:, 0, :]
        self.smax = np.zeros(self.shape)
        for j in range(1, self.shape[1]):
            for i in range(self.shape[0]):
                for k in range(self.shape[2]):
                    s = sum(out[m] ** self.P for m in self.region(i, j, k))
                    self.smax[i, j, k] = s ** (1.0 / self.Q)
                    out[i, j, k] = self.smin(x[i, j, k], self.smax[i, j, k])
        self.filt = out.copy()
        return out.copy()

    def backprop(self, g, vars_):
        g = np.asarray(g, dtype=np.float64).reshape(self.shape)
        v = np.asarray(vars_, dtype=np.float64).reshape(self.shape)
        P, Q, E = self.P, self.Q, self.EPS
        lam = np.zeros(self.shape)
        ny = self.shape[1]
        for layer in range(ny - 1, -1, -1):
            lam[:, layer, :] = g[:, layer, :]
            if layer < ny - 1:
                for i in range(self.shape[0]):
                    for k in range(self.shape[2]):
                        e = (i, layer + 1, k)
                        S = sum(self.filt[m] ** P for m in self.region(*e))
                        d2 = 0.5 * (1 + (v[e] - self.smax[e]) / np.sqrt((v[e] - self.smax[e]) ** 2 + E))
                        for m in self.region(*e):
                            lam[m] += lam[e] * d2 * (P * self.filt[m] ** (P - 1) / Q * S ** (1.0 / Q - 1))
        out = lam.copy()
        d1 = 0.5 * (1 - (v - self.smax) / np.sqrt((v - self.smax) ** 2 + E))
        out[:, 1:, :] = lam[:, 1:, :] * d1[:, 1:, :]
        return out


def _flat3(a):
    a = np.asarray(a, dtype=np.float64)
    return a[:, :, None]


def upsample_2d(a, F):
    """UpsampleFilter::ApplyImpl<1, 1>: bilinear upsampling of an (x, y) node grid."""
    a = np.asarray(a, dtype=np.float64)
    out = np.zeros(tuple((s - 1) * F + 1 for s in a.shape))
    t = np.arange(F + 1) / F
    w = [1.0 - t, t]
    for i in range(a.shape[0] - 1):
        for j in range(a.shape[1] - 1):
            blk = np.zeros((F + 1, F + 1))
            for c in range(4):
                b0, b1 = (c >> 1) & 1, c & 1
                blk += a[i + b0, j + b1] * (w[b0][:, None] * w[b1][None, :])
            out[i * F:i * F + F + 1, j * F:j * F + F + 1] = blk
    return out


def upsample_backprop_2d(g, in_shape, F):
    """UpsampleFilter::BackpropImpl<1, 1>."""
    return upsample_backprop(_flat3(g), tuple(in_shape) + (1,), F)[:, :, 0]


def vertex_to_cell_2d(v):
    v = np.asarray(v, dtype=np.float64)
    return 0.25 * sum(v[a:a + v.shape[0] - 1, b:b + v.shape[1] - 1] for a in (0, 1) for b in (0, 1))


def vertex_to_cell_backprop_2d(g):
    g = np.asarray(g, dtype=np.float64)
    out = np.zeros(tuple(s + 1 for s in g.shape))
    for a in (0, 1):
        for b in (0, 1):
            out[a:a + g.shape[0], b:b + g.shape[1]] += g
    return 0.25 * out
