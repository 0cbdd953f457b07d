"""UpsampleFilter, VertexToCellFilter and LangelaarFilter on the GPU against the oracle's numpy
restatements (oracle/filters.py): apply and backprop to 1e-13 (Langelaar 1e-11: pow-heavy),
the adjoint identity <A x, y> = <x, A^T y> for the linear filters, the Langelaar filter's state
across applications, and dimension propagation through a FilterChain."""
import numpy as np
import pytest

from oracle import filters as of
from voxelfem_gb300 import pyVoxelFEM as pv

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("shape,factor", [((3, 4, 5), 2), ((2, 3, 2), 3), ((4, 4, 4), 1)])
def test_upsample(gpu, shape, factor):
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 1, shape)
    f = pv.UpsampleFilter(factor)
    f.setInputDimensions(shape)
    out_shape = tuple((s - 1) * factor + 1 for s in shape)
    np.testing.assert_array_equal(f.outputDimensions, out_shape)
    y = f.apply(x.ravel())
    assert rel(y, of.upsample(x, factor)) < 1e-14
    g = rng.standard_normal(out_shape)
    b = f.backprop(g.ravel())
    assert rel(b, of.upsample_backprop(g, shape, factor)) < 1e-13
    assert abs(np.dot(y, g.ravel()) - np.dot(x.ravel(), b)) < 1e-12 * abs(np.dot(y, g.ravel()))


def test_vertex_to_cell(gpu):
    rng = np.random.default_rng(1)
    shape = (5, 4, 6)
    v = rng.uniform(0, 1, shape)
    f = pv.VertexToCellFilter()
    f.setInputDimensions(shape)
    y = f.apply(v.ravel())
    assert rel(y, of.vertex_to_cell(v)) < 1e-15
    g = rng.standard_normal(tuple(s - 1 for s in shape))
    b = f.backprop(g.ravel())
    assert rel(b, of.vertex_to_cell_backprop(g)) < 1e-15
    assert abs(np.dot(y, g.ravel()) - np.dot(v.ravel(), b)) < 1e-12 * abs(np.dot(y, g.ravel()))


@pytest.mark.parametrize("shape", [(5, 6, 4), (40, 7, 3)])
def test_langelaar(gpu, shape):
    rng = np.random.default_rng(2)
    f = pv.LangelaarFilter()
    f.setInputDimensions(shape)
    o = of.Langelaar(shape)
    for it in range(2):  # the second application sees the first one's output (own-voxel term)
        x = rng.uniform(0.05, 1.0, shape)
        y = f.apply(x.ravel())
        assert rel(y, o.apply(x)) < 1e-11, it
        g = rng.standard_normal(shape)
        assert rel(f.backprop(g.ravel(), x.ravel()), o.backprop(g, x)) < 1e-11, it


def test_filter_chain_dimensions(gpu):
    """A chain that upsamples node values and converts them to cells: the design grid is sized
    backwards from the density grid, and the chain matches the composition of the oracle's
    filters."""
    out = (8, 8, 8)
    chain = pv.FilterChain([pv.UpsampleFilter(2), pv.VertexToCellFilter(),
                            pv.ProjectionFilter(2.0)], out)
    np.testing.assert_array_equal(chain.gridDims(), (5, 5, 5))
    np.testing.assert_array_equal(chain.physicalGridDims(), out)
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, (5, 5, 5))
    chain.setDesignVars(x.ravel())
    from oracle import pyoracle as po
    ref = po.projection_apply(of.vertex_to_cell(of.upsample(x, 2)).ravel(), 2.0)
    assert rel(chain.physicalVars(), ref) < 1e-14
    g = rng.standard_normal(int(np.prod(out)))
    gb = chain.backprop(g)
    assert gb.size == 125


# ---- 2D instantiations ----
@pytest.mark.parametrize("shape,factor", [((5, 4), 2), ((3, 6), 3)])
def test_upsample_2d(gpu, shape, factor):
    rng = np.random.default_rng(10)
    x = rng.uniform(0, 1, shape)
    f = pv.UpsampleFilter(factor)
    f.setInputDimensions(shape)
    y = f.apply(x.ravel())
    assert rel(y, of.upsample_2d(x, factor)) < 1e-14
    g = rng.standard_normal(tuple((s - 1) * factor + 1 for s in shape))
    assert rel(f.backprop(g.ravel()), of.upsample_backprop_2d(g, shape, factor)) < 1e-13


def test_vertex_to_cell_2d(gpu):
    rng = np.random.default_rng(11)
    v = rng.uniform(0, 1, (7, 5))
    f = pv.VertexToCellFilter()
    f.setInputDimensions(v.shape)
    np.testing.assert_array_equal(f.outputDimensions, (6, 4))
    assert rel(f.apply(v.ravel()), of.vertex_to_cell_2d(v)) < 1e-15
    g = rng.standard_normal((6, 4))
    assert rel(f.backprop(g.ravel()), of.vertex_to_cell_backprop_2d(g)) < 1e-15


def test_langelaar_2d(gpu):
    rng = np.random.default_rng(12)
    shape = (9, 7)
    f = pv.LangelaarFilter()
    f.setInputDimensions(shape)
    ref = of.Langelaar(shape, ndim=2)
    for _ in range(2):
        x = rng.uniform(0.05, 1, shape)
        assert rel(f.apply(x.ravel()), ref.apply(x).ravel()) < 1e-11
        g = rng.standard_normal(shape)
        assert rel(f.backprop(g.ravel(), x.ravel()), ref.backprop(g, x).ravel()) < 1e-11
