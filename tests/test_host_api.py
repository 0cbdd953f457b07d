"""Host-side behaviour of the pyVoxelFEM mirror that needs no GPU: the factory's dispatch
errors (VoxelFEM.cc:423-430), the ElasticityTensor value object the reference's scripts use,
and FilterChain's backward sizing of dimension-changing filters."""
import pytest


@pytest.fixture(scope="module")
def pv():
    from voxelfem_gb300 import pyVoxelFEM
    return pyVoxelFEM


@pytest.mark.parametrize("degs", [[2, 2], [1, 2, 1], [3, 3, 3], [1]])
def test_factory_rejects_unregistered_instantiations(pv, degs):
    bbox = [[0.0] * len(degs), [1.0] * len(degs)]
    with pytest.raises(RuntimeError, match="No template instantiation matching degreesPerDimension/number type!"):
        pv.TensorProductSimulator(degs, bbox, [4] * len(degs))


def test_factory_rejects_float_number_type(pv):
    with pytest.raises(RuntimeError, match="No template instantiation"):
        pv.TensorProductSimulator([1, 1, 1], [[0, 0, 0], [1, 1, 1]], [4, 4, 4], numberType=pv.NumberType.FLOAT)


def test_elasticity_tensor_value_semantics(pv):
    e = pv.ElasticityTensor()
    assert tuple(e) == (1.0, 0.0)
    e.setIsotropic(2, 0.3)
    young, poisson = e
    assert (young, poisson) == (2.0, 0.3)
    assert e == (2.0, 0.3) and e == pv.ElasticityTensor(2.0, 0.3) and e != (2.0, 0.25)
    assert len(e) == 2 and e[0] == 2.0 and e[1] == 0.3
    assert "young=2" in repr(e)


def test_filter_chain_sizes_dimension_changing_filters_backwards(pv):
    # TopologyOptimizationFilter.hh:90-187: the chain ends on the physical grid and each
    # filter's input size follows from its output size
    chain = pv.FilterChain([pv.UpsampleFilter(2), pv.VertexToCellFilter(), pv.SmoothingFilter(2)], (8, 4, 4))
    assert tuple(chain.physicalGridDims()) == (8, 4, 4) and chain.numPhysicalVars() == 128
    # smoothing keeps (8, 4, 4); vertex-to-cell needs the (9, 5, 5) vertex grid; upsampling by 2
    # reaches (9, 5, 5) from (5, 3, 3)
    assert tuple(chain.gridDims()) == (5, 3, 3) and chain.numVars() == 45


def test_upsample_output_must_be_reachable(pv):
    with pytest.raises(RuntimeError, match="Output size is not divisible by factor"):
        pv.FilterChain([pv.UpsampleFilter(2)], (8, 4, 4))
    with pytest.raises(RuntimeError, match="2\\^d grid or larger"):
        pv.UpsampleFilter(2).setInputDimensions((1, 4, 4))


def test_filter_use_before_sizing_is_an_error(pv):
    with pytest.raises(RuntimeError, match="Filter grid dimensions not set"):
        pv.VertexToCellFilter().apply([0.0] * 8)
