"""Host-side behaviour of the pyVoxelFEM mirror that needs no GPU: the factory's dispatch
errors (VoxelFEM.cc:423-430) and the ElasticityTensor value object the reference's scripts use."""
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
