"""The tensor-core outer matvec (integer-slice bf16 MMAs, exact FP32 accumulation) against
the oracle's FP64 applyK: 1e-12 relative to max |K u| on operands spanning ten decades, the
residual form, masked layers, NaN propagation, the fallback to the double-float kernel when K0
has no small-integer form, and MG-PCG with the same iteration count as FP64 (compliance to
1e-9)."""
import numpy as np
import pytest

from voxelfem_gb300 import pyVoxelFEM as pv
from voxelfem_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def setup(oracle, ne, levels=1, rho_lo=0.01, mask_layer=None, nu=0.3, bbox=None):
    if bbox is None:
        bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    g = pv.TensorProductSimulator([1, 1, 1], bbox, ne)
    o = oracle.Sim(ne, bbox)
    wl.setup_cantilever(g, ne, rho_lo, 0)
    wl.setup_cantilever(o, ne, rho_lo, 0)
    if nu != 0.3:
        g.ETensor = (1.0, nu)
        o.setMaterial(1.0, nu)
    if mask_layer is not None:
        g.setFabricationMaskHeightByLayer(mask_layer)
        o.setFabricationMaskHeightByLayer(mask_layer)
    mg = g.multigridSolver(levels)
    if mask_layer is not None:
        mg.setFabricationMaskHeightByLayer(mask_layer)
    mg.setPrecision("mixed", "df")
    return g, o, mg


def wide_operand(nn, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nn, 3)) * 10.0 ** rng.uniform(-8, 2, (nn, 3))


@pytest.mark.parametrize("ne", [(4, 2, 2), (14, 10, 22), (64, 32, 32), (20, 40, 8)])
def test_tensor_matvec_matches_fp64(gpu, oracle, ne):
    g, o, mg = setup(oracle, ne)
    assert mg.outerMatvecKind() == "tensor"
    mask = g.getDirichletMask()
    for seed in (1, 2):
        u = wide_operand(g.numNodes(), seed)
        ref = o.applyK(u)
        ref[mask] = 0.0
        assert rel(mg.outerApply(u), ref) < 1e-12
    # residual form
    b = np.random.default_rng(3).standard_normal((g.numNodes(), 3))
    r = b - o.applyK(u)
    r[mask] = 0.0
    assert rel(mg.outerApply(u, b), r) < 1e-12
    # a zero operand
    assert np.max(np.abs(mg.outerApply(np.zeros_like(u)))) == 0.0


def test_tensor_matvec_masked_layer(gpu, oracle):
    ne = (12, 16, 10)
    g, o, mg = setup(oracle, ne, mask_layer=7)
    assert mg.outerMatvecKind() == "tensor"
    u = wide_operand(g.numNodes(), 4)
    ref = o.applyK(u)
    ref[g.getDirichletMask()] = 0.0
    out = mg.outerApply(u)
    assert rel(out, ref) < 1e-12
    nn = [v + 1 for v in ne]
    j = (np.arange(g.numNodes()) // nn[2]) % nn[1]
    assert np.all(out[j > 8] == 0.0)  # detached rows


def test_tensor_matvec_nan_propagates(gpu, oracle):
    g, o, mg = setup(oracle, (8, 6, 6))
    u = wide_operand(g.numNodes(), 5)
    u[17, 1] = np.nan
    assert np.isnan(mg.outerApply(u)).any()


def test_fallback_to_double_float(gpu, oracle):
    # nu = 0.33 makes lambda / mu = 66 / 34: the integer matrix exceeds the exactness bound
    g, o, mg = setup(oracle, (8, 4, 6), nu=0.33)
    assert mg.outerMatvecKind() == "df-simt"
    u = wide_operand(g.numNodes(), 6)
    ref = o.applyK(u)
    ref[g.getDirichletMask()] = 0.0
    assert rel(mg.outerApply(u), ref) < 1e-12
    # stretched voxels: K0 is not a scaled integer matrix either
    g2, o2, mg2 = setup(oracle, (8, 4, 6), bbox=[[0.0, 0.0, 0.0], [8.0, 6.0, 6.0]])
    assert mg2.outerMatvecKind() == "df-simt"
    # back to a cube material: the tensor path returns
    g.ETensor = (1.0, 0.3)
    assert mg.outerMatvecKind() == "tensor"


def test_mixed_pcg_outer_matvecs(gpu, oracle):
    """Tensor-core and double-float outer matvecs under the same FP32 preconditioner follow the
    same iterations; both meet the FP64 solve."""
    ne = (64, 32, 32)
    g, o, mg = setup(oracle, ne, levels=3, rho_lo=0.3)
    f = g.buildLoadVector()
    mg.setPrecision("fp64")
    x64 = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 100, 1e-8, None, 1, 2, False)
    c64 = np.sum(f * x64)
    res = {}
    for matvec, kind in (("df-simt", "df-simt"), ("df", "tensor")):
        mg.setPrecision("mixed", matvec)
        assert mg.outerMatvecKind() == kind
        x = mg.preconditionedConjugateGradient(np.zeros_like(f), f, 100, 1e-8, None, 1, 2, False)
        assert mg.lastStats.relres <= 1e-8
        r = f - o.applyK(x)
        r[g.getDirichletMask()] = 0.0
        assert np.linalg.norm(r) / np.linalg.norm(f) < 2e-8  # true residual, FP64
        assert abs(np.sum(f * x) - c64) / abs(c64) < 1e-7
        res[kind] = (x, mg.lastStats.iterations)
    assert res["tensor"][1] == res["df-simt"][1]
    assert rel(res["tensor"][0], res["df-simt"][0]) < 1e-8
