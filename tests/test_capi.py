"""C-ABI boundary checks that need no GPU: the library loads and exports every
symbol that include/vfem.h declares, and the Python binding covers them all."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "vfem.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\s*\*)\s*(vfem_\w+)\s*\(", text, re.M)))


def test_header_parses():
    syms = header_symbols()
    assert len(syms) > 40
    assert "vfem_mg_pcg" in syms and "vfem_grid_apply_k" in syms


def test_library_exports_every_declared_symbol():
    from voxelfem_gb300 import _capi
    lib = _capi.load()  # builds with nvcc when stale; loading needs no GPU
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from voxelfem_gb300 import _capi
    assert sorted(_capi.EXPORTED) == header_symbols()


def test_error_path_without_device_work():
    from voxelfem_gb300 import _capi
    lib = _capi.load()
    out = ctypes.c_void_p()
    bad = (ctypes.c_int64 * 3)(0, 1, 1)
    lo = (ctypes.c_double * 3)(0, 0, 0)
    hi = (ctypes.c_double * 3)(1, 1, 1)
    rc = lib.vfem_grid_create(bad, lo, hi, ctypes.byref(out))
    assert rc == 1
    assert b"elementsPerDimension" in lib.vfem_last_error()


def test_api_rejects_unsupported_instantiations():
    from voxelfem_gb300 import pyVoxelFEM as pv
    with pytest.raises(RuntimeError, match="No template instantiation"):
        pv.TensorProductSimulator([2, 2], [[0, 0], [1, 1]], [2, 2])
    with pytest.raises(RuntimeError, match="No template instantiation"):
        pv.TensorProductSimulator([1, 1, 1], [[0, 0, 0], [1, 1, 1]], [2, 2, 2], pv.NumberType.FLOAT)
