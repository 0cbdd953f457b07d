"""GB300-native VoxelFEM solve-and-sensitivity path.

``voxelfem_gb300.pyVoxelFEM`` mirrors the reference's ``pyVoxelFEM`` module on
the hot path; ``voxelfem_gb300.autograd`` wraps the solve, compliance and
volume in a ``torch.autograd.Function``. All computation runs in the CUDA
library ``_lib/libvfem.so`` (C ABI: include/vfem.h).
"""
from . import pyVoxelFEM  # noqa: F401
from ._capi import LIB_PATH, VoxelFEMError, load  # noqa: F401

__all__ = ["pyVoxelFEM", "load", "LIB_PATH", "VoxelFEMError"]
