"""ctypes binding of the C ABI declared in include/vfem.h (libvfem.so).

The library is the only compute path: if it cannot be loaded, every call
raises. There is no CPU fallback.
"""
import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libvfem.so")

_lib = None
_lock = threading.Lock()

_d = C.POINTER(C.c_double)
_i64 = C.POINTER(C.c_int64)
_i32 = C.POINTER(C.c_int)
_u8 = C.POINTER(C.c_uint8)
_vp = C.c_void_p


class PcgStats(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("relres", C.c_double), ("rsq", C.c_double), ("bnorm2", C.c_double)]


PCG_CALLBACK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p)

_SIGS = {
    "vfem_last_error": (C.c_char_p, []),
    "vfem_version": (C.c_int, []),
    "vfem_device_synchronize": (C.c_int, []),
    "vfem_grid_create": (C.c_int, [_i64, _d, _d, C.POINTER(_vp)]),
    "vfem_grid_destroy": (C.c_int, [_vp]),
    "vfem_grid_dims": (C.c_int, [_vp, _i64, _i64, _i64]),
    "vfem_grid_set_etensor": (C.c_int, [_vp, C.c_double, C.c_double]),
    "vfem_grid_get_etensor": (C.c_int, [_vp, _d, _d]),
    "vfem_grid_get_k0": (C.c_int, [_vp, _d]),
    "vfem_grid_k0_is_cube": (C.c_int, [_vp, _i32]),
    "vfem_grid_set_material_params": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
    "vfem_grid_get_material_params": (C.c_int, [_vp, _d, _d, _d, _d, _i32]),
    "vfem_grid_set_densities": (C.c_int, [_vp, _vp]),
    "vfem_grid_get_densities": (C.c_int, [_vp, _vp]),
    "vfem_grid_set_uniform_densities": (C.c_int, [_vp, C.c_double]),
    "vfem_grid_get_young_moduli": (C.c_int, [_vp, _vp]),
    "vfem_grid_add_dirichlet": (C.c_int, [_vp, _d, _d, _d, C.c_uint32]),
    "vfem_grid_apply_symmetry": (C.c_int, [_vp, _i32, _i32]),
    "vfem_grid_set_nodal_forces": (C.c_int, [_vp, _vp]),
    "vfem_grid_get_dirichlet_mask": (C.c_int, [_vp, _u8]),
    "vfem_grid_set_gravity": (C.c_int, [_vp, _d]),
    "vfem_grid_get_gravity": (C.c_int, [_vp, _d]),
    "vfem_grid_set_mask_layer": (C.c_int, [_vp, C.c_int64]),
    "vfem_grid_get_mask_height": (C.c_int, [_vp, _d]),
    "vfem_grid_apply_k": (C.c_int, [_vp, _vp, _vp]),
    "vfem_grid_build_load": (C.c_int, [_vp, _vp]),
    "vfem_grid_compliance_gradient": (C.c_int, [_vp, _vp, _vp]),
    "vfem_grid_adjoint_sensitivity": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, _vp]),
    "vfem_lbl_create": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "vfem_q2_create": (C.c_int, [_vp, _vp, _vp, C.POINTER(C.c_void_p)]),
    "vfem_q2_destroy": (C.c_int, [_vp]),
    "vfem_q2_dims": (C.c_int, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "vfem_q2_set_etensor": (C.c_int, [_vp, C.c_double, C.c_double]),
    "vfem_q2_set_material_params": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
    "vfem_q2_set_densities": (C.c_int, [_vp, _vp]),
    "vfem_q2_get_k0": (C.c_int, [_vp, _vp]),
    "vfem_q2_add_dirichlet": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "vfem_q2_get_dirichlet_mask": (C.c_int, [_vp, _vp]),
    "vfem_q2_apply_k": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int]),
    "vfem_q2_smooth": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int]),
    "vfem_q2_restrict": (C.c_int, [_vp, _vp, _vp]),
    "vfem_q2_interpolate": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "vfem_q2_time_apply_k": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "vfem_q2_time_smooth": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "vfem_q2_set_outer_matvec": (C.c_int, [_vp, C.c_int]),
    "vfem_q2_set_hierarchy": (C.c_int, [_vp, C.c_int]),
    "vfem_q2_set_precision": (C.c_int, [_vp, C.c_int]),
    "vfem_q2_mg_num_nodes": (C.c_int, [_vp, C.c_int64, C.c_int, _vp]),
    "vfem_q2_mg_level_dirichlet": (C.c_int, [_vp, C.c_int64, C.c_int, _vp]),
    "vfem_q2_mg_level_ke": (C.c_int, [_vp, C.c_int64, C.c_int, C.c_int, _vp]),
    "vfem_q2_mg_smooth": (C.c_int, [_vp, C.c_int64, C.c_int, _vp, _vp, C.c_int, C.c_int]),
    "vfem_q2_mg_residual": (C.c_int, [_vp, C.c_int64, C.c_int, _vp, _vp, _vp, C.c_int]),
    "vfem_q2_mg_coarse_solve": (C.c_int, [_vp, C.c_int64, _vp, _vp, C.c_int]),
    "vfem_q2_mg_vcycle": (C.c_int, [_vp, C.c_int64, _vp, _vp, C.c_int64, C.c_int]),
    "vfem_q2_pcg": (C.c_int, [_vp, C.c_int64, _vp, _vp, C.c_int64, C.c_double, C.c_int64, _vp]),
    "vfem_mg_outer_matvec_kind": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "vfem_mg_outer_apply": (C.c_int, [_vp, _vp, _vp, _vp]),
    "vfem_tc_fit_k0": (C.c_int, [_vp, C.POINTER(C.c_double), _vp, C.POINTER(C.c_int)]),
    "vfem_lbl_destroy": (C.c_int, [_vp]),
    "vfem_lbl_run": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int,
                               _vp, _vp, _vp]),
    "vfem_lbl_set_init": (C.c_int, [_vp, C.c_int, C.c_int]),
    "vfem_mma_create": (C.c_int, [C.c_int64, C.c_int, _vp, _vp, _vp, _vp, _vp, C.POINTER(C.c_void_p)]),
    "vfem_mma_destroy": (C.c_int, [_vp]),
    "vfem_mma_set_initial_var": (C.c_int, [_vp, _vp]),
    "vfem_mma_enable_gcmma": (C.c_int, [_vp, C.c_int]),
    "vfem_mma_step": (C.c_int, [_vp]),
    "vfem_mma_get_optimal_var": (C.c_int, [_vp, _vp]),
    "vfem_upsample_filter": (C.c_int, [_vp, C.c_int64, _vp, _vp]),
    "vfem_upsample_filter_backprop": (C.c_int, [_vp, C.c_int64, _vp, _vp]),
    "vfem_vertex_to_cell_filter": (C.c_int, [_vp, _vp, _vp]),
    "vfem_vertex_to_cell_filter_backprop": (C.c_int, [_vp, _vp, _vp]),
    "vfem_langelaar_create": (C.c_int, [_vp, C.POINTER(C.c_void_p)]),
    "vfem_langelaar_destroy": (C.c_int, [_vp]),
    "vfem_langelaar_apply": (C.c_int, [_vp, _vp, _vp]),
    "vfem_langelaar_backprop": (C.c_int, [_vp, _vp, _vp, _vp]),
    "vfem_grid_element_energy": (C.c_int, [_vp, _vp, _vp]),
    "vfem_mg_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "vfem_mg_destroy": (C.c_int, [_vp]),
    "vfem_mg_num_levels": (C.c_int, [_vp, _i32]),
    "vfem_mg_level_dims": (C.c_int, [_vp, C.c_int, _i64]),
    "vfem_mg_level_dirichlet_mask": (C.c_int, [_vp, C.c_int, _u8]),
    "vfem_mg_set_precision": (C.c_int, [_vp, C.c_int, C.c_int]),
    "vfem_mg_set_use_graphs": (C.c_int, [_vp, C.c_int]),
    "vfem_mg_set_device_loop": (C.c_int, [_vp, C.c_int]),
    "vfem_mg_stiffness_rebuilds": (C.c_int, [_vp, _i64, _i64]),
    "vfem_mg_set_sweep_form": (C.c_int, [_vp, C.c_int]),
    "vfem_mg_set_stencil_bf16": (C.c_int, [_vp, C.c_int]),
    "vfem_lbl_set_sweep_form": (C.c_int, [_vp, C.c_int]),
    "vfem_mg_set_symmetric_gs": (C.c_int, [_vp, C.c_int]),
    "vfem_mg_set_mask_layer": (C.c_int, [_vp, C.c_int64]),
    "vfem_mg_update_stiffness": (C.c_int, [_vp]),
    "vfem_mg_apply_k": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "vfem_mg_residual": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "vfem_mg_smooth": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int]),
    "vfem_mg_restrict": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "vfem_mg_interpolate": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int]),
    "vfem_mg_coarse_solve": (C.c_int, [_vp, _vp, _vp]),
    "vfem_mg_zero_dirichlet": (C.c_int, [_vp, C.c_int, _vp]),
    "vfem_mg_solve": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int, C.c_int, _vp]),
    "vfem_mg_pcg": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int,
                              PCG_CALLBACK, _vp, C.POINTER(PcgStats)]),
    "vfem_mg_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "vfem_mg_time_kernel": (C.c_int, [_vp, C.c_int, C.c_int, _d, _d]),
    "vfem_kernel_launch_count": (C.c_int, [C.POINTER(C.c_uint64)]),
    "vfem_mg_profile": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int, C.c_char_p, C.c_int64, _d, C.c_int, _i32]),
    "vfem_smoothing_filter": (C.c_int, [_i64, C.c_int, C.c_int, _vp, _vp]),
    "vfem_debug_pivot_reciprocals": (C.c_int, [_vp, C.c_int64, _vp, _vp]),
    "vfem_smoothing_filter_noalloc": (C.c_int, [_i64, C.c_int, C.c_int, _vp, _vp, _vp]),
    "vfem_projection_apply": (C.c_int, [C.c_int64, C.c_double, _vp, _vp]),
    "vfem_projection_backprop": (C.c_int, [C.c_int64, C.c_double, _vp, _vp, _vp]),
    "vfem_problem_create": (C.c_int, [_vp, C.c_int, _i32, _i32, _i32, _d, C.c_double, C.POINTER(_vp)]),
    "vfem_problem_destroy": (C.c_int, [_vp]),
    "vfem_problem_set_solver": (C.c_int, [_vp, C.c_int64, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int]),
    "vfem_problem_set_vars": (C.c_int, [_vp, _vp]),
    "vfem_problem_get_vars": (C.c_int, [_vp, _vp]),
    "vfem_problem_objective": (C.c_int, [_vp, _d]),
    "vfem_problem_gradient": (C.c_int, [_vp, _vp]),
    "vfem_problem_constraint": (C.c_int, [_vp, _d]),
    "vfem_problem_jacobian": (C.c_int, [_vp, _vp]),
    "vfem_problem_get_u": (C.c_int, [_vp, _vp]),
    "vfem_problem_get_physical": (C.c_int, [_vp, _vp]),
    "vfem_problem_last_solve": (C.c_int, [_vp, C.POINTER(PcgStats)]),
    "vfem_problem_oc_step": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, _i64]),
    "vfem_problem_oc_step_with_gradient": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, _vp, _i64]),
    # ---- 2D (bilinear quadrilaterals) ----
    "vfem_grid2_create": (C.c_int, [_i64, _d, _d, C.POINTER(_vp)]),
    "vfem_grid2_destroy": (C.c_int, [_vp]),
    "vfem_grid2_dims": (C.c_int, [_vp, _i64, _i64, _i64]),
    "vfem_grid2_set_etensor": (C.c_int, [_vp, C.c_double, C.c_double]),
    "vfem_grid2_get_etensor": (C.c_int, [_vp, _d, _d]),
    "vfem_grid2_get_k0": (C.c_int, [_vp, _d]),
    "vfem_grid2_set_material_params": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
    "vfem_grid2_get_material_params": (C.c_int, [_vp, _d, _d, _d, _d, _i32]),
    "vfem_grid2_set_densities": (C.c_int, [_vp, _vp]),
    "vfem_grid2_get_densities": (C.c_int, [_vp, _vp]),
    "vfem_grid2_set_uniform_densities": (C.c_int, [_vp, C.c_double]),
    "vfem_grid2_get_young_moduli": (C.c_int, [_vp, _vp]),
    "vfem_grid2_add_dirichlet": (C.c_int, [_vp, _d, _d, _d, C.c_uint32]),
    "vfem_grid2_apply_symmetry": (C.c_int, [_vp, _i32, _i32]),
    "vfem_grid2_set_nodal_forces": (C.c_int, [_vp, _vp]),
    "vfem_grid2_get_dirichlet_mask": (C.c_int, [_vp, _u8]),
    "vfem_grid2_get_dirichlet_values": (C.c_int, [_vp, _vp]),
    "vfem_grid2_set_gravity": (C.c_int, [_vp, _d]),
    "vfem_grid2_get_gravity": (C.c_int, [_vp, _d]),
    "vfem_grid2_set_mask_layer": (C.c_int, [_vp, C.c_int64]),
    "vfem_grid2_get_mask_height": (C.c_int, [_vp, _d]),
    "vfem_grid2_apply_k": (C.c_int, [_vp, _vp, _vp]),
    "vfem_grid2_build_load": (C.c_int, [_vp, _vp]),
    "vfem_grid2_compliance_gradient": (C.c_int, [_vp, _vp, _vp]),
    "vfem_grid2_adjoint_sensitivity": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, _vp]),
    "vfem_grid2_element_energy": (C.c_int, [_vp, _vp, _vp]),
    "vfem_mg2_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "vfem_mg2_destroy": (C.c_int, [_vp]),
    "vfem_mg2_num_levels": (C.c_int, [_vp, _i32]),
    "vfem_mg2_level_dims": (C.c_int, [_vp, C.c_int, _i64]),
    "vfem_mg2_level_dirichlet_mask": (C.c_int, [_vp, C.c_int, _u8]),
    "vfem_mg2_set_use_graphs": (C.c_int, [_vp, C.c_int]),
    "vfem_mg2_set_symmetric_gs": (C.c_int, [_vp, C.c_int]),
    "vfem_mg2_set_mask_layer": (C.c_int, [_vp, C.c_int64]),
    "vfem_mg2_update_stiffness": (C.c_int, [_vp]),
    "vfem_mg2_apply_k": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "vfem_mg2_residual": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "vfem_mg2_smooth": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int]),
    "vfem_mg2_restrict": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "vfem_mg2_interpolate": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int]),
    "vfem_mg2_coarse_solve": (C.c_int, [_vp, _vp, _vp]),
    "vfem_mg2_zero_dirichlet": (C.c_int, [_vp, C.c_int, _vp]),
    "vfem_mg2_solve": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int, C.c_int, _vp]),
    "vfem_mg2_pcg": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int,
                              PCG_CALLBACK, C.c_void_p, C.POINTER(PcgStats)]),
    "vfem_mg2_time_kernel": (C.c_int, [_vp, C.c_int, C.c_int, _d]),
    "vfem_lbl2_create": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "vfem_mg2_set_precision": (C.c_int, [_vp, C.c_int]),
    "vfem_mg2_set_outer_matvec": (C.c_int, [_vp, C.c_int]),
    "vfem_lbl2_destroy": (C.c_int, [_vp]),
    "vfem_lbl2_set_init": (C.c_int, [_vp, C.c_int, C.c_int]),
    "vfem_lbl2_run": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int,
                                _vp, _vp, _vp]),
    "vfem_upsample_filter2": (C.c_int, [_i64, C.c_int64, _vp, _vp]),
    "vfem_upsample_filter2_backprop": (C.c_int, [_i64, C.c_int64, _vp, _vp]),
    "vfem_vertex_to_cell_filter2": (C.c_int, [_i64, _vp, _vp]),
    "vfem_vertex_to_cell_filter2_backprop": (C.c_int, [_i64, _vp, _vp]),
    "vfem_langelaar2_create": (C.c_int, [_i64, C.POINTER(_vp)]),
    "vfem_smoothing_filter2": (C.c_int, [_i64, C.c_int, C.c_int, _vp, _vp]),
    "vfem_problem2_create": (C.c_int, [_vp, C.c_int, _i32, _i32, _i32, _d, C.c_double, C.POINTER(_vp)]),
}

EXPORTED = sorted(_SIGS)


def load(path: str = LIB_PATH):
    """Load libvfem.so (building it first when absent or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path) or path == LIB_PATH:
            from . import build as _build
            try:
                path = _build.build()
            except Exception as exc:  # no nvcc: the library must already exist
                if not os.path.exists(path):
                    raise RuntimeError("libvfem.so is missing and could not be built: %s" % exc)
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


class VoxelFEMError(RuntimeError):
    """Raised for a nonzero status of the C ABI (the reference's std::runtime_error)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def check(rc):
    if rc != 0:
        raise VoxelFEMError(rc, load().vfem_last_error().decode())


def ptr(a):
    """Raw address of a numpy array or a CUDA torch tensor (device pointers pass through)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError("expected a numpy array or a tensor, got %r" % type(a))


def dptr(a):
    return a.ctypes.data_as(_d)
