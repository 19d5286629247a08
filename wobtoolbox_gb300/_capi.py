"""ctypes binding of libwob_gb300.so (the C ABI declared in include/wob_capi.h).

The library is loaded from the package's in-tree build directory. There is no fallback: if the
library is missing or a CUDA call fails, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libwob_gb300.so")

WOB_OK = 0
STATUS_NAMES = {
    0: "WOB_OK",
    1: "WOB_ERR_INVALID_ARGUMENT",
    2: "WOB_ERR_UNSUPPORTED",
    3: "WOB_ERR_CUDA",
    4: "WOB_ERR_OUT_OF_MEMORY",
    5: "WOB_ERR_DEVICE_LIMIT",
}

# Every symbol the header declares, for load checks.
EXPORTED = [
    "wob_last_error", "wob_version", "wob_device_info", "wob_scene_create", "wob_scene_destroy",
    "wob_scene_get_info", "wob_scene_get_element_order", "wob_scene_poll_error",
    "wob_scene_set_volume_cache", "wob_scene_clear_volume_cache", "wob_solve_domain",
    "wob_solve_domain_host", "wob_solve_boundary", "wob_line_query", "wob_debug_domain_paths",
    "wob_debug_boundary_paths", "wob_solve_domain_host_noalloc", "wob_noalloc_max_points",
    "wob_autotune_domain", "wob_tunable_variant", "wob_set_domain_config", "wob_get_domain_config",
    "wob_batch_create", "wob_batch_solve", "wob_batch_destroy", "wob_solve_unknown_boundary",
    "wob_scene_set_control_variate", "wob_solve_domain_cv", "wob_cv_residual_data", "wob_cv_potential",
    "wob_scene_clone", "wob_scene_add_boundary_offsets", "wob_scene_element_frames", "wob_scene_sample_boundary", "wob_clip_magnitude_quantile", "wob_measure_gather_peak", "wob_scene_set_step_limits", "wob_mlp_create", "wob_mlp_destroy",
    "wob_mlp_num_params", "wob_mlp_get_params", "wob_mlp_set_params", "wob_mlp_forward", "wob_mlp_gradient",
    "wob_mlp_adam_step", "wob_mlp_train", "wob_mlp_gradient_fused", "wob_mlp_inject_wait_timeout", "wob_scene_set_rhs", "wob_solve_domain_multi",
    "wob_solve_unknown_boundary_multi",
    "wob_scene_set_rhs_control_variate", "wob_solve_domain_multi_cv", "wob_scene_create_device",
    "wob_vpl_paths", "wob_vpl_aggregate", "wob_solve_wos", "wob_closest_point",
]


class WobError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class wob_params(C.Structure):
    _fields_ = [
        ("bie_model", C.c_int32), ("domain", C.c_int32), ("estimator", C.c_int32), ("problem", C.c_int32),
        ("path_length", C.c_uint32), ("num_sample_paths", C.c_uint32),
        ("num_resampling_candidates", C.c_uint32), ("num_volume_samples", C.c_uint32),
        ("eps", C.c_float), ("first_kind_equation_scaling_constant", C.c_float),
        ("seed", C.c_uint64), ("path_offset", C.c_uint64),
        ("point_offset", C.c_uint32), ("flags", C.c_uint32),
    ]


class wob_scene_info(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n_elems", C.c_uint32), ("n_nodes", C.c_uint32), ("bvh_depth", C.c_uint32),
        ("total_area", C.c_float), ("total_boundary_value", C.c_float), ("has_volume_cache", C.c_int32),
        ("bytes_on_device", C.c_uint32), ("line_grid_bins", C.c_uint32), ("line_grid_cells", C.c_uint32),
    ]


_lib = None


def load() -> C.CDLL:
    """Loads the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise WobError(3, f"engine library not built: {LIB_PATH} (run __graft_entry__.build())")
    _lib = load_library(LIB_PATH)
    return _lib


def load_library(path: str) -> C.CDLL:
    """Loads a build of the engine library from `path` with every signature set (a second build,
    such as the contraction-enabled measurement variant, lives beside the default one in the same
    process: each library has its own device code and state)."""
    lib = C.CDLL(path)
    vp, u32, u64, i32, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32, C.c_float
    P = C.POINTER
    sigs = {
        "wob_last_error": (C.c_char_p, []),
        "wob_version": (C.c_int, []),
        "wob_device_info": (C.c_int, [P(C.c_int), P(C.c_int)]),
        "wob_scene_create": (C.c_int, [C.c_int, u32, vp, vp, vp, vp, vp, P(vp)]),
        "wob_scene_destroy": (C.c_int, [vp]),
        "wob_scene_get_info": (C.c_int, [vp, P(wob_scene_info)]),
        "wob_scene_get_element_order": (C.c_int, [vp, vp]),
        "wob_scene_poll_error": (C.c_int, [vp, P(u32)]),
        "wob_scene_set_volume_cache": (C.c_int, [vp, u32, f32, vp]),
        "wob_scene_clear_volume_cache": (C.c_int, [vp]),
        "wob_solve_domain": (C.c_int, [vp, P(wob_params), vp, u32, vp, vp, vp, vp]),
        "wob_solve_domain_host": (C.c_int, [vp, P(wob_params), vp, u32, vp, vp, vp]),
        "wob_solve_boundary": (C.c_int, [vp, P(wob_params), vp, vp, vp, vp, vp, vp, u32, vp, vp, vp, vp]),
        "wob_line_query": (C.c_int, [vp, vp, vp, u32, vp, vp, vp, vp]),
        "wob_debug_domain_paths": (C.c_int, [vp, P(wob_params), vp, u32, vp, vp]),
        "wob_debug_boundary_paths": (C.c_int, [vp, P(wob_params), vp, vp, vp, vp, vp, vp, u32, vp, vp]),
        "wob_solve_domain_host_noalloc": (C.c_int, [vp, P(wob_params), vp, u32, vp, vp, vp, vp]),
        "wob_noalloc_max_points": (C.c_int, [C.c_int, P(u32)]),
        "wob_autotune_domain": (C.c_int, [vp, P(wob_params), vp, u32, P(i32), vp, P(i32), vp]),
        "wob_tunable_variant": (C.c_int, [vp, P(wob_params), P(i32)]),
        "wob_set_domain_config": (C.c_int, [i32, i32]),
        "wob_get_domain_config": (C.c_int, [i32, P(i32)]),
        "wob_batch_create": (C.c_int, [vp, vp, vp, u32, P(vp)]),
        "wob_batch_solve": (C.c_int, [vp, vp, vp, vp, vp, u64, vp]),
        "wob_batch_destroy": (C.c_int, [vp]),
        "wob_solve_unknown_boundary": (C.c_int, [vp, P(wob_params), vp, vp, vp, vp, vp, vp, u32, vp, vp, vp, vp]),
        "wob_scene_set_control_variate": (C.c_int, [vp, vp, u32]),
        "wob_cv_residual_data": (C.c_int, [vp, vp, C.c_int, f32, f32, vp, vp]),
        "wob_cv_potential": (C.c_int, [vp, vp, f32, f32, vp, u32, vp, vp]),
        "wob_scene_clone": (C.c_int, [vp, P(vp)]),
        "wob_scene_add_boundary_offsets": (C.c_int, [vp, vp, u32, C.c_int, vp]),
        "wob_scene_element_frames": (C.c_int, [vp, vp, vp]),
        "wob_scene_sample_boundary": (C.c_int, [vp, u32, u64, vp, vp, vp, vp, vp, vp, vp]),
        "wob_clip_magnitude_quantile": (C.c_int, [vp, u32, f32, vp, vp]),
        "wob_measure_gather_peak": (C.c_int, [u32, u32, u32, P(C.c_double), P(f32)]),
        "wob_scene_set_step_limits": (C.c_int, [vp, u32, u32]),
        "wob_solve_domain_cv": (C.c_int, [vp, P(wob_params), u32, u32, vp, u32, vp, vp, vp, vp, vp]),
        "wob_mlp_create": (C.c_int, [u32, u32, u32, f32, u64, P(vp)]),
        "wob_mlp_destroy": (C.c_int, [vp]),
        "wob_mlp_num_params": (C.c_int, [vp, P(u32)]),
        "wob_mlp_get_params": (C.c_int, [vp, vp, vp]),
        "wob_mlp_set_params": (C.c_int, [vp, vp]),
        "wob_mlp_forward": (C.c_int, [vp, vp, u32, vp, vp]),
        "wob_mlp_gradient": (C.c_int, [vp, vp, vp, u32, vp, vp, vp]),
        "wob_mlp_adam_step": (C.c_int, [vp, vp, vp, u32, f32, vp, vp]),
        "wob_mlp_train": (C.c_int, [vp, vp, vp, u32, u32, u32, f32, u64, vp, vp]),
        "wob_mlp_gradient_fused": (C.c_int, [vp, vp, vp, u32, vp, vp, vp]),
        "wob_mlp_inject_wait_timeout": (C.c_int, [vp, u32]),
        "wob_scene_set_rhs": (C.c_int, [vp, vp, u32]),
        "wob_solve_domain_multi": (C.c_int, [vp, P(wob_params), vp, u32, vp, vp, vp, vp, vp]),
        "wob_solve_unknown_boundary_multi": (C.c_int, [vp, P(wob_params), vp, vp, vp, vp, vp, vp, u32, vp, vp, vp,
                                                       vp, vp]),
        "wob_scene_set_rhs_control_variate": (C.c_int, [vp, vp, u32, u32]),
        "wob_scene_create_device": (C.c_int, [C.c_int, u32, vp, vp, vp, vp, vp, vp, P(vp)]),
        "wob_vpl_paths": (C.c_int, [vp, P(wob_params), u32, vp, vp, vp, vp]),
        "wob_vpl_aggregate": (C.c_int, [vp, f32, vp, vp, u32, vp, u32, vp, vp]),
        "wob_solve_wos": (C.c_int, [vp, P(wob_params), vp, u32, vp, vp, vp, vp, vp]),
        "wob_closest_point": (C.c_int, [vp, vp, u32, vp, vp, vp, vp]),
        "wob_solve_domain_multi_cv": (C.c_int, [vp, P(wob_params), u32, vp, u32, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def check(status: int) -> None:
    if status != WOB_OK:
        msg = load().wob_last_error()
        raise WobError(status, msg.decode() if msg else "")
