"""ctypes binding of libgishadow.so (the C ABI declared in include/gi_shadow.h).

The library is built in-tree by globalillumination_gb300/build.py.  Loading
fails loudly when it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgishadow.so")

# gi_status
GI_OK = 0
GI_ERR_INVALID_ARG = 1
GI_ERR_IO = 2
GI_ERR_PARSE = 3
GI_ERR_CUDA = 4
GI_ERR_CAPACITY = 5
GI_ERR_OOM = 6
GI_ERR_DEVICE = 7
GI_ERR_UNSUPPORTED = 8

STATUS_NAMES = {
    0: "GI_OK", 1: "GI_ERR_INVALID_ARG", 2: "GI_ERR_IO", 3: "GI_ERR_PARSE", 4: "GI_ERR_CUDA",
    5: "GI_ERR_CAPACITY", 6: "GI_ERR_OOM", 7: "GI_ERR_DEVICE", 8: "GI_ERR_UNSUPPORTED",
}

# gi_bias_mode
GI_BIAS_NONE = 0
GI_BIAS_CONSTANT = 1
GI_BIAS_POLYGON_OFFSET = 2

# gi_technique
GI_TECH_HARD = 0
GI_TECH_PCF = 1
GI_TECH_PCF_TRICUBIC = 2
GI_TECH_PCSS_GRID = 3
GI_TECH_PCSS_POISSON = 4
GI_TECH_SMSR_CONSERVATIVE = 5
GI_TECH_SMSR_NONCONSERVATIVE = 6
GI_TECH_RPCF_CONSERVATIVE = 7
GI_TECH_RPCF_SMSR = 8
GI_TECH_RSMSS = 9
GI_TECH_HARD_SOFTAPP = 10
GI_PBA_MARKER = -32768
GI_TECH_RBSSM = 11
GI_TECH_VSM = 12
GI_TECH_ESM = 13
GI_TECH_EVSM = 14
GI_TECH_MSM = 15
GI_TECH_SAVSM = 16
GI_TECH_VSSM = 17
GI_TECH_ESSM = 18
GI_TECH_MSSM = 19
GI_TECH_COUNT = 20
GI_ACT_NONE = 0
GI_ACT_RELU = 1

# gi_pretest_mode
GI_PRETEST_REFERENCE = 0
GI_PRETEST_OFF = 1

# gi_depth_func
GI_DEPTH_LESS = 0
GI_DEPTH_LEQUAL = 1

F3 = C.c_float * 3
F9 = C.c_float * 9
F16 = C.c_float * 16


class SceneInfo(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int),
        ("num_triangles", C.c_int),
        ("camera_eye", F3),
        ("camera_at", F3),
        ("light_eye", F3),
        ("light_at", F3),
        ("depth_threshold", C.c_float),
        ("hsm_alpha", C.c_float),
        ("hsm_beta", C.c_float),
        ("num_objects", C.c_int),
    ]


class View(C.Structure):
    _fields_ = [
        ("eye", F3),
        ("at", F3),
        ("up", F3),
        ("fovy_deg", C.c_float),
        ("znear", C.c_float),
        ("zfar", C.c_float),
        ("width", C.c_int),
        ("height", C.c_int),
    ]


class FrameMatrices(C.Structure):
    _fields_ = [
        ("light_mvp", F16),
        ("light_mvp_biased", F16),
        ("camera_mvp", F16),
        ("camera_mv", F16),
        ("normal_matrix", F9),
        ("light_position", F3),
    ]


class MapParams(C.Structure):
    _fields_ = [
        ("width", C.c_int),
        ("height", C.c_int),
        ("bias_mode", C.c_int),
        ("constant_bias", C.c_float),
        ("offset_factor", C.c_float),
        ("offset_units", C.c_float),
    ]


class VisParams(C.Structure):
    _fields_ = [
        ("technique", C.c_int),
        ("pretest", C.c_int),
        ("shadow_intensity", C.c_float),
        ("kernel_order", C.c_int),
        ("penumbra_size", C.c_int),
        ("max_search", C.c_int),
        ("depth_threshold", C.c_float),
        ("blocker_search_size", C.c_int),
        ("kernel_size", C.c_int),
        ("light_radius", C.c_float),
        ("znear", C.c_float),
        ("pcss_min_blocker_depth", C.c_float),
        ("poisson_blocker_taps", C.c_int),
        ("poisson_filter_taps", C.c_int),
        ("summed_area_table", C.c_int),
        ("hsm_alpha", C.c_float),
        ("hsm_beta", C.c_float),
        ("light_mvp_biased", F16),
        ("camera_mv", F16),
        ("normal_matrix", F9),
        ("light_position", F3),
    ]


class BatchTuning(C.Structure):
    _fields_ = [
        ("tiny_px", C.c_int),
        ("coop_px", C.c_int),
        ("streams", C.c_int),
        ("frames", C.c_int),
        ("kernel_launches", C.c_uint64),
        ("best_ms", C.c_float),
        ("persistent", C.c_int),
        ("tile_w", C.c_int),
        ("tile_h", C.c_int),
        ("work_items", C.c_uint32),
    ]


# Every function the header declares, with its ctypes prototype.
_VP = C.c_void_p
_PROTOS = {
    "gi_last_error_string": (C.c_char_p, []),
    "gi_debug_fail_allocation": (C.c_int, [C.c_int]),
    "gi_version": (C.c_char_p, []),
    "gi_context_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "gi_context_destroy": (None, [_VP]),
    "gi_context_launch_count": (C.c_uint64, [_VP]),
    "gi_context_set_profiling": (C.c_int, [_VP, C.c_int]),
    "gi_context_phase_ms": (C.c_int, [_VP, C.c_float * 3]),
    "gi_context_set_tuning": (C.c_int, [_VP, C.c_int, C.c_int]),
    "gi_scene_load_config": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(_VP)]),
    "gi_scene_create": (C.c_int, [C.POINTER(_VP)]),
    "gi_scene_destroy": (None, [_VP]),
    "gi_scene_object_load_obj": (C.c_int, [_VP, C.c_char_p]),
    "gi_scene_object_from_arrays": (C.c_int, [_VP, _VP, C.c_int, _VP, C.c_int]),
    "gi_scene_object_scale": (C.c_int, [_VP, C.c_float, C.c_float, C.c_float]),
    "gi_scene_object_translate": (C.c_int, [_VP, C.c_float, C.c_float, C.c_float]),
    "gi_scene_object_rotate": (C.c_int, [_VP, C.c_float, C.c_float, C.c_float]),
    "gi_scene_object_commit": (C.c_int, [_VP]),
    "gi_scene_set_views": (C.c_int, [_VP, F3, F3, F3, F3, C.c_float]),
    "gi_scene_get_info": (C.c_int, [_VP, C.POINTER(SceneInfo)]),
    "gi_scene_get_arrays": (C.c_int, [_VP, _VP, _VP, _VP]),
    "gi_gen_ground": (C.c_int, [_VP, C.c_float, C.c_float]),
    "gi_gen_uv_sphere": (C.c_int, [_VP, C.c_int, C.c_int, C.c_float, F3]),
    "gi_gen_icosphere": (C.c_int, [_VP, C.c_int, C.c_float, F3]),
    "gi_gen_displaced_sphere": (C.c_int, [_VP, C.c_int, C.c_int, C.c_float, C.c_float, F3, C.c_uint64]),
    "gi_gen_icosphere_field": (C.c_int, [_VP, C.c_int, C.c_int, F3, F3, C.c_float, C.c_float, C.c_uint64]),
    "gi_scene_upload": (C.c_int, [_VP, _VP, _VP]),
    "gi_scene_upload_from": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int, _VP, C.c_int, _VP]),
    "gi_scene_device_arrays": (C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP)]),
    "gi_view_matrices": (C.c_int, [C.POINTER(View), F16, F16]),
    "gi_frame_setup": (C.c_int, [C.POINTER(View), C.POINTER(View), C.POINTER(FrameMatrices)]),
    "gi_shadow_map": (C.c_int, [_VP, _VP, C.POINTER(MapParams), F16, _VP, _VP]),
    "gi_gbuffer": (C.c_int, [_VP, _VP, F16, C.c_int, C.c_int, _VP, _VP, _VP]),
    "gi_gbuffer_noalloc": (C.c_int, [_VP, _VP, C.c_int, _VP, C.c_int, F16, C.c_int, C.c_int, _VP, _VP, _VP]),
    "gi_vis_params_default": (C.c_int, [C.c_int, C.POINTER(VisParams)]),
    "gi_visibility": (C.c_int, [_VP, C.POINTER(VisParams), _VP, C.c_int, C.c_int, _VP, _VP, _VP,
                                C.c_int, C.c_int, _VP]),
    "gi_render_frame": (C.c_int, [_VP, _VP, C.POINTER(MapParams), F16, F16, C.POINTER(VisParams), C.c_int,
                                  C.c_int, _VP, _VP, _VP, _VP, _VP]),
    "gi_poisson_table": (C.c_int, [C.c_int, _VP]),
    "gi_soft_moment_map": (C.c_int, [_VP, C.POINTER(VisParams), _VP, C.c_int, C.c_int, _VP, _VP]),
    "gi_hierarchical_shadow_map": (C.c_int, [_VP, C.POINTER(VisParams), _VP, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_shadow_volume_counts": (C.c_int, [_VP, _VP, F3, C.c_float, F16, C.c_int, C.c_int, C.c_int,
                                          _VP, _VP, _VP]),
    "gi_shadow_volume_geometry": (C.c_int, [_VP, _VP, F3, C.c_float, _VP, _VP]),
    "gi_shadow_volume_counts_silhouette": (C.c_int, [_VP, _VP, F3, C.c_float, F16, C.c_int, C.c_int, C.c_int,
                                                     _VP, _VP, C.POINTER(C.c_int), _VP]),
    "gi_light_map_minmax": (C.c_int, [_VP, _VP, C.c_int, C.c_int, _VP, _VP]),
    "gi_context_set_tap_pyramid": (C.c_int, [_VP, C.c_int]),
    "gi_context_set_frame_graph": (C.c_int, [_VP, C.c_int]),
    "gi_phong_shade": (C.c_int, [_VP, C.POINTER(VisParams), _VP, _VP, _VP, _VP, C.c_int, C.c_int, _VP, _VP]),
    "gi_pba_voronoi": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_edt_soft_shadows": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                      C.c_float, _VP, _VP, _VP]),
    "gi_edt_mean_filter": (C.c_int, [_VP, C.POINTER(VisParams), _VP, _VP, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_pba_chain_rows": (C.c_int, [_VP, C.POINTER(C.c_uint32), C.c_int]),
    "gi_edt_inputs": (C.c_int, [_VP, C.POINTER(VisParams), F16, _VP, _VP, _VP, C.c_int, C.c_int, _VP, _VP, _VP]),
    "gi_area_light_samples": (C.c_int, [C.POINTER(View), C.c_float, C.c_int, _VP]),
    "gi_area_light_visibility": (C.c_int, [_VP, _VP, _VP, C.c_int, C.POINTER(MapParams), F16, C.c_float, C.c_int,
                                           C.c_int, _VP, _VP]),
    "gi_area_light_adaptive": (C.c_int, [_VP, _VP, C.POINTER(View), C.c_float, C.c_int, C.c_int, C.POINTER(MapParams),
                                         F16,
                                         C.c_float, C.c_int, C.c_int, _VP, _VP, _VP, C.POINTER(C.c_int), _VP]),
    "gi_batch_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "gi_batch_destroy": (None, [_VP]),
    "gi_batch_add_frame": (C.c_int, [_VP, _VP, C.POINTER(View), C.POINTER(View), C.POINTER(MapParams), C.c_int,
                                     C.POINTER(VisParams), _VP]),
    "gi_batch_build": (C.c_int, [_VP, C.c_int]),
    "gi_batch_run": (C.c_int, [_VP, _VP]),
    "gi_batch_autotune": (C.c_int, [_VP, _VP, C.c_int, C.POINTER(BatchTuning)]),
    "gi_batch_build_persistent": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int]),
    "gi_batch_autotune_persistent": (C.c_int, [_VP, _VP, C.c_int, C.POINTER(BatchTuning)]),
    "gi_batch_info": (C.c_int, [_VP, C.POINTER(BatchTuning)]),
    # gi_surrogate.h
    "gi_tc_set_wait_limit": (C.c_int, [C.c_uint32]),
    "gi_tc_wait_limit": (C.c_uint32, []),
    "gi_tc_set_test_withhold": (C.c_int, [C.c_int]),
    "gi_conv2d_bf16": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP, C.c_int, C.c_int, C.c_int, _VP,
                                 _VP, C.c_int, C.c_int, _VP, _VP, _VP]),
    "gi_conv2d_wgrad_scratch_floats": (C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "gi_conv2d_wgrad_bf16": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP,
                                       _VP, _VP, _VP]),
    "gi_pack_conv_weights": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_unpack_conv_grad": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_maxpool2_bf16": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_maxpool2_bwd_bf16": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_upsample2_bf16": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, C.c_int, C.c_int, _VP]),
    "gi_upsample2_bwd_bf16": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_channel_slice_bf16": (C.c_int, [_VP, C.c_size_t, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "gi_channel_slice_add_bf16": (C.c_int, [_VP, C.c_size_t, C.c_int, _VP, C.c_int, C.c_int, _VP]),
    "gi_surrogate_features": (C.c_int, [_VP, _VP, C.POINTER(MapParams), F16, F16, C.POINTER(VisParams), C.c_int,
                                        C.c_int, _VP, _VP, _VP]),
    "gi_surrogate_finish": (C.c_int, [_VP, _VP, C.c_int, C.c_int, _VP, F16, C.POINTER(VisParams), C.c_int, C.c_int,
                                      _VP, C.c_int, _VP, C.c_float, _VP, _VP, _VP]),
    "gi_conv2d_head_bf16": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP, C.c_int, C.c_int, _VP, _VP,
                                      _VP, _VP, _VP]),
    "gi_conv2d_fused_bf16": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP, C.c_int, C.c_int, _VP,
                                       C.c_int, C.c_int, _VP, C.c_int, _VP, _VP]),
    "gi_surrogate_loss": (C.c_int, [_VP, _VP, _VP, C.c_size_t, C.c_float, _VP, _VP, _VP]),
    "gi_adam_f32": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                              C.c_float, _VP]),
}

_lib = None


def load() -> C.CDLL:
    """Loads libgishadow.so (building is the caller's job: __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class GIError(RuntimeError):
    def __init__(self, status: int, where: str, text: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {text}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != GI_OK:
        raise GIError(status, where, load().gi_last_error_string().decode(errors="replace"))


def exported_symbols() -> list[str]:
    return list(_PROTOS)
