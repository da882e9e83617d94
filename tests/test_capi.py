"""The C ABI library loads, exports every symbol the header declares, and
reports argument errors through gi_status without touching a GPU."""
import ctypes as C
import os
import re

import pytest

from globalillumination_gb300 import _capi as api

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
HEADERS = [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE)) if f.endswith(".h")]


def header_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names.update(re.findall(r"\b(gi_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    fns = header_functions()
    for name in ("gi_shadow_map", "gi_gbuffer", "gi_visibility", "gi_shadow_volume_counts",
                 "gi_scene_load_config", "gi_frame_setup", "gi_context_create"):
        assert name in fns


def test_library_exports_every_declared_symbol():
    lib = api.load()
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_bindings_cover_header():
    assert set(header_functions()) == set(api.exported_symbols())


def test_struct_layouts():
    # the ctypes mirrors must match the C layout (checked through sizes)
    assert C.sizeof(api.VisParams) == 17 * 4 + 16 * 4 * 2 + 9 * 4 + 3 * 4
    assert C.sizeof(api.View) == 12 * 4 + 2 * 4
    assert C.sizeof(api.MapParams) == 6 * 4


def test_version_and_error_string():
    lib = api.load()
    assert lib.gi_version().startswith(b"gi_shadow")
    st = lib.gi_frame_setup(None, None, None)
    assert st == api.GI_ERR_INVALID_ARG
    assert b"NULL" in lib.gi_last_error_string()


def test_invalid_views_rejected():
    lib = api.load()
    bad = api.View(api.F3(0, 0, 0), api.F3(0, 0, 1), api.F3(0, 1, 0), 45.0, 0.0, 1000.0, 64, 64)
    P, V = api.F16(), api.F16()
    assert lib.gi_view_matrices(C.byref(bad), P, V) == api.GI_ERR_INVALID_ARG
    bad.znear, bad.width = 1.0, 0
    assert lib.gi_view_matrices(C.byref(bad), P, V) == api.GI_ERR_INVALID_ARG
    bad.width, bad.fovy_deg = 64, 180.0
    assert lib.gi_view_matrices(C.byref(bad), P, V) == api.GI_ERR_INVALID_ARG


def test_pass_argument_checks_before_device_work():
    lib = api.load()
    p = api.VisParams()
    assert lib.gi_vis_params_default(api.GI_TECH_PCF, C.byref(p)) == api.GI_OK
    assert lib.gi_vis_params_default(99, C.byref(p)) == api.GI_ERR_INVALID_ARG
    # NULL context / buffers
    assert lib.gi_visibility(None, C.byref(p), None, 4, 4, None, None, None, 4, 4, None) == api.GI_ERR_INVALID_ARG
    assert lib.gi_shadow_map(None, None, None, api.F16(), None, None) == api.GI_ERR_INVALID_ARG
    assert lib.gi_gbuffer(None, None, api.F16(), 4, 4, None, None, None) == api.GI_ERR_INVALID_ARG
    # context switches reject a NULL context
    assert lib.gi_context_set_frame_graph(None, 1) == api.GI_ERR_INVALID_ARG
    assert lib.gi_context_set_tap_pyramid(None, 1) == api.GI_ERR_INVALID_ARG
    assert lib.gi_context_set_tuning(None, 96, 1024) == api.GI_ERR_INVALID_ARG


def test_poisson_table():
    lib = api.load()
    import numpy as np

    t = np.empty(128, np.float32)
    assert lib.gi_poisson_table(64, t.ctypes.data) == api.GI_OK
    xy = t.reshape(64, 2)
    r = np.hypot(xy[:, 0], xy[:, 1])
    assert (r <= 1.0).all()
    d = np.hypot(xy[:, None, 0] - xy[None, :, 0], xy[:, None, 1] - xy[None, :, 1]) + np.eye(64) * 9
    assert d[:16, :16].min() > 0.3  # the 16-tap prefix is well spread
    assert lib.gi_poisson_table(65, t.ctypes.data) == api.GI_ERR_INVALID_ARG
    assert lib.gi_poisson_table(0, t.ctypes.data) == api.GI_ERR_INVALID_ARG


def test_context_without_device_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = api.load()
    h = C.c_void_p()
    assert lib.gi_context_create(0, C.byref(h)) == api.GI_ERR_CUDA
    assert lib.gi_last_error_string()


def test_batch_argument_checks():
    lib = api.load()
    assert lib.gi_batch_create(0, None) == api.GI_ERR_INVALID_ARG
    assert lib.gi_batch_build(None, 4) == api.GI_ERR_INVALID_ARG
    assert lib.gi_batch_run(None, None) == api.GI_ERR_INVALID_ARG
    assert lib.gi_batch_add_frame(None, None, None, None, None, 1, None, None) == api.GI_ERR_INVALID_ARG
    assert lib.gi_batch_info(None, None) == api.GI_ERR_INVALID_ARG
    assert C.sizeof(api.BatchTuning) == 4 * 4 + 8 + 4 + 3 * 4 + 4 + 4  # + padding to 8


def test_training_helpers_reject_bad_shapes_before_device_work():
    """Every call below breaks a host-side shape check, so none launches a
    kernel (the dummy pointers are never dereferenced)."""
    lib = api.load()
    P = C.c_void_p(256)
    bad = api.GI_ERR_INVALID_ARG
    # max-pool: negative or empty batch / image, odd sizes, no channels
    assert lib.gi_maxpool2_bf16(P, -1, -2, 4, 8, P, None) == bad
    assert lib.gi_maxpool2_bf16(P, 1, 0, 4, 8, P, None) == bad
    assert lib.gi_maxpool2_bf16(P, 1, 3, 4, 8, P, None) == bad
    assert lib.gi_maxpool2_bf16(P, 1, 4, 4, 0, P, None) == bad
    assert lib.gi_maxpool2_bwd_bf16(P, P, P, -1, -2, 4, 8, P, None) == bad
    assert lib.gi_maxpool2_bwd_bf16(P, P, P, 1, 4, 4, -8, P, None) == bad
    # upsampling and its gradient: negative sizes, offsets outside the stride
    assert lib.gi_upsample2_bf16(P, -1, -4, 4, 8, P, 8, 0, None) == bad
    assert lib.gi_upsample2_bf16(P, 1, 4, 4, 0, P, 8, 0, None) == bad
    assert lib.gi_upsample2_bf16(P, 1, 4, 4, 8, P, 16, -8, None) == bad
    assert lib.gi_upsample2_bwd_bf16(P, -1, -4, 4, 8, 8, 0, P, None) == bad
    assert lib.gi_upsample2_bwd_bf16(P, 1, 4, 4, 8, 16, -8, P, None) == bad
    assert lib.gi_upsample2_bwd_bf16(P, 1, 4, 4, 0, 16, 0, P, None) == bad
    # channel slices
    assert lib.gi_channel_slice_bf16(P, 16, 16, -8, 8, P, None) == bad
    assert lib.gi_channel_slice_bf16(P, 16, 16, 0, 0, P, None) == bad
    assert lib.gi_channel_slice_add_bf16(P, 16, 8, P, 16, -8, None) == bad
    assert lib.gi_channel_slice_add_bf16(P, 16, 0, P, 16, 0, None) == bad
    # weight (un)packing with negative sizes
    assert lib.gi_unpack_conv_grad(P, -1, -1, 8, 3, P, None) == bad
    assert lib.gi_pack_conv_weights(P, -1, 1, 8, 3, 0, P, None) == bad


def test_shadow_params_to_c_follows_field_changes():
    """ShadowParams.to_c caches the scalar part of the C struct per set of
    field values: every change, down to a zero's sign, reaches the struct."""
    import math

    import numpy as np

    from globalillumination_gb300.shadow import Frame, ShadowParams

    p = ShadowParams.defaults(api.GI_TECH_PCSS_POISSON)
    first = bytes(p.to_c(None))
    assert bytes(p.to_c(None)) == first
    p.light_radius = 0.25
    assert p.to_c(None).light_radius == 0.25 and bytes(p.to_c(None)) != first
    p.depth_threshold = 0.0
    plus = bytes(p.to_c(None))
    p.depth_threshold = -0.0
    assert bytes(p.to_c(None)) != plus
    assert math.copysign(1.0, p.to_c(None).depth_threshold) == -1.0
    p.technique = api.GI_TECH_PCF
    assert p.to_c(None).technique == api.GI_TECH_PCF
    m = np.arange(16, dtype=np.float32)
    fr = Frame(m, m + 1, m + 2, m + 3, m[:9] + 4, m[:3] + 5)
    c = p.to_c(fr)
    assert list(c.light_mvp_biased) == list(m + 1) and list(c.light_position) == list(m[:3] + 5)
    assert list(c.normal_matrix) == list(m[:9] + 4) and list(c.camera_mv) == list(m + 3)
