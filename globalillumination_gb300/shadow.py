"""Host-side mirror of the reference's shadow technique interface.

The reference drives its passes from GLUT callbacks
(ShadowMapping/src/main.cpp:459-472 display(), SoftShadowMapping/src/main.cpp
:925-1022 renderSoftShadows(), ShadowVolumes/src/main.cpp:120-206) and keeps
the technique choice in a ShadowParams struct
(ShadowMapping/include/Viewers/ShadowParams.h:6-37,
SoftShadowMapping/include/Viewers/ShadowParams.h:6-69) set from menus.  This
module keeps those names and meanings on top of the C ABI of libgishadow.so:

  Scene                 SceneLoader + Mesh (Configs/<name>.txt and OBJ files)
  ShadowParams          the parameter block, with the technique as an enum
  render_shadow_map     renderShadowMap / displaySceneFromLightPOV
  render_gbuffer        renderGBuffer
  compute_hard_shadows  computeHardShadows (visibility into a float buffer)
  render_soft_shadows   renderSoftShadows (G-buffer, light map, PCSS)
  shadow_volume_counts  the ShadowVolumes stencil passes

Device buffers are torch CUDA tensors (torch provides memory and streams
only; all the work runs in the library's own kernels).  Every call raises
GIError on failure; nothing falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np

from . import _capi as api
from ._capi import check


def _lib():
    return api.load()


def _f3(v) -> api.F3:
    return api.F3(*[float(x) for x in v])


def _f16(m) -> api.F16:
    a = np.ascontiguousarray(m, dtype=np.float32).reshape(-1)
    if a.size != 16:
        raise ValueError("a 4x4 matrix needs 16 values")
    return api.F16.from_buffer_copy(a)


def _stream_ptr(stream) -> C.c_void_p:
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return C.c_void_p(int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream))


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(int(t.data_ptr()))


def debug_fail_allocation(countdown: int) -> None:
    """Test hook: let `countdown` more allocations succeed and fail the next (-1: off)."""
    check(_lib().gi_debug_fail_allocation(int(countdown)), "gi_debug_fail_allocation")


class Context:
    """Owns the scratch memory of the passes on one CUDA device."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(_lib().gi_context_create(int(device), C.byref(h)), "gi_context_create")
        self.handle = h
        self.device = int(device)

    @property
    def launch_count(self) -> int:
        return int(_lib().gi_context_launch_count(self.handle))

    def set_tuning(self, tiny_px: int, coop_px: int) -> None:
        """Rasteriser tier thresholds (results do not depend on them)."""
        check(_lib().gi_context_set_tuning(self.handle, int(tiny_px), int(coop_px)), "gi_context_set_tuning")

    def set_tap_pyramid(self, enable: bool) -> None:
        """Build the light map's min-max pyramid for exact tap skipping of larger boxes."""
        check(_lib().gi_context_set_tap_pyramid(self.handle, 1 if enable else 0), "gi_context_set_tap_pyramid")

    def set_frame_graph(self, enable: bool) -> None:
        """Replay repeated render_frame calls (same arguments) as one captured CUDA graph."""
        check(_lib().gi_context_set_frame_graph(self.handle, 1 if enable else 0), "gi_context_set_frame_graph")

    def set_profiling(self, enable: bool) -> None:
        check(_lib().gi_context_set_profiling(self.handle, int(bool(enable))), "gi_context_set_profiling")

    def phase_ms(self):
        """(light map, visibility keys, resolve + visibility) of the last render_frame, in ms."""
        out = (C.c_float * 3)()
        check(_lib().gi_context_phase_ms(self.handle, out), "gi_context_phase_ms")
        return tuple(float(v) for v in out)

    def close(self) -> None:
        if self.handle:
            _lib().gi_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """Scene geometry with the SceneLoader / Mesh semantics of the reference."""

    def __init__(self, handle: C.c_void_p | None = None):
        if handle is None:
            handle = C.c_void_p()
            check(_lib().gi_scene_create(C.byref(handle)), "gi_scene_create")
        self.handle = handle

    @classmethod
    def from_config(cls, cfg_path: str, base_dir: str | None = None) -> "Scene":
        h = C.c_void_p()
        check(_lib().gi_scene_load_config(cfg_path.encode(), base_dir.encode() if base_dir else None,
                                          C.byref(h)), "gi_scene_load_config")
        return cls(h)

    # config keys o / s / t / r / +
    def load_obj(self, path: str) -> "Scene":
        check(_lib().gi_scene_object_load_obj(self.handle, path.encode()), "load_obj")
        return self

    def object_from_arrays(self, points, indices) -> "Scene":
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1)
        i = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1)
        check(_lib().gi_scene_object_from_arrays(self.handle, p.ctypes.data, p.size // 3, i.ctypes.data,
                                                 i.size // 3), "object_from_arrays")
        return self

    def scale(self, x, y, z) -> "Scene":
        check(_lib().gi_scene_object_scale(self.handle, x, y, z), "scale")
        return self

    def translate(self, x, y, z) -> "Scene":
        check(_lib().gi_scene_object_translate(self.handle, x, y, z), "translate")
        return self

    def rotate(self, x, y, z) -> "Scene":
        check(_lib().gi_scene_object_rotate(self.handle, x, y, z), "rotate")
        return self

    def commit(self) -> "Scene":
        check(_lib().gi_scene_object_commit(self.handle), "commit")
        return self

    # procedural objects
    def ground(self, half_size: float, y: float = 0.0) -> "Scene":
        check(_lib().gi_gen_ground(self.handle, half_size, y), "gi_gen_ground")
        return self.commit()

    def uv_sphere(self, slices: int, stacks: int, radius: float, centre) -> "Scene":
        check(_lib().gi_gen_uv_sphere(self.handle, slices, stacks, radius, _f3(centre)), "gi_gen_uv_sphere")
        return self.commit()

    def icosphere(self, level: int, radius: float, centre) -> "Scene":
        check(_lib().gi_gen_icosphere(self.handle, level, radius, _f3(centre)), "gi_gen_icosphere")
        return self.commit()

    def displaced_sphere(self, slices: int, stacks: int, radius: float, amplitude: float, centre,
                         seed: int) -> "Scene":
        check(_lib().gi_gen_displaced_sphere(self.handle, slices, stacks, radius, amplitude, _f3(centre),
                                             int(seed)), "gi_gen_displaced_sphere")
        return self.commit()

    def icosphere_field(self, count: int, level: int, lo, hi, rmin: float, rmax: float,
                        seed: int) -> "Scene":
        check(_lib().gi_gen_icosphere_field(self.handle, count, level, _f3(lo), _f3(hi), rmin, rmax,
                                            int(seed)), "gi_gen_icosphere_field")
        return self

    def set_views(self, camera_eye, camera_at, light_eye, light_at, depth_threshold=0.0) -> "Scene":
        check(_lib().gi_scene_set_views(self.handle, _f3(camera_eye), _f3(camera_at), _f3(light_eye),
                                        _f3(light_at), float(depth_threshold)), "gi_scene_set_views")
        return self

    def info(self) -> api.SceneInfo:
        out = api.SceneInfo()
        check(_lib().gi_scene_get_info(self.handle, C.byref(out)), "gi_scene_get_info")
        return out

    def arrays(self):
        """(points float32[V,3], normals float32[V,3], indices int32[T,3])."""
        inf = self.info()
        p = np.empty((inf.num_vertices, 3), np.float32)
        n = np.empty((inf.num_vertices, 3), np.float32)
        i = np.empty((inf.num_triangles, 3), np.int32)
        check(_lib().gi_scene_get_arrays(self.handle, p.ctypes.data, n.ctypes.data, i.ctypes.data),
              "gi_scene_get_arrays")
        return p, n, i

    def upload(self, ctx: Context, stream=None) -> "Scene":
        check(_lib().gi_scene_upload(self.handle, ctx.handle, _stream_ptr(stream)), "gi_scene_upload")
        return self

    def upload_from(self, ctx: Context, points_ptr: int, normals_ptr: int, num_vertices: int,
                    indices_ptr: int, num_triangles: int, stream=None) -> "Scene":
        """Replaces the device geometry with caller-owned host arrays (pinned for async copies)."""
        check(_lib().gi_scene_upload_from(self.handle, ctx.handle, C.c_void_p(points_ptr), C.c_void_p(normals_ptr),
                                          int(num_vertices), C.c_void_p(indices_ptr), int(num_triangles),
                                          _stream_ptr(stream)), "gi_scene_upload_from")
        return self

    def close(self) -> None:
        if self.handle:
            _lib().gi_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class ViewSpec:
    """Eye / look / up plus the projection configureAmbient builds."""
    eye: tuple
    at: tuple
    width: int
    height: int
    fovy_deg: float = 45.0
    znear: float = 1.0
    zfar: float = 1000.0
    up: tuple = (0.0, 0.0, 1.0)

    def to_c(self) -> api.View:
        return api.View(_f3(self.eye), _f3(self.at), _f3(self.up), self.fovy_deg, self.znear, self.zfar,
                        int(self.width), int(self.height))


@dataclass
class Frame:
    light_mvp: np.ndarray
    light_mvp_biased: np.ndarray
    camera_mvp: np.ndarray
    camera_mv: np.ndarray
    normal_matrix: np.ndarray
    light_position: np.ndarray


def frame_setup(light: ViewSpec, camera: ViewSpec) -> Frame:
    out = api.FrameMatrices()
    lv, cv = light.to_c(), camera.to_c()
    check(_lib().gi_frame_setup(C.byref(lv), C.byref(cv), C.byref(out)), "gi_frame_setup")
    f = lambda a, n: np.frombuffer(bytes(a), dtype=np.float32, count=n).copy()
    return Frame(f(out.light_mvp, 16), f(out.light_mvp_biased, 16), f(out.camera_mvp, 16),
                 f(out.camera_mv, 16), f(out.normal_matrix, 9), f(out.light_position, 3))


@dataclass
class MapParams:
    width: int
    height: int
    bias_mode: int = api.GI_BIAS_POLYGON_OFFSET
    constant_bias: float = 0.0
    offset_factor: float = 4.0
    offset_units: float = 20.0

    def to_c(self) -> api.MapParams:
        return api.MapParams(self.width, self.height, self.bias_mode, self.constant_bias,
                             self.offset_factor, self.offset_units)


TECHNIQUES = {
    "hard": api.GI_TECH_HARD,
    "pcf": api.GI_TECH_PCF,
    "pcf_tricubic": api.GI_TECH_PCF_TRICUBIC,
    "pcss_grid": api.GI_TECH_PCSS_GRID,
    "pcss_poisson": api.GI_TECH_PCSS_POISSON,
    "smsr_conservative": api.GI_TECH_SMSR_CONSERVATIVE,
    "smsr_nonconservative": api.GI_TECH_SMSR_NONCONSERVATIVE,
    "rpcf_conservative": api.GI_TECH_RPCF_CONSERVATIVE,
    "rpcf_smsr": api.GI_TECH_RPCF_SMSR,
    "rsmss": api.GI_TECH_RSMSS,
    "hard_softapp": api.GI_TECH_HARD_SOFTAPP,
    "rbssm": api.GI_TECH_RBSSM,
    "vsm": api.GI_TECH_VSM,
    "esm": api.GI_TECH_ESM,
    "evsm": api.GI_TECH_EVSM,
    "msm": api.GI_TECH_MSM,
    "savsm": api.GI_TECH_SAVSM,
    "vssm": api.GI_TECH_VSSM,
    "essm": api.GI_TECH_ESSM,
    "mssm": api.GI_TECH_MSSM,
}


# ShadowParams.to_c's cache key: the scalar fields in declaration order
# (integers as int64, reals as float64, the SAT switch as a bool).
_SCALAR_KEY = struct.Struct("<qqdqqqdqqdddqq?dd")


@dataclass
class ShadowParams:
    """ShadowParams of the reference with the technique as one enum value."""
    technique: int = api.GI_TECH_HARD
    shadow_intensity: float = 0.25
    kernel_order: int = 7
    penumbra_size: int = 1
    max_search: int = 16
    depth_threshold: float = 0.0
    blocker_search_size: int = 7
    kernel_size: int = 15
    light_radius: float = 8.0
    znear: float = 1.0
    pcss_min_blocker_depth: float = 0.99
    poisson_blocker_taps: int = 16
    poisson_filter_taps: int = 32
    summed_area_table: bool = False
    hsm_alpha: float = 0.0
    hsm_beta: float = 0.0
    pretest: int = api.GI_PRETEST_REFERENCE

    @classmethod
    def defaults(cls, technique: int) -> "ShadowParams":
        p = api.VisParams()
        check(_lib().gi_vis_params_default(int(technique), C.byref(p)), "gi_vis_params_default")
        return cls(technique=p.technique, shadow_intensity=p.shadow_intensity, kernel_order=p.kernel_order,
                   penumbra_size=p.penumbra_size, max_search=p.max_search, depth_threshold=p.depth_threshold,
                   blocker_search_size=p.blocker_search_size, kernel_size=p.kernel_size,
                   light_radius=p.light_radius, znear=p.znear, pcss_min_blocker_depth=p.pcss_min_blocker_depth,
                   poisson_blocker_taps=p.poisson_blocker_taps, poisson_filter_taps=p.poisson_filter_taps,
                   summed_area_table=bool(p.summed_area_table), hsm_alpha=p.hsm_alpha, hsm_beta=p.hsm_beta,
                   pretest=p.pretest)

    def to_c(self, frame: Frame) -> api.VisParams:
        # The scalar part is built once per set of field values (fields may
        # change between calls) and copied; the frame's matrices are copied
        # straight from their float32 buffers.
        # The key is the fields' bytes, so values that compare equal in
        # Python but differ in bits (-0.0 and 0.0) get their own struct.
        key = _SCALAR_KEY.pack(
            self.technique, self.pretest, self.shadow_intensity, self.kernel_order, self.penumbra_size,
            self.max_search, self.depth_threshold, self.blocker_search_size, self.kernel_size,
            self.light_radius, self.znear, self.pcss_min_blocker_depth, self.poisson_blocker_taps,
            self.poisson_filter_taps, self.summed_area_table, self.hsm_alpha, self.hsm_beta)
        cached = self.__dict__.get("_c_scalars")
        if cached is None or cached[0] != key:
            cached = (key, bytes(self._scalars_to_c()))
            self.__dict__["_c_scalars"] = cached
        p = api.VisParams.from_buffer_copy(cached[1])
        if frame is not None:  # the light-side maps need no matrices
            for dst, src, n in ((p.light_mvp_biased, frame.light_mvp_biased, 64), (p.camera_mv, frame.camera_mv, 64),
                                (p.normal_matrix, frame.normal_matrix, 36), (p.light_position, frame.light_position, 12)):
                b = (src if src.dtype == np.float32 else src.astype(np.float32)).tobytes()
                if len(b) != n:
                    raise ValueError("frame matrix of the wrong size")
                C.memmove(dst, b, n)
        return p

    def _scalars_to_c(self) -> api.VisParams:
        p = api.VisParams()
        p.technique = int(self.technique)
        p.pretest = int(self.pretest)
        p.shadow_intensity = self.shadow_intensity
        p.kernel_order = self.kernel_order
        p.penumbra_size = self.penumbra_size
        p.max_search = self.max_search
        p.depth_threshold = self.depth_threshold
        p.blocker_search_size = self.blocker_search_size
        p.kernel_size = self.kernel_size
        p.light_radius = self.light_radius
        p.znear = self.znear
        p.pcss_min_blocker_depth = self.pcss_min_blocker_depth
        p.poisson_blocker_taps = self.poisson_blocker_taps
        p.poisson_filter_taps = self.poisson_filter_taps
        p.summed_area_table = 1 if self.summed_area_table else 0
        p.hsm_alpha = self.hsm_alpha
        p.hsm_beta = self.hsm_beta
        return p


def poisson_table(n: int) -> np.ndarray:
    out = np.empty((n, 2), np.float32)
    check(_lib().gi_poisson_table(int(n), out.ctypes.data), "gi_poisson_table")
    return out


# ---------------------------------------------------------------------------
# Passes (device tensors in, device tensors out; stream-ordered)
# ---------------------------------------------------------------------------
def render_shadow_map(ctx: Context, scene: Scene, mp: MapParams, light_mvp, depth, stream=None):
    """renderShadowMap: depth is a float32 CUDA tensor of mp.height * mp.width."""
    assert depth.is_cuda and depth.dtype.itemsize == 4 and depth.numel() >= mp.width * mp.height
    c = mp.to_c()
    check(_lib().gi_shadow_map(ctx.handle, scene.handle, C.byref(c), _f16(light_mvp), _ptr(depth),
                               _stream_ptr(stream)), "gi_shadow_map")
    return depth


def render_gbuffer(ctx: Context, scene: Scene, camera_mvp, width: int, height: int, pos, nrm, stream=None):
    """renderGBuffer: pos / nrm are float32 CUDA tensors of height * width * 4."""
    n = width * height * 4
    assert pos.is_cuda and nrm.is_cuda and pos.numel() >= n and nrm.numel() >= n
    check(_lib().gi_gbuffer(ctx.handle, scene.handle, _f16(camera_mvp), width, height, _ptr(pos), _ptr(nrm),
                            _stream_ptr(stream)), "gi_gbuffer")
    return pos, nrm


def compute_visibility(ctx: Context, params: ShadowParams, frame: Frame, depth, map_w: int, map_h: int,
                       pos, nrm, vis, width: int, height: int, stream=None):
    """computeHardShadows / the soft visibility pass: vis is float32[height * width]."""
    assert vis.is_cuda and vis.numel() >= width * height
    p = params.to_c(frame)
    check(_lib().gi_visibility(ctx.handle, C.byref(p), _ptr(depth), map_w, map_h, _ptr(pos), _ptr(nrm),
                               _ptr(vis), width, height, _stream_ptr(stream)), "gi_visibility")
    return vis


compute_hard_shadows = compute_visibility


def soft_moment_map(ctx: Context, params: ShadowParams, depth, map_w: int, map_h: int, out, stream=None):
    """The light-side map of a moment soft-shadow technique (SAVSM..MSSM): the moment map, or its
    summed-area table when params.summed_area_table is set; out is float32[map_h * map_w * 4]."""
    assert out.is_cuda and out.numel() >= map_w * map_h * 4
    p = params.to_c(None)
    check(_lib().gi_soft_moment_map(ctx.handle, C.byref(p), _ptr(depth), map_w, map_h, _ptr(out),
                                    _stream_ptr(stream)), "gi_soft_moment_map")
    return out


def hierarchical_shadow_map(ctx: Context, params: ShadowParams, depth, map_w: int, map_h: int, level: int, out,
                            stream=None):
    """Level `level` of renderHSM's min-max map: out is float32[(map_h >> level) * (map_w >> level) * 2]."""
    assert out.is_cuda and out.numel() >= (map_w >> level) * (map_h >> level) * 2
    p = params.to_c(None)
    check(_lib().gi_hierarchical_shadow_map(ctx.handle, C.byref(p), _ptr(depth), map_w, map_h, int(level),
                                            _ptr(out), _stream_ptr(stream)), "gi_hierarchical_shadow_map")
    return out


def shadow_volume_counts(ctx: Context, scene: Scene, light_pos, camera_mvp, width: int, height: int,
                         stencil, depth=None, depth_func: int = api.GI_DEPTH_LEQUAL, infinity: float = 100.0,
                         stream=None):
    """The ShadowVolumes stencil passes: stencil is a uint8 CUDA tensor of height * width."""
    assert stencil.is_cuda and stencil.numel() >= width * height
    check(_lib().gi_shadow_volume_counts(ctx.handle, scene.handle, _f3(light_pos), float(infinity),
                                         _f16(camera_mvp), width, height, int(depth_func), _ptr(stencil),
                                         _ptr(depth) if depth is not None else None, _stream_ptr(stream)),
          "gi_shadow_volume_counts")
    return stencil


def shadow_volume_counts_silhouette(ctx: Context, scene: Scene, light_pos, camera_mvp, width: int, height: int,
                                    stencil, depth=None, depth_func: int = api.GI_DEPTH_LEQUAL,
                                    infinity: float = 100.0, stream=None) -> int:
    """The stencil passes with silhouette extraction (opt-in, see gi_shadow.h): fills stencil
    and returns the number of volume triangles drawn."""
    assert stencil.is_cuda and stencil.numel() >= width * height
    drawn = C.c_int(0)
    check(_lib().gi_shadow_volume_counts_silhouette(ctx.handle, scene.handle, _f3(light_pos), float(infinity),
                                                    _f16(camera_mvp), width, height, int(depth_func), _ptr(stencil),
                                                    _ptr(depth) if depth is not None else None, C.byref(drawn),
                                                    _stream_ptr(stream)), "gi_shadow_volume_counts_silhouette")
    return drawn.value


def shadow_volume_geometry(ctx: Context, scene: Scene, light_pos, out, infinity: float = 100.0, stream=None):
    """ShadowVolume::build's triangles as the stencil pass draws them: out is a float32
    CUDA tensor of 6T * 9 values (entry 6t + k = side k of triangle t, three vertices)."""
    nt = scene.info().num_triangles
    assert out.is_cuda and out.dtype.is_floating_point and out.numel() >= 6 * nt * 9
    check(_lib().gi_shadow_volume_geometry(ctx.handle, scene.handle, _f3(light_pos), float(infinity), _ptr(out),
                                           _stream_ptr(stream)), "gi_shadow_volume_geometry")
    return out


def light_map_minmax(ctx: Context, depth, width: int, height: int, stream=None) -> list:
    """The light map's min-max pyramid (levels 1..6) as a list of float32 CUDA tensors
    [(height >> L), (width >> L), 2] holding (min, max) per 2^L x 2^L block."""
    import torch

    sizes = [(height >> L, width >> L) for L in range(1, 7)]
    out = torch.empty(sum(h * w for h, w in sizes) * 2, dtype=torch.float32, device=depth.device)
    check(_lib().gi_light_map_minmax(ctx.handle, _ptr(depth), int(width), int(height), _ptr(out), _stream_ptr(stream)),
          "gi_light_map_minmax")
    levels, off = [], 0
    for h, w in sizes:
        levels.append(out[off:off + h * w * 2].view(h, w, 2))
        off += h * w * 2
    return levels


@dataclass
class FrameBuffers:
    depth: object
    pos: object
    nrm: object
    vis: object


def allocate_frame(map_w: int, map_h: int, width: int, height: int, device: int = 0) -> FrameBuffers:
    import torch
    dev = torch.device("cuda", device)
    return FrameBuffers(
        depth=torch.empty(map_h * map_w, dtype=torch.float32, device=dev),
        pos=torch.empty(height * width * 4, dtype=torch.float32, device=dev),
        nrm=torch.empty(height * width * 4, dtype=torch.float32, device=dev),
        vis=torch.empty(height * width, dtype=torch.float32, device=dev),
    )


def render_frame(ctx: Context, scene: Scene, frame: Frame, mp: MapParams, params: ShadowParams, width: int,
                 height: int, bufs: FrameBuffers, stream=None, store_gbuffer: bool = False):
    """One shadowed frame (display() up to the visibility target) through gi_render_frame.

    The G-buffer is resolved and shaded in one kernel; it is written to
    bufs.pos / bufs.nrm only when store_gbuffer is true.
    """
    c = mp.to_c()
    p = params.to_c(frame)
    pos = _ptr(bufs.pos) if store_gbuffer else None
    nrm = _ptr(bufs.nrm) if store_gbuffer else None
    check(_lib().gi_render_frame(ctx.handle, scene.handle, C.byref(c), _f16(frame.light_mvp), _f16(frame.camera_mvp),
                                 C.byref(p), width, height, _ptr(bufs.depth), _ptr(bufs.vis), pos, nrm,
                                 _stream_ptr(stream)), "gi_render_frame")
    return bufs.vis


def render_frame_passes(ctx: Context, scene: Scene, frame: Frame, mp: MapParams, params: ShadowParams,
                        width: int, height: int, bufs: FrameBuffers, stream=None):
    """The same frame as three separate passes (light map, G-buffer, visibility)."""
    render_shadow_map(ctx, scene, mp, frame.light_mvp, bufs.depth, stream)
    render_gbuffer(ctx, scene, frame.camera_mvp, width, height, bufs.pos, bufs.nrm, stream)
    compute_visibility(ctx, params, frame, bufs.depth, mp.width, mp.height, bufs.pos, bufs.nrm, bufs.vis,
                       width, height, stream)
    return bufs.vis


render_soft_shadows = render_frame


def phong_shade(ctx: Context, params: ShadowParams, frame: Frame, pos, nrm, vis, width: int, height: int, out,
                color=None, stream=None):
    """shadeScene: deferred Phong of the G-buffer with vis as shadow term; out is float4 per pixel."""
    assert out.is_cuda and out.numel() >= 4 * width * height
    p = params.to_c(frame)
    check(_lib().gi_phong_shade(ctx.handle, C.byref(p), _ptr(pos), _ptr(nrm), _ptr(vis),
                                _ptr(color) if color is not None else None, width, height, _ptr(out),
                                _stream_ptr(stream)), "gi_phong_shade")
    return out


def _need(t, numel: int, dtype, what: str) -> None:
    if not t.is_cuda or t.dtype != dtype or not t.is_contiguous() or t.numel() < numel:
        raise ValueError(f"{what}: need a contiguous CUDA {dtype} tensor of >= {numel} elements")


def pba_voronoi(ctx: Context, sites, nearest, bands=(16, 16, 16), stream=None):
    """pba2DVoronoiDiagram: nearest site of every pixel (int16 [H, W, 2] in and out).

    A site is any pixel whose x is not GI_PBA_MARKER; bands are PBA's
    (phase1Band, phase2Band, phase3Band), (16, 16, 16) in the reference.
    """
    import torch

    H, W = sites.shape[0], sites.shape[1]
    _need(sites, 2 * W * H, torch.int16, "sites")
    _need(nearest, 2 * W * H, torch.int16, "nearest")
    check(_lib().gi_pba_voronoi(ctx.handle, _ptr(sites), W, H, int(bands[0]), int(bands[1]), int(bands[2]),
                                _ptr(nearest), _stream_ptr(stream)), "gi_pba_voronoi")
    return nearest


def pba_chain_rows(ctx: Context, reset: bool = False) -> int:
    """Rows colored by replaying the reference's group chain (lists that are not strict envelopes)."""
    n = C.c_uint32(0)
    check(_lib().gi_pba_chain_rows(ctx.handle, C.byref(n), 1 if reset else 0), "gi_pba_chain_rows")
    return int(n.value)


def edt_mean_filter(ctx: Context, params: ShadowParams, frame: Frame, image, pos, out, width: int, height: int,
                    order: int = 7, stream=None):
    """MeanFilter.frag's x and y passes over the EDT image (float4) into out (float4)."""
    import torch

    for t, what in ((image, "image"), (pos, "pos"), (out, "out")):
        _need(t, 4 * width * height, torch.float32, what)
    p = params.to_c(frame)
    check(_lib().gi_edt_mean_filter(ctx.handle, C.byref(p), _ptr(image), _ptr(pos), width, height, int(order),
                                    _ptr(out), _stream_ptr(stream)), "gi_edt_mean_filter")
    return out


def edt_inputs(ctx: Context, params: ShadowParams, frame: Frame, pos, nrm, vis, width: int, height: int, image,
               position, stream=None):
    """The SMSR shaders' EDTSM outputs: hard-shadow image and clip position (float4 each)."""
    import torch

    for t, n, what in ((pos, 4, "pos"), (nrm, 4, "nrm"), (vis, 1, "vis"), (image, 4, "image"),
                       (position, 4, "position")):
        _need(t, n * width * height, torch.float32, what)
    p = params.to_c(frame)
    check(_lib().gi_edt_inputs(ctx.handle, C.byref(p), _f16(frame.camera_mvp), _ptr(pos), _ptr(nrm), _ptr(vis),
                               width, height, _ptr(image), _ptr(position), _stream_ptr(stream)), "gi_edt_inputs")
    return image, position


def edt_soft_shadows(ctx: Context, image, position, out, penumbra_size: float = 1.0, shadow_intensity: float = 0.25,
                     bands=(16, 16, 16), nearest=None, stream=None):
    """filterHardShadowsUsingEDT's CUDA part: sites, PBA, normalisation into out (float4, channels 0-1).

    penumbra_size is shadowParams.penumbraSize; like the reference, the
    kernels get penumbra_size / 5.
    """
    import torch

    H, W = image.shape[0], image.shape[1]
    for t, what in ((image, "image"), (position, "position"), (out, "out")):
        _need(t, 4 * W * H, torch.float32, what)
    if nearest is not None:
        _need(nearest, 2 * W * H, torch.int16, "nearest")
    check(_lib().gi_edt_soft_shadows(ctx.handle, _ptr(image), _ptr(position), W, H, int(bands[0]), int(bands[1]),
                                     int(bands[2]), float(penumbra_size / 5.0), float(shadow_intensity), _ptr(out),
                                     _ptr(nearest) if nearest is not None else None, _stream_ptr(stream)),
          "gi_edt_soft_shadows")
    return out


def area_light_samples(light: ViewSpec, size: float, n_side: int = 17) -> list:
    """The reference's uniform point-light samples of an area light (n_side^2 views)."""
    n = n_side * n_side
    out = (api.View * n)()
    lv = light.to_c()
    check(_lib().gi_area_light_samples(C.byref(lv), float(size), int(n_side), out), "gi_area_light_samples")
    views = []
    for v in out:
        views.append(ViewSpec(eye=tuple(v.eye), at=tuple(v.at), width=v.width, height=v.height, fovy_deg=v.fovy_deg,
                              znear=v.znear, zfar=v.zfar, up=tuple(v.up)))
    return views


def area_light_visibility(ctx: Context, scene: Scene, samples, mp: MapParams, camera_mvp, intensity: float,
                          width: int, height: int, vis, stream=None):
    """Monte-Carlo area-light ground truth (renderMonteCarlo + AccurateSoftShadow.frag)."""
    assert vis.is_cuda and vis.numel() >= width * height
    arr = (api.View * len(samples))(*[v.to_c() for v in samples])
    c = mp.to_c()
    check(_lib().gi_area_light_visibility(ctx.handle, scene.handle, arr, len(samples), C.byref(c), _f16(camera_mvp),
                                          float(intensity), width, height, _ptr(vis), _stream_ptr(stream)),
          "gi_area_light_visibility")
    return vis


def area_light_adaptive(ctx: Context, scene: Scene, light: ViewSpec, size: float, mp: MapParams, camera_mvp,
                        intensity: float, width: int, height: int, vis, max_level: int = 4,
                        lower_accuracy: bool = False, stream=None):
    """Adaptive (quad-tree) area-light ground truth (SoftShadowMapping adaptiveSampling).

    Returns (vis, samples, levels): the sample views in the order the final pass sums them and the
    quad-tree level each map is weighted with (1 / (2^level + 1)^2)."""
    assert vis.is_cuda and vis.numel() >= width * height
    lv, c = light.to_c(), mp.to_c()
    out = (api.View * 289)()
    levels = np.zeros(289, np.float32)
    n = C.c_int(0)
    check(_lib().gi_area_light_adaptive(ctx.handle, scene.handle, C.byref(lv), float(size), int(max_level),
                                        1 if lower_accuracy else 0, C.byref(c), _f16(camera_mvp), float(intensity), width, height, _ptr(vis),
                                        out, levels.ctypes.data, C.byref(n), _stream_ptr(stream)),
          "gi_area_light_adaptive")
    views = [ViewSpec(eye=tuple(v.eye), at=tuple(v.at), width=v.width, height=v.height, fovy_deg=v.fovy_deg,
                      znear=v.znear, zfar=v.zfar, up=tuple(v.up)) for v in out[:n.value]]
    return vis, views, levels[:n.value].copy()


class Batch:
    """Many frames (scene, camera, lights) replayed as one CUDA graph (gi_batch_*).

    Every light of a frame writes its visibility image into its own slice of
    the frame's output tensor (lights x height x width); the result of each
    light equals render_frame for that light.  Scenes and output tensors
    must outlive the batch.
    """

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(_lib().gi_batch_create(device, C.byref(h)), "gi_batch_create")
        self.handle = h
        self._keep = []

    def add_frame(self, scene: Scene, camera: ViewSpec, lights, maps, params: ShadowParams, out) -> None:
        lights, maps = list(lights), list(maps)
        if len(lights) != len(maps) or not lights:
            raise ValueError("one map per light, at least one light")
        import torch
        if out.dtype != torch.float32 or not out.is_cuda or out.numel() < len(lights) * camera.width * camera.height:
            raise ValueError("out must be a CUDA float32 tensor of lights x height x width")
        lv = (api.View * len(lights))(*[l.to_c() for l in lights])
        mv = (api.MapParams * len(maps))(*[m.to_c() for m in maps])
        cv = camera.to_c()
        p = params.to_c(frame_setup(lights[0], camera))
        check(_lib().gi_batch_add_frame(self.handle, scene.handle, C.byref(cv), lv, mv, len(lights), C.byref(p),
                                        _ptr(out)), "gi_batch_add_frame")
        self._keep.append((scene, out))

    def build(self, streams: int = 8) -> None:
        check(_lib().gi_batch_build(self.handle, streams), "gi_batch_build")

    def build_persistent(self, streams: int = 8, tile_w: int = 64, tile_h: int = 8) -> None:
        """Persistent mode: all maps and G-buffers resident, one persistent visibility launch."""
        check(_lib().gi_batch_build_persistent(self.handle, streams, tile_w, tile_h), "gi_batch_build_persistent")

    def autotune_persistent(self, stream=None, repeats: int = 3) -> dict:
        t = api.BatchTuning()
        check(_lib().gi_batch_autotune_persistent(self.handle, _stream_ptr(stream), repeats, C.byref(t)),
              "gi_batch_autotune_persistent")
        return self._tuning(t)

    def run(self, stream=None) -> None:
        check(_lib().gi_batch_run(self.handle, _stream_ptr(stream)), "gi_batch_run")

    def autotune(self, stream=None, repeats: int = 3) -> dict:
        t = api.BatchTuning()
        check(_lib().gi_batch_autotune(self.handle, _stream_ptr(stream), repeats, C.byref(t)), "gi_batch_autotune")
        return self._tuning(t)

    def info(self) -> dict:
        t = api.BatchTuning()
        check(_lib().gi_batch_info(self.handle, C.byref(t)), "gi_batch_info")
        return self._tuning(t)

    @staticmethod
    def _tuning(t) -> dict:
        return {"tiny_px": t.tiny_px, "coop_px": t.coop_px, "streams": t.streams, "frames": t.frames,
                "kernel_launches": int(t.kernel_launches), "best_ms": float(t.best_ms),
                "persistent": bool(t.persistent), "tile_w": t.tile_w, "tile_h": t.tile_h,
                "work_items": int(t.work_items)}

    def close(self) -> None:
        if self.handle:
            _lib().gi_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
