"""Python wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
import this package, to check or time the CUDA path; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build_oracle import ORACLE_LIB, build_oracle

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        lib.or_shadow_map.argtypes = [vp, i, vp, i, vp, i, i, i, f, f, f, vp, i]
        lib.or_gbuffer.argtypes = [vp, vp, i, vp, i, vp, i, i, vp, vp, i]
        lib.or_visibility.argtypes = [vp, vp, i, i, vp, vp, vp, i, i, vp, i]
        lib.or_shadow_volume_counts.argtypes = [vp, vp, i, vp, i, vp, f, vp, i, i, i, vp, vp, i]
        lib.or_shadow_volume_geometry.argtypes = [vp, vp, vp, i, vp, f, vp]
        lib.or_shadow_volume_geometry.restype = None
        lib.or_rbssm_hits.argtypes = [vp, i]
        lib.or_phong_shade.argtypes = [vp, vp, vp, vp, vp, i, i, vp]
        lib.or_area_light_visibility.argtypes = [vp, vp, i, vp, i, vp, vp, i, i, i, f, f, f, vp, f, i, i, vp, i]
        lib.or_pba_voronoi.argtypes = [vp, i, i, i, i, i, vp, i]
        lib.or_edt_sites.argtypes = [vp, i, i, vp]
        lib.or_edt_normalize.argtypes = [vp, vp, vp, i, i, f, f, vp]
        lib.or_edt_soft_shadows.argtypes = [vp, vp, i, i, i, i, i, f, f, vp, vp, vp, i]
        lib.or_edt_inputs.argtypes = [vp, vp, vp, vp, vp, i, i, vp, vp]
        lib.or_edt_mean_filter.argtypes = [vp, vp, vp, i, i, i, vp]
        lib.or_soft_moment_map.argtypes = [vp, vp, i, i, vp]
        lib.or_area_light_adaptive.argtypes = [vp, vp, i, vp, i, vp, vp, f, i, i, VIEW_MVP_FN, vp, i, i, f, f, f,
                                               vp, f, i, i, vp, vp, vp, i]
        lib.or_area_light_adaptive.restype = i
        lib.or_hierarchical_shadow_map.argtypes = [vp, vp, i, i, i, vp]
        for fn in (lib.or_shadow_map, lib.or_gbuffer, lib.or_visibility, lib.or_shadow_volume_counts):
            fn.restype = None
        _lib = lib
    return _lib


VIEW_MVP_FN = C.CFUNCTYPE(None, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                          C.POINTER(C.c_float), C.c_void_p)


def area_light_adaptive(points, normals, indices, light_eye, light_at, size, max_level, view_mvp, S, bias_mode,
                        cbias, factor, units, camera_mvp, intensity, width, height, lower_accuracy=False, threads=0):
    """Adaptive (quad-tree) area-light ground truth.  view_mvp(eye, at) -> (mvp[16], biased[16]) gives a
    sample's light matrices.  Returns (vis, eyes [n, 6] (eye, at), levels [n])."""
    p, n = _f32(points), _f32(normals)
    ix, cm = np.ascontiguousarray(indices, dtype=np.int32), _f32(camera_mvp).reshape(16)
    le, la = _f32(light_eye).reshape(3), _f32(light_at).reshape(3)

    def cb(eye, at, mvp, biased, _user):
        m, b = view_mvp(tuple(eye[k] for k in range(3)), tuple(at[k] for k in range(3)))
        m, b = _f32(m).reshape(16), _f32(b).reshape(16)
        for k in range(16):
            mvp[k] = float(m[k])
            biased[k] = float(b[k])

    fn = VIEW_MVP_FN(cb)
    out = np.empty(height * width, np.float32)
    eyes = np.empty((289, 6), np.float32)
    levels = np.empty(289, np.float32)
    cnt = load().or_area_light_adaptive(p.ctypes.data, n.ctypes.data, p.size // 3, ix.ctypes.data, ix.size // 3,
                                        le.ctypes.data, la.ctypes.data, float(size), int(max_level),
                                        1 if lower_accuracy else 0, fn, None, S,
                                        bias_mode, cbias, factor, units, cm.ctypes.data, float(intensity), width,
                                        height, out.ctypes.data, eyes.ctypes.data, levels.ctypes.data, threads)
    return out, eyes[:cnt].copy(), levels[:cnt].copy()


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def shadow_map(points, indices, mvp, width, height, bias_mode=0, constant_bias=0.0, factor=0.0, units=0.0,
               threads=0):
    p, ix, m = _f32(points), np.ascontiguousarray(indices, dtype=np.int32), _f32(mvp).reshape(16)
    out = np.empty(height * width, np.float32)
    load().or_shadow_map(p.ctypes.data, p.size // 3, ix.ctypes.data, ix.size // 3, m.ctypes.data, width, height,
                         bias_mode, constant_bias, factor, units, out.ctypes.data, threads)
    return out


def gbuffer(points, normals, indices, mvp, width, height, threads=0):
    p, n = _f32(points), _f32(normals)
    ix, m = np.ascontiguousarray(indices, dtype=np.int32), _f32(mvp).reshape(16)
    pos = np.empty(height * width * 4, np.float32)
    nrm = np.empty(height * width * 4, np.float32)
    load().or_gbuffer(p.ctypes.data, n.ctypes.data, p.size // 3, ix.ctypes.data, ix.size // 3, m.ctypes.data,
                      width, height, pos.ctypes.data, nrm.ctypes.data, threads)
    return pos, nrm


def visibility(vis_params, depth, map_w, map_h, pos, nrm, width, height, poisson_xy=None, threads=0):
    """vis_params is a globalillumination_gb300._capi.VisParams (same layout as gi_vis_params)."""
    d, ps, ns = _f32(depth), _f32(pos), _f32(nrm)
    out = np.empty(height * width, np.float32)
    tab = _f32(poisson_xy) if poisson_xy is not None else None
    load().or_visibility(C.addressof(vis_params), d.ctypes.data, map_w, map_h, ps.ctypes.data, ns.ctypes.data,
                         out.ctypes.data, width, height, tab.ctypes.data if tab is not None else None, threads)
    return out


def soft_moment_map(vis_params, depth, S, T):
    """Moment map (or its summed-area table) of a SoftShadowMapping moment technique, float32 [T, S, 4]."""
    d = _f32(depth)
    out = np.empty((T, S, 4), np.float32)
    load().or_soft_moment_map(C.addressof(vis_params), d.ctypes.data, S, T, out.ctypes.data)
    return out


def hierarchical_shadow_map(vis_params, depth, S, T, level):
    """Level `level` of the min-max shadow map, float32 [T >> level, S >> level, 2]."""
    d = _f32(depth)
    out = np.empty((T >> level, S >> level, 2), np.float32)
    load().or_hierarchical_shadow_map(C.addressof(vis_params), d.ctypes.data, S, T, level, out.ctypes.data)
    return out


def shadow_volume_counts(points, normals, indices, light_pos, infinity, mvp, width, height, depth_func,
                         threads=0):
    p, n = _f32(points), _f32(normals)
    ix, m, L = np.ascontiguousarray(indices, dtype=np.int32), _f32(mvp).reshape(16), _f32(light_pos)
    st = np.empty(height * width, np.uint8)
    dp = np.empty(height * width, np.float32)
    load().or_shadow_volume_counts(p.ctypes.data, n.ctypes.data, p.size // 3, ix.ctypes.data, ix.size // 3,
                                   L.ctypes.data, infinity, m.ctypes.data, width, height, depth_func,
                                   st.ctypes.data, dp.ctypes.data, threads)
    return st, dp


def shadow_volume_geometry(points, normals, indices, light_pos, infinity):
    """ShadowVolume::build's triangles: float32 [6T, 3, 3] (entry 6t + k is side k of triangle t)."""
    p, n = _f32(points), _f32(normals)
    ix, L = np.ascontiguousarray(indices, dtype=np.int32), _f32(light_pos)
    nt = ix.size // 3
    out = np.empty((6 * nt, 3, 3), np.float32)
    load().or_shadow_volume_geometry(p.ctypes.data, n.ctypes.data, ix.ctypes.data, nt, L.ctypes.data, infinity,
                                     out.ctypes.data)
    return out


# ---------------------------------------------------------------------------
# The reference's own scene C++ (oracle/_ref/libscene_ref_<app>.so, built by
# build_oracle.build_scene_ref where the reference tree is present).
# ---------------------------------------------------------------------------
class _PinScene(C.Structure):
    _fields_ = [("num_vertices", C.c_int), ("num_triangles", C.c_int), ("points", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_int)), ("views", C.c_float * 13)]


_scene_refs: dict = {}


def scene_ref(app: str = "ShadowMapping"):
    """The reference's scene loader of `app` ("ShadowMapping" or "ShadowVolumes"), or None if not built."""
    from .build_oracle import scene_ref_lib

    if app not in _scene_refs:
        path = scene_ref_lib(app)
        if not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        lib.pin_scene_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(_PinScene)]
        lib.pin_scene_load.restype = C.c_int
        lib.pin_scene_free.argtypes = [C.POINTER(_PinScene)]
        lib.pin_scene_free.restype = None
        if hasattr(lib, "pin_shadow_volume_build"):
            vp, i = C.c_void_p, C.c_int
            lib.pin_shadow_volume_build.argtypes = [vp, vp, i, vp, i, vp, i, vp, vp]
            lib.pin_shadow_volume_build.restype = C.c_int
        _scene_refs[app] = lib
    return _scene_refs[app]


def ref_load_config(cfg_path: str, base_dir: str, app: str = "ShadowMapping"):
    """SceneLoader::load + Mesh of the reference itself: (points [V,3], normals [V,3], indices [T,3], views[13])."""
    lib = scene_ref(app)
    if lib is None:
        raise RuntimeError(f"the reference scene pin for {app} is not built")
    sc = _PinScene()
    if lib.pin_scene_load(cfg_path.encode(), base_dir.encode(), C.byref(sc)) != 0:
        raise OSError(f"reference SceneLoader could not open {cfg_path}")
    nv, nt = sc.num_vertices, sc.num_triangles
    p = np.ctypeslib.as_array(sc.points, (nv * 3,)).copy().reshape(nv, 3)
    n = np.ctypeslib.as_array(sc.normals, (nv * 3,)).copy().reshape(nv, 3)
    ix = np.ctypeslib.as_array(sc.indices, (nt * 3,)).copy().reshape(nt, 3)
    views = np.array(sc.views[:], np.float32)
    lib.pin_scene_free(C.byref(sc))
    return p, n, ix, views


def ref_shadow_volume_build(points, normals, indices, light_pos, infinity: int = 100):
    """ShadowVolume::build of the reference itself: (quad points [6T, 3], index buffer [6T, 3])."""
    lib = scene_ref("ShadowVolumes")
    if lib is None:
        raise RuntimeError("the reference ShadowVolumes pin is not built")
    p, n = _f32(points), _f32(normals)
    ix, L = np.ascontiguousarray(indices, dtype=np.int32), _f32(light_pos)
    nv, nt = p.size // 3, ix.size // 3
    out_p = np.empty((6 * nt, 3), np.float32)
    out_i = np.empty((6 * nt, 3), np.int32)
    rc = lib.pin_shadow_volume_build(p.ctypes.data, n.ctypes.data, nv, ix.ctypes.data, nt, L.ctypes.data,
                                     int(infinity), out_p.ctypes.data, out_i.ctypes.data)
    if rc != 0:
        raise ValueError("empty mesh")
    return out_p, out_i


def rbssm_hits(reset=False):
    """Hit counts of the RBSSM smoothONDS return sites: {source line: hits}."""
    out = np.zeros(4096, np.uint64)
    load().or_rbssm_hits(out.ctypes.data, 1 if reset else 0)
    return {int(k): int(out[k]) for k in np.nonzero(out)[0]}


def rbssm_return_sites():
    """Source lines of the RBSSM smoothONDS return sites in gi_oracle.cpp."""
    import os

    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gi_oracle.cpp")
    with open(src) as f:
        lines = f.read().split("\n")
    return [i + 1 for i, l in enumerate(lines) if "RB_RET(" in l and "#define" not in l]


def area_light_visibility(points, normals, indices, mvps, biased, S, bias_mode, cbias, factor, units, camera_mvp,
                          intensity, width, height, threads=0):
    p, n = _f32(points), _f32(normals)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    mv, bs, cm = _f32(mvps).reshape(-1), _f32(biased).reshape(-1), _f32(camera_mvp).reshape(16)
    out = np.empty(height * width, np.float32)
    load().or_area_light_visibility(p.ctypes.data, n.ctypes.data, p.size // 3, ix.ctypes.data, ix.size // 3,
                                    mv.ctypes.data,
                                    bs.ctypes.data, mv.size // 16, S, bias_mode, cbias, factor, units, cm.ctypes.data,
                                    intensity, width, height, out.ctypes.data, threads)
    return out


def phong_shade(vis_params, pos, nrm, vis, width, height, color=None):
    ps, ns, vs = _f32(pos), _f32(nrm), _f32(vis)
    cs = _f32(color) if color is not None else None
    out = np.empty(height * width * 4, np.float32)
    load().or_phong_shade(C.byref(vis_params), ps.ctypes.data, ns.ctypes.data, vs.ctypes.data,
                          cs.ctypes.data if cs is not None else None, width, height, out.ctypes.data)
    return out


PBA_MARKER = -32768


def pba_voronoi(sites, m=(16, 16, 16), threads=0):
    """sites: int16 [H, W, 2] ((x, y) at a site, MARKER elsewhere) -> nearest site [H, W, 2]."""
    s = np.ascontiguousarray(sites, dtype=np.int16)
    H, W = s.shape[:2]
    out = np.zeros_like(s)
    load().or_pba_voronoi(s.ctypes.data, W, H, m[0], m[1], m[2], out.ctypes.data, threads)
    return out


def edt_sites(image):
    im = _f32(image)
    H, W = im.shape[:2]
    out = np.empty((H, W, 2), np.int16)
    load().or_edt_sites(im.ctypes.data, W, H, out.ctypes.data)
    return out


def edt_normalize(nearest, image, position, penumbra, intensity, out4=None):
    nn = np.ascontiguousarray(nearest, dtype=np.int16)
    im, po = _f32(image), _f32(position)
    H, W = im.shape[:2]
    out = np.zeros((H, W, 4), np.float32) if out4 is None else out4
    load().or_edt_normalize(nn.ctypes.data, im.ctypes.data, po.ctypes.data, W, H, penumbra, intensity,
                            out.ctypes.data)
    return out


def edt_soft_shadows(image, position, penumbra, intensity, m=(16, 16, 16), threads=0):
    """Returns (out4 [H, W, 4] with channels 0-1 written, sites, nearest)."""
    im, po = _f32(image), _f32(position)
    H, W = im.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    sites = np.empty((H, W, 2), np.int16)
    nearest = np.empty((H, W, 2), np.int16)
    load().or_edt_soft_shadows(im.ctypes.data, po.ctypes.data, W, H, m[0], m[1], m[2], penumbra, intensity,
                               sites.ctypes.data, nearest.ctypes.data, out.ctypes.data, threads)
    return out, sites, nearest


def edt_inputs(vis_params, camera_mvp, pos, nrm, vis, width, height):
    ps, ns, vs, cm = _f32(pos), _f32(nrm), _f32(vis), _f32(camera_mvp).reshape(16)
    image = np.empty((height, width, 4), np.float32)
    position = np.empty((height, width, 4), np.float32)
    load().or_edt_inputs(C.addressof(vis_params), cm.ctypes.data, ps.ctypes.data, ns.ctypes.data, vs.ctypes.data,
                         width, height, image.ctypes.data, position.ctypes.data)
    return image, position


def edt_mean_filter(vis_params, image, pos, width, height, order=7):
    im, ps = _f32(image), _f32(pos)
    out = np.empty((height, width, 4), np.float32)
    load().or_edt_mean_filter(C.addressof(vis_params), im.ctypes.data, ps.ctypes.data, width, height, order,
                              out.ctypes.data)
    return out
