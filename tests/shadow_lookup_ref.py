"""A second, numpy restatement of the per-pixel shadow lookups (test helper).

The hard test, PCF and PCSS of the reference's visibility shaders written
again with numpy float32 scalars (every operation rounds to float32, in the
order the shader text writes it), independently of the C++ oracle, so the
CPU tests can hold the oracle to it bit for bit:

* main() of ShadowMapping/Shaders/Shadow.frag:240-272 and of
  SoftShadowMapping/Shaders/SoftShadow/PlausibleSoftShadow.frag:605-632:
  background where vertex.x == 0, shadowCoord = lightMVP * vertex divided by
  its w, the pre-test, and the lookup only where w > 0 and the pre-test
  passed;
* computePreEvaluationBasedOnNormalOrientation (Shadow.frag:222-238), with
  normalize(v) fixed as v * (1 / sqrt(dot(v, v))) and dot / matrix products
  summed left to right;
* the naive hard test (Shadow.frag:253-256; the soft app's
  HardShadow.frag:36-58, background for failed pre-tests) and PCF's float loop
  (Shadow.frag:86-116), bilinear (one texture2D) or tricubic
  (textureBicubic, :41-84), over a NEAREST, CLAMP_TO_BORDER (border 0) map:
  the texel of (s, t) is (floor(s * W), floor(t * H));
* PCSS (PlausibleSoftShadow.frag:166-194 blocker search, 365-374 penumbra
  width, 376-398 filter, 556-563), with the light radius a float and the
  0.99 average-blocker cut-off a parameter;
* the Poisson-disk PCSS of this library (no reference counterpart): the
  same blocker search and filter with the grid offsets replaced by the
  Poisson points times the blocker search width / the penumbra width, the
  filter averaging over its own tap count;
* deferred Phong shading (ShadowMapping/Shaders/GBuffer/PhongShading.frag:
  11-46, shadeScene);
* the uniform area-light ground truth (AccurateSoftShadow.frag:52-133) and
  the adaptive quad-tree one (SoftShadowMapping/src/main.cpp:423-690,
  Shaders/QuadTree/{Reprojection,Evaluation}.frag, QuadTreeLightSource.cpp),
  their maps and G-buffer drawn by raster_ref's brute-force rasteriser;
* EDTSM's inputs written by the SMSR shaders and its screen-space mean
  filter (Shaders/Filter/MeanFilter.frag).
"""
from __future__ import annotations

import numpy as np

f32 = np.float32

TECH_HARD, TECH_PCF, TECH_PCF_TRICUBIC, TECH_PCSS_GRID, TECH_PCSS_POISSON = 0, 1, 2, 3, 4
TECH_HARD_SOFTAPP = 10
PRETEST_REFERENCE, PRETEST_OFF = 0, 1


def mat4_mul(m, v):
    """Column-major mat4 times vec4, each row summed left to right."""
    return [((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * v[3] for r in range(4)]


def fetch(depth, W, H, s, t):
    """texture2D(shadowMap, (s, t)).z with NEAREST filtering and a border of 0."""
    fi = np.floor(s * f32(W))
    fj = np.floor(t * f32(H))
    if not (fi >= 0 and fi < f32(W) and fj >= 0 and fj < f32(H)):
        return f32(0.0)
    return depth[int(fj) * W + int(fi)]


def pretest(p, vertex, normal):
    if p["pretest"] == PRETEST_OFF:
        return f32(1.0)
    ev = mat4_mul(p["camera_mv"], vertex)
    nm = p["normal_matrix"]
    nx = (nm[0] * normal[0] + nm[3] * normal[1]) + nm[6] * normal[2]
    ny = (nm[1] * normal[0] + nm[4] * normal[1]) + nm[7] * normal[2]
    nz = (nm[2] * normal[0] + nm[5] * normal[1]) + nm[8] * normal[2]
    inv = f32(1.0) / np.sqrt((nx * nx + ny * ny) + nz * nz)
    nx, ny, nz = nx * inv, ny * inv, nz * inv
    lp = p["light_position"]
    lx, ly, lz = lp[0] - ev[0], lp[1] - ev[1], lp[2] - ev[2]
    linv = f32(1.0) / np.sqrt((lx * lx + ly * ly) + lz * lz)
    lx, ly, lz = lx * linv, ly * linv, lz * linv
    if not normal[3] != 0:  # !bool(normal.w)
        nx, ny, nz = nx * f32(-1.0), ny * f32(-1.0), nz * f32(-1.0)
    d = (nx * lx + ny * ly) + nz * lz
    return p["intensity"] if max(d, f32(0.0)) == 0 else f32(1.0)


def cubic(v):
    """cubic() of Shadow.frag:41-52."""
    n = [f32(1.0) - v, f32(2.0) - v, f32(3.0) - v, f32(4.0) - v]
    s = [(k * k) * k for k in n]
    x = s[0]
    y = s[1] - f32(4.0) * s[0]
    z = (s[2] - f32(4.0) * s[1]) + f32(6.0) * s[0]
    w = ((f32(6.0) - x) - y) - z
    k = f32(1.0 / 6.0)
    return [x * k, y * k, z * k, w * k]


def texture_bicubic(depth, W, H, u, v):
    """textureBicubic (Shadow.frag:54-84): four NEAREST fetches blended."""
    inv_w, inv_h = f32(1.0) / f32(W), f32(1.0) / f32(H)
    tx, ty = u * f32(W) - f32(0.5), v * f32(H) - f32(0.5)
    fx, fy = tx - np.floor(tx), ty - np.floor(ty)
    tx, ty = tx - fx, ty - fy
    xc, yc = cubic(fx), cubic(fy)
    c = [tx + f32(-0.5), tx + f32(1.5), ty + f32(-0.5), ty + f32(1.5)]
    s = [xc[0] + xc[1], xc[2] + xc[3], yc[0] + yc[1], yc[2] + yc[3]]
    num = [xc[1], xc[3], yc[1], yc[3]]
    off = [c[i] + num[i] / s[i] for i in range(4)]
    off = [off[0] * inv_w, off[1] * inv_w, off[2] * inv_h, off[3] * inv_h]
    s0, s1 = fetch(depth, W, H, off[0], off[2]), fetch(depth, W, H, off[1], off[2])
    s2, s3 = fetch(depth, W, H, off[0], off[3]), fetch(depth, W, H, off[1], off[3])
    sx = s[0] / (s[0] + s[1])
    sy = s[2] / (s[2] + s[3])

    def mix(a, b, t):
        return a * (f32(1.0) - t) + b * t

    return mix(mix(s3, s2, sx), mix(s1, s0, sx), sy)


def pcf(p, depth, W, H, n, tricubic=False):
    incr_w, incr_h = f32(1.0) / f32(W), f32(1.0) / f32(H)
    illum = f32(0.0)
    offset = f32(p["penumbra_size"])
    step = (f32(2.0) * offset) / f32(p["kernel_order"])
    count = 0
    w = -offset
    while w < offset:
        h = -offset
        while h < offset:
            u, v = n[0] + w * incr_w, n[1] + h * incr_h
            d = texture_bicubic(depth, W, H, u, v) if tricubic else fetch(depth, W, H, u, v)
            illum = illum + (f32(1.0) if n[2] <= d else p["intensity"])
            count += 1
            h = h + step
        w = w + step
    return illum / f32(count)


def blocker_search_width(p, W):
    R = p["light_radius"]
    return R / f32(W) if f32(W) <= f32(1024.0) else R / f32(1024.0)


def grid_range(fw):
    """for (int h = -filterWidth; h <= filterWidth; h++) with a float filterWidth."""
    h = int(-fw)  # float to int conversion truncates
    while f32(h) <= fw:
        yield h
        h += 1


def avg_blocker(p, depth, W, H, n, taps=None):
    avg, nb = f32(0.0), 0
    bsw = blocker_search_width(p, W)
    if taps is None:
        fw = (f32(p["blocker_search_size"]) - f32(1.0)) * f32(0.5)
        offs = [((f32(w) * bsw) / fw, (f32(h) * bsw) / fw) for h in grid_range(fw) for w in grid_range(fw)]
    else:
        offs = [(x * bsw, y * bsw) for x, y in taps]
    for ox, oy in offs:
        d = fetch(depth, W, H, n[0] + ox, n[1] + oy)
        if n[2] > d:
            avg = avg + d
            nb += 1
    return f32(1.0) if nb == 0 else avg / f32(nb)


def penumbra_width(p, avg, z):
    if avg < p["min_blocker_depth"]:
        return f32(0.0)
    pw = ((z - avg) / avg) * p["light_radius"]
    return (p["znear"] * pw) / z


def pcss_filter(p, depth, W, H, n, pw, taps=None):
    K = p["kernel_size"]
    step = (f32(2.0) * pw) / f32(K)
    if step <= 0 or step >= 1:
        return f32(1.0)
    illum = f32(0.0)
    if taps is None:
        fw = (f32(K) - f32(1.0)) * f32(0.5)
        offs = [((f32(w) * pw) / fw, (f32(h) * pw) / fw) for h in grid_range(fw) for w in grid_range(fw)]
        count = f32(K * K)
    else:
        offs = [(x * pw, y * pw) for x, y in taps]
        count = f32(len(taps))
    for ox, oy in offs:
        d = fetch(depth, W, H, n[0] + ox, n[1] + oy)
        illum = illum + (f32(1.0) if n[2] <= d else p["intensity"])
    return illum / count


def shade(p, depth, W, H, vertex, normal, blocker_taps=None, filter_taps=None):
    """Visibility of one G-buffer pixel (vertex, normal: 4 float32 each)."""
    if vertex[0] == 0:
        return f32(0.0)
    sc = mat4_mul(p["light_mvp_biased"], vertex)
    n = [sc[0] / sc[3], sc[1] / sc[3], sc[2] / sc[3], sc[3] / sc[3]]
    shadow = pretest(p, vertex, normal)
    tech = p["technique"]
    if tech == TECH_HARD_SOFTAPP:  # SoftShadowMapping HardShadow.frag:36-58
        r = shadow
        if sc[3] > 0 and r == 1:
            r = f32(1.0) if n[2] <= fetch(depth, W, H, n[0], n[1]) else p["intensity"]
        return f32(0.0) if pretest(p, vertex, normal) == p["intensity"] else r
    if not (sc[3] > 0 and shadow == 1):
        return shadow
    if tech == TECH_HARD:
        return f32(1.0) if n[2] <= fetch(depth, W, H, n[0], n[1]) else p["intensity"]
    if tech == TECH_PCF:
        return pcf(p, depth, W, H, n)
    if tech == TECH_PCF_TRICUBIC:
        return pcf(p, depth, W, H, n, tricubic=True)
    if tech == TECH_PCSS_GRID:
        return pcss_filter(p, depth, W, H, n, penumbra_width(p, avg_blocker(p, depth, W, H, n), n[2]))
    if tech == TECH_PCSS_POISSON:
        avg = avg_blocker(p, depth, W, H, n, blocker_taps)
        return pcss_filter(p, depth, W, H, n, penumbra_width(p, avg, n[2]), filter_taps)
    raise ValueError(f"technique {tech} is not restated here")


def params_of(c):
    """The fields of a gi_vis_params (ctypes) this restatement reads, as float32 / int."""
    return {
        "technique": int(c.technique), "pretest": int(c.pretest), "intensity": f32(c.shadow_intensity),
        "kernel_order": int(c.kernel_order), "penumbra_size": int(c.penumbra_size),
        "blocker_search_size": int(c.blocker_search_size), "kernel_size": int(c.kernel_size),
        "light_radius": f32(c.light_radius), "znear": f32(c.znear), "min_blocker_depth": f32(c.pcss_min_blocker_depth),
        "light_mvp_biased": [f32(x) for x in c.light_mvp_biased], "camera_mv": [f32(x) for x in c.camera_mv],
        "normal_matrix": [f32(x) for x in c.normal_matrix], "light_position": [f32(x) for x in c.light_position],
    }


def phong(p, vertex, normal, shadow, color=(1.0, 1.0, 1.0, 1.0)):
    """shadeScene's PhongShading.frag:11-46 for one pixel (RGBA float32):
    shadow * fragmentColor * (Idiff + Ispec + Iamb), with reflect(I, N) =
    I - 2 dot(N, I) N, E = normalize(-vertex) over the 4-component eye-space
    vertex, pow(x, 0.3 * 10) as x * x * x; background keeps the clear colour."""
    if vertex[0] == 0:
        return [f32(0.63), f32(0.82), f32(0.96), f32(1.0)]
    spec_shadow = shadow - p["intensity"]
    v = mat4_mul(p["camera_mv"], vertex)
    nm = p["normal_matrix"]
    nx = (nm[0] * normal[0] + nm[3] * normal[1]) + nm[6] * normal[2]
    ny = (nm[1] * normal[0] + nm[4] * normal[1]) + nm[7] * normal[2]
    nz = (nm[2] * normal[0] + nm[5] * normal[1]) + nm[8] * normal[2]
    inv = f32(1.0) / np.sqrt((nx * nx + ny * ny) + nz * nz)
    nx, ny, nz = nx * inv, ny * inv, nz * inv
    lp = p["light_position"]
    lx, ly, lz = lp[0] - v[0], lp[1] - v[1], lp[2] - v[2]
    inv = f32(1.0) / np.sqrt((lx * lx + ly * ly) + lz * lz)
    lx, ly, lz = lx * inv, ly * inv, lz * inv
    e = [-v[0], -v[1], -v[2], -v[3]]
    inv = f32(1.0) / np.sqrt(((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]) + e[3] * e[3])
    ex, ey, ez = e[0] * inv, e[1] * inv, e[2] * inv
    ndl = (nx * lx + ny * ly) + nz * lz
    two = f32(2.0)
    rx, ry, rz = -(lx - (two * ndl) * nx), -(ly - (two * ndl) * ny), -(lz - (two * ndl) * nz)
    inv = f32(1.0) / np.sqrt((rx * rx + ry * ry) + rz * rz)
    rx, ry, rz = rx * inv, ry * inv, rz * inv
    diff = max(ndl, f32(0.0))
    re = max((rx * ex + ry * ey) + rz * ez, f32(0.0))
    spec = (re * re) * re
    amb, dif, spc = (0.4, 0.4, 0.4, 1.0), (0.5, 0.5, 0.5, 1.0), (0.25, 0.25, 0.25, 1.0)
    out = []
    for k in range(4):
        idiff = f32(dif[k]) * diff
        ispec = (spec_shadow * f32(spc[k])) * spec
        out.append((shadow * f32(color[k])) * ((idiff + ispec) + f32(amb[k])))
    return out


def area_light_visibility(points, normals, indices, mvps, biased, S, bias_mode, cbias, factor, units, camera_mvp,
                          intensity, W, H):
    """renderMonteCarlo's uniform branch (SoftShadowMapping/src/main.cpp:756-811,
    AccurateSoftShadow.frag:52-133) with the light maps and the G-buffer drawn
    by the brute-force rasteriser of raster_ref: per pixel the common
    coordinate from columns 0-2 of the LAST sample's biased MVP, plus each
    sample's translation column, divided by w, one NEAREST fetch from that
    sample's map, accShadow += (z <= d ? 1 : intensity) * 1, shadow =
    accShadow / count; no pre-test, background 0."""
    import raster_ref

    pos, _ = raster_ref.gbuffer(points, normals, indices, camera_mvp, W, H)
    pos = pos.reshape(-1, 4)
    I = f32(intensity)
    m = [f32(v) for v in np.asarray(biased[-1], np.float32).reshape(16)]
    acc = np.zeros(W * H, np.float32)
    fg = np.flatnonzero(pos[:, 0] != 0)
    for k in range(len(mvps)):
        depth = raster_ref.shadow_map(points, indices, mvps[k], S, S, bias_mode, cbias, factor, units)
        t = [f32(v) for v in np.asarray(biased[k], np.float32).reshape(16)[12:]]
        for q in fg:
            x, y, z = pos[q, 0], pos[q, 1], pos[q, 2]
            c = [((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + t[r] for r in range(4)]
            d = fetch(depth, S, S, c[0] / c[3], c[1] / c[3])
            acc[q] = acc[q] + (f32(1.0) if c[2] / c[3] <= d else I) * f32(1.0)
    count = f32(0.0)
    for _ in range(len(mvps)):
        count = count + f32(1.0)
    out = np.zeros(W * H, np.float32)
    out[fg] = acc[fg] / count
    return out


def area_light_adaptive(points, normals, indices, light_eye, light_at, size, max_level, view_mvp, S, bias_mode,
                        cbias, factor, units, camera_mvp, intensity, W, H, lower_accuracy=False):
    """SoftShadowMapping's adaptive light-source sampling without temporal
    coherency (src/main.cpp:423-690, 820-870): evaluateAreaLightSource
    depth first from the root node, each node rendering its four corner
    samples (QuadTreeLightSource::getEye / getAt, the light's 17 x 17 grid,
    one map per grid position), the reprojection pass
    (Shaders/QuadTree/Reprojection.frag: the four corners' hard tests summed,
    background the clear red 0.63), the evaluation pass
    (Shaders/QuadTree/Evaluation.frag over a (W / div) x (H / div) viewport,
    div 4 in the lower-accuracy mode, each coarse pixel reading the count
    texel at its centre, the border 0) whose occlusion query decides the
    subdivision (children's reference samples: computeReferenceSamples), then
    renderAreaLightSource setting each leaf corner's level and the final
    AccurateSoftShadow.frag pass with weights 1 / (2^level + 1)^2 carried in
    the translation's w.  Maps and G-buffer come from raster_ref's
    rasteriser.  Returns (vis, eyes [n, 6], levels [n])."""
    import raster_ref

    pos, _ = raster_ref.gbuffer(points, normals, indices, camera_mvp, W, H)
    pos = pos.reshape(-1, 4)
    fg = np.flatnonzero(pos[:, 0] != 0)
    I = f32(intensity)
    fsize = f32(size)
    grid = {}  # quadTreeHash: grid position -> sample index
    maps, biased, eyes, level = [], [], [], []

    def offset(ref_, div_pow, index):
        div = int(np.float32(2.0) ** np.float32(div_pow))
        step = fsize / f32(div)
        out = list(ref_)
        out[0] = out[0] + (-step + (f32(2.0) * step) * f32(index % 2))
        out[1] = out[1] + (-step + (f32(2.0) * step) * f32(index // 2))
        return out

    def corner(lvl, node, index):
        cf, pf = int(16.0 / 2.0 ** lvl), int(2.0 ** lvl)
        return (index % 2) * cf + (node % pf) * cf, (index // 2) * cf + (node // pf) * cf

    def children(lvl, node):
        div = int(2.0 ** lvl)
        x, y = node % div, node // div
        base = 2 * x + int(2.0 ** (lvl + 2)) * y
        row = int(2.0 ** (lvl + 1))
        return [base, base + 1, base + row, base + row + 1]

    def sample(nd, index, x, y):
        if (x, y) in grid:
            return grid[(x, y)]
        e = offset(nd["eye"], nd["level"] + 1, index) + offset(nd["at"], nd["level"] + 1, index)
        mvp, b = view_mvp(tuple(e[:3]), tuple(e[3:]))
        maps.append(raster_ref.shadow_map(points, indices, mvp, S, S, bias_mode, cbias, factor, units))
        biased.append([f32(v) for v in np.asarray(b, np.float32).reshape(16)])
        eyes.append(e)
        level.append(f32(0.0))
        grid[(x, y)] = len(maps) - 1
        return grid[(x, y)]

    def needs_subdivision(idx):
        count = np.full(W * H, f32(0.63), np.float32)
        for p in fg:
            v = [f32(c) for c in pos[p]]
            s = f32(0.0)
            for k in range(4):
                c = mat4_mul(biased[idx[k]], v)
                lit = c[2] / c[3] <= fetch(maps[idx[k]], S, S, c[0] / c[3], c[1] / c[3])
                s = s + (f32(1.0) if lit else f32(0.0))
            count[p] = s
        div = 4 if lower_accuracy else 1
        Wq, Hq = W // div, H // div

        def coarse(i, j):
            if not (0 <= i < Wq and 0 <= j < Hq):
                return f32(0.0)
            return count[((2 * j + 1) * H // (2 * Hq)) * W + (2 * i + 1) * W // (2 * Wq)]

        for y in range(Hq):
            for x in range(Wq):
                s = coarse(x, y)
                if s in (f32(0.63), f32(0.0), f32(4.0), f32(5.0)):
                    continue
                if all(coarse(x + dx, y + dy) == s for dy in (-1, 0, 1) for dx in (-1, 0, 1)):
                    return True
        return False

    def evaluate(nd, node):
        if nd["level"] == max_level:
            return
        kids = children(nd["level"], node)
        idx = [sample(nd, k, *corner(nd["level"], node, k)) for k in range(4)]
        if not needs_subdivision(idx):
            return
        nd["kids"] = [{"level": nd["level"] + 1, "eye": offset(nd["eye"], nd["level"] + 2, c),
                       "at": offset(nd["at"], nd["level"] + 2, c), "kids": None} for c in range(4)]
        for c in range(4):
            evaluate(nd["kids"][c], kids[c])

    def render(nd, node):
        if nd["kids"] is not None:
            for c, k in enumerate(children(nd["level"], node)):
                render(nd["kids"][c], k)
            return
        for k in range(4):
            level[sample(nd, k, *corner(nd["level"], node, k))] = f32(nd["level"])

    root = {"level": 0, "eye": [f32(v) for v in light_eye], "at": [f32(v) for v in light_at], "kids": None}
    evaluate(root, 0)
    render(root, 0)
    m = biased[-1]
    acc = np.zeros(W * H, np.float32)
    count = f32(0.0)
    offs = []
    if lower_accuracy:
        o, st = f32(1.0), (f32(2.0) * f32(1.0)) / f32(3.0)
        w = -o
        while w <= o:
            offs.append(w)
            w = w + st
    incr = f32(1.0) / f32(S)
    for i in range(len(maps)):
        b = biased[i]
        w_enc = b[15] + level[i] * f32(10000.0)
        ql = min(int(w_enc / f32(10000.0)), 4)
        wv = w_enc - f32(ql * 10000)
        f = f32(1.0)
        for _ in range(ql):
            f = f * f32(2.0)
        f = f + f32(1.0)
        wt = f32(1.0) / (f * f)
        for p in fg:
            v = [f32(c) for c in pos[p]]
            c = [(m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2] for r in range(4)]
            sx, sy, sz, sw = c[0] + b[12], c[1] + b[13], c[2] + b[14], c[3] + wv
            if not lower_accuracy:
                d = fetch(maps[i], S, S, sx / sw, sy / sw)
                acc[p] = acc[p] + (f32(1.0) if sz / sw <= d else I) * wt
            else:
                ux, uy, uz = sx / sw, sy / sw, sz / sw
                illum = f32(0.0)
                for ow in offs:
                    for oh in offs:
                        illum = illum + (f32(1.0) if uz <= fetch(maps[i], S, S, ux + ow * incr, uy + oh * incr) else I)
                acc[p] = acc[p] + (illum / f32(len(offs) * len(offs))) * wt
        count = count + wt
    out = np.zeros(W * H, np.float32)
    out[fg] = acc[fg] / count
    return out, np.array(eyes, np.float32), np.array(level, np.float32)


def edt_mean_filter(p, image, pos, W, H, order=7):
    """filterHardShadowsUsingEDT's two MeanFilter.frag passes
    (ShadowMapping/src/main.cpp:424-447; Shaders/Filter/MeanFilter.frag) with
    the library's sampling choices: the centre of pixel i at (i + 0.5) /
    size; the x pass NEAREST (texel floor(u size)), the y pass bilinear along
    y at level 0; a zero border; at most 2049 samples; dscreen = 1 / (2
    tan(45 / 2)) with the 45-degree fov uniform taken as radians, tan in
    double.  image, pos: float32 [H, W, 4]; returns float32 [H, W, 4]."""
    import math

    dscreen = f32(1.0) / (f32(2.0) * f32(math.tan(float(f32(45.0) / f32(2.0)))))
    m = p["camera_mv"]
    thr = f32(0.0005)

    def lin(d):
        return f32(2.0) / (f32(1001.0) - d * f32(999.0))

    src = image.astype(np.float32)
    for vertical in (False, True):
        dst = np.zeros((H, W, 4), np.float32)
        size = f32(H if vertical else W)
        step = f32(1.0) / size
        for y in range(H):
            for x in range(W):
                v = pos[y, x]
                if v[0] == 0:
                    dst[y, x] = (0.0, 0.0, 0.0, 1.0)
                    continue
                color = src[y, x]
                ez = ((m[2] * v[0] + m[6] * v[1]) + m[10] * v[2]) + m[14] * v[3]
                kc = ((dscreen * f32(order)) * f32(50.0)) / (-ez * f32(2.0))
                cs = (f32(y if vertical else x) + f32(0.5)) / size
                Lc = lin(color[1])
                total, count = f32(0.0), 0
                s = -kc
                while s <= kc and count < 2049:
                    u = cs + s * step
                    if not vertical:
                        fi = np.floor(u * size)
                        r, g = (src[y, int(fi), 0], src[y, int(fi), 1]) if 0 <= fi < size else (f32(0.0), f32(0.0))
                    else:
                        uu = u * size - f32(0.5)
                        f0 = np.floor(uu)
                        w1 = uu - f0
                        w0 = f32(1.0) - w1
                        j0 = int(f0)
                        t0 = src[j0, x, :2] if 0 <= j0 < H else np.zeros(2, np.float32)
                        t1 = src[j0 + 1, x, :2] if 0 <= j0 + 1 < H else np.zeros(2, np.float32)
                        r, g = w0 * t0[0] + w1 * t1[0], w0 * t0[1] + w1 * t1[1]
                    if r == 0 or abs(lin(g) - Lc) >= thr:
                        r = color[0]
                    total = total + r
                    count += 1
                    s = s + f32(1.0)
                dst[y, x] = (total / f32(count), color[1], 0.0, 0.0)
        src = dst
    return src


def edt_inputs(p, camera_mvp, vertex, normal, shadow):
    """The EDTSM outputs of NonConservativeSMSR.frag:367-397 (and
    ConservativeSMSR.frag's) for one pixel: image (shadow, depth,
    preEvaluatedShadow, 1) with depth = position.z / position.w * 0.5 + 0.5,
    and position = MVP * vertex; background keeps (0, 0, 0, 1) in both."""
    if vertex[0] == 0:
        bg = [f32(0.0), f32(0.0), f32(0.0), f32(1.0)]
        return bg, list(bg)
    pre = pretest(p, vertex, normal)
    cp = mat4_mul([f32(v) for v in np.asarray(camera_mvp, np.float32).reshape(16)], vertex)
    depth = cp[2] / cp[3]
    depth = depth * f32(0.5) + f32(0.5)
    return [shadow, depth, pre, f32(1.0)], cp
