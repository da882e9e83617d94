"""A second restatement of the depth-map rasterisation rules (test helper).

The light-map pass written again with numpy, independently of the C++
oracle, so the CPU tests can hold the oracle's rasteriser to it bit for bit.
It follows the rules the library fixes where the reference leaves them to
the GL driver (clip = MVP (x, y, z, 1); Sutherland-Hodgman clipping against
z >= -w, z <= w and the |x|, |y| <= 16 w guard band, intersections taken from
the inside vertex, the polygon fanned from vertex 0; window coordinates
snapped to 8 sub-pixel bits, round to nearest even; integer edge functions
at pixel centres with the top-left rule of the counter-clockwise triangle;
depth linear in window space from l_i = E_i (1 / area); polygon offset
m factor + 2^(e - 23) units; depth clamped to [0, 1], cleared to 1, test
LESS; for the G-buffer the nearest fragment, first in draw order among
equals, its attributes interpolated perspective-correct), but tests EVERY
pixel of a triangle's bounding box with exact integers, where the oracle
scans a narrowed span per row.  float32
arithmetic rounds once per operation in the written order (numpy scalars
and arrays, no fused multiply-add).
"""
from __future__ import annotations

import numpy as np

f32 = np.float32
SUB_BITS = 8
SUB = 1 << SUB_BITS
GUARD = f32(16.0)
BIAS_NONE, BIAS_CONSTANT, BIAS_POLYGON_OFFSET = 0, 1, 2


def transform(m, p):
    """Column-major mat4 times (x, y, z, 1), rows summed left to right."""
    x, y, z = f32(p[0]), f32(p[1]), f32(p[2])
    return [((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] for r in range(4)]


def plane_distance(c, k):
    x, y, z, w = c
    return (z + w, w - z, x + GUARD * w, GUARD * w - x, y + GUARD * w, GUARD * w - y)[k]


def clip(tri):
    """Sutherland-Hodgman against the six planes.  tri: three clip-space
    vertices; returns the polygon as (clip coordinates, barycentric weights
    with respect to the source triangle) pairs."""
    one = [f32(1.0), f32(0.0), f32(0.0)]
    poly = [(list(tri[k]), [one[(j - k) % 3] for j in range(3)]) for k in range(3)]
    for k in range(6):
        d = [plane_distance(v[0], k) for v in poly]
        inside = [di >= 0 for di in d]
        if not any(inside):
            return []
        if all(inside):
            continue
        out = []
        n = len(poly)
        for i in range(n):
            j = (i + 1) % n
            if inside[i]:
                out.append(poly[i])
            if inside[i] != inside[j]:
                a, b, da, db = (i, j, d[i], d[j]) if inside[i] else (j, i, d[j], d[i])
                t = da / (da - db)
                (ca, ba), (cb, bb) = poly[a], poly[b]
                out.append(([ca[q] + t * (cb[q] - ca[q]) for q in range(4)],
                            [ba[q] + t * (bb[q] - ba[q]) for q in range(3)]))
        poly = out
        if len(poly) < 3:
            return []
    return poly


def setup(v0, v1, v2, W, H):
    """Window coordinates of one (sub-)triangle, reordered counter-clockwise:
    a dict with X, Y (sub-pixel integers), Z (window depth), iw (1 / clip w),
    b (source barycentric rows), area and front (counter-clockwise as drawn);
    None if culled."""
    hw, hh = f32(0.5) * f32(W), f32(0.5) * f32(H)
    X, Y, Z, Wc, Bw = [], [], [], [], []
    for c, bary in (v0, v1, v2):
        w = c[3]
        if not w > 0:
            return None
        xd, yd, zd = c[0] / w, c[1] / w, c[2] / w
        X.append(int(np.rint(f32(xd * hw + hw) * f32(SUB))))
        Y.append(int(np.rint(f32(yd * hh + hh) * f32(SUB))))
        Z.append(f32(zd * f32(0.5) + f32(0.5)))
        Wc.append(w)
        Bw.append(bary)
    area = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0])
    if area == 0:
        return None
    front = area > 0
    if area < 0:  # clockwise: reorder to counter-clockwise
        for L in (X, Y, Z, Wc, Bw):
            L[1], L[2] = L[2], L[1]
        area = -area
    return {"X": X, "Y": Y, "Z": Z, "iw": [f32(1.0) / w for w in Wc], "b": Bw, "area": area, "front": front,
            "inv_area": f32(1.0) / f32(area)}


def edges(s, px, py):
    """Edge values (opposite vertex 0, 1, 2) at pixel centres px, py and the inside mask."""
    X, Y = s["X"], s["Y"]
    E, inside = [], True
    for k in range(3):
        a, b = (k + 1) % 3, (k + 2) % 3
        A, B = X[b] - X[a], Y[b] - Y[a]
        e = A * (py - Y[a]) - B * (px - X[a])
        top_left = B < 0 or (B == 0 and A < 0)
        inside = inside & ((e > 0) | ((e == 0) & top_left))
        E.append(e)
    return E, inside


def fragments(points, indices, mvp, W, H):
    """Every covered pixel of every (sub-)triangle, each bounding-box pixel
    tested: yields (triangle, sub-triangle, setup, rows, columns, E, depth)."""
    m = [f32(v) for v in np.asarray(mvp, np.float32).reshape(16)]
    pts = np.asarray(points, np.float32).reshape(-1, 3)
    tris = np.asarray(indices, np.int64).reshape(-1, 3)
    for t, tri in enumerate(tris):
        poly = clip([transform(m, pts[k]) for k in tri])
        for i in range(1, len(poly) - 1):
            s = setup(poly[0], poly[i], poly[i + 1], W, H)
            if s is None:
                continue
            X, Y, Z = s["X"], s["Y"], s["Z"]
            x0 = max(0, -((-(min(X) - SUB // 2)) // SUB))
            x1 = min(W - 1, (max(X) - SUB // 2) // SUB)
            y0 = max(0, -((-(min(Y) - SUB // 2)) // SUB))
            y1 = min(H - 1, (max(Y) - SUB // 2) // SUB)
            if x0 > x1 or y0 > y1:
                continue
            px = np.arange(x0, x1 + 1, dtype=np.int64)[None, :] * SUB + SUB // 2
            py = np.arange(y0, y1 + 1, dtype=np.int64)[:, None] * SUB + SUB // 2
            E, inside = edges(s, px, py)
            if not inside.any():
                continue
            ys, xs = np.nonzero(inside)
            E = [e[inside] for e in E]
            l1 = E[1].astype(np.float32) * s["inv_area"]
            l2 = E[2].astype(np.float32) * s["inv_area"]
            z = Z[0] + (l1 * (Z[1] - Z[0]) + l2 * (Z[2] - Z[0]))
            yield t, i - 1, s, ys + y0, xs + x0, E, z


def clamp01(z):
    return np.where(z > 0, np.minimum(z, f32(1.0)), f32(0.0)).astype(np.float32)


def polygon_offset(s, factor, units):
    X, Y, Z, area = s["X"], s["Y"], s["Z"], s["area"]
    fx1, fy1 = f32(X[1] - X[0]), f32(Y[1] - Y[0])
    fx2, fy2 = f32(X[2] - X[0]), f32(Y[2] - Y[0])
    dz1, dz2 = Z[1] - Z[0], Z[2] - Z[0]
    fa = f32(area)
    dzdx = ((dz1 * fy2 - dz2 * fy1) / fa) * f32(SUB)
    dzdy = ((dz2 * fx1 - dz1 * fx2) / fa) * f32(SUB)
    m = max(abs(dzdx), abs(dzdy))
    zmax = max(Z)
    e = -126
    if zmax > 0:
        mant, ex = np.frexp(zmax)  # zmax = mant 2^ex, mant in [0.5, 1)
        e = max(int(ex) - 1, -126)
    return m * f32(factor) + f32(2.0 ** (e - 23)) * f32(units)


def shadow_map(points, indices, mvp, W, H, bias_mode=BIAS_NONE, constant_bias=0.0, factor=0.0, units=0.0):
    """Depth map (float32 [H * W], cleared to 1, LESS) of a triangle mesh."""
    depth = np.ones(H * W, np.float32)
    for _, _, s, ys, xs, _, z in fragments(points, indices, mvp, W, H):
        if bias_mode == BIAS_CONSTANT:
            z = z + f32(constant_bias)
        elif bias_mode == BIAS_POLYGON_OFFSET:
            z = z + polygon_offset(s, factor, units)
        z = clamp01(z)
        keep = z < 1
        np.minimum.at(depth, ys[keep] * W + xs[keep], z[keep])
    return depth


def gbuffer(points, normals, indices, mvp, W, H):
    """Positions and normals (float32 [H * W, 4] each) of the nearest
    fragment, the first in draw order among equals: the key of a fragment
    is its depth bits above triangle * 8 + sub-triangle, the smallest wins;
    the winner's attributes are interpolated perspective-correct."""
    clear = (np.uint64(0x3F800000) << np.uint64(32)) | np.uint64(0xFFFFFFFF)
    keys = np.full(H * W, clear, np.uint64)
    setups = {}
    for t, sub, s, ys, xs, _, z in fragments(points, indices, mvp, W, H):
        setups[(t, sub)] = s
        z = clamp01(z)
        keep = z < 1
        k = (z[keep].view(np.uint32).astype(np.uint64) << np.uint64(32)) | np.uint64(t * 8 + sub)
        np.minimum.at(keys, ys[keep] * W + xs[keep], k)
    pts = np.asarray(points, np.float32).reshape(-1, 3)
    nrm = np.asarray(normals, np.float32).reshape(-1, 3)
    tris = np.asarray(indices, np.int64).reshape(-1, 3)
    pos = np.zeros((H * W, 4), np.float32)
    out_n = np.zeros((H * W, 4), np.float32)
    pos[:, 3] = 1.0
    out_n[:, 3] = 1.0
    for p in np.flatnonzero(keys != clear):
        prim = int(keys[p] & np.uint64(0xFFFFFFFF))
        t, sub = prim >> 3, prim & 7
        s = setups[(t, sub)]
        y, x = divmod(int(p), W)
        E, _ = edges(s, x * SUB + SUB // 2, y * SUB + SUB // 2)
        q = [(f32(E[j]) * s["inv_area"]) * s["iw"][j] for j in range(3)]
        total = (q[0] + q[1]) + q[2]
        pc = [q[j] / total for j in range(3)]
        B = [(pc[0] * s["b"][0][j] + pc[1] * s["b"][1][j]) + pc[2] * s["b"][2][j] for j in range(3)]
        P = [pts[v] for v in tris[t]]
        N = [nrm[v] for v in tris[t]]
        for j in range(3):
            pos[p, j] = (B[0] * P[0][j] + B[1] * P[1][j]) + B[2] * P[2][j]
            out_n[p, j] = (B[0] * N[0][j] + B[1] * N[1][j]) + B[2] * N[2][j]
        out_n[p, 3] = 1.0 if s["front"] else 0.0
    return pos.reshape(-1), out_n.reshape(-1)


def stencil_counts(points, indices, volume_triangles, mvp, W, H, less_equal):
    """ShadowVolumes' stencil pass (ShadowVolumes/src/main.cpp:150-172): the
    depth prepass (no bias), then every volume triangle drawn against it with
    LESS (or LEQUAL), +1 for a front-facing and -1 for a back-facing
    fragment that passes, the sum wrapped to 8 bits.  volume_triangles:
    float32 [n, 3, 3] world-space triangles."""
    depth = shadow_map(points, indices, mvp, W, H)
    count = np.zeros(H * W, np.int64)
    vt = np.asarray(volume_triangles, np.float32).reshape(-1, 3)
    tri = np.arange(len(vt), dtype=np.int64).reshape(-1, 3)
    for _, _, s, ys, xs, _, z in fragments(vt, tri, mvp, W, H):
        z = clamp01(z)
        idx = ys * W + xs
        d = depth[idx]
        passed = (z <= d) if less_equal else (z < d)
        np.add.at(count, idx[passed], 1 if s["front"] else -1)
    return (count & 0xFF).astype(np.uint8), depth
