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
LESS), but tests EVERY pixel of a triangle's bounding box with exact Python
integers, where the oracle scans a narrowed span per row.  float32
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
    """Sutherland-Hodgman against the six planes; returns the polygon's clip coordinates."""
    poly = [list(v) for v in tri]
    for k in range(6):
        d = [plane_distance(v, k) for v in poly]
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
                out.append([poly[a][q] + t * (poly[b][q] - poly[a][q]) for q in range(4)])
        poly = out
        if len(poly) < 3:
            return []
    return poly


def setup(v0, v1, v2, W, H):
    """Window coordinates of one (sub-)triangle, counter-clockwise; None if culled."""
    hw, hh = f32(0.5) * f32(W), f32(0.5) * f32(H)
    X, Y, Z = [], [], []
    for c in (v0, v1, v2):
        w = c[3]
        if not w > 0:
            return None
        xd, yd, zd = c[0] / w, c[1] / w, c[2] / w
        X.append(int(np.rint(f32(xd * hw + hw) * f32(SUB))))
        Y.append(int(np.rint(f32(yd * hh + hh) * f32(SUB))))
        Z.append(f32(zd * f32(0.5) + f32(0.5)))
    area = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0])
    if area == 0:
        return None
    if area < 0:  # clockwise: reorder to counter-clockwise
        X[1], X[2], Y[1], Y[2], Z[1], Z[2] = X[2], X[1], Y[2], Y[1], Z[2], Z[1]
        area = -area
    return X, Y, Z, area


def polygon_offset(X, Y, Z, area, factor, units):
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
    m = [f32(v) for v in np.asarray(mvp, np.float32).reshape(16)]
    pts = np.asarray(points, np.float32).reshape(-1, 3)
    tris = np.asarray(indices, np.int64).reshape(-1, 3)
    depth = np.ones(H * W, np.float32)
    for t in tris:
        poly = clip([transform(m, pts[k]) for k in t])
        for i in range(1, len(poly) - 1):
            s = setup(poly[0], poly[i], poly[i + 1], W, H)
            if s is None:
                continue
            X, Y, Z, area = s
            x0 = max(0, -((-(min(X) - SUB // 2)) // SUB))
            x1 = min(W - 1, (max(X) - SUB // 2) // SUB)
            y0 = max(0, -((-(min(Y) - SUB // 2)) // SUB))
            y1 = min(H - 1, (max(Y) - SUB // 2) // SUB)
            if x0 > x1 or y0 > y1:
                continue
            px = np.arange(x0, x1 + 1, dtype=np.int64)[None, :] * SUB + SUB // 2
            py = np.arange(y0, y1 + 1, dtype=np.int64)[:, None] * SUB + SUB // 2
            E, inside = [], np.ones((y1 - y0 + 1, x1 - x0 + 1), bool)
            for k in range(3):
                a, b = (k + 1) % 3, (k + 2) % 3
                A, B = X[b] - X[a], Y[b] - Y[a]
                e = A * (py - Y[a]) - B * (px - X[a])
                top_left = B < 0 or (B == 0 and A < 0)
                inside &= (e > 0) | ((e == 0) & top_left)
                E.append(e)
            if not inside.any():
                continue
            inv_area = f32(1.0) / f32(area)
            l1 = E[1].astype(np.float32) * inv_area
            l2 = E[2].astype(np.float32) * inv_area
            z = Z[0] + (l1 * (Z[1] - Z[0]) + l2 * (Z[2] - Z[0]))
            if bias_mode == BIAS_CONSTANT:
                z = z + f32(constant_bias)
            elif bias_mode == BIAS_POLYGON_OFFSET:
                z = z + polygon_offset(X, Y, Z, area, factor, units)
            z = np.where(z > 0, np.minimum(z, f32(1.0)), f32(0.0)).astype(np.float32)
            keep = inside & (z < 1)
            ys, xs = np.nonzero(keep)
            idx = (ys + y0) * W + (xs + x0)
            np.minimum.at(depth, idx, z[keep])
    return depth
