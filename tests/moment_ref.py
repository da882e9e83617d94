"""A second, numpy restatement of the filtered moment shadow maps (test helper).

ShadowMapping's VSM, ESM, EVSM and MSM path written again with numpy
float32 arithmetic, independently of the C++ oracle: the light pass's moment
targets (Shaders/ShadowMap/Moments.frag, Exponential.frag,
ExponentialMoments.frag), the separable 7-tap Gaussian blur into the window-
size targets (src/main.cpp:374-396; Shaders/Filter/GaussianFilter.frag and,
for ESM, LogGaussianFilter.frag) and the lookups of Shaders/Shadow.frag:
118-220.  The choices GL leaves to the driver are the library's: moments
from the depth map's values (an empty texel, depth 1, keeps the clear
colour (0, 0, 0, 1)); dFdx / dFdy as the differences inside each 2 x 2
quad, 0 next to an empty texel; the map reduced to the window size by 2 x 2
box averages ((a + b) + (c + d)) * 0.25; the 7 taps on texel centres with a
zero border, each product and sum rounded in tap order; lookups bilinear at
level 0 with float32 weights and a zero border.  exp and log are the C
library's expf / logf (ctypes), as the oracle calls them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

f32 = np.float32
VSM, ESM, EVSM, MSM = 12, 13, 14, 15
GAUSS7 = [f32(1.0 / 64.0), f32(6.0 / 64.0), f32(15.0 / 64.0), f32(20.0 / 64.0), f32(15.0 / 64.0),
          f32(6.0 / 64.0), f32(1.0 / 64.0)]
Q_ROWS = [[-2.07224649, 32.2370378, -68.5710746, 39.3703274],
          [13.7948857, -59.4683976, 82.035975, -35.3649032],
          [0.105877704, -1.90774663, 9.34965551, -6.65434907],
          [9.79240621, -33.76521106, 47.9456097, -23.9728048]]
TQ0 = f32(0.0359558848)

_libm = C.CDLL("libm.so.6")
for _name in ("expf", "logf"):
    getattr(_libm, _name).restype = C.c_float
    getattr(_libm, _name).argtypes = [C.c_float]


def expf(x):
    return f32(_libm.expf(float(x)))


def logf(x):
    return f32(_libm.logf(float(x)))


def linearize(d):
    """Shadow.frag / Moments.frag linearize with zNear 1, zFar 1000."""
    return f32(2.0) / (f32(1001.0) - d * f32(999.0))


def quantization():
    """MyGLGeometryViewer::configureMoments' matrix (column-major float32) and
    its inverse, Gauss-Jordan with partial pivoting in double on the float
    matrix, rounded to float32."""
    q = [[float(f32(v)) for v in row] for row in Q_ROWS]
    mq = [f32(0.0)] * 16
    for r in range(4):
        for c in range(4):
            mq[c * 4 + r] = f32(q[r][c])
    a = [q[r][:] + [1.0 if r == c else 0.0 for c in range(4)] for r in range(4)]
    for c in range(4):
        piv = c
        for r in range(c + 1, 4):
            if abs(a[r][c]) > abs(a[piv][c]):
                piv = r
        a[c], a[piv] = a[piv], a[c]
        inv = 1.0 / a[c][c]
        a[c] = [v * inv for v in a[c]]
        for r in range(4):
            if r != c:
                f = a[r][c]
                a[r] = [a[r][k] - f * a[c][k] for k in range(8)]
    mqi = [f32(0.0)] * 16
    for r in range(4):
        for c in range(4):
            mqi[c * 4 + r] = f32(a[r][c + 4])
    return mq, mqi


def moment_map(tech, depth, S):
    """The light pass's moment target, float32 [S, S, 4]."""
    d = depth.reshape(S, S).astype(np.float32)
    empty = ~(d < 1)
    lin = linearize(d)
    out = np.zeros((S, S, 4), np.float32)
    if tech == ESM:
        out[..., 0] = lin
        out[..., 3] = 1.0
    elif tech == MSM:
        mq, _ = quantization()
        d2 = lin * lin
        d3 = d2 * lin
        d4 = d3 * lin
        for r in range(4):
            v = mq[r] * lin + mq[4 + r] * d2
            v = v + mq[8 + r] * d3
            v = v + mq[12 + r] * d4
            out[..., r] = v + (TQ0 if r == 0 else f32(0.0))
    else:
        xs = np.arange(S)
        left = xs & ~1
        right = np.where((xs | 1) < S, xs | 1, xs)
        dx = np.where(empty[:, left] | empty[:, right], f32(0.0), lin[:, right] - lin[:, left]).astype(np.float32)
        dy = np.where(empty[left, :] | empty[right, :], f32(0.0), lin[right, :] - lin[left, :]).astype(np.float32)
        m2 = lin * lin
        m2 = m2 + f32(0.25) * (dx * dx + dy * dy)
        out[..., 0] = lin
        out[..., 1] = m2
        if tech == EVSM:
            out[..., 2] = lin
            out[..., 3] = 1.0
    out[empty] = (0.0, 0.0, 0.0, 1.0)
    return out


def filtered(tech, depth, S, W):
    """The blurred window-size target, float32 [W, W, 4]."""
    m = moment_map(tech, depth, S)
    side = S
    while side > W:
        a, b = m[0::2, 0::2], m[0::2, 1::2]
        c, d = m[1::2, 0::2], m[1::2, 1::2]
        m = ((a + b) + (c + d)) * f32(0.25)
        side //= 2

    def blur(img, dx, dy):
        pad = np.zeros((W + 6, W + 6, 4), np.float32)
        pad[3:3 + W, 3:3 + W] = img

        def tap(k):
            return pad[3 + dy * k:3 + dy * k + W, 3 + dx * k:3 + dx * k + W]

        if tech != ESM:
            r = np.zeros((W, W, 4), np.float32)
            for k in range(-3, 4):
                r = r + tap(k) * GAUSS7[3 + k]
            return r
        out = np.zeros((W, W, 4), np.float32)
        t = [tap(k)[..., 0] for k in range(-3, 4)]
        for y in range(W):
            for x in range(W):
                s0, s1 = t[0][y, x], t[1][y, x]
                s = s0 + logf(GAUSS7[0] + GAUSS7[1] * expf(s1 - s0))
                for i in range(2, 7):
                    s = s + logf(f32(1.0) + GAUSS7[i] * expf(t[i][y, x] - s))
                out[y, x] = s
        return out

    return blur(blur(m, 1, 0), 0, 1)


def fetch(mm, W, s, t):
    """Bilinear at level 0, float32 weights, zero border."""
    u, v = s * f32(W) - f32(0.5), t * f32(W) - f32(0.5)
    if not (u > -2 and u < f32(W) + 1 and v > -2 and v < f32(W) + 1):
        return [f32(0.0)] * 4
    fu, fv = np.floor(u), np.floor(v)
    i0, j0 = int(fu), int(fv)
    a, b = u - fu, v - fv
    w = [(f32(1.0) - a) * (f32(1.0) - b), a * (f32(1.0) - b), (f32(1.0) - a) * b, a * b]
    T = []
    for k in range(4):
        i, j = i0 + (k & 1), j0 + (k >> 1)
        T.append(mm[j, i] if 0 <= i < W and 0 <= j < W else np.zeros(4, np.float32))
    return [((w[0] * T[0][ch] + w[1] * T[1][ch]) + w[2] * T[2][ch]) + w[3] * T[3][ch] for ch in range(4)]


def mix(x, y, a):
    return x * (f32(1.0) - a) + y * a


def clamp(x, lo, hi):
    return min(max(x, lo), hi)


def chebyshev(mx, my, z, I):
    if z <= mx:
        return f32(1.0)
    variance = my - mx * mx
    d = z - mx
    p_max = variance / (variance + d * d)
    p = f32(1.0) if z <= mx else f32(0.0)
    return mix(max(p, p_max), f32(1.0), I)


def lookup(tech, mm, W, n, I):
    """The Shadow.frag lookup at the normalised light coordinate n."""
    if tech == VSM:
        m = fetch(mm, W, n[0], n[1])
        return chebyshev(m[0], m[1], linearize(n[2]), I)
    if tech == ESM:
        e2 = expf(f32(80.0) * fetch(mm, W, n[0], n[1])[0])
        e1 = expf(-f32(80.0) * linearize(n[2]))
        return clamp(e1 * e2, I, f32(1.0))
    if tech == EVSM:
        z = linearize(n[2])
        m = fetch(mm, W, n[0], n[1])
        variance = chebyshev(m[0], m[1], z, I)
        e1 = expf(-f32(60.0) * z)
        e2 = expf(f32(60.0) * m[2])
        return min(variance, clamp(e1 * e2, I, f32(1.0)))
    _, mqi = quantization()
    b = fetch(mm, W, n[0], n[1])
    b = [b[0] - TQ0, b[1] - f32(0.0), b[2] - f32(0.0), b[3] - f32(0.0)]
    b = [((mqi[r] * b[0] + mqi[4 + r] * b[1]) + mqi[8 + r] * b[2]) + mqi[12 + r] * b[3] for r in range(4)]
    bias = f32(0.00003)
    ob, hb = f32(1.0) - bias, bias * f32(0.5)
    b = [ob * v + hb for v in b]
    z0 = linearize(n[2])
    dx, dy, dz = f32(1.0), z0, z0 * z0
    L10, L20 = b[0], b[1]
    D11 = b[1] - L10 * L10
    L21 = (b[2] - L20 * L10) / D11
    D22 = (b[3] - L20 * L20) - (L21 * L21) * D11
    y0 = dx
    y1 = dy - L10 * y0
    y2 = (dz - L20 * y0) - L21 * y1
    y1 = y1 / D11
    y2 = y2 / D22
    cz = y2
    cy = y1 - L21 * cz
    cx = (y0 - L10 * cy) - L20 * cz
    p, q = cy / cz, cx / cz
    D = ((p * p) / f32(4.0)) - q
    with np.errstate(invalid="ignore"):  # D < 0 gives NaN, as sqrt does in the shader
        r = np.sqrt(D)
    zy, zz = -(p / f32(2.0)) - r, -(p / f32(2.0)) + r
    if z0 <= zy:
        return f32(1.0)
    if z0 <= zz:
        return clamp(f32(1.0) - clamp((z0 * zz - b[0] * (z0 + zz) + b[1]) / ((zz - zy) * (z0 - zy)), f32(0.0), f32(1.0)),
                     I, f32(1.0))
    return clamp(f32(1.0) - clamp(f32(1.0) - (zy * zz - b[0] * (zy + zz) + b[1]) / ((z0 - zy) * (z0 - zz)), f32(0.0),
                                  f32(1.0)), I, f32(1.0))
