"""A second, numpy restatement of the moment soft shadows (test helper).

SoftShadowMapping's SAVSM / VSSM / ESSM / MSSM path written again with
numpy float32 arithmetic (every operation rounds to float32, in the order
the shaders write it), independently of the C++ oracle, so the CPU tests can
pin the oracle bit for bit: the light-pass moment map (Shaders/Moments/
Moments.frag, Shaders/Exponential.frag), the summed-area table
(SAT{Horizontal,Vertical}Pass.frag, src/main.cpp:943-971), the min-max map
(PrepareMinMax.frag, MinMax.frag, main.cpp:696-751) and the per-pixel
lookups of Shaders/SoftShadow/PlausibleSoftShadow.frag for single probes.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

f32 = np.float32
ZERO = f32(0.0)

# MyGLGeometryViewer::configureMoments: rows of the 4MSM quantisation
Q_ROWS = [[-2.07224649, 32.2370378, -68.5710746, 39.3703274],
          [13.7948857, -59.4683976, 82.035975, -35.3649032],
          [0.105877704, -1.90774663, 9.34965551, -6.65434907],
          [9.79240621, -33.76521106, 47.9456097, -23.9728048]]
TQ0 = f32(0.0359558848)


def logf(x: float) -> float:
    libm = C.CDLL("libm.so.6")
    libm.logf.restype = C.c_float
    libm.logf.argtypes = [C.c_float]
    return libm.logf(x)


def sat_iterations(S: int) -> int:
    """main.cpp:943: int m = std::logf(shadowMapWidth) / std::logf(2), in float."""
    return int(f32(logf(float(S))) / f32(logf(2.0)))


def linearize(d):
    return f32(2.0) / (f32(1001.0) - d * f32(999.0))


def nonlinearize(d):
    # d == 0 divides by zero and gives -inf, as the shader's IEEE division does
    with np.errstate(divide="ignore"):
        return -(f32(2.0) - d * f32(1001.0)) / (d * f32(999.0))


def msm_inverse():
    """The float quantisation matrix inverted in double (column-major, as the shader gets it)."""
    q = np.array(Q_ROWS, np.float32).astype(np.float64)
    a = np.concatenate([q, np.eye(4)], axis=1)
    for c in range(4):
        piv = c + int(np.argmax(np.abs(a[c:, c])))  # the first of equal magnitudes
        a[[c, piv]] = a[[piv, c]]
        a[c] *= 1.0 / a[c, c]
        for r in range(4):
            if r != c:
                a[r] -= a[r, c] * a[c]
    inv = a[:, 4:].astype(np.float32)
    return inv.T.reshape(-1)  # column-major


def moment_map(tech: str, depth: np.ndarray) -> np.ndarray:
    """depth: float32 [T, S] light map -> float32 [T, S, 4]."""
    T, S = depth.shape
    empty = ~(depth < f32(1.0))
    lin = linearize(depth.astype(np.float32))
    out = np.zeros((T, S, 4), np.float32)
    if tech == "essm":
        with np.errstate(over="ignore"):
            e = np.exp(f32(80.0) * lin)
        m = np.stack([lin, e, e * lin, np.zeros_like(lin)], -1)
    elif tech == "mssm":
        q = np.array(Q_ROWS, np.float32)
        d2 = lin * lin
        d3 = d2 * lin
        d4 = d3 * lin
        m = np.stack([q[r, 0] * lin + q[r, 1] * d2 + q[r, 2] * d3 + q[r, 3] * d4 + (TQ0 if r == 0 else ZERO)
                      for r in range(4)], -1)
    else:
        xs, ys = np.arange(S), np.arange(T)
        xl, xr = xs & ~1, np.where((xs | 1) < S, xs | 1, xs)
        yb, yt = ys & ~1, np.where((ys | 1) < T, ys | 1, ys)
        l, r = lin[:, xl], lin[:, xr]
        b, t = lin[yb, :], lin[yt, :]
        dx = np.where(empty[:, xl] | empty[:, xr], ZERO, r - l)
        dy = np.where(empty[yb, :] | empty[yt, :], ZERO, t - b)
        m = np.stack([lin - f32(0.5), lin * lin + (f32(0.25) * (dx * dx + dy * dy) - f32(0.5)),
                      np.zeros_like(lin), np.zeros_like(lin)], -1)
    out[~empty] = m[~empty]
    return out


def summed_area_table(m: np.ndarray) -> np.ndarray:
    """Interleaved horizontal / vertical passes at offsets 2^i, border 0."""
    s = m.astype(np.float32).copy()
    T, S = s.shape[:2]
    for i in range(sat_iterations(S)):
        d = 1 << i
        t = s + ZERO
        t[:, d:] = s[:, d:] + s[:, :S - d] if d < S else t[:, d:]
        s = t + ZERO
        if d < T:
            s[d:] = t[d:] + t[:T - d]
    return s


def hsm_levels(depth: np.ndarray, alpha: float, beta: float, L: int):
    """Levels 0..L of the min-max map, float32 [h, w, 2] each."""
    d = depth.astype(np.float32)
    lv = [np.stack([np.where(d == f32(0.0), f32(1.0), d) + f32(alpha), d + f32(beta)], -1)]
    q = f32(0.25)
    for _ in range(L):
        p = lv[-1]
        ph, pw = p.shape[:2]
        h, w = ph // 2, pw // 2
        pad = np.zeros((ph + 8, pw + 8, 2), np.float32)  # border 0, 4 texels each side
        pad[4:4 + ph, 4:4 + pw] = p

        def quad(i0, j0):  # 2 x 2 blocks from (i0, j0) for all output texels, bilinear weights 0.25
            ii = 2 * np.arange(w)[None, :] + i0 + 4
            jj = 2 * np.arange(h)[:, None] + j0 + 4
            return ((q * pad[jj, ii] + q * pad[jj, ii + 1]) + q * pad[jj + 1, ii]) + q * pad[jj + 1, ii + 1]

        v0, v1, v2, v3 = quad(-2, -2), quad(-2, 2), quad(2, -2), quad(2, 2)
        gmin = lambda a, b: np.where(b < a, b, a)
        gmax = lambda a, b: np.where(a < b, b, a)
        mn = gmin(v0[..., 0], gmin(v1[..., 0], gmin(v2[..., 0], v3[..., 0])))
        mx = gmax(v0[..., 1], gmax(v1[..., 1], gmax(v2[..., 1], v3[..., 1])))
        lv.append(np.stack([mn, mx], -1))
    return lv


# ---- per-probe lookups (numpy float32 scalars) --------------------------------
def bilinear(tex: np.ndarray, s, t):
    H, W = tex.shape[:2]
    u, v = s * f32(W) - f32(0.5), t * f32(H) - f32(0.5)
    nch = tex.shape[2]
    if not (u > f32(-2.0) and u < f32(W) + f32(1.0) and v > f32(-2.0) and v < f32(H) + f32(1.0)):
        return np.zeros(nch, np.float32)
    fu, fv = f32(math.floor(u)), f32(math.floor(v))
    i0, j0 = int(fu), int(fv)
    a, b = u - fu, v - fv
    one = f32(1.0)
    w = [(one - a) * (one - b), a * (one - b), (one - a) * b, a * b]
    T = []
    for k in range(4):
        i, j = i0 + (k & 1), j0 + (k >> 1)
        T.append(tex[j, i] if 0 <= i < W and 0 <= j < H else np.zeros(nch, np.float32))
    return ((w[0] * T[0] + w[1] * T[1]) + w[2] * T[2]) + w[3] * T[3]


def gmin(x, y):
    return y if y < x else x


def gmax(x, y):
    return y if x < y else x


def gclamp(x, lo, hi):
    return gmin(gmax(x, lo), hi)


def cheb(mx, my, z):
    if z <= mx:
        return f32(1.0)
    var = my - mx * mx
    d = z - mx
    pm = var / (var + d * d)
    return gmax(f32(1.0) if z <= mx else ZERO, pm)


class Probe:
    """Lookups of one technique over one light map (square S x S)."""

    def __init__(self, tech, depth, *, sat, intensity=0.25, light_radius=8.0, blocker=7, kernel=7,
                 min_blocker=0.99, alpha=0.0, beta=0.0):
        self.tech, self.depth, self.sat = tech, depth.astype(np.float32), sat
        self.S = depth.shape[1]
        self.I, self.R = f32(intensity), f32(light_radius)
        self.B, self.K, self.minb = blocker, kernel, f32(min_blocker)
        m = moment_map(tech, depth)
        self.mom = summed_area_table(m) if sat else m
        if tech == "vssm":
            lod = f32(1.75) if self.S > 1024 else f32(self.S) / f32(1024.0) + f32(0.5)
            lo = int(math.floor(lod))
            lv = hsm_levels(depth, alpha, beta, lo + 1)
            self.lo, self.hi, self.frac = lv[lo], lv[lo + 1], lod - f32(lo)
        self.mqi = msm_inverse()

    def fetch_depth(self, s, t):
        W = self.S
        fi, fj = f32(math.floor(s * f32(W))), f32(math.floor(t * f32(W)))
        if not (fi >= 0 and fi < W and fj >= 0 and fj < W):
            return ZERO
        return self.depth[int(fj), int(fi)]

    def bsw(self):
        return self.R / f32(self.S) if f32(self.S) <= f32(1024.0) else self.R / f32(1024.0)

    def box(self, n, width, step, count):
        if self.sat:
            div = f32(2.0) * width / step
            size = div / f32(2.0)
            xmax, xmin = n[0] + div * step, n[0] - (div + f32(1.0)) * step
            ymax, ymin = n[1] + div * step, n[1] - (div + f32(1.0)) * step
            A, B = bilinear(self.mom, xmin, ymin), bilinear(self.mom, xmax, ymin)
            Cc, D = bilinear(self.mom, xmin, ymax), bilinear(self.mom, xmax, ymax)
            return (((D + A) - B) - Cc) / (size * size)
        fw = (f32(count) - f32(1.0)) * f32(0.5)
        acc = np.zeros(4, np.float32)
        h = int(-fw)
        while f32(h) <= fw:
            w = int(-fw)
            while f32(w) <= fw:
                acc = acc + bilinear(self.mom, n[0] + (f32(w) * width) / fw, n[1] + (f32(h) * width) / fw)
                w += 1
            h += 1
        return acc / f32(count * count)

    def blocker_pcf(self, n):
        avg, nb = ZERO, 0
        bsw = self.bsw()
        fw = (f32(self.B) - f32(1.0)) * f32(0.5)
        h = int(-fw)
        while f32(h) <= fw:
            w = int(-fw)
            while f32(w) <= fw:
                d = self.fetch_depth(n[0] + (f32(w) * bsw) / fw, n[1] + (f32(h) * bsw) / fw)
                if n[2] > d:
                    avg = avg + d
                    nb += 1
                w += 1
            h += 1
        return f32(1.0) if nb == 0 else avg / f32(nb)

    def penumbra(self, avg, z):
        if avg < self.minb:
            return ZERO
        pw = ((z - avg) / avg) * self.R
        return (f32(1.0) * pw) / z

    def vsm(self, pw, n):
        step = f32(2.0) * pw / f32(self.K)
        if step <= 0 or step >= 1:
            return f32(1.0)
        m = self.box(n, pw, step, self.K)
        mx, my = m[0] + f32(0.5), m[1] + f32(0.5)
        c = cheb(mx, my, linearize(n[2]))
        return gclamp(c * (f32(1.0) - self.I) + f32(1.0) * self.I, ZERO, f32(1.0))

    def vsm_blocker(self, n):
        bsw = self.bsw()
        step = f32(2.0) * bsw / f32(self.B)
        zun = linearize(n[2])
        m = self.box(n, bsw, step, self.B)
        mx, my = m[0] + f32(0.5), m[1] + f32(0.5)
        prob = cheb(mx, my, zun)
        with np.errstate(divide="ignore", invalid="ignore"):
            zocc = nonlinearize((mx - prob * zun) / (f32(1.0) - prob))
        return f32(1.0) if prob > f32(0.99) else zocc

    def hsm(self, n):
        lo, hi, f = bilinear(self.lo, n[0], n[1]), bilinear(self.hi, n[0], n[1]), self.frac
        one = f32(1.0)
        mn, mx = (one - f) * lo[0] + f * hi[0], (one - f) * lo[1] + f * hi[1]
        if n[2] <= mn:
            return one
        if n[2] > mx:
            return self.I
        return f32(0.555)

    def msm_solve(self, m, lz):
        b = m - np.array([TQ0, 0, 0, 0], np.float32)
        mi = self.mqi
        b = np.array([mi[r] * b[0] + mi[4 + r] * b[1] + mi[8 + r] * b[2] + mi[12 + r] * b[3] for r in range(4)],
                     np.float32)
        bias = f32(0.00003)
        b = (f32(1.0) - bias) * b + bias * f32(0.5)
        L10, L20 = b[0], b[1]
        D11 = b[1] - L10 * L10
        L21 = (b[2] - L20 * L10) / D11
        D22 = b[3] - L20 * L20 - L21 * L21 * D11
        y0 = f32(1.0)
        y1 = lz - L10 * y0
        y2 = lz * lz - L20 * y0 - L21 * y1
        y1, y2 = y1 / D11, y2 / D22
        cz = y2
        cy = y1 - L21 * cz
        cx = y0 - L10 * cy - L20 * cz
        p, q = cy / cz, cx / cz
        with np.errstate(invalid="ignore"):
            r = np.sqrt(((p * p) / f32(4.0)) - q)
        return b, lz, -(p / f32(2.0)) - r, -(p / f32(2.0)) + r

    def msm(self, pw, n):
        step = f32(2.0) * pw / f32(self.K)
        if step <= 0 or step >= 1:
            return f32(1.0)
        b, zx, zy, zz = self.msm_solve(self.box(n, pw, step, self.K), linearize(n[2]))
        one = f32(1.0)
        if zx <= zy:
            return one
        if zx <= zz:
            return gclamp(one - gclamp((zx * zz - b[0] * (zx + zz) + b[1]) / ((zz - zy) * (zx - zy)), ZERO, one),
                          self.I, one)
        return gclamp(one - gclamp(one - (zy * zz - b[0] * (zy + zz) + b[1]) / ((zx - zy) * (zx - zz)), ZERO, one),
                      self.I, one)

    def msm_blocker(self, n):
        bias = f32(0.01)
        bsw = self.R / f32(self.S)
        step = f32(2.0) * bsw / f32(self.B)
        b, zx, zy, zz = self.msm_solve(self.box(n, bsw, step, self.B), linearize(n[2]))
        wx = (zy * zz - b[0] * (zy + zz) + b[1]) / ((zx - zy) * (zx - zz))
        wy = (zx * zz - b[0] * (zx + zz) + b[1]) / ((zz - zy) * (zx - zy))
        wz = f32(1.0) - wx - wy
        ky, kz = f32(1.0) - wy, f32(1.0) - wz
        avg, sm = ZERO, ZERO
        if zx > zy:
            avg, sm = avg + ky * zy, sm + ky
        if zx > zz:
            avg, sm = avg + kz * zz, sm + kz
        avg, sm = avg + bias * zx, sm + bias
        if sm > f32(1.0) - bias:
            return f32(1.0)
        return nonlinearize(avg / sm)

    def esm_blocker(self, n):
        bsw = self.bsw()
        step = f32(2.0) * bsw / f32(self.B)
        s = self.box(n, bsw, step, self.B)
        lz = linearize(n[2])
        prob = np.exp(f32(-80.0) * lz) * s[1]
        if prob > f32(0.91):
            return f32(1.0)
        return nonlinearize((s[0] - np.exp(f32(-80.0) * lz) * s[2]) / (f32(1.0) - prob))

    def esm(self, pw, n):
        step = f32(2.0) * pw / f32(self.K)
        if step <= 0 or step >= 1:
            return f32(1.0)
        avg = self.box(n, pw, step, self.K)[1]
        dist = bilinear(self.mom, n[0], n[1])[0] + f32(0.0001)
        lz = linearize(n[2])
        v = gclamp(np.exp(f32(-80.0) * lz) * avg, self.I, f32(1.0))
        return f32(1.0) if (dist > lz and v == self.I) else v

    def __call__(self, s, t, z):
        n = (f32(s), f32(t), f32(z))
        if self.tech == "savsm":
            return self.vsm(self.penumbra(self.blocker_pcf(n), n[2]), n)
        if self.tech == "vssm":
            v = self.hsm(n)
            if v == self.I or v == f32(1.0):
                return v
            return self.vsm(self.penumbra(self.vsm_blocker(n), n[2]), n)
        if self.tech == "essm":
            return self.esm(self.penumbra(self.esm_blocker(n), n[2]), n)
        return self.msm(self.penumbra(self.msm_blocker(n), n[2]), n)
