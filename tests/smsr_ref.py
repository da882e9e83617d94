"""A second, numpy restatement of the non-conservative shadow-map
silhouette revectorisation (test helper).

ShadowMapping/Shaders/RBSM/NonConservativeSMSR.frag written again with
numpy float32 scalars, independently of the C++ oracle, in the shader's
operation order: computeShadowFromSMSR (:279-303, the SMSR technique) and
computeShadowFromAccurateRPCF (:305-348, RPCF + SMSR; with FilteredRBSM.frag's
relative position and revectorisation, RSMSS), with getDisc's three
overloads (:23-174), computeDiscontinuityLength (:176-225, including the
shader's global newDepth), estimateRelativePosition (:227-236, 249-256),
orientateDS (:238-247), revectorizeShadow (:258-266) and
computeDiscontinuity (:268-277).  GLSL's mix(x, y, a) is x (1 - a) + y a and
fract(x) is x - floor(x); shadowMapStep is (1 / W, 1 / H) rounded from
double, as glUniform2f receives it.  Lookups are shadow_lookup_ref.fetch
(NEAREST, border 0).
"""
from __future__ import annotations

import numpy as np

from shadow_lookup_ref import fetch

f32 = np.float32
ONE, ZERO, TWO = f32(1.0), f32(0.0), f32(2.0)


def mix(x, y, a):
    return x * (ONE - a) + y * a


def fract(x):
    return x - np.floor(x)


class Smsr:
    """NonConservativeSMSR.frag; with filtered=True FilteredRBSM.frag (RSMSS),
    whose relative position drops the shadow factor (:241) and whose
    revectorisation returns a fractional fill (:268-272)."""

    def __init__(self, depth, W, H, intensity, depth_threshold, max_search, kernel_order=3, penumbra_size=1,
                 filtered=False):
        self.filtered = filtered
        self.depth, self.W, self.H = depth, W, H
        self.sx, self.sy = f32(1.0 / W), f32(1.0 / H)
        self.I = f32(intensity)
        self.thr = f32(depth_threshold)
        self.max_search = int(max_search)
        self.kernel_order, self.penumbra_size = int(kernel_order), int(penumbra_size)
        self.new_depth = ZERO
        self.discontinuities = 0  # lookups that found a discontinuity (coverage)

    def tex(self, x, y):
        return fetch(self.depth, self.W, self.H, x, y)

    def lit(self, z, d):
        return ONE if z <= d else ZERO

    # getDisc(vec4, vec2 shadowMapStep, float, false, false): all four neighbours
    def disc_all(self, c):
        x, y, z = c[0], c[1], c[2]
        x = x - self.sx
        left = self.lit(z, self.tex(x, y))
        x = x + TWO * self.sx
        right = self.lit(z, self.tex(x, y))
        x = x - self.sx
        y = y + self.sy
        bottom = self.lit(z, self.tex(x, y))
        y = y - TWO * self.sy
        top = self.lit(z, self.tex(x, y))
        return [left, right, bottom, top]

    # getDisc(vec4, vec2 dir, float discType)
    def disc_type(self, c, dir_, disc_type):
        x, y, z = c[0], c[1], c[2]
        if dir_[0] == 0:
            x = x - self.sx
            if self.lit(z, self.tex(x, y)) == disc_type:
                return True
            x = x + TWO * self.sx
            if self.lit(z, self.tex(x, y)) == disc_type:
                return True
            x = x - self.sx
        if dir_[1] == 0:
            y = y + self.sy
            if self.lit(z, self.tex(x, y)) == disc_type:
                return True
            y = y - TWO * self.sy
            if self.lit(z, self.tex(x, y)) == disc_type:
                return True
        return False

    # getDisc(vec4, vec2 dir, vec4 discType): sets the global newDepth
    def disc_vec(self, c, dir_, disc):
        x, y, z = c[0], c[1], c[2]
        rx, ry = x, y
        self.new_depth = z

        def probe(px, py, z):
            d = self.tex(px, py)
            if disc[2] == 1 and abs(z - d) < self.thr:
                z = z - self.thr
                self.new_depth = z
            return self.lit(z, d) == disc[2], z

        if dir_[0] == 0:
            if disc[0] == f32(0.5) or disc[0] == f32(0.75):
                rx = x - self.sx
                hit, z = probe(rx, ry, z)
                if hit:
                    return True
            if disc[0] == f32(0.75) or disc[0] == f32(0.25):
                rx = x + self.sx
                hit, z = probe(rx, ry, z)
                if hit:
                    return True
        if dir_[1] == 0:
            if disc[1] == f32(0.5) or disc[1] == f32(0.75):
                ry = y + self.sy
                hit, z = probe(rx, ry, z)
                if hit:
                    return True
            if disc[1] == f32(0.75) or disc[1] == f32(0.25):
                ry = y - self.sy
                hit, z = probe(rx, ry, z)
                if hit:
                    return True
        return False

    def disc_length(self, disc, c, dir_, sub):
        cx, cy, cz = c[0], c[1], c[2]
        found = ZERO
        dist = ZERO
        stx, sty = f32(dir_[0]) * self.sx, f32(dir_[1]) * self.sy
        cx, cy = cx + stx, cy + sty
        for _ in range(self.max_search):
            d = self.tex(cx, cy)
            if disc[2] == 0 and abs(cz - d) < self.thr:
                cz = cz - self.thr
            if self.lit(cz, d) == disc[2]:
                found = ONE if self.disc_type((cx, cy, cz), (0.0, 0.0), disc[2]) else ZERO
                break
            if not self.disc_vec((cx, cy, cz), dir_, disc):
                break
            dist = dist + ONE
            cx, cy = cx + stx, cy + sty
            if disc[2] == 1:
                cz = self.new_depth
        e = dist + (ONE - sub)
        return mix(-e, e, found)

    def orientate(self, c, disc, sub):
        return [self.disc_length(disc, c, (-1.0, 0.0), ONE - sub[0]),
                self.disc_length(disc, c, (1.0, 0.0), sub[0]),
                self.disc_length(disc, c, (0.0, -1.0), ONE - sub[1]),
                self.disc_length(disc, c, (0.0, 1.0), sub[1])]

    def relative_position(self, dx, dy, shadow):
        T = ONE
        if dx < 0 and dy < 0:
            T = ZERO
        if dx > 0 and dy > 0:
            T = f32(-2.0)
        edge_length = min(abs(dx) + abs(dy), f32(self.max_search))
        if self.filtered:
            return (T * abs(max(T * dx, T * dy))) / edge_length
        return (max(T, TWO * shadow - ONE) * abs(max(T * dx, T * dy))) / edge_length

    def revectorize(self, r, shadow):
        if self.filtered:
            if r[0] * r[1] < 0:
                return (ONE - shadow) + (TWO * shadow - ONE) * max(r[0], r[1])
            if r[0] * r[1] == 0:
                return shadow
            v = (ONE - shadow) + (TWO * shadow - ONE) * (r[0] + r[1])
            return min(max(v, ZERO), ONE)
        if (r[0] * r[1] == TWO * shadow) or (
                (abs(r[0]) * abs(r[1]) > 0) and ((ONE - shadow) + (TWO * shadow - ONE) * (abs(r[0]) + abs(r[1])) < f32(0.5))):
            return ZERO
        return ONE

    def discontinuity(self, c, d):
        center = self.lit(c[2], d)
        dirs = self.disc_all(c)
        disc = [abs(v - center) for v in dirs]
        return [(TWO * disc[0] + disc[1]) / f32(4.0), (TWO * disc[2] + disc[3]) / f32(4.0), ONE - center, ONE]

    def revectorized(self, c, d, shadow, disc):
        self.discontinuities += 1
        sub = (fract(c[0] * f32(self.W)), fract(c[1] * f32(self.H)))
        ds = self.orientate(c, disc, sub)
        r = (self.relative_position(ds[0], ds[1], shadow), self.relative_position(ds[2], ds[3], shadow))
        return mix(self.revectorize(r, shadow), ONE, self.I)

    def smsr(self, c):
        """computeShadowFromSMSR at the normalised light coordinate c."""
        d = self.tex(c[0], c[1])
        disc = self.discontinuity(c, d)
        shadow = self.lit(c[2], d)
        if disc[0] > 0 or disc[1] > 0:
            if disc[0] == f32(0.75) and disc[1] == f32(0.75):
                self.discontinuities += 1
                return mix(ONE - shadow, ONE, self.I)
            return self.revectorized(c, d, shadow, disc)
        return mix(shadow, ONE, self.I)

    def rpcf(self, c):
        """computeShadowFromAccurateRPCF at the normalised light coordinate c."""
        incr_w, incr_h = ONE / f32(self.W), ONE / f32(self.H)
        illum = ZERO
        offset = f32(self.penumbra_size)
        step = (TWO * offset) / f32(self.kernel_order)
        count = 0
        w = -offset
        while w <= offset:
            h = -offset
            while h <= offset:
                s = (c[0] + w * incr_w, c[1] + h * incr_h, c[2], c[3])
                d = self.tex(s[0], s[1])
                shadow = self.lit(s[2], d)
                disc = self.discontinuity(s, d)
                if disc[0] > 0 or disc[1] > 0:
                    illum = illum + self.revectorized(s, d, shadow, disc)
                else:
                    illum = illum + mix(shadow, ONE, self.I)
                count += 1
                h = h + step
            w = w + step
        return illum / f32(count)


class ConservativeSmsr:
    """ShadowMapping/Shaders/RBSM/ConservativeSMSR.frag: computeShadowFromSMSR
    (:127-144, the conservative SMSR technique) and computeShadowFromRPCF
    (:146-198, conservative RPCF), with computeDiscontinuity (:23-47: 1 for a
    shadowed neighbour), computeRelativeDistance (:49-94), its normalisation
    (:96-115) and revectorizeShadow (:117-125)."""

    def __init__(self, depth, W, H, intensity, depth_threshold, max_search, kernel_order=3, penumbra_size=1):
        self.depth, self.W, self.H = depth, W, H
        self.sx, self.sy = f32(1.0 / W), f32(1.0 / H)
        self.I = f32(intensity)
        self.thr = f32(depth_threshold)
        self.max_search = int(max_search)
        self.kernel_order, self.penumbra_size = int(kernel_order), int(penumbra_size)
        self.discontinuities = 0

    def tex(self, x, y):
        return fetch(self.depth, self.W, self.H, x, y)

    def disc(self, c):
        x, y, z = c[0], c[1], c[2]
        out = []
        x = x - self.sx
        out.append(ONE if z <= self.tex(x, y) else ZERO)
        x = x + TWO * self.sx
        out.append(ONE if z <= self.tex(x, y) else ZERO)
        x = x - self.sx
        y = y + self.sy
        out.append(ONE if z <= self.tex(x, y) else ZERO)
        y = y - TWO * self.sy
        out.append(ONE if z <= self.tex(x, y) else ZERO)
        return [abs(v - ONE) for v in out]

    def distance(self, c, dir_, sub):
        x, y, z = c[0], c[1], c[2]
        found = ZERO
        dist = ZERO
        stx, sty = f32(dir_[0]) * self.sx, f32(dir_[1]) * self.sy
        x, y = x + stx, y + sty
        for _ in range(self.max_search):
            d = self.tex(x, y)
            if abs(z - d) < self.thr:
                z = z - self.thr
            if not (z <= d):  # the centre is in umbra: the silhouette ends here
                found = ONE
                break
            dd = self.disc((x, y, z))
            if ((dd[0] + dd[1]) + dd[2]) + dd[3] == 0:
                break
            dist = dist + ONE
            x, y = x + stx, y + sty
        dist = dist + (ONE - sub)
        return mix(-dist, dist, found)

    def normalise(self, dx, dy):
        T = ONE
        if dx < 0 and dy < 0:
            T = ZERO
        if dx > 0 and dy > 0:
            T = f32(-2.0)
        length = min(abs(dx) + abs(dy), f32(self.max_search))
        return abs(max(T * dx, T * dy)) / length

    def revectorized(self, c):
        self.discontinuities += 1
        sub = (fract(c[0] * f32(self.W)), fract(c[1] * f32(self.H)))
        ds = [self.distance(c, (-1.0, 0.0), ONE - sub[0]), self.distance(c, (1.0, 0.0), sub[0]),
              self.distance(c, (0.0, -1.0), ONE - sub[1]), self.distance(c, (0.0, 1.0), sub[1])]
        r = (self.normalise(ds[0], ds[1]), self.normalise(ds[2], ds[3]))
        if (r[0] * r[1] > 0) and (ONE - r[0] > r[1]):
            return self.I
        return ONE

    def smsr(self, c):
        d = self.tex(c[0], c[1])
        if not (c[2] <= d):
            return self.I
        dd = self.disc(c)
        if ((dd[0] + dd[1]) + dd[2]) + dd[3] == 0:
            return ONE
        if dd[0] + dd[1] == TWO or dd[2] + dd[3] == TWO:
            return self.I
        return self.revectorized(c)

    def rpcf(self, c):
        incr_w, incr_h = ONE / f32(self.W), ONE / f32(self.H)
        illum = ZERO
        offset = f32(self.penumbra_size)
        step = (TWO * offset) / f32(self.kernel_order)
        count = 0
        w = -offset
        while w <= offset:
            h = -offset
            while h <= offset:
                d = self.tex(c[0] + w * incr_w, c[1] + h * incr_h)
                if c[2] <= d:
                    s = (c[0] + w * incr_w, c[1] + h * incr_h, c[2], c[3])
                    dd = self.disc(s)
                    if dd[0] == 0 and dd[1] == 0:
                        illum = illum + ONE
                    else:
                        illum = illum + self.revectorized(s)
                else:
                    illum = illum + self.I
                count += 1
                h = h + step
            w = w + step
        return illum / f32(count)
