// Device-side triangle setup shared by the raster kernels.
//
// The arithmetic follows the rasterisation rules stated at the top of
// raster.cu operation for operation (the file is compiled with
// -fmad=false so no multiply-add is fused): clip coordinates in glm's
// order, near/far/guard-band clipping, 8 sub-pixel bits, integer edge
// functions with the top-left rule, window-space linear depth and
// perspective-correct attributes.
#pragma once

#include <cstdint>
#include "launch.cuh"

namespace gi {
namespace dev {

constexpr float kGuard = 16.0f;
constexpr int kSubBits = 8;
constexpr int64_t kSub = 1 << kSubBits;

struct Mat4 {
    float m[16];
};

struct CV {
    float c[4];
    float b[3];
};

__device__ __forceinline__ void transform(const Mat4& M, float x, float y, float z, float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r)
        out[r] = M.m[0 * 4 + r] * x + M.m[1 * 4 + r] * y + M.m[2 * 4 + r] * z + M.m[3 * 4 + r];
}

__device__ __forceinline__ float plane_dist(const float c[4], int k) {
    const float x = c[0], y = c[1], z = c[2], w = c[3];
    switch (k) {
        case 0: return z + w;
        case 1: return w - z;
        case 2: return x + kGuard * w;
        case 3: return kGuard * w - x;
        case 4: return y + kGuard * w;
        default: return kGuard * w - y;
    }
}

// True if no vertex is outside any of the six planes (no clipping needed).
__device__ __forceinline__ bool all_inside(const float c0[4], const float c1[4], const float c2[4]) {
#pragma unroll
    for (int k = 0; k < 6; ++k)
        if (!(plane_dist(c0, k) >= 0.0f) || !(plane_dist(c1, k) >= 0.0f) ||
            !(plane_dist(c2, k) >= 0.0f))
            return false;
    return true;
}

__device__ __forceinline__ CV intersect(const CV& in, const CV& out, float din, float dout) {
    float t = din / (din - dout);
    CV r;
#pragma unroll
    for (int k = 0; k < 4; ++k) r.c[k] = in.c[k] + t * (out.c[k] - in.c[k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) r.b[k] = in.b[k] + t * (out.b[k] - in.b[k]);
    return r;
}

// Sutherland-Hodgman against the planes some vertex violates, in the fixed
// plane order; returns the polygon size (0 = culled).
static __device__ __noinline__ int clip_polygon(const float c0[4], const float c1[4], const float c2[4],
                                         CV poly[9]) {
    CV a[9], b[9];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[0].c[k] = c0[k];
        a[1].c[k] = c1[k];
        a[2].c[k] = c2[k];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) a[i].b[k] = (i == k) ? 1.0f : 0.0f;
    int n = 3;
    CV* src = a;
    CV* dst = b;
    for (int plane = 0; plane < 6; ++plane) {
        bool any_out = false, all_out = true;
        for (int i = 0; i < n; ++i) {
            bool out = !(plane_dist(src[i].c, plane) >= 0.0f);
            any_out |= out;
            all_out &= out;
        }
        if (all_out) return 0;
        if (!any_out) continue;
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const CV& cur = src[i];
            const CV& nxt = src[(i + 1 == n) ? 0 : i + 1];
            float dc = plane_dist(cur.c, plane), dn = plane_dist(nxt.c, plane);
            bool cin = dc >= 0.0f, nin = dn >= 0.0f;
            if (cin) dst[m++] = cur;
            if (cin != nin) {
                if (cin) dst[m++] = intersect(cur, nxt, dc, dn);
                else dst[m++] = intersect(nxt, cur, dn, dc);
            }
        }
        n = m;
        CV* t = src;
        src = dst;
        dst = t;
        if (n < 3) return 0;
    }
    for (int i = 0; i < n; ++i) poly[i] = src[i];
    return n;
}

struct Setup {
    int64_t X[3], Y[3];
    float z[3];
    float iw[3];
    float b[3][3];
    int64_t area;
    float inv_area;
    bool front;
    bool swapped;  // vertices 1 and 2 exchanged to make the triangle CCW
};

// Window transform, snapping and orientation of one (sub-)triangle whose
// vertices are given in clip space with their source barycentric rows.
__device__ __forceinline__ bool setup_triangle(const float* c0, const float* c1, const float* c2,
                                               const float* b0, const float* b1, const float* b2,
                                               int W, int H, Setup& s) {
    const float* cv[3] = {c0, c1, c2};
    const float* bv[3] = {b0, b1, b2};
    const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
    float wv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float w = cv[i][3];
        if (!(w > 0.0f)) return false;
        float xd = cv[i][0] / w, yd = cv[i][1] / w, zd = cv[i][2] / w;
        float xw = xd * hw + hw;
        float yw = yd * hh + hh;
        float zw = zd * 0.5f + 0.5f;
        s.X[i] = __float2ll_rn(xw * (float)kSub);
        s.Y[i] = __float2ll_rn(yw * (float)kSub);
        s.z[i] = zw;
        wv[i] = w;
#pragma unroll
        for (int k = 0; k < 3; ++k) s.b[i][k] = bv[i][k];
    }
    int64_t area = (s.X[1] - s.X[0]) * (s.Y[2] - s.Y[0]) - (s.X[2] - s.X[0]) * (s.Y[1] - s.Y[0]);
    if (area == 0) return false;
    s.front = area > 0;
    s.swapped = area < 0;
    if (area < 0) {
        int64_t t;
        t = s.X[1]; s.X[1] = s.X[2]; s.X[2] = t;
        t = s.Y[1]; s.Y[1] = s.Y[2]; s.Y[2] = t;
        float f;
        f = s.z[1]; s.z[1] = s.z[2]; s.z[2] = f;
        f = wv[1]; wv[1] = wv[2]; wv[2] = f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            f = s.b[1][k]; s.b[1][k] = s.b[2][k]; s.b[2][k] = f;
        }
        area = -area;
    }
    s.area = area;
#pragma unroll
    for (int i = 0; i < 3; ++i) s.iw[i] = 1.0f / wv[i];
    s.inv_area = 1.0f / (float)area;
    return true;
}

// Edge i opposite vertex i; (a, b) = (1, 2), (2, 0), (0, 1).
struct Edges {
    int64_t A[3];  // Xb - Xa : coefficient of (py - Ya)
    int64_t B[3];  // Yb - Ya : coefficient of (px - Xa)
    int64_t Xa[3], Ya[3];
    bool topleft[3];
};

__device__ __forceinline__ void make_edges(const Setup& s, Edges& e) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        int a = (i + 1) % 3, b = (i + 2) % 3;
        e.A[i] = s.X[b] - s.X[a];
        e.B[i] = s.Y[b] - s.Y[a];
        e.Xa[i] = s.X[a];
        e.Ya[i] = s.Y[a];
        e.topleft[i] = (e.B[i] < 0) || (e.B[i] == 0 && e.A[i] < 0);
    }
}

__device__ __forceinline__ int64_t edge_at(const Edges& e, int i, int64_t px, int64_t py) {
    return e.A[i] * (py - e.Ya[i]) - e.B[i] * (px - e.Xa[i]);
}

__device__ __forceinline__ bool inside3(const Edges& e, const int64_t E[3]) {
    return (E[0] > 0 || (E[0] == 0 && e.topleft[0])) && (E[1] > 0 || (E[1] == 0 && e.topleft[1])) &&
           (E[2] > 0 || (E[2] == 0 && e.topleft[2]));
}

// int64 -> float with round-to-nearest-even, off the FP64 pipe (a narrow
// unit on this GPU): for |v| < 2^47, v = h * 2^24 + l with h = v >> 24
// (|h| < 2^23) and 0 <= l < 2^24, both exact in FP32; h * 2^24 is exact and
// the one addition rounds once, giving the correctly rounded v, the same
// value as the (float) cast.
//
// Below 2^45 in magnitude the two halves are split at bit 23 instead and
// converted with exponent tricks rather than conversion instructions:
// 12582912 + h (|h| < 2^22) and 8388608 + l (0 <= l < 2^23) are exact FP32
// integers whose bit patterns are plain integer sums, so subtracting the
// constants recovers h and l exactly; h * 2^23 + l rounds once, to the same
// correctly rounded v.
__device__ __forceinline__ float i2f(int64_t v) {
    if (v >= -(1LL << 45) && v < (1LL << 45)) {
        const int h = (int)(v >> 23);
        const int l = (int)(v & 0x7FFFFF);
        const float fh = __int_as_float(0x4B400000 + h) - 12582912.0f;
        const float fl = __int_as_float(0x4B000000 | l) - 8388608.0f;
        return fh * 8388608.0f + fl;
    }
    if (v >= -(1LL << 47) && v < (1LL << 47)) {
        const int h = (int)(v >> 24);
        const int l = (int)(v & 0xFFFFFF);
        return __int2float_rn(h) * 16777216.0f + __int2float_rn(l);
    }
    return (float)v;
}

// The top-left rule as a bias: an edge value E passes when E > 0, or
// E == 0 on a top or left edge, that is when E - tl_bias >= 0.  With the
// bias folded into the stepped values, a pixel is inside when none of the
// three is negative.
__device__ __forceinline__ int tl_bias(bool tl) { return tl ? 0 : 1; }


__device__ __forceinline__ bool inside_biased(const int64_t E[3]) {
    return ((int)(E[0] >> 32) | (int)(E[1] >> 32) | (int)(E[2] >> 32)) >= 0;
}

__device__ __forceinline__ float depth_at(const Setup& s, const int64_t E[3]) {
    float l1 = i2f(E[1]) * s.inv_area;
    float l2 = i2f(E[2]) * s.inv_area;
    return s.z[0] + (l1 * (s.z[1] - s.z[0]) + l2 * (s.z[2] - s.z[0]));
}

__device__ __forceinline__ float pow2i(int k) {
    uint32_t bits = (k >= -126) ? ((uint32_t)(k + 127) << 23) : (1u << (k + 149));
    return __uint_as_float(bits);
}

// glPolygonOffset for a float depth buffer: m * factor + r * units.
__device__ __forceinline__ float polygon_offset(const Setup& s, float factor, float units) {
    float fx1 = (float)(s.X[1] - s.X[0]), fy1 = (float)(s.Y[1] - s.Y[0]);
    float fx2 = (float)(s.X[2] - s.X[0]), fy2 = (float)(s.Y[2] - s.Y[0]);
    float dz1 = s.z[1] - s.z[0], dz2 = s.z[2] - s.z[0];
    float area_f = (float)s.area;
    float dzdx = ((dz1 * fy2 - dz2 * fy1) / area_f) * (float)kSub;
    float dzdy = ((dz2 * fx1 - dz1 * fx2) / area_f) * (float)kSub;
    float ax = fabsf(dzdx), ay = fabsf(dzdy);
    float m = ax > ay ? ax : ay;
    float zmax = s.z[0];
    if (s.z[1] > zmax) zmax = s.z[1];
    if (s.z[2] > zmax) zmax = s.z[2];
    int e = -126;
    if (zmax > 0.0f) {
        uint32_t bits = __float_as_uint(zmax);
        int be = (int)((bits >> 23) & 0xFF);
        e = be == 0 ? -126 : be - 127;
    }
    float r = pow2i(e - 23);
    return m * factor + r * units;
}

__device__ __forceinline__ float clamp01(float z) {
    if (!(z > 0.0f)) return 0.0f;
    if (z > 1.0f) return 1.0f;
    return z;
}

__device__ __forceinline__ int64_t floor_div256(int64_t a) {
    // floor(a / 256) for signed a (arithmetic shift rounds toward -inf)
    return a >> 8;
}


// Set-up record of one (sub-)triangle, 64 bytes: snapped CCW window
// vertices, window depth plane (z0 + l1 dz1 + l2 dz2 with l = E / area),
// bias, key / stencil primitive id, pixel bounding box, flags.
constexpr unsigned kFlagFront = 1u;
struct __align__(16) BRec {
    int X[3];
    int Y[3];
    float z0, dz1, dz2, inv_area;
    float zoff;
    unsigned prim;     // key / stencil primitive id
    unsigned short x0, x1, y0, y1;
    unsigned flags;
    unsigned spill_id; // (primitive << 3) | sub-triangle
};
static_assert(sizeof(BRec) == 64, "BRec is four 16-byte words");

__device__ __forceinline__ void ldg3(const float* p, int idx, float out[3]) {
    out[0] = __ldg(p + 3 * (size_t)idx + 0);
    out[1] = __ldg(p + 3 * (size_t)idx + 1);
    out[2] = __ldg(p + 3 * (size_t)idx + 2);
}

// Resolve from a stored record of an unclipped triangle: X / Y are the
// snapped (CCW-ordered) window vertices, inv_area = 1 / area, iw = 1 / clip w
// of the CCW-ordered vertices, swapped = vertices 1 and 2 were exchanged.
// Performs the same operations as resolve_key's interpolation.
__device__ __forceinline__ void resolve_record(const int X[3], const int Y[3], float inv_area,
                                               const float iw[3], bool swapped, bool front, int t,
                                               const float* points, const float* normals,
                                               const int* indices, int x, int y, float4& pos,
                                               float4& nrm) {
    const int64_t px = (int64_t)x * kSub + kSub / 2, py = (int64_t)y * kSub + kSub / 2;
    float q[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int a = (j + 1) % 3, b = (j + 2) % 3;
        const int64_t e = ((int64_t)X[b] - X[a]) * (py - Y[a]) - ((int64_t)Y[b] - Y[a]) * (px - X[a]);
        const float l = i2f(e) * inv_area;
        q[j] = l * iw[j];
    }
    const float sum = (q[0] + q[1]) + q[2];
    const float pc[3] = {q[0] / sum, q[1] / sum, q[2] / sum};
    // identity source rows (exchanged for a swapped triangle): B = pc permuted
    const float B[3] = {pc[0], swapped ? pc[2] : pc[1], swapped ? pc[1] : pc[2]};
    const int* tri = indices + 3 * (size_t)t;
    const int ids[3] = {__ldg(tri), __ldg(tri + 1), __ldg(tri + 2)};
    float P[3][3], N[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        ldg3(points, ids[j], P[j]);
        ldg3(normals, ids[j], N[j]);
    }
    float o[3], on[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o[j] = (B[0] * P[0][j] + B[1] * P[1][j]) + B[2] * P[2][j];
        on[j] = (B[0] * N[0][j] + B[1] * N[1][j]) + B[2] * N[2][j];
    }
    pos = make_float4(o[0], o[1], o[2], 1.0f);
    nrm = make_float4(on[0], on[1], on[2], front ? 1.0f : 0.0f);
}

// The G-buffer texel of pixel (x, y) from its 64-bit visibility key
// (depth bits << 32 | triangle * 8 + sub-triangle): the winning
// sub-triangle is re-derived (transform, clip, set up) and the object
// position and vertex normal are interpolated perspective-correctly
// (GBuffer.frag:32-38: (position, 1), (normal, gl_FrontFacing)).
// Background keys give (0, 0, 0, 1) for both, the G-buffer's clear colour.
// Returns false for background.
__device__ __forceinline__ bool resolve_key(unsigned long long k, const float* points,
                                            const float* normals, const int* indices,
                                            const Mat4& mvp, int W, int H, int x, int y,
                                            float4& pos, float4& nrm) {
    const unsigned long long clear = ((unsigned long long)__float_as_uint(1.0f) << 32) | 0xFFFFFFFFull;
    const float4 bg = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (k == clear) {
        pos = bg;
        nrm = bg;
        return false;
    }
    const unsigned prim = (unsigned)(k & 0xFFFFFFFFull);
    const int t = (int)(prim >> 3), sub = (int)(prim & 7);
    const int* tri = indices + 3 * (size_t)t;
    const int ids[3] = {__ldg(tri), __ldg(tri + 1), __ldg(tri + 2)};
    float P[3][3];
    float c[3][4];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        ldg3(points, ids[j], P[j]);
        transform(mvp, P[j][0], P[j][1], P[j][2], c[j]);
    }
    const float id[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
    Setup s;
    bool ok;
    if (all_inside(c[0], c[1], c[2])) {
        ok = sub == 0 && setup_triangle(c[0], c[1], c[2], id[0], id[1], id[2], W, H, s);
    } else {
        CV poly[9];
        const int n = clip_polygon(c[0], c[1], c[2], poly);
        ok = (sub + 2 < n) && setup_triangle(poly[0].c, poly[sub + 1].c, poly[sub + 2].c, poly[0].b,
                                             poly[sub + 1].b, poly[sub + 2].b, W, H, s);
    }
    if (!ok) {
        pos = bg;
        nrm = bg;
        return false;
    }
    Edges e;
    make_edges(s, e);
    const int64_t px = (int64_t)x * kSub + kSub / 2, py = (int64_t)y * kSub + kSub / 2;
    float q[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float l = i2f(edge_at(e, j, px, py)) * s.inv_area;
        q[j] = l * s.iw[j];
    }
    const float sum = (q[0] + q[1]) + q[2];
    const float pc[3] = {q[0] / sum, q[1] / sum, q[2] / sum};
    float B[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) B[j] = (pc[0] * s.b[0][j] + pc[1] * s.b[1][j]) + pc[2] * s.b[2][j];
    float N[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) ldg3(normals, ids[j], N[j]);
    float o[3], on[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o[j] = (B[0] * P[0][j] + B[1] * P[1][j]) + B[2] * P[2][j];
        on[j] = (B[0] * N[0][j] + B[1] * N[1][j]) + B[2] * N[2][j];
    }
    pos = make_float4(o[0], o[1], o[2], 1.0f);
    nrm = make_float4(on[0], on[1], on[2], s.front ? 1.0f : 0.0f);
    return true;
}

// resolve_key with a shortcut: when the key names the unclipped triangle t
// and rec_of[t] holds its record (written by the light-map / G-buffer
// set-up), the interpolation starts from the stored set-up instead of
// re-deriving it.  Same values either way.
__device__ __forceinline__ bool resolve_pixel(unsigned long long k, const float* points,
                                              const float* normals, const int* indices,
                                              const Mat4& mvp, int W, int H, int x, int y,
                                              const unsigned* rec_of, const BRec* recs,
                                              const uint4* rres, float4& pos, float4& nrm) {
    const unsigned long long clear = ((unsigned long long)__float_as_uint(1.0f) << 32) | 0xFFFFFFFFull;
    if (k != clear && rec_of) {
        const unsigned prim = (unsigned)(k & 0xFFFFFFFFull);
        const int t = (int)(prim >> 3);
        if ((prim & 7) == 0) {
            const unsigned ri = __ldg(rec_of + t);
            if (ri != ~0u) {
                const uint4* rp = reinterpret_cast<const uint4*>(recs + ri);
                const uint4 q0 = __ldg(rp), q1 = __ldg(rp + 1), q2 = __ldg(rp + 2), q3 = __ldg(rp + 3);
                const int X[3] = {(int)q0.x, (int)q0.y, (int)q0.z};
                const int Y[3] = {(int)q0.w, (int)q1.x, (int)q1.y};
                const float inv_area = __uint_as_float(q2.y);
                const uint4 rr = __ldg(rres + ri);
                const float iw[3] = {__uint_as_float(rr.x), __uint_as_float(rr.y), __uint_as_float(rr.z)};
                resolve_record(X, Y, inv_area, iw, rr.w != 0u, (q3.z & kFlagFront) != 0, t, points, normals,
                               indices, x, y, pos, nrm);
                return true;
            }
        }
    }
    return resolve_key(k, points, normals, indices, mvp, W, H, x, y, pos, nrm);
}

}  // namespace dev
}  // namespace gi
