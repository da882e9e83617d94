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
__device__ __noinline__ int clip_polygon(const float c0[4], const float c1[4], const float c2[4],
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

__device__ __forceinline__ float depth_at(const Setup& s, const int64_t E[3]) {
    float l1 = (float)E[1] * s.inv_area;
    float l2 = (float)E[2] * s.inv_area;
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

}  // namespace dev
}  // namespace gi
