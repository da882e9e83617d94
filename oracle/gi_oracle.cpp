// gi_oracle.cpp -- CPU oracle (test infrastructure; see gi_oracle.h).
//
// Scalar restatement of the reference's shadow passes.  Build with
// -O2 -ffp-contract=off and without -ffast-math: every FP32 operation below
// is meant to round exactly once, in the order written.
//
// Rasterisation rules (OpenGL 4.6 core spec, sections 13.6 / 14.6 / 14.9;
// the choices the spec leaves open are fixed here):
//   * clip coordinates c = MVP * (x, y, z, 1), glm's operation order;
//   * triangles are clipped against the near (z >= -w) and far (z <= w)
//     planes and against a guard band |x|, |y| <= 16 w (Sutherland-Hodgman,
//     intersection computed from the inside vertex); the clipped polygon is
//     fanned from its first vertex;
//   * window coordinates x_w = x_ndc * W/2 + W/2 (same for y),
//     z_w = z_ndc * 0.5 + 0.5, snapped to 8 sub-pixel bits (round to nearest
//     even);
//   * integer edge functions; pixel centres at (x + 1/2, y + 1/2); a centre
//     on an edge belongs to the triangle iff the edge is a top or left edge
//     of the counter-clockwise-ordered triangle (y up);
//   * gl_FrontFacing = counter-clockwise window-space area > 0, no culling;
//   * depth is interpolated linearly in window space from the barycentrics
//     l_i = E_i * (1 / area); attributes perspective-correctly;
//   * polygon offset o = m * factor + r * units, m = max(|dz/dx|, |dz/dy|),
//     r = 2^(e - 23) with e the exponent of the primitive's largest z_w;
//   * depth is clamped to [0, 1] after the offset; the depth buffer is
//     cleared to 1 and the test is LESS, so a buffer texel ends as the
//     minimum fragment depth below 1;
//   * for the G-buffer the surviving fragment is the first one in draw
//     order among those with the minimum depth (LESS keeps the earlier).
// Texture fetches: GL_NEAREST, i = floor(s * width), CLAMP_TO_BORDER with
// border depth 0 (ShadowMapping/src/Viewers/MyGLTextureViewer.cpp:3-28).
#include "gi_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const float kGuard = 16.0f;
const int kSubBits = 8;
const int64_t kSub = 1 << kSubBits;

// ---------------------------------------------------------------------------
// Clipping
// ---------------------------------------------------------------------------
struct CV {
    float c[4];  // clip x, y, z, w
    float b[3];  // barycentric weights with respect to the source triangle
};

float plane_dist(const CV& v, int k) {
    const float x = v.c[0], y = v.c[1], z = v.c[2], w = v.c[3];
    switch (k) {
        case 0: return z + w;
        case 1: return w - z;
        case 2: return x + kGuard * w;
        case 3: return kGuard * w - x;
        case 4: return y + kGuard * w;
        default: return kGuard * w - y;
    }
}

CV intersect(const CV& in, const CV& out, float din, float dout) {
    float t = din / (din - dout);
    CV r;
    for (int k = 0; k < 4; ++k) r.c[k] = in.c[k] + t * (out.c[k] - in.c[k]);
    for (int k = 0; k < 3; ++k) r.b[k] = in.b[k] + t * (out.b[k] - in.b[k]);
    return r;
}

// Returns the clipped polygon size (0 if culled); poly holds <= 9 vertices.
int clip_polygon(const float c0[4], const float c1[4], const float c2[4], CV poly[9]) {
    CV a[9], b[9];
    for (int k = 0; k < 4; ++k) {
        a[0].c[k] = c0[k];
        a[1].c[k] = c1[k];
        a[2].c[k] = c2[k];
    }
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) a[i].b[k] = (i == k) ? 1.0f : 0.0f;
    int n = 3;
    CV* src = a;
    CV* dst = b;
    for (int plane = 0; plane < 6; ++plane) {
        bool any_out = false, all_out = true;
        for (int i = 0; i < n; ++i) {
            bool out = !(plane_dist(src[i], plane) >= 0.0f);
            any_out |= out;
            all_out &= out;
        }
        if (all_out) return 0;
        if (!any_out) continue;
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const CV& cur = src[i];
            const CV& nxt = src[(i + 1) % n];
            float dc = plane_dist(cur, plane), dn = plane_dist(nxt, plane);
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

// ---------------------------------------------------------------------------
// Triangle setup for one (sub-)triangle
// ---------------------------------------------------------------------------
struct Setup {
    int64_t X[3], Y[3];
    float z[3];
    float iw[3];     // 1 / clip w
    float b[3][3];   // source barycentric rows of the three vertices
    int64_t area;    // > 0 after reordering
    bool front;
    bool topleft[3];
    float inv_area;
};

float f_of_ll(int64_t v) { return (float)v; }

bool setup_triangle(const CV& v0, const CV& v1, const CV& v2, int W, int H, Setup& s) {
    const CV* v[3] = {&v0, &v1, &v2};
    const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
    float wv[3];
    for (int i = 0; i < 3; ++i) {
        float w = v[i]->c[3];
        if (!(w > 0.0f)) return false;
        float xd = v[i]->c[0] / w, yd = v[i]->c[1] / w, zd = v[i]->c[2] / w;
        float xw = xd * hw + hw;
        float yw = yd * hh + hh;
        float zw = zd * 0.5f + 0.5f;
        s.X[i] = (int64_t)std::nearbyint(xw * (float)kSub);
        s.Y[i] = (int64_t)std::nearbyint(yw * (float)kSub);
        s.z[i] = zw;
        wv[i] = w;
        for (int k = 0; k < 3; ++k) s.b[i][k] = v[i]->b[k];
    }
    int64_t area = (s.X[1] - s.X[0]) * (s.Y[2] - s.Y[0]) - (s.X[2] - s.X[0]) * (s.Y[1] - s.Y[0]);
    if (area == 0) return false;
    s.front = area > 0;
    if (area < 0) {
        std::swap(s.X[1], s.X[2]);
        std::swap(s.Y[1], s.Y[2]);
        std::swap(s.z[1], s.z[2]);
        std::swap(wv[1], wv[2]);
        for (int k = 0; k < 3; ++k) std::swap(s.b[1][k], s.b[2][k]);
        area = -area;
    }
    s.area = area;
    for (int i = 0; i < 3; ++i) s.iw[i] = 1.0f / wv[i];
    // Edge i is the edge opposite vertex i: (1,2), (2,0), (0,1).
    for (int i = 0; i < 3; ++i) {
        int a = (i + 1) % 3, bb = (i + 2) % 3;
        int64_t dy = s.Y[bb] - s.Y[a], dx = s.X[bb] - s.X[a];
        s.topleft[i] = (dy < 0) || (dy == 0 && dx < 0);
    }
    s.inv_area = 1.0f / f_of_ll(area);
    return true;
}

int64_t edge(const Setup& s, int i, int64_t px, int64_t py) {
    int a = (i + 1) % 3, b = (i + 2) % 3;
    return (s.X[b] - s.X[a]) * (py - s.Y[a]) - (s.Y[b] - s.Y[a]) * (px - s.X[a]);
}

int64_t floor_div(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}

float pow2i(int k) {
    // exact 2^k for k in [-149, 127]
    uint32_t bits;
    if (k >= -126) bits = (uint32_t)(k + 127) << 23;
    else bits = 1u << (k + 149);
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

float polygon_offset(const Setup& s, float factor, float units) {
    float fx1 = f_of_ll(s.X[1] - s.X[0]), fy1 = f_of_ll(s.Y[1] - s.Y[0]);
    float fx2 = f_of_ll(s.X[2] - s.X[0]), fy2 = f_of_ll(s.Y[2] - s.Y[0]);
    float dz1 = s.z[1] - s.z[0], dz2 = s.z[2] - s.z[0];
    float area_f = f_of_ll(s.area);
    float dzdx = ((dz1 * fy2 - dz2 * fy1) / area_f) * (float)kSub;
    float dzdy = ((dz2 * fx1 - dz1 * fx2) / area_f) * (float)kSub;
    float ax = std::fabs(dzdx), ay = std::fabs(dzdy);
    float m = ax > ay ? ax : ay;
    float zmax = s.z[0];
    if (s.z[1] > zmax) zmax = s.z[1];
    if (s.z[2] > zmax) zmax = s.z[2];
    int e = -126;
    if (zmax > 0.0f) {
        uint32_t bits;
        std::memcpy(&bits, &zmax, 4);
        int be = (int)((bits >> 23) & 0xFF);
        e = be == 0 ? -126 : be - 127;
    }
    float r = pow2i(e - 23);
    return m * factor + r * units;
}

float clamp01(float z) {
    if (!(z > 0.0f)) return 0.0f;
    if (z > 1.0f) return 1.0f;
    return z;
}

uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

void transform(const float m[16], const float* p, float out[4]) {
    const float x = p[0], y = p[1], z = p[2];
    for (int r = 0; r < 4; ++r)
        out[r] = m[0 * 4 + r] * x + m[1 * 4 + r] * y + m[2 * 4 + r] * z + m[3 * 4 + r];
}

// Visits every covered pixel of every sub-triangle of one clipped triangle:
// fn(sub_index, setup, x, y, E0, E1, E2).
template <class Fn>
void raster_clipped(const float c0[4], const float c1[4], const float c2[4], int W, int H, Fn fn) {
    CV poly[9];
    int n = clip_polygon(c0, c1, c2, poly);
    for (int i = 1; i + 1 < n; ++i) {
        Setup s;
        if (!setup_triangle(poly[0], poly[i], poly[i + 1], W, H, s)) continue;
        int64_t minX = std::min(s.X[0], std::min(s.X[1], s.X[2]));
        int64_t maxX = std::max(s.X[0], std::max(s.X[1], s.X[2]));
        int64_t minY = std::min(s.Y[0], std::min(s.Y[1], s.Y[2]));
        int64_t maxY = std::max(s.Y[0], std::max(s.Y[1], s.Y[2]));
        int64_t x0 = std::max<int64_t>(0, -floor_div(-(minX - kSub / 2), kSub));
        int64_t x1 = std::min<int64_t>(W - 1, floor_div(maxX - kSub / 2, kSub));
        int64_t y0 = std::max<int64_t>(0, -floor_div(-(minY - kSub / 2), kSub));
        int64_t y1 = std::min<int64_t>(H - 1, floor_div(maxY - kSub / 2, kSub));
        for (int64_t y = y0; y <= y1; ++y) {
            // Scan only the row's span: each edge with B != 0 bounds px on
            // one side at A (py - Ya) / B + Xa, found in double and widened
            // by two pixels, so that no covered pixel is skipped; the exact
            // test below still decides every pixel of the span.
            int64_t xl = x0, xr = x1;
            const int64_t pyc = y * kSub + kSub / 2;
            for (int k = 0; k < 3; ++k) {
                const int a = (k + 1) % 3, b = (k + 2) % 3;
                const int64_t A = s.X[b] - s.X[a], B = s.Y[b] - s.Y[a];
                if (B == 0) continue;
                const double lim = (double)A * (double)(pyc - s.Y[a]) / (double)B + (double)s.X[a];
                const double xb = (lim - kSub / 2) / kSub;
                if (!(std::fabs(xb) < 1e15)) continue;
                if (B > 0) xr = std::min<int64_t>(xr, (int64_t)std::floor(xb) + 2);
                else xl = std::max<int64_t>(xl, (int64_t)std::ceil(xb) - 2);
            }
            for (int64_t x = xl; x <= xr; ++x) {
                int64_t px = x * kSub + kSub / 2, py = pyc;
                int64_t e[3];
                bool inside = true;
                for (int k = 0; k < 3 && inside; ++k) {
                    e[k] = edge(s, k, px, py);
                    inside = e[k] > 0 || (e[k] == 0 && s.topleft[k]);
                }
                if (inside) fn(i - 1, s, (int)x, (int)y, e);
            }
        }
    }
}

float depth_at(const Setup& s, const int64_t e[3]) {
    float l1 = f_of_ll(e[1]) * s.inv_area;
    float l2 = f_of_ll(e[2]) * s.inv_area;
    return s.z[0] + (l1 * (s.z[1] - s.z[0]) + l2 * (s.z[2] - s.z[0]));
}

template <class T>
void atomic_min(std::atomic<T>& a, T v) {
    T cur = a.load(std::memory_order_relaxed);
    while (v < cur && !a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
    }
}

int nthreads(int t) {
#ifdef _OPENMP
    return t > 0 ? t : omp_get_max_threads();
#else
    (void)t;
    return 1;
#endif
}

// Depth-only rasterisation of a whole mesh into `buf` (uint32 depth bits,
// pre-cleared), with the given bias; used by the light map and the
// shadow-volume prepass.
void raster_depth(const float* points, const int* indices, int nt, const float mvp[16], int W,
                  int H, int bias_mode, float cbias, float factor, float units,
                  std::atomic<uint32_t>* buf, int threads) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))
    for (int t = 0; t < nt; ++t) {
        float c[3][4];
        for (int k = 0; k < 3; ++k) transform(mvp, points + 3 * (size_t)indices[3 * (size_t)t + k], c[k]);
        float offset = 0.0f;
        bool offset_done = false;
        int last_sub = -1;
        raster_clipped(c[0], c[1], c[2], W, H,
                       [&](int sub, const Setup& s, int x, int y, const int64_t e[3]) {
                           if (bias_mode == GI_BIAS_POLYGON_OFFSET && (!offset_done || sub != last_sub)) {
                               offset = polygon_offset(s, factor, units);
                               offset_done = true;
                               last_sub = sub;
                           }
                           float z = depth_at(s, e);
                           if (bias_mode == GI_BIAS_CONSTANT) z = z + cbias;
                           else if (bias_mode == GI_BIAS_POLYGON_OFFSET) z = z + offset;
                           z = clamp01(z);
                           if (z < 1.0f) atomic_min(buf[(size_t)y * W + x], fbits(z));
                       });
    }
}

}  // namespace

extern "C" void or_shadow_map(const float* points, int nv, const int* indices, int nt,
                              const float mvp[16], int W, int H, int bias_mode, float cbias,
                              float factor, float units, float* out_depth, int threads) {
    (void)nv;
    std::vector<std::atomic<uint32_t>> buf((size_t)W * H);
    for (auto& b : buf) b.store(fbits(1.0f), std::memory_order_relaxed);
    raster_depth(points, indices, nt, mvp, W, H, bias_mode, cbias, factor, units, buf.data(),
                 threads);
    for (size_t i = 0; i < buf.size(); ++i) {
        uint32_t u = buf[i].load(std::memory_order_relaxed);
        std::memcpy(&out_depth[i], &u, 4);
    }
}

extern "C" void or_gbuffer(const float* points, const float* normals, int nv, const int* indices,
                           int nt, const float mvp[16], int W, int H, float* out_pos,
                           float* out_nrm, int threads) {
    (void)nv;
    const uint64_t clear = ((uint64_t)fbits(1.0f) << 32) | 0xFFFFFFFFull;
    std::vector<std::atomic<uint64_t>> key((size_t)W * H);
    for (auto& k : key) k.store(clear, std::memory_order_relaxed);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))
    for (int t = 0; t < nt; ++t) {
        float c[3][4];
        for (int k = 0; k < 3; ++k) transform(mvp, points + 3 * (size_t)indices[3 * (size_t)t + k], c[k]);
        raster_clipped(c[0], c[1], c[2], W, H,
                       [&](int sub, const Setup& s, int x, int y, const int64_t e[3]) {
                           float z = clamp01(depth_at(s, e));
                           if (!(z < 1.0f)) return;
                           uint64_t k = ((uint64_t)fbits(z) << 32) | (uint32_t)(t * 8 + sub);
                           atomic_min(key[(size_t)y * W + x], k);
                       });
    }
    // Resolve: re-derive the winning sub-triangle and interpolate.
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads(threads))
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            size_t p = (size_t)y * W + x;
            uint64_t k = key[p].load(std::memory_order_relaxed);
            float* op = out_pos + 4 * p;
            float* on = out_nrm + 4 * p;
            if (k == clear) {
                op[0] = op[1] = op[2] = 0.0f;
                op[3] = 1.0f;
                on[0] = on[1] = on[2] = 0.0f;
                on[3] = 1.0f;
                continue;
            }
            uint32_t prim = (uint32_t)(k & 0xFFFFFFFFull);
            int t = (int)(prim >> 3), sub = (int)(prim & 7);
            const int* tri = indices + 3 * (size_t)t;
            float c[3][4];
            for (int j = 0; j < 3; ++j) transform(mvp, points + 3 * (size_t)tri[j], c[j]);
            CV poly[9];
            int n = clip_polygon(c[0], c[1], c[2], poly);
            Setup s;
            bool ok = (sub + 2 < n) && setup_triangle(poly[0], poly[sub + 1], poly[sub + 2], W, H, s);
            if (!ok) continue;  // unreachable for keys the raster wrote
            int64_t px = (int64_t)x * kSub + kSub / 2, py = (int64_t)y * kSub + kSub / 2;
            int64_t e[3];
            for (int j = 0; j < 3; ++j) e[j] = edge(s, j, px, py);
            float l[3], q[3];
            for (int j = 0; j < 3; ++j) {
                l[j] = f_of_ll(e[j]) * s.inv_area;
                q[j] = l[j] * s.iw[j];
            }
            float sum = (q[0] + q[1]) + q[2];
            float pc[3] = {q[0] / sum, q[1] / sum, q[2] / sum};
            float B[3];
            for (int j = 0; j < 3; ++j) B[j] = (pc[0] * s.b[0][j] + pc[1] * s.b[1][j]) + pc[2] * s.b[2][j];
            const float* P0 = points + 3 * (size_t)tri[0];
            const float* P1 = points + 3 * (size_t)tri[1];
            const float* P2 = points + 3 * (size_t)tri[2];
            const float* N0 = normals + 3 * (size_t)tri[0];
            const float* N1 = normals + 3 * (size_t)tri[1];
            const float* N2 = normals + 3 * (size_t)tri[2];
            for (int j = 0; j < 3; ++j) {
                op[j] = (B[0] * P0[j] + B[1] * P1[j]) + B[2] * P2[j];
                on[j] = (B[0] * N0[j] + B[1] * N1[j]) + B[2] * N2[j];
            }
            op[3] = 1.0f;
            on[3] = s.front ? 1.0f : 0.0f;
        }
}

// ShadowVolume::build/update (ShadowVolumes/src/ShadowVolume.cpp:15-194):
// the six quad vertices of triangle t (near copies, far (v - L) * infinity)
// and the index pattern its winding rule picks (dot of the averaged vertex
// normal with the light position, :55-61).
namespace {
const int kVolPatA[6][3] = {{1, 0, 3}, {1, 3, 4}, {2, 1, 4}, {2, 4, 5}, {0, 2, 5}, {0, 5, 3}};
const int kVolPatB[6][3] = {{4, 3, 0}, {4, 0, 1}, {5, 4, 1}, {5, 1, 2}, {3, 5, 2}, {3, 2, 0}};

const int (*volume_quad(const float* points, const float* normals, const int* indices, int t, const float L[3],
                        float infinity, float q[6][3]))[3] {
    const int* tri = indices + 3 * (size_t)t;
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) {
            q[k][a] = points[3 * (size_t)tri[k] + a];
            q[k + 3][a] = (points[3 * (size_t)tri[k] + a] - L[a]) * infinity;
        }
    const float* n0 = normals + 3 * (size_t)tri[0];
    const float* n1 = normals + 3 * (size_t)tri[1];
    const float* n2 = normals + 3 * (size_t)tri[2];
    float n[3];
    for (int a = 0; a < 3; ++a) n[a] = ((n0[a] + n1[a]) + n2[a]) / 3.0f;
    float d = n[0] * L[0] + n[1] * L[1] + n[2] * L[2];
    return d >= 0.0f ? kVolPatA : kVolPatB;
}
}  // namespace

extern "C" void or_shadow_volume_geometry(const float* points, const float* normals, const int* indices, int nt,
                                          const float L[3], float infinity, float* out) {
    for (int t = 0; t < nt; ++t) {
        float q[6][3];
        const int(*pat)[3] = volume_quad(points, normals, indices, t, L, infinity, q);
        for (int k = 0; k < 6; ++k)
            for (int j = 0; j < 3; ++j)
                for (int a = 0; a < 3; ++a) out[((size_t)t * 6 + k) * 9 + j * 3 + a] = q[pat[k][j]][a];
    }
}

extern "C" void or_shadow_volume_counts(const float* points, const float* normals, int nv,
                                        const int* indices, int nt, const float L[3],
                                        float infinity, const float mvp[16], int W, int H,
                                        int depth_func, uint8_t* out_stencil, float* out_depth,
                                        int threads) {
    (void)nv;
    const size_t npx = (size_t)W * H;
    std::vector<std::atomic<uint32_t>> depth(npx);
    for (auto& d : depth) d.store(fbits(1.0f), std::memory_order_relaxed);
    raster_depth(points, indices, nt, mvp, W, H, GI_BIAS_NONE, 0, 0, 0, depth.data(), threads);
    std::vector<std::atomic<int>> count(npx);
    for (auto& c : count) c.store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads(threads))
    for (int t = 0; t < nt; ++t) {
        float q[6][3];
        const int(*pat)[3] = volume_quad(points, normals, indices, t, L, infinity, q);
        for (int k = 0; k < 6; ++k) {
            float c[3][4];
            for (int j = 0; j < 3; ++j) transform(mvp, q[pat[k][j]], c[j]);
            raster_clipped(c[0], c[1], c[2], W, H,
                           [&](int, const Setup& s, int x, int y, const int64_t e[3]) {
                               float z = clamp01(depth_at(s, e));
                               size_t p = (size_t)y * W + x;
                               uint32_t db = depth[p].load(std::memory_order_relaxed);
                               float dv;
                               std::memcpy(&dv, &db, 4);
                               bool pass = depth_func == GI_DEPTH_LEQUAL ? (z <= dv) : (z < dv);
                               if (pass) count[p].fetch_add(s.front ? 1 : -1, std::memory_order_relaxed);
                           });
        }
    }
    for (size_t p = 0; p < npx; ++p) {
        out_stencil[p] = (uint8_t)((uint32_t)count[p].load(std::memory_order_relaxed) & 0xFFu);
        if (out_depth) {
            uint32_t u = depth[p].load(std::memory_order_relaxed);
            std::memcpy(&out_depth[p], &u, 4);
        }
    }
}

// ===========================================================================
// Per-pixel visibility: restatement of the fragment shaders.
// ===========================================================================
namespace {

struct V4 {
    float x, y, z, w;
};
struct V2 {
    float x, y;
};

// GLSL built-ins as the GLSL 1.20 spec defines them.
float gmin(float x, float y) { return y < x ? y : x; }
float gmax(float x, float y) { return x < y ? y : x; }
float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
float gfract(float x) { return x - std::floor(x); }
float gabs(float x) { return std::fabs(x); }

struct Ctx {
    const gi_vis_params* p;
    const float* map;
    int W, H;
    float sx, sy;  // shadowMapStep = (1/W, 1/H)
    float I;       // shadowIntensity
    // moment soft shadows: the moment map or its summed-area table (W x H
    // float4) and the two min-max levels VSSM's lookup blends
    const float* mom = nullptr;
    const float* hsm_lo = nullptr;
    const float* hsm_hi = nullptr;
    int lo_w = 0, lo_h = 0, hi_w = 0, hi_h = 0;
    float hsm_frac = 0.0f;
};

float fetch(const Ctx& c, float s, float t) {
    float fi = std::floor(s * (float)c.W);
    float fj = std::floor(t * (float)c.H);
    if (!(fi >= 0.0f && fi < (float)c.W && fj >= 0.0f && fj < (float)c.H)) return 0.0f;
    return c.map[(size_t)(int)fj * c.W + (int)fi];
}

V4 mat4_mul(const float m[16], V4 v) {
    V4 r;
    float* o = &r.x;
    for (int row = 0; row < 4; ++row)
        o[row] = m[0 * 4 + row] * v.x + m[1 * 4 + row] * v.y + m[2 * 4 + row] * v.z +
                 m[3 * 4 + row] * v.w;
    return r;
}

// computePreEvaluationBasedOnNormalOrientation (Shadow.frag:222-238 and its
// copies in every visibility shader).
float pretest(const Ctx& c, V4 vertex, V4 normal) {
    if (c.p->pretest == GI_PRETEST_OFF) return 1.0f;
    V4 ev = mat4_mul(c.p->camera_mv, vertex);
    const float* nm = c.p->normal_matrix;
    float nx = nm[0] * normal.x + nm[3] * normal.y + nm[6] * normal.z;
    float ny = nm[1] * normal.x + nm[4] * normal.y + nm[7] * normal.z;
    float nz = nm[2] * normal.x + nm[5] * normal.y + nm[8] * normal.z;
    float inv = 1.0f / std::sqrt(nx * nx + ny * ny + nz * nz);
    nx = nx * inv;
    ny = ny * inv;
    nz = nz * inv;
    float lx = c.p->light_position[0] - ev.x;
    float ly = c.p->light_position[1] - ev.y;
    float lz = c.p->light_position[2] - ev.z;
    float linv = 1.0f / std::sqrt(lx * lx + ly * ly + lz * lz);
    lx = lx * linv;
    ly = ly * linv;
    lz = lz * linv;
    if (!(normal.w != 0.0f)) {
        nx = nx * -1.0f;
        ny = ny * -1.0f;
        nz = nz * -1.0f;
    }
    float d = nx * lx + ny * ly + nz * lz;
    if (gmax(d, 0.0f) == 0.0f) return c.I;
    return 1.0f;
}

// ---- Shadow.frag ----------------------------------------------------------
float pcf_bilinear(const Ctx& c, V4 n) {
    float incrW = 1.0f / (float)c.W, incrH = 1.0f / (float)c.H;
    float illum = 0.0f;
    float offset = (float)c.p->penumbra_size;
    float step = 2.0f * offset / (float)c.p->kernel_order;
    int count = 0;
    for (float w = -offset; w < offset; w += step)
        for (float h = -offset; h < offset; h += step) {
            float d = fetch(c, n.x + w * incrW, n.y + h * incrH);
            if (n.z <= d) illum = illum + 1.0f;
            else illum += c.I;
            count++;
        }
    return illum / (float)count;
}

void cubic(float v, float out[4]) {
    float n[4] = {1.0f - v, 2.0f - v, 3.0f - v, 4.0f - v};
    float s[4];
    for (int i = 0; i < 4; ++i) s[i] = n[i] * n[i] * n[i];
    float x = s[0];
    float y = s[1] - 4.0f * s[0];
    float z = s[2] - 4.0f * s[1] + 6.0f * s[0];
    float w = 6.0f - x - y - z;
    const float k = 1.0f / 6.0f;
    out[0] = x * k;
    out[1] = y * k;
    out[2] = z * k;
    out[3] = w * k;
}

// textureBicubic (Shadow.frag:54-84) over a NEAREST depth texture.
float texture_bicubic(const Ctx& c, float u, float v) {
    float tsx = (float)c.W, tsy = (float)c.H;
    float itx = 1.0f / tsx, ity = 1.0f / tsy;
    float tx = u * tsx - 0.5f, ty = v * tsy - 0.5f;
    float fx = gfract(tx), fy = gfract(ty);
    tx -= fx;
    ty -= fy;
    float xc[4], yc[4];
    cubic(fx, xc);
    cubic(fy, yc);
    float cc[4] = {tx + -0.5f, tx + 1.5f, ty + -0.5f, ty + 1.5f};
    float s[4] = {xc[0] + xc[1], xc[2] + xc[3], yc[0] + yc[1], yc[2] + yc[3]};
    float num[4] = {xc[1], xc[3], yc[1], yc[3]};
    float off[4];
    for (int i = 0; i < 4; ++i) off[i] = cc[i] + num[i] / s[i];
    off[0] *= itx;
    off[1] *= itx;
    off[2] *= ity;
    off[3] *= ity;
    float s0 = fetch(c, off[0], off[2]);
    float s1 = fetch(c, off[1], off[2]);
    float s2 = fetch(c, off[0], off[3]);
    float s3 = fetch(c, off[1], off[3]);
    float sx = s[0] / (s[0] + s[1]);
    float sy = s[2] / (s[2] + s[3]);
    return gmix(gmix(s3, s2, sx), gmix(s1, s0, sx), sy);
}

float pcf_tricubic(const Ctx& c, V4 n) {
    float incrW = 1.0f / (float)c.W, incrH = 1.0f / (float)c.H;
    float illum = 0.0f;
    float offset = (float)c.p->penumbra_size;
    float step = 2.0f * offset / (float)c.p->kernel_order;
    int count = 0;
    for (float w = -offset; w < offset; w += step)
        for (float h = -offset; h < offset; h += step) {
            float d = texture_bicubic(c, n.x + w * incrW, n.y + h * incrH);
            if (n.z <= d) illum = illum + 1.0f;
            else illum += c.I;
            count++;
        }
    return illum / (float)count;
}

// ---- PlausibleSoftShadow.frag ----------------------------------------------
float blocker_search_width(const Ctx& c) {
    float R = c.p->light_radius;
    if ((float)c.W <= 1024.0f) return R / (float)c.W;
    return R / 1024.0f;
}

float avg_blocker_grid(const Ctx& c, V4 n) {
    float avg = 0.0f;
    int nb = 0;
    float bsw = blocker_search_width(c);
    float fw = ((float)c.p->blocker_search_size - 1.0f) * 0.5f;
    for (int h = (int)(-fw); (float)h <= fw; h++)
        for (int w = (int)(-fw); (float)w <= fw; w++) {
            float d = fetch(c, n.x + ((float)w * bsw) / fw, n.y + ((float)h * bsw) / fw);
            if (n.z > d) {
                avg += d;
                nb++;
            }
        }
    return nb == 0 ? 1.0f : avg / (float)nb;
}

float avg_blocker_poisson(const Ctx& c, V4 n, const float* tab) {
    float avg = 0.0f;
    int nb = 0;
    float bsw = blocker_search_width(c);
    for (int i = 0; i < c.p->poisson_blocker_taps; ++i) {
        float d = fetch(c, n.x + tab[2 * i] * bsw, n.y + tab[2 * i + 1] * bsw);
        if (n.z > d) {
            avg += d;
            nb++;
        }
    }
    return nb == 0 ? 1.0f : avg / (float)nb;
}

float penumbra_width(const Ctx& c, float avg, float z) {
    if (avg < c.p->pcss_min_blocker_depth) return 0.0f;
    float pw = ((z - avg) / avg) * c.p->light_radius;
    return (c.p->znear * pw) / z;
}

float pcss_filter_grid(const Ctx& c, float pw, V4 n) {
    float illum = 0.0f;
    int K = c.p->kernel_size;
    float step = 2.0f * pw / (float)K;
    float fw = ((float)K - 1.0f) * 0.5f;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    for (int h = (int)(-fw); (float)h <= fw; h++)
        for (int w = (int)(-fw); (float)w <= fw; w++) {
            float d = fetch(c, n.x + ((float)w * pw) / fw, n.y + ((float)h * pw) / fw);
            if (n.z <= d) illum = illum + 1.0f;
            else illum += c.I;
        }
    return illum / (float)(K * K);
}

float pcss_filter_poisson(const Ctx& c, float pw, V4 n, const float* tab) {
    float illum = 0.0f;
    int K = c.p->kernel_size;
    float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const int nf = c.p->poisson_filter_taps;
    for (int j = 0; j < nf; ++j) {
        float d = fetch(c, n.x + tab[2 * j] * pw, n.y + tab[2 * j + 1] * pw);
        if (n.z <= d) illum = illum + 1.0f;
        else illum += c.I;
    }
    return illum / (float)nf;
}

// ---- RBSM/NonConservativeSMSR.frag and FilteredRBSM.frag ---------------------
V4 nc_get_disc_all(const Ctx& c, V4 n) {  // getDisc(vec4, ..., false, false)
    V4 dir = {0, 0, 0, 0};
    n.x -= c.sx;
    dir.x = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
    n.x += 2.0f * c.sx;
    dir.y = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
    n.x -= c.sx;
    n.y += c.sy;
    dir.z = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
    n.y -= 2.0f * c.sy;
    dir.w = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
    return dir;
}

bool nc_get_disc_type(const Ctx& c, V4 n, V2 dir, float disc_type) {  // getDisc(vec4, vec2, float)
    if (dir.x == 0.0f) {
        n.x -= c.sx;
        float left = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (gabs(left - disc_type) == 0.0f) return true;
        n.x += 2.0f * c.sx;
        float right = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (gabs(right - disc_type) == 0.0f) return true;
        n.x -= c.sx;
    }
    if (dir.y == 0.0f) {
        n.y += c.sy;
        float bottom = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (gabs(bottom - disc_type) == 0.0f) return true;
        n.y -= 2.0f * c.sy;
        float top = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (gabs(top - disc_type) == 0.0f) return true;
    }
    return false;
}

// getDisc(vec4, vec2, vec4) with its write to the global newDepth.
bool nc_get_disc_vec(const Ctx& c, V4 n, V2 dir, V4 dt, float& new_depth) {
    V4 rel = n;
    new_depth = n.z;
    const float thr = c.p->depth_threshold;
    auto probe = [&](float s, float t) -> bool {
        float d = fetch(c, s, t);
        if (dt.z == 1.0f) {
            if (gabs(n.z - d) < thr) {
                n.z -= thr;
                new_depth = n.z;
            }
        }
        float v = (n.z <= d) ? 1.0f : 0.0f;
        return gabs(v - dt.z) == 0.0f;
    };
    if (dir.x == 0.0f) {
        if (dt.x == 0.5f || dt.x == 0.75f) {
            rel.x = n.x - c.sx;
            if (probe(rel.x, rel.y)) return true;
        }
        if (dt.x == 0.75f || dt.x == 0.25f) {
            rel.x = n.x + c.sx;
            if (probe(rel.x, rel.y)) return true;
        }
    }
    if (dir.y == 0.0f) {
        if (dt.y == 0.5f || dt.y == 0.75f) {
            rel.y = n.y + c.sy;
            if (probe(rel.x, rel.y)) return true;
        }
        if (dt.y == 0.75f || dt.y == 0.25f) {
            rel.y = n.y - c.sy;
            if (probe(rel.x, rel.y)) return true;
        }
    }
    return false;
}

float nc_disc_length(const Ctx& c, V4 in_disc, V4 lc, V2 dir, float sub) {
    V4 cc = lc;
    float found = 0.0f;
    float dist = 0.0f;
    float new_depth = 0.0f;
    V2 st = {dir.x * c.sx, dir.y * c.sy};
    cc.x += st.x;
    cc.y += st.y;
    const float thr = c.p->depth_threshold;
    for (int it = 0; it < c.p->max_search; it++) {
        float d = fetch(c, cc.x, cc.y);
        if (in_disc.z == 0.0f)
            if (gabs(cc.z - d) < thr) cc.z -= thr;
        float center = (cc.z <= d) ? 1.0f : 0.0f;
        if (gabs(center - in_disc.z) == 0.0f) {
            bool has = nc_get_disc_type(c, cc, V2{0.0f, 0.0f}, in_disc.z);
            found = has ? 1.0f : 0.0f;
            break;
        } else {
            bool has = nc_get_disc_vec(c, cc, dir, in_disc, new_depth);
            if (!has) break;
        }
        dist = dist + 1.0f;
        cc.x += st.x;
        cc.y += st.y;
        if (in_disc.z == 1.0f) cc.z = new_depth;
    }
    float a = dist + (1.0f - sub);
    return gmix(-a, a, found);
}

V4 nc_orientate(const Ctx& c, V4 lc, V4 disc, V2 sub) {
    V4 r;
    r.x = nc_disc_length(c, disc, lc, V2{-1.0f, 0.0f}, 1.0f - sub.x);
    r.y = nc_disc_length(c, disc, lc, V2{1.0f, 0.0f}, sub.x);
    r.z = nc_disc_length(c, disc, lc, V2{0.0f, -1.0f}, 1.0f - sub.y);
    r.w = nc_disc_length(c, disc, lc, V2{0.0f, 1.0f}, sub.y);
    return r;
}

float nc_rel_pos(const Ctx& c, V2 dir, float shadow, bool filtered) {
    float T = 1.0f;
    if (dir.x < 0.0f && dir.y < 0.0f) T = 0.0f;
    if (dir.x > 0.0f && dir.y > 0.0f) T = -2.0f;
    float edge_len = gmin(gabs(dir.x) + gabs(dir.y), (float)c.p->max_search);
    if (filtered) return (T * gabs(gmax(T * dir.x, T * dir.y))) / edge_len;
    return (gmax(T, 2.0f * shadow - 1.0f) * gabs(gmax(T * dir.x, T * dir.y))) / edge_len;
}

float nc_revectorize(V2 r, float shadow, bool filtered) {
    if (filtered) {
        if (r.x * r.y < 0.0f) return (1.0f - shadow) + (2.0f * shadow - 1.0f) * gmax(r.x, r.y);
        else if (r.x * r.y == 0.0f) return shadow;
        return gclamp((1.0f - shadow) + (2.0f * shadow - 1.0f) * (r.x + r.y), 0.0f, 1.0f);
    }
    if ((r.x * r.y == 2.0f * shadow) ||
        ((gabs(r.x) * gabs(r.y) > 0.0f) &&
         ((1.0f - shadow) + (2.0f * shadow - 1.0f) * (gabs(r.x) + gabs(r.y)) < 0.5f)))
        return 0.0f;
    return 1.0f;
}

V4 nc_compute_disc(const Ctx& c, V4 n, float dist) {
    float center = (n.z <= dist) ? 1.0f : 0.0f;
    float disc_type = 1.0f - center;
    V4 dir = nc_get_disc_all(c, n);
    float dx = gabs(dir.x - center), dy = gabs(dir.y - center);
    float dz = gabs(dir.z - center), dw = gabs(dir.w - center);
    return V4{(2.0f * dx + dy) / 4.0f, (2.0f * dz + dw) / 4.0f, disc_type, 1.0f};
}

float nc_revectorized_tap(const Ctx& c, V4 n, V4 disc, float shadow, bool filtered) {
    V2 sub = {gfract(n.x * (float)c.W), gfract(n.y * (float)c.H)};
    V4 ds = nc_orientate(c, n, disc, sub);
    V2 r = {nc_rel_pos(c, V2{ds.x, ds.y}, shadow, filtered),
            nc_rel_pos(c, V2{ds.z, ds.w}, shadow, filtered)};
    return gmix(nc_revectorize(r, shadow, filtered), 1.0f, c.I);
}

float nc_smsr(const Ctx& c, V4 n) {  // computeShadowFromSMSR
    float dist = fetch(c, n.x, n.y);
    V4 disc = nc_compute_disc(c, n, dist);
    float shadow = (n.z <= dist) ? 1.0f : 0.0f;
    if (disc.x > 0.0f || disc.y > 0.0f) {
        if (disc.x == 0.75f && disc.y == 0.75f) return gmix(1.0f - shadow, 1.0f, c.I);
        return nc_revectorized_tap(c, n, disc, shadow, false);
    }
    return gmix(shadow, 1.0f, c.I);
}

float nc_rpcf(const Ctx& c, V4 n, bool filtered) {  // computeShadowFromAccurateRPCF
    float incrW = 1.0f / (float)c.W, incrH = 1.0f / (float)c.H;
    float illum = 0.0f;
    float offset = (float)c.p->penumbra_size;
    float step = 2.0f * offset / (float)c.p->kernel_order;
    int count = 0;
    for (float w = -offset; w <= offset; w += step)
        for (float h = -offset; h <= offset; h += step) {
            V4 s = {n.x + w * incrW, n.y + h * incrH, n.z, n.w};
            float d = fetch(c, s.x, s.y);
            float shadow = (s.z <= d) ? 1.0f : 0.0f;
            V4 disc = nc_compute_disc(c, s, d);
            if (disc.x > 0.0f || disc.y > 0.0f) {
                illum += nc_revectorized_tap(c, s, disc, shadow, filtered);
            } else {
                shadow = gmix(shadow, 1.0f, c.I);
                illum += shadow;
            }
            count++;
        }
    return illum / (float)count;
}

// ---- SoftShadow/RBSSM.frag -----------------------------------------------------
// Revectorization-based soft shadow mapping.  getDisc(vec4, vec2, float) and
// getDisc(vec4, vec2, vec4) are the same functions as in
// NonConservativeSMSR.frag (nc_get_disc_type / nc_get_disc_vec above); the
// four-neighbour getDisc(vec4, float) (RBSSM.frag:37-61) is nc_get_disc_all
// without early exits.
float gstep(float edge, float x) { return x < edge ? 0.0f : 1.0f; }

// compressPositiveDiscontinuity / decompressPositiveDiscontinuity
// (RBSSM.frag:25-35).
float rb_compress(float nd) { return -2.0f - ((0.5f - nd) * 2.0f); }
float rb_decompress(float nd) { return 0.5f - ((nd + 2.0f) * -1.0f) / 2.0f; }

bool rb_disc_t(const Ctx& c, V4 n, float dx, float dy, float type) {
    return nc_get_disc_type(c, n, V2{dx, dy}, type);
}
bool rb_disc_v(const Ctx& c, V4 n, float dx, float dy, V4 type) {
    float unused = 0.0f;
    return nc_get_disc_vec(c, n, V2{dx, dy}, type, unused);
}

// computeDiscontinuityLength (RBSSM.frag:193-253).
float rb_disc_length(const Ctx& c, V4 in_disc, V4 lc, V2 dir) {
    V4 cc = lc;
    float found = 0.0f;
    if (dir.x == 0.0f && in_disc.x == 0.0f && in_disc.y != 0.0f) return -1.0f;
    if (dir.y == 0.0f && in_disc.x != 0.0f && in_disc.y == 0.0f) return -1.0f;
    if (((0.5f - in_disc.x) * 8.0f - 1.0f) == dir.x) return 1.0f;
    if (((in_disc.y - 0.5f) * 8.0f + 1.0f) == dir.y) return 1.0f;
    float dist = 1.0f;
    float new_depth = 0.0f;
    V2 st = {dir.x * c.sx, dir.y * c.sy};
    cc.x += st.x;
    cc.y += st.y;
    const float thr = c.p->depth_threshold;
    for (int it = 0; it < c.p->max_search; it++) {
        float d = fetch(c, cc.x, cc.y);
        if (in_disc.z == 0.0f)
            if (gabs(cc.z - d) < thr) cc.z -= thr;
        float center = (cc.z <= d) ? 1.0f : 0.0f;
        if (gabs(center - in_disc.z) == 0.0f) {
            bool has = nc_get_disc_type(c, cc, V2{0.0f, 0.0f}, in_disc.z);
            found = has ? 1.0f : 0.0f;
            break;
        } else {
            bool has = nc_get_disc_vec(c, cc, dir, in_disc, new_depth);
            if (!has) break;
        }
        dist = dist + 1.0f;
        cc.x += st.x;
        cc.y += st.y;
        if (in_disc.z == 1.0f) cc.z = new_depth;
    }
    return gmix(-dist, dist, found);
}

// normalizeDiscontinuitySpace (RBSSM.frag:255-280).
float rb_normalize_space(const Ctx& c, V2 dir, float sub) {
    if (dir.x < 0.0f && dir.y < 0.0f) return -1.0f;
    float edge = gmin(gabs(dir.x) + gabs(dir.y) - 1.0f, (float)c.p->max_search);
    float nd = 1.0f - gmax(dir.x, dir.y) / edge;
    if (dir.x == dir.y) nd += gmix(sub / edge, (1.0f - sub) / edge, gstep(0.5f, sub));
    else if (dir.x == gmax(dir.x, dir.y)) nd += (1.0f - sub) / edge;
    else nd += sub / edge;
    if (dir.x > 0.0f && dir.y > 0.0f) return rb_compress(nd);
    return nd;
}

// Branch coverage of smoothONDS for the tests: every return site counts
// its hits (indexed by source line).
std::atomic<unsigned long long> g_rb_hits[4096];
#define RB_RET(v)                                                    \
    do {                                                             \
        g_rb_hits[__LINE__ & 4095].fetch_add(1, std::memory_order_relaxed); \
        return (v);                                                  \
    } while (0)

// smoothONDS (RBSSM.frag:311-1117): the fill of one discontinuity tap.
// lc, nd and disc are by-value copies that the cases modify in place, as
// the shader does; a case that does not return leaves its changes for the
// cases below it.
float rb_smooth_onds(const Ctx& c, V4 lc, V4 nd, V4 disc, V2 sub) {
    const float sx = c.sx, sy = c.sy;
    if (disc.z == 0.0f) {
        // entering discontinuity: positive on both axes, both sides of one axis
        if (nd.x <= -2.0f && nd.y <= -2.0f && (disc.x == 0.75f || disc.y == 0.75f)) {
            bool left = true, right = true, bottom = true, top = true;
            if (disc.x == 0.75f) {
                if (disc.y == 0.0f) {
                    lc.y += sy;
                    top = rb_disc_t(c, lc, 0.0f, 1.0f, disc.z);
                    lc.y -= 2.0f * sy;
                    bottom = rb_disc_t(c, lc, 0.0f, 1.0f, disc.z);
                    lc.y += sy;
                    if (top && bottom) RB_RET(0.0f);
                    lc.y += gmix(-sy, sy, gstep(1.0f, top ? 1.0f : 0.0f));
                    left = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, 0.0f});
                    right = !left;
                } else {
                    if (disc.y == 0.5f) top = false;
                    else if (disc.y == 0.25f) bottom = false;
                    lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
                    left = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    right = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                    if (left && right) {
                        if (nd.y <= -2.0f) nd.y = rb_decompress(nd.y) + 0.5f;
                        float a = gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f);
                        float b = gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f);
                        float cc = gmix(1.0f - sub.y, sub.y, gstep(disc.y, 1.0f));
                        RB_RET(gmin(gmin(a, b), cc));
                    }
                }
            }
            if (disc.y == 0.75f) {
                if (disc.x == 0.0f) {
                    lc.x -= sx;
                    left = rb_disc_t(c, lc, 1.0f, 0.0f, disc.z);
                    lc.x += 2.0f * sx;
                    right = rb_disc_t(c, lc, 1.0f, 0.0f, disc.z);
                    lc.x -= sx;
                    if (left && right) RB_RET(0.0f);
                    lc.x += gmix(sx, -sx, gstep(1.0f, left ? 1.0f : 0.0f));
                    bottom = rb_disc_v(c, lc, 0.0f, 0.25f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    top = !bottom;
                } else {
                    if (disc.x == 0.5f) right = false;
                    else if (disc.x == 0.25f) left = false;
                    lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                    bottom = rb_disc_v(c, lc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                    top = rb_disc_v(c, lc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                    if (bottom && top) {
                        if (nd.x <= -2.0f) nd.x = rb_decompress(nd.x) + 0.5f;
                        float a = gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f);
                        float b = gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f);
                        float cc = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 1.0f));
                        RB_RET(gmin(gmin(a, b), cc));
                    }
                }
            }
            if (!left && !bottom) RB_RET(gclamp((1.0f - sub.x) - (1.0f - sub.y), 0.0f, 1.0f));
            else if (!right && !bottom) RB_RET(gclamp(sub.x - (1.0f - sub.y), 0.0f, 1.0f));
            else if (!left && !top) RB_RET(gclamp((1.0f - sub.y) - sub.x, 0.0f, 1.0f));
            else if (!right && !top) RB_RET(gclamp((1.0f - sub.y) - (1.0f - sub.x), 0.0f, 1.0f));
        }
        if (disc.x == 0.75f || disc.y == 0.75f) {
            // entering left and right, plus top or bottom
            if (disc.x == 0.75f && disc.y != 0.0f) {
                lc.y += ((disc.y - 0.75f) * 4.0f) * sy;
                bool left = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                bool right = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                if (!left && !right) RB_RET(gclamp(1.0f - nd.y, 0.0f, 1.0f));
                float s = gmix(1.0f - sub.y, sub.y, gstep(1.0f, disc.y));
                float a = gmix(s, gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f),
                               gstep(1.0f, right ? 1.0f : 0.0f));
                float b = gmix(s, gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f),
                               gstep(1.0f, left ? 1.0f : 0.0f));
                RB_RET(gmin(a, b));
            }
            // entering left and right only
            if (disc.x == 0.75f && disc.y == 0.0f) {
                bool topLeft = true, topRight = true, bottomLeft = true, bottomRight = true;
                bool topCenter = false, bottomCenter = false;
                V4 tlc = lc, blc = lc;
                if (!topCenter) {
                    tlc.y += sy;
                    float center = (tlc.z <= fetch(c, tlc.x, tlc.y)) ? 1.0f : 0.0f;
                    topCenter = !(center != 0.0f);
                    topLeft = rb_disc_v(c, tlc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    topRight = rb_disc_v(c, tlc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                }
                if (!bottomCenter) {
                    blc.y -= sy;
                    float center = (blc.z <= fetch(c, blc.x, blc.y)) ? 1.0f : 0.0f;
                    bottomCenter = !(center != 0.0f);
                    bottomLeft = rb_disc_v(c, blc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    bottomRight = rb_disc_v(c, blc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                }
                if (topCenter) {
                    topLeft = true;
                    topRight = true;
                }
                if (bottomCenter) {
                    bottomLeft = true;
                    bottomRight = true;
                }
                if (nd.y <= -2.0f) {
                    nd.y = rb_decompress(nd.y) + 0.5f;
                    float a = gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f);
                    float b = gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f);
                    if (!bottomRight || !topRight) RB_RET(a);
                    else if (!bottomLeft || !topLeft) RB_RET(b);
                    else RB_RET(gmin(a, b));
                }
                if ((!bottomRight && !bottomLeft) || (!topRight && !topLeft))
                    RB_RET(gclamp(1.0f - nd.y, 0.0f, 1.0f));
                else if (!bottomRight || !topRight)
                    RB_RET(gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f));
                else
                    RB_RET(gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f));
            }
            // entering top and bottom, plus left or right
            if (disc.x != 0.0f && disc.y == 0.75f) {
                lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                bool bottom = rb_disc_v(c, lc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                bool top = rb_disc_v(c, lc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                if (!bottom && !top) RB_RET(gclamp(1.0f - nd.x, 0.0f, 1.0f));
                float s = gmix(sub.x, 1.0f - sub.x, gstep(disc.x, 0.25f));
                float a = gmix(s, gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f), gstep(1.0f, top ? 1.0f : 0.0f));
                float b = gmix(s, gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f),
                               gstep(1.0f, bottom ? 1.0f : 0.0f));
                RB_RET(gmin(a, b));
            }
            // entering top and bottom only
            if (disc.x == 0.0f && disc.y == 0.75f) {
                bool topLeft = true, topRight = true, bottomLeft = true, bottomRight = true;
                bool leftCenter = false, rightCenter = false;
                V4 llc = lc, rlc = lc;
                if (!rightCenter) {
                    rlc.x += sx;
                    float center = (rlc.z <= fetch(c, rlc.x, rlc.y)) ? 1.0f : 0.0f;
                    rightCenter = !(center != 0.0f);
                    bottomRight = rb_disc_v(c, rlc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                    topRight = rb_disc_v(c, rlc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                }
                if (!leftCenter) {
                    llc.x -= sx;
                    float center = (llc.z <= fetch(c, llc.x, llc.y)) ? 1.0f : 0.0f;
                    leftCenter = !(center != 0.0f);
                    bottomLeft = rb_disc_v(c, llc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                    topLeft = rb_disc_v(c, llc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                }
                if (rightCenter) {
                    bottomRight = true;
                    topRight = true;
                }
                if (leftCenter) {
                    topLeft = true;
                    bottomLeft = true;
                }
                if (nd.x <= -2.0f) {
                    nd.x = rb_decompress(nd.x) + 0.5f;
                    float a = gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f);
                    float b = gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f);
                    if (!bottomRight || !bottomLeft) RB_RET(a);
                    else if (!topRight || !topLeft) RB_RET(b);
                    else RB_RET(gmin(a, b));
                }
                if ((!bottomRight && !topRight) || (!bottomLeft && !topLeft))
                    RB_RET(gclamp(1.0f - nd.x, 0.0f, 1.0f));
                else if (!bottomRight || !bottomLeft)
                    RB_RET(gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f));
                else
                    RB_RET(gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f));
            }
        }
        // corner: discontinuity on both axes
        if (disc.x > 0.0f && disc.y > 0.0f) {
            lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
            bool horizontal = rb_disc_t(c, lc, 1.0f, 0.0f, 0.0f);
            lc.x += ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
            lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
            bool vertical = rb_disc_t(c, lc, 0.0f, 1.0f, 0.0f);
            if (horizontal && !vertical) {
                disc.x = 0.0f;
            } else if (!horizontal && vertical) {
                disc.y = 0.0f;
            } else if (!horizontal && !vertical) {
                if (disc.y == 0.5f) RB_RET(gclamp((1.0f - nd.x) - (sub.y - 1.0f), 0.0f, 1.0f));
                else if (disc.y == 0.25f) RB_RET(gclamp((1.0f - nd.x) + sub.y, 0.0f, 1.0f));
            } else {
                float a, b;
                if (disc.x == 0.5f && disc.y == 0.5f) {
                    a = gmix(1.0f - sub.y, gclamp(1.0f - (nd.x - (1.0f - sub.y)), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(1.0f - (nd.y - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmin(a, b));
                } else if (disc.x == 0.5f && disc.y == 0.25f) {
                    a = gmix(sub.y, gclamp(1.0f - (nd.x - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(1.0f - (nd.y - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmin(a, b));
                } else if (disc.x == 0.25f && disc.y == 0.5f) {
                    a = gmix(1.0f - sub.y, gclamp(1.0f - (nd.x - (1.0f - sub.y)), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(1.0f - (nd.y - (1.0f - sub.x)), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmin(a, b));
                } else if (disc.x == 0.25f && disc.y == 0.25f) {
                    a = gmix(sub.y, gclamp(1.0f - (nd.x - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(1.0f - (nd.y - (1.0f - sub.x)), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmin(a, b));
                }
            }
        }
        if (nd.x <= -2.0f) RB_RET(gmix(1.0f - sub.y, sub.y, gstep(disc.y, 0.25f)));
        if (nd.y <= -2.0f) RB_RET(gmix(sub.x, 1.0f - sub.x, gstep(disc.x, 0.25f)));
        if (disc.y > 0.0f) {
            if (disc.y == 0.5f) RB_RET(gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f));
            else RB_RET(gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f));
        }
        if (disc.x > 0.0f) {
            if (disc.x == 0.5f) RB_RET(gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f));
            else RB_RET(gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f));
        }
    } else {
        // exiting discontinuity
        if (disc.x == 0.75f || disc.y == 0.75f) {
            // exiting left and right only
            if (disc.x == 0.75f && disc.y == 0.0f) {
                V4 ref = lc;
                ref.x = lc.x - sx;
                bool left = rb_disc_v(c, ref, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                ref.x = lc.x + sx;
                bool right = rb_disc_v(c, ref, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                if (left && right) {
                    RB_RET(gclamp(nd.y, 0.0f, 1.0f));
                } else if (left || right) {
                    if (!left) RB_RET(gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y)));
                    else RB_RET(gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y)));
                } else {
                    // one pass of the commented-out while loop: count = 0, mult = 1
                    const int count = 0;
                    const int mult = (count / 2) + 1;
                    if (std::fmod((float)count, 2.0f) == 0.0f) ref.y = lc.y + (float)mult * sy;
                    else ref.y = lc.y - (float)mult * sy;
                    ref.x = lc.x - sx;
                    left = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    ref.x = lc.x + sx;
                    right = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    if (left && right) {
                        RB_RET(gclamp(nd.y, 0.0f, 1.0f));
                    } else {
                        if (!left) RB_RET(gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y)));
                        else RB_RET(gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y)));
                    }
                }
            }
            // exiting left and right, plus top or bottom
            if (disc.x == 0.75f && disc.y != 0.0f) {
                lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
                bool left = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                bool right = rb_disc_v(c, lc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                float a = 0.0f, b = 0.0f;
                if (left && right) {
                    RB_RET(gclamp(nd.y, 0.0f, 1.0f));
                } else if (left || right) {
                    if (left) a = gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
                    else a = gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    if (right) b = gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
                    else b = gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmax(a, b));
                } else {
                    if (disc.y == 0.75f) RB_RET(0.0f);
                    V4 ref = lc;
                    ref.x = lc.x - sx;
                    left = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    ref.x = lc.x + sx;
                    right = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
                    if (left && right) {
                        RB_RET(gclamp(nd.y, 0.0f, 1.0f));
                    } else {
                        a = gmix(1.0f - sub.x, sub.x, gstep(1.0f, left ? 1.0f : 0.0f));
                        b = gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
                        RB_RET(gmax(a, b));
                    }
                }
            }
            // exiting top and bottom only
            if (disc.x == 0.0f && disc.y == 0.75f) {
                V4 ref = lc;
                ref.y = lc.y - sy;
                bool top = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                ref.y = lc.y + sy;
                bool bottom = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                if (bottom && top) {
                    RB_RET(gclamp(nd.x, 0.0f, 1.0f));
                } else if (bottom || top) {
                    if (!top) RB_RET(gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x)));
                    else RB_RET(gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x)));
                } else {
                    const int count = 0;
                    const int mult = (count / 2) + 1;
                    if (std::fmod((float)count, 2.0f) == 0.0f) ref.x = lc.x + (float)mult * sx;
                    else ref.x = lc.x - (float)mult * sx;
                    ref.y = lc.y - sy;
                    top = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    ref.y = lc.y + sy;
                    bottom = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    if (top && bottom) {
                        RB_RET(gclamp(nd.x, 0.0f, 1.0f));
                    } else {
                        if (!top) RB_RET(gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x)));
                        else RB_RET(gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x)));
                    }
                }
            }
            // exiting top and bottom, plus left or right
            if (disc.x != 0.0f && disc.y == 0.75f) {
                lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                bool bottom = rb_disc_v(c, lc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                bool top = rb_disc_v(c, lc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                float a = 0.0f, b = 0.0f;
                if (bottom && top) {
                    RB_RET(gclamp(nd.x, 0.0f, 1.0f));
                } else if (bottom || top) {
                    if (top) a = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
                    else a = gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    if (bottom) b = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
                    else b = gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    RB_RET(gmax(a, b));
                } else {
                    if (disc.x == 0.75f) RB_RET(0.0f);
                    V4 ref = lc;
                    ref.y = lc.y - sy;
                    top = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    ref.y = lc.y + sy;
                    bottom = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                    if (top && bottom) {
                        RB_RET(gclamp(nd.x, 0.0f, 1.0f));
                    } else {
                        a = gmix(1.0f - sub.y, sub.y, gstep(1.0f, top ? 1.0f : 0.0f));
                        b = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
                        RB_RET(gmax(a, b));
                    }
                }
            }
        }
        // corner: discontinuity on both axes (the x step is added twice, as
        // in the shader)
        if (disc.x > 0.0f && disc.y > 0.0f) {
            lc.x += ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
            bool horizontal = rb_disc_t(c, lc, 1.0f, 0.0f, disc.z);
            lc.x += ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
            lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
            bool vertical = rb_disc_t(c, lc, 0.0f, 1.0f, disc.z);
            if (horizontal && !vertical) {
                disc.x = 0.0f;
            } else if (!horizontal && vertical) {
                disc.y = 0.0f;
            } else if (!horizontal && !vertical) {
                if (disc.y == 0.5f) RB_RET(gclamp(sub.y - (1.0f - nd.x), 0.0f, 1.0f));
                else if (disc.y == 0.25f) RB_RET(gclamp((1.0f - sub.y) - (1.0f - nd.x), 0.0f, 1.0f));
            } else {
                float a, b;
                if (disc.x == 0.5f && disc.y == 0.5f) {
                    a = gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmax(a, b));
                } else if (disc.x == 0.5f && disc.y == 0.25f) {
                    a = gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmax(a, b));
                } else if (disc.x == 0.25f && disc.y == 0.5f) {
                    a = gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmax(a, b));
                } else if (disc.x == 0.25f && disc.y == 0.25f) {
                    a = gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    RB_RET(gmax(a, b));
                }
            }
        }
        if (nd.x <= -2.0f) RB_RET(gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f)));
        if (nd.y <= -2.0f) RB_RET(gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f)));
        if (disc.y > 0.0f) {
            if (disc.y == 0.5f) RB_RET(gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f));
            else RB_RET(gclamp(nd.x - sub.y, 0.0f, 1.0f));
        }
        if (disc.x > 0.0f) {
            if (disc.x == 0.5f) RB_RET(gclamp(nd.y - sub.x, 0.0f, 1.0f));
            else RB_RET(gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f));
        }
    }
    RB_RET(1.0f - disc.z);
}

// RBSSM (RBSSM.frag:1202-1339, the commented-out branches left out): K x K
// taps over the penumbra; a discontinuity tap is filled by smoothONDS.
float rb_filter(const Ctx& c, float pw, V4 n) {
    float illum = 0.0f;
    const int K = c.p->kernel_size;
    float fw = ((float)K - 1.0f) * 0.5f;
    for (int h = (int)(-fw); (float)h <= fw; h++)
        for (int w = (int)(-fw); (float)w <= fw; w++) {
            V4 lc = {n.x + ((float)w * pw) / fw, n.y + ((float)h * pw) / fw, n.z, n.w};
            V2 sub = {gfract(lc.x * (float)c.W), gfract(lc.y * (float)c.H)};
            float d = fetch(c, lc.x, lc.y);
            V4 disc = nc_compute_disc(c, lc, d);
            if (disc.x > 0.0f || disc.y > 0.0f) {
                V4 ds;
                ds.x = rb_disc_length(c, disc, lc, V2{-1.0f, 0.0f});
                ds.y = rb_disc_length(c, disc, lc, V2{1.0f, 0.0f});
                ds.z = rb_disc_length(c, disc, lc, V2{0.0f, -1.0f});
                ds.w = rb_disc_length(c, disc, lc, V2{0.0f, 1.0f});
                V4 nd = {rb_normalize_space(c, V2{ds.x, ds.y}, sub.x),
                         rb_normalize_space(c, V2{ds.z, ds.w}, sub.y), 0.0f, 0.0f};
                float fill = rb_smooth_onds(c, lc, nd, disc, sub);
                fill = gmix(fill, 1.0f, c.I);
                illum += fill;
            } else {
                float shadow = (lc.z <= d) ? 1.0f : c.I;
                illum += shadow;
            }
        }
    return illum / (float)(K * K);
}

// revectorizationBasedShadowMappingSmoothing (RBSSM.frag:1341-1360).
float rb_rbssm(const Ctx& c, V4 n) {
    float avg = avg_blocker_grid(c, n);
    float pw = penumbra_width(c, avg, n.z);
    float step = 2.0f * pw / (float)c.p->kernel_size;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    return rb_filter(c, pw, n);
}

// ---- RBSM/ConservativeSMSR.frag ---------------------------------------------
V4 cs_compute_disc(const Ctx& c, V4 s) {
    V4 dir = {0, 0, 0, 0};
    s.x -= c.sx;
    dir.x = (s.z <= fetch(c, s.x, s.y)) ? 1.0f : 0.0f;
    s.x += 2.0f * c.sx;
    dir.y = (s.z <= fetch(c, s.x, s.y)) ? 1.0f : 0.0f;
    s.x -= c.sx;
    s.y += c.sy;
    dir.z = (s.z <= fetch(c, s.x, s.y)) ? 1.0f : 0.0f;
    s.y -= 2.0f * c.sy;
    dir.w = (s.z <= fetch(c, s.x, s.y)) ? 1.0f : 0.0f;
    return V4{gabs(dir.x - 1.0f), gabs(dir.y - 1.0f), gabs(dir.z - 1.0f), gabs(dir.w - 1.0f)};
}

float cs_rel_dist(const Ctx& c, V4 s, V2 dir, float cc) {
    V4 t = s;
    float found = 0.0f, distance = 0.0f;
    V2 st = {dir.x * c.sx, dir.y * c.sy};
    t.x += st.x;
    t.y += st.y;
    const float thr = c.p->depth_threshold;
    for (int it = 0; it < c.p->max_search; it++) {
        float d = fetch(c, t.x, t.y);
        if (gabs(t.z - d) < thr) t.z -= thr;
        float center = (t.z <= d) ? 1.0f : 0.0f;
        bool umbra = !(center != 0.0f);
        if (umbra) {
            found = 1.0f;
            break;
        } else {
            V4 dd = cs_compute_disc(c, t);
            if ((dd.x + dd.y + dd.z + dd.w) == 0.0f) break;
        }
        distance = distance + 1.0f;
        t.x += st.x;
        t.y += st.y;
    }
    distance = distance + (1.0f - cc);
    return gmix(-distance, distance, found);
}

float cs_normalize(const Ctx& c, V2 d) {
    float T = 1.0f;
    if (d.x < 0.0f && d.y < 0.0f) T = 0.0f;
    if (d.x > 0.0f && d.y > 0.0f) T = -2.0f;
    float len = gmin(gabs(d.x) + gabs(d.y), (float)c.p->max_search);
    return gabs(gmax(T * d.x, T * d.y)) / len;
}

float cs_revectorize(const Ctx& c, V2 r) {
    if ((r.x * r.y > 0.0f) && (1.0f - r.x > r.y)) return c.I;
    return 1.0f;
}

float cs_revectorized(const Ctx& c, V4 s) {
    V2 sub = {gfract(s.x * (float)c.W), gfract(s.y * (float)c.H)};
    float dl = cs_rel_dist(c, s, V2{-1.0f, 0.0f}, 1.0f - sub.x);
    float dr = cs_rel_dist(c, s, V2{1.0f, 0.0f}, sub.x);
    float db = cs_rel_dist(c, s, V2{0.0f, -1.0f}, 1.0f - sub.y);
    float dt = cs_rel_dist(c, s, V2{0.0f, 1.0f}, sub.y);
    V2 r = {cs_normalize(c, V2{dl, dr}), cs_normalize(c, V2{db, dt})};
    return cs_revectorize(c, r);
}

float cs_smsr(const Ctx& c, V4 s) {  // computeShadowFromSMSR (conservative)
    float d = fetch(c, s.x, s.y);
    float shadow = (s.z <= d) ? 1.0f : 0.0f;
    if (shadow == 0.0f) return c.I;
    V4 dd = cs_compute_disc(c, s);
    if ((dd.x + dd.y + dd.z + dd.w) == 0.0f) return 1.0f;
    else if ((dd.x + dd.y) == 2.0f || (dd.z + dd.w) == 2.0f) return c.I;
    return cs_revectorized(c, s);
}

float cs_rpcf(const Ctx& c, V4 n) {  // computeShadowFromRPCF (conservative)
    float incrW = 1.0f / (float)c.W, incrH = 1.0f / (float)c.H;
    float illum = 0.0f;
    float offset = (float)c.p->penumbra_size;
    float step = 2.0f * offset / (float)c.p->kernel_order;
    int count = 0;
    for (float w = -offset; w <= offset; w += step)
        for (float h = -offset; h <= offset; h += step) {
            float d = fetch(c, n.x + w * incrW, n.y + h * incrH);
            float shadow = (n.z <= d) ? 1.0f : c.I;
            if (shadow == 1.0f) {
                V4 s = {n.x + w * incrW, n.y + h * incrH, n.z, n.w};
                V4 dd = cs_compute_disc(c, s);
                if (dd.x == 0.0f && dd.y == 0.0f) illum = illum + 1.0f;
                else illum += cs_revectorized(c, s);
            } else {
                illum += c.I;
            }
            count++;
        }
    return illum / (float)count;
}

// ---- filtered moment maps (VSM, ESM, EVSM, MSM) ------------------------------
// ShadowMapping/src/main.cpp:220-240 (moment shaders), 374-396 (filters),
// Shadow.frag:118-220 (lookups).  The choices GL leaves to the driver are
// made as in the CUDA path: moments from the depth map's value; dFdx / dFdy
// as differences inside each 2 x 2 quad (0 next to an empty texel); mip
// levels as 2 x 2 box averages ((a + b) + (c + d)) * 0.25; the 7 Gaussian
// taps on texel centres with a zero border, products and sums rounded
// separately in tap order; lookups bilinear at level 0 with FP32 weights.
const float kGauss7[7] = {1.0f / 64.0f, 6.0f / 64.0f, 15.0f / 64.0f, 20.0f / 64.0f,
                          15.0f / 64.0f, 6.0f / 64.0f, 1.0f / 64.0f};

float gl_linearize(float depth) { return 2.0f / (1001.0f - depth * 999.0f); }

// MyGLGeometryViewer::configureMoments: the optimised 4MSM quantisation
// (rows as written), column-major as the shader receives it, and its
// inverse computed in double from the float matrix.
void msm_quantization(float mq[16], float mqi[16]) {
    const double Q[4][4] = {{-2.07224649, 32.2370378, -68.5710746, 39.3703274},
                            {13.7948857, -59.4683976, 82.035975, -35.3649032},
                            {0.105877704, -1.90774663, 9.34965551, -6.65434907},
                            {9.79240621, -33.76521106, 47.9456097, -23.9728048}};
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            const float q = (float)Q[r][c];
            mq[c * 4 + r] = q;
            a[r][c] = (double)q;
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        const double inv = 1.0 / a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] *= inv;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) mqi[c * 4 + r] = (float)a[r][c + 4];
}

// The blurred window-size moment map (W x W float4) of an S x S depth map.
std::vector<float> moment_filtered(int tech, const float* depth, int S, int W) {
    std::vector<float> m((size_t)S * S * 4);
    float mq[16], mqi[16];
    msm_quantization(mq, mqi);
    const float tq0 = 0.0359558848f;
    auto lin_at = [&](int x, int y, bool& empty) {
        const float d = depth[(size_t)y * S + x];
        empty = !(d < 1.0f);
        return gl_linearize(d);
    };
    for (int y = 0; y < S; ++y)
        for (int x = 0; x < S; ++x) {
            float* o = &m[4 * ((size_t)y * S + x)];
            bool empty;
            const float d = lin_at(x, y, empty);
            if (empty) {
                o[0] = o[1] = o[2] = 0.0f;
                o[3] = 1.0f;
            } else if (tech == GI_TECH_ESM) {
                o[0] = d;
                o[1] = o[2] = 0.0f;
                o[3] = 1.0f;
            } else if (tech == GI_TECH_MSM) {
                const float d2 = d * d, d3 = d2 * d, d4 = d3 * d;
                for (int r = 0; r < 4; ++r)
                    o[r] = mq[r] * d + mq[4 + r] * d2 + mq[8 + r] * d3 + mq[12 + r] * d4 + (r == 0 ? tq0 : 0.0f);
            } else {
                bool el, er, eb, et;
                const int xr = (x | 1) < S ? (x | 1) : x, yt = (y | 1) < S ? (y | 1) : y;
                const float l = lin_at(x & ~1, y, el), rr = lin_at(xr, y, er);
                const float b = lin_at(x, y & ~1, eb), t = lin_at(x, yt, et);
                const float dx = (el || er) ? 0.0f : rr - l;
                const float dy = (eb || et) ? 0.0f : t - b;
                float m2 = d * d;
                m2 = m2 + 0.25f * (dx * dx + dy * dy);
                o[0] = d;
                o[1] = m2;
                o[2] = tech == GI_TECH_EVSM ? d : 0.0f;
                o[3] = tech == GI_TECH_EVSM ? 1.0f : 0.0f;
            }
        }
    for (int side = S; side > W; side /= 2) {
        const int h = side / 2;
        std::vector<float> n((size_t)h * h * 4);
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < h; ++x)
                for (int k = 0; k < 4; ++k) {
                    const float a = m[4 * ((size_t)(2 * y) * side + 2 * x) + k];
                    const float b = m[4 * ((size_t)(2 * y) * side + 2 * x + 1) + k];
                    const float c = m[4 * ((size_t)(2 * y + 1) * side + 2 * x) + k];
                    const float d = m[4 * ((size_t)(2 * y + 1) * side + 2 * x + 1) + k];
                    n[4 * ((size_t)y * h + x) + k] = ((a + b) + (c + d)) * 0.25f;
                }
        m.swap(n);
    }
    auto blur = [&](const std::vector<float>& in, int dx, int dy) {
        std::vector<float> out((size_t)W * W * 4);
        for (int y = 0; y < W; ++y)
            for (int x = 0; x < W; ++x) {
                auto tap = [&](int k, int ch) {
                    const int xx = x + dx * k, yy = y + dy * k;
                    if (xx < 0 || xx >= W || yy < 0 || yy >= W) return 0.0f;
                    return in[4 * ((size_t)yy * W + xx) + ch];
                };
                float* o = &out[4 * ((size_t)y * W + x)];
                if (tech != GI_TECH_ESM) {
                    for (int ch = 0; ch < 4; ++ch) {
                        float r = 0.0f;
                        for (int k = -3; k <= 3; ++k) r = r + tap(k, ch) * kGauss7[3 + k];
                        o[ch] = r;
                    }
                } else {
                    const float s0 = tap(-3, 0), s1 = tap(-2, 0);
                    float sum = s0 + std::log(kGauss7[0] + kGauss7[1] * std::exp(s1 - s0));
                    for (int i = 2; i < 7; ++i) sum = sum + std::log(1.0f + kGauss7[i] * std::exp(tap(i - 3, 0) - sum));
                    o[0] = o[1] = o[2] = o[3] = sum;
                }
            }
        return out;
    };
    return blur(blur(m, 1, 0), 0, 1);
}

V4 moment_fetch(const Ctx& c, float s, float t) {
    const float u = s * (float)c.W - 0.5f, v = t * (float)c.H - 0.5f;
    V4 r{0.0f, 0.0f, 0.0f, 0.0f};
    if (!(u > -2.0f && u < (float)c.W + 1.0f && v > -2.0f && v < (float)c.H + 1.0f)) return r;
    const float fu = std::floor(u), fv = std::floor(v);
    const int i0 = (int)fu, j0 = (int)fv;
    const float a = u - fu, b = v - fv;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float T[4][4];
    for (int k = 0; k < 4; ++k) {
        const int i = i0 + (k & 1), j = j0 + (k >> 1);
        for (int ch = 0; ch < 4; ++ch)
            T[k][ch] = (i >= 0 && i < c.W && j >= 0 && j < c.H) ? c.map[4 * ((size_t)j * c.W + i) + ch] : 0.0f;
    }
    float* o = &r.x;
    for (int ch = 0; ch < 4; ++ch) o[ch] = ((w00 * T[0][ch] + w10 * T[1][ch]) + w01 * T[2][ch]) + w11 * T[3][ch];
    return r;
}

// chebyshevUpperBound (Shadow.frag:118-131)
float chebyshev(float mx, float my, float z, float I) {
    if (z <= mx) return 1.0f;
    const float variance = my - mx * mx;
    const float d = z - mx;
    float p_max = variance / (variance + d * d);
    const float p = z <= mx ? 1.0f : 0.0f;
    p_max = gmax(p, p_max);
    return gmix(p_max, 1.0f, I);
}

float moment_lookup(const Ctx& c, V4 n) {
    const int tech = c.p->technique;
    if (tech == GI_TECH_VSM) {  // varianceShadowMapping (:133-141)
        const V4 m = moment_fetch(c, n.x, n.y);
        return chebyshev(m.x, m.y, gl_linearize(n.z), c.I);
    }
    if (tech == GI_TECH_ESM) {  // exponentialShadowMapping (:144-157)
        const float k = 80.0f;
        float e2 = moment_fetch(c, n.x, n.y).x;
        e2 = std::exp(k * e2);
        const float z = gl_linearize(n.z);
        const float e1 = std::exp(-k * z);
        return gclamp(e1 * e2, c.I, 1.0f);
    }
    if (tech == GI_TECH_EVSM) {  // exponentialVarianceShadowMapping (:160-176)
        const float z = gl_linearize(n.z);
        const V4 m = moment_fetch(c, n.x, n.y);
        const float variance = chebyshev(m.x, m.y, z, c.I);
        const float k = 60.0f;
        const float e1 = std::exp(-k * z);
        const float e2 = std::exp(k * m.z);
        return gmin(variance, gclamp(e1 * e2, c.I, 1.0f));
    }
    // hamburger4MSM (:178-220)
    float mq[16], mqi[16];
    msm_quantization(mq, mqi);
    V4 b = moment_fetch(c, n.x, n.y);
    b = V4{b.x - 0.0359558848f, b.y - 0.0f, b.z - 0.0f, b.w - 0.0f};
    b = mat4_mul(mqi, b);
    const float bias = 0.00003f;
    const float z0 = gl_linearize(n.z);
    const float ob = 1.0f - bias, hb = bias * 0.5f;
    b = V4{ob * b.x + hb, ob * b.y + hb, ob * b.z + hb, ob * b.w + hb};
    const float dx = 1.0f, dy = z0, dz = z0 * z0;
    const float L10 = b.x, L20 = b.y;
    const float D11 = b.y - L10 * L10;
    const float L21 = (b.z - L20 * L10) / D11;
    const float D22 = b.w - L20 * L20 - L21 * L21 * D11;
    const float y0 = dx;
    float y1 = dy - L10 * y0;
    float y2 = dz - L20 * y0 - L21 * y1;
    y1 = y1 / D11;
    y2 = y2 / D22;
    const float cz = y2, cy = y1 - L21 * cz, cx = y0 - L10 * cy - L20 * cz;
    const float p = cy / cz, q = cx / cz;
    const float D = ((p * p) / 4.0f) - q;
    const float r = std::sqrt(D);
    const float zy = -(p / 2.0f) - r, zz = -(p / 2.0f) + r;
    if (z0 <= zy) return 1.0f;
    if (z0 <= zz)
        return gclamp(1.0f - gclamp((z0 * zz - b.x * (z0 + zz) + b.y) / ((zz - zy) * (z0 - zy)), 0.0f, 1.0f), c.I,
                      1.0f);
    return gclamp(1.0f - gclamp(1.0f - (zy * zz - b.x * (zy + zz) + b.y) / ((z0 - zy) * (z0 - zz)), 0.0f, 1.0f),
                  c.I, 1.0f);
}

// ---- moment soft shadows (SoftShadowMapping PlausibleSoftShadow.frag) --------
// SAVSM, VSSM, ESSM and MSSM with or without the summed-area table.  The
// choices GL leaves to the driver are those of the filtered moment maps
// above (moments from the depth map's value, dFdx / dFdy inside 2 x 2
// quads, lookups bilinear at level 0 with a zero border) plus: the SAT
// passes read exact texels (their coordinates are texel centres); the
// min-max levels read level k - 1 at the half-texel positions MinMax.frag's
// offsets give (each read the 0.25-weighted average of a 2 x 2 block); the
// min-max lookup at lod L blends levels floor(L) and floor(L) + 1 as
// (1 - f) t1 + f t2 with f = L - floor(L).
bool is_soft_moment(int t) { return t >= GI_TECH_SAVSM && t <= GI_TECH_MSSM; }

// Moments.frag (SAVSM / VSSM / MSSM) or Exponential.frag (ESSM) per texel
// of the light map; texels no fragment reached keep the clear colour 0.
std::vector<float> soft_moment_map(int tech, const float* depth, int S, int T) {
    std::vector<float> m((size_t)S * T * 4, 0.0f);
    float mq[16], mqi[16];
    msm_quantization(mq, mqi);
    const float tq0 = 0.0359558848f;
    auto lin_at = [&](int x, int y, bool& empty) {
        const float d = depth[(size_t)y * S + x];
        empty = !(d < 1.0f);
        return gl_linearize(d);
    };
    for (int y = 0; y < T; ++y)
        for (int x = 0; x < S; ++x) {
            float* o = &m[4 * ((size_t)y * S + x)];
            bool empty;
            const float d = lin_at(x, y, empty);
            if (empty) continue;
            if (tech == GI_TECH_ESSM) {
                const float e = std::exp(80.0f * d);
                o[0] = d;
                o[1] = e;
                o[2] = e * d;
            } else if (tech == GI_TECH_MSSM) {
                const float d2 = d * d, d3 = d2 * d, d4 = d3 * d;
                for (int r = 0; r < 4; ++r)
                    o[r] = mq[r] * d + mq[4 + r] * d2 + mq[8 + r] * d3 + mq[12 + r] * d4 + (r == 0 ? tq0 : 0.0f);
            } else {
                bool el, er, eb, et;
                const int xr = (x | 1) < S ? (x | 1) : x, yt = (y | 1) < T ? (y | 1) : y;
                const float l = lin_at(x & ~1, y, el), rr = lin_at(xr, y, er);
                const float b = lin_at(x, y & ~1, eb), t = lin_at(x, yt, et);
                const float dx = (el || er) ? 0.0f : rr - l;
                const float dy = (eb || et) ? 0.0f : t - b;
                o[0] = d - 0.5f;
                o[1] = d * d + (0.25f * (dx * dx + dy * dy) - 0.5f);
            }
        }
    return m;
}

// main.cpp:943-971: int m = logf(width) / logf(2); for i < m a horizontal
// then a vertical pass at offset 2^i, reads outside the map giving 0.
int sat_iterations(int S) { return (int)(std::log((float)S) / std::log(2.0f)); }

void summed_area_table(std::vector<float>& s, int S, int T) {
    std::vector<float> t(s.size());
    const int m = sat_iterations(S);
    for (int i = 0; i < m; ++i) {
        const int d = 1 << i;
        for (int y = 0; y < T; ++y)
            for (int x = 0; x < S; ++x)
                for (int ch = 0; ch < 4; ++ch)
                    t[4 * ((size_t)y * S + x) + ch] =
                        s[4 * ((size_t)y * S + x) + ch] + (x >= d ? s[4 * ((size_t)y * S + x - d) + ch] : 0.0f);
        for (int y = 0; y < T; ++y)
            for (int x = 0; x < S; ++x)
                for (int ch = 0; ch < 4; ++ch)
                    s[4 * ((size_t)y * S + x) + ch] =
                        t[4 * ((size_t)y * S + x) + ch] + (y >= d ? t[4 * ((size_t)(y - d) * S + x) + ch] : 0.0f);
    }
}

// renderHSM: level 0 (PrepareMinMax.frag) and levels 1..L (MinMax.frag),
// float2 per texel; level k is (S >> k) x (T >> k).
std::vector<std::vector<float>> hsm_levels(const float* depth, int S, int T, float alpha, float beta, int L) {
    std::vector<std::vector<float>> lv(L + 1);
    lv[0].resize((size_t)S * T * 2);
    for (size_t i = 0; i < (size_t)S * T; ++i) {
        const float d = depth[i];
        const float mn = d == 0.0f ? 1.0f : d;
        lv[0][2 * i] = mn + alpha;
        lv[0][2 * i + 1] = d + beta;
    }
    for (int k = 1; k <= L; ++k) {
        const int pw = S >> (k - 1), ph = T >> (k - 1), w = S >> k, h = T >> k;
        const std::vector<float>& in = lv[k - 1];
        lv[k].resize((size_t)w * h * 2);
        auto tex = [&](int i, int j, int ch) {
            return (i >= 0 && i < pw && j >= 0 && j < ph) ? in[2 * ((size_t)j * pw + i) + ch] : 0.0f;
        };
        // a read at a half-texel position: the 2 x 2 block from (i0, j0),
        // bilinear weights 0.25 in moment_fetch's order
        auto quad = [&](int i0, int j0, int ch) {
            return ((0.25f * tex(i0, j0, ch) + 0.25f * tex(i0 + 1, j0, ch)) + 0.25f * tex(i0, j0 + 1, ch)) +
                   0.25f * tex(i0 + 1, j0 + 1, ch);
        };
        for (int j = 0; j < h; ++j)
            for (int i = 0; i < w; ++i) {
                // shadowValues[0..3]: (-, -), (-, +), (+, -), (+, +) offsets
                // of one output texel = two input texels
                const int xa = 2 * i - 2, xb = 2 * i + 2, ya = 2 * j - 2, yb = 2 * j + 2;
                const float mn = gmin(quad(xa, ya, 0), gmin(quad(xa, yb, 0), gmin(quad(xb, ya, 0), quad(xb, yb, 0))));
                const float mx = gmax(quad(xa, ya, 1), gmax(quad(xa, yb, 1), gmax(quad(xb, ya, 1), quad(xb, yb, 1))));
                lv[k][2 * ((size_t)j * w + i)] = mn;
                lv[k][2 * ((size_t)j * w + i) + 1] = mx;
            }
    }
    return lv;
}

// computeVisibilityFromHSM's lod (PlausibleSoftShadow.frag:538-539)
float hsm_lod(int S) { return S > 1024 ? 1.75f : (float)S / 1024.0f + 0.5f; }

// bilinear read of an n-channel level (the formula of moment_fetch)
void bilinear(const float* tex, int W, int H, int nch, float s, float t, float* out) {
    const float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    for (int ch = 0; ch < nch; ++ch) out[ch] = 0.0f;
    if (!(u > -2.0f && u < (float)W + 1.0f && v > -2.0f && v < (float)H + 1.0f)) return;
    const float fu = std::floor(u), fv = std::floor(v);
    const int i0 = (int)fu, j0 = (int)fv;
    const float a = u - fu, b = v - fv;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    for (int ch = 0; ch < nch; ++ch) {
        float T[4];
        for (int k = 0; k < 4; ++k) {
            const int i = i0 + (k & 1), j = j0 + (k >> 1);
            T[k] = (i >= 0 && i < W && j >= 0 && j < H) ? tex[nch * ((size_t)j * W + i) + ch] : 0.0f;
        }
        out[ch] = ((w00 * T[0] + w10 * T[1]) + w01 * T[2]) + w11 * T[3];
    }
}

V4 mom_at(const Ctx& c, float s, float t) {
    V4 r;
    bilinear(c.mom, c.W, c.H, 4, s, t, &r.x);
    return r;
}

float nonlinearize(float d) { return -(2.0f - d * 1001.0f) / (d * 999.0f); }

// chebyshevUpperBound (PlausibleSoftShadow.frag:78-91)
float chebyshev_soft(float mx, float my, float z) {
    if (z <= mx) return 1.0f;
    const float variance = my - mx * mx;
    const float d = z - mx;
    float p_max = variance / (variance + d * d);
    const float p = z <= mx ? 1.0f : 0.0f;
    return gmax(p, p_max);
}

// The SAT branch shared by the filters and blocker estimates: the box from
// the four corner reads, (D + A - B - C) / (SATFilterSize^2).
V4 sat_box(const Ctx& c, V4 n, float width, float step) {
    const float div = 2.0f * width / step;
    const float size = div / 2.0f;
    const float xmax = n.x + div * step, xmin = n.x - (div + 1.0f) * step;
    const float ymax = n.y + div * step, ymin = n.y - (div + 1.0f) * step;
    const V4 A = mom_at(c, xmin, ymin), B = mom_at(c, xmax, ymin), C = mom_at(c, xmin, ymax), D = mom_at(c, xmax, ymax);
    const float den = size * size;
    return V4{(((D.x + A.x) - B.x) - C.x) / den, (((D.y + A.y) - B.y) - C.y) / den, (((D.z + A.z) - B.z) - C.z) / den,
              (((D.w + A.w) - B.w) - C.w) / den};
}

// The tap loop: for h, w in [-fw, fw] sum the bilinear reads at
// n.xy + (w, h) * width / fw, then / float(count * count).
V4 loop_box(const Ctx& c, V4 n, float width, int count) {
    const float fw = ((float)count - 1.0f) * 0.5f;
    V4 acc{0.0f, 0.0f, 0.0f, 0.0f};
    for (int h = (int)(-fw); (float)h <= fw; h++)
        for (int w = (int)(-fw); (float)w <= fw; w++) {
            const V4 t = mom_at(c, n.x + ((float)w * width) / fw, n.y + ((float)h * width) / fw);
            acc = V4{acc.x + t.x, acc.y + t.y, acc.z + t.z, acc.w + t.w};
        }
    const float den = (float)(count * count);
    return V4{acc.x / den, acc.y / den, acc.z / den, acc.w / den};
}

V4 box(const Ctx& c, V4 n, float width, float step, int count) {
    return c.p->summed_area_table ? sat_box(c, n, width, step) : loop_box(c, n, width, count);
}

// VSM (:400-440)
float soft_vsm(const Ctx& c, float pw, V4 n) {
    const int K = c.p->kernel_size;
    const float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const V4 m = box(c, n, pw, step, K);
    const float mx = m.x + 0.5f, my = m.y + 0.5f;
    return gclamp(gmix(chebyshev_soft(mx, my, gl_linearize(n.z)), 1.0f, c.I), 0.0f, 1.0f);
}

// computeAverageBlockerDepthBasedOnVSM (:196-244)
float vsm_blocker(const Ctx& c, V4 n) {
    const float bsw = blocker_search_width(c);
    const int B = c.p->blocker_search_size;
    const float step = 2.0f * bsw / (float)B;
    const float zun = gl_linearize(n.z);
    const V4 m = box(c, n, bsw, step, B);
    const float mx = m.x + 0.5f, my = m.y + 0.5f;
    const float prob = chebyshev_soft(mx, my, zun);
    float zocc = nonlinearize((mx - prob * zun) / (1.0f - prob));
    if (prob > 0.99f) zocc = 1.0f;
    return zocc;
}

// computeAverageBlockerDepthBasedOnESM (:246-301)
float esm_blocker(const Ctx& c, V4 n) {
    const float bsw = blocker_search_width(c);
    const int B = c.p->blocker_search_size;
    const float step = 2.0f * bsw / (float)B;
    const V4 s = box(c, n, bsw, step, B);
    const float lz = gl_linearize(n.z);
    const float prob = std::exp(-80.0f * lz) * s.y;
    if (prob > 0.91f) return 1.0f;
    const float zocc = (s.x - std::exp(-80.0f * lz) * s.z) / (1.0f - prob);
    return nonlinearize(zocc);
}

// ESM (:442-490)
float soft_esm(const Ctx& c, float pw, V4 n) {
    const int K = c.p->kernel_size;
    const float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const float avg = box(c, n, pw, step, K).y;
    const float dist = mom_at(c, n.x, n.y).x + 0.0001f;
    const float lz = gl_linearize(n.z);
    float vis = std::exp(-80.0f * lz) * avg;
    vis = gclamp(vis, c.I, 1.0f);
    if (dist > lz && vis == c.I) return 1.0f;
    return vis;
}

// computeMomentDepthsFromMSM / computeWeightsFromMSM /
// computeShadowIntensityFromMSM (:93-164): b, then the three depths
struct Msm {
    V4 b;
    float zx, zy, zz;
};

Msm msm_solve(const V4& moments, float lz) {
    float mq[16], mqi[16];
    msm_quantization(mq, mqi);
    V4 b = V4{moments.x - 0.0359558848f, moments.y - 0.0f, moments.z - 0.0f, moments.w - 0.0f};
    b = mat4_mul(mqi, b);
    const float bias = 0.00003f;
    const float ob = 1.0f - bias, hb = bias * 0.5f;
    b = V4{ob * b.x + hb, ob * b.y + hb, ob * b.z + hb, ob * b.w + hb};
    const float dx = 1.0f, dy = lz, dz = lz * lz;
    const float L10 = b.x, L20 = b.y;
    const float D11 = b.y - L10 * L10;
    const float L21 = (b.z - L20 * L10) / D11;
    const float D22 = b.w - L20 * L20 - L21 * L21 * D11;
    const float y0 = dx;
    float y1 = dy - L10 * y0;
    float y2 = dz - L20 * y0 - L21 * y1;
    y1 = y1 / D11;
    y2 = y2 / D22;
    const float cz = y2, cy = y1 - L21 * cz, cx = y0 - L10 * cy - L20 * cz;
    const float p = cy / cz, q = cx / cz;
    const float D = ((p * p) / 4.0f) - q;
    const float r = std::sqrt(D);
    return Msm{b, lz, -(p / 2.0f) - r, -(p / 2.0f) + r};
}

// computeAverageBlockerDepthBasedOnMSM (:303-363)
float msm_blocker(const Ctx& c, V4 n) {
    const float bias = 0.01f;
    const float bsw = c.p->light_radius / (float)c.W;
    const int B = c.p->blocker_search_size;
    const float step = 2.0f * bsw / (float)B;
    const Msm z = msm_solve(box(c, n, bsw, step, B), gl_linearize(n.z));
    const V4& b = z.b;
    const float wx = (z.zy * z.zz - b.x * (z.zy + z.zz) + b.y) / ((z.zx - z.zy) * (z.zx - z.zz));
    const float wy = (z.zx * z.zz - b.x * (z.zx + z.zz) + b.y) / ((z.zz - z.zy) * (z.zx - z.zy));
    const float wz = 1.0f - wx - wy;
    const float ky = 1.0f - wy, kz = 1.0f - wz;
    float avg = 0.0f, sum = 0.0f;
    if (z.zx > z.zy) {
        avg += ky * z.zy;
        sum += ky;
    }
    if (z.zx > z.zz) {
        avg += kz * z.zz;
        sum += kz;
    }
    avg += bias * z.zx;
    sum += bias;
    if (sum > 1.0f - bias) return 1.0f;
    return nonlinearize(avg / sum);
}

// MSM (:492-533)
float soft_msm(const Ctx& c, float pw, V4 n) {
    const int K = c.p->kernel_size;
    const float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const Msm z = msm_solve(box(c, n, pw, step, K), gl_linearize(n.z));
    const V4& b = z.b;
    if (z.zx <= z.zy) return 1.0f;
    if (z.zx <= z.zz)
        return gclamp(1.0f - gclamp((z.zx * z.zz - b.x * (z.zx + z.zz) + b.y) / ((z.zz - z.zy) * (z.zx - z.zy)),
                                    0.0f, 1.0f),
                      c.I, 1.0f);
    return gclamp(1.0f - gclamp(1.0f - (z.zy * z.zz - b.x * (z.zy + z.zz) + b.y) / ((z.zx - z.zy) * (z.zx - z.zz)),
                                0.0f, 1.0f),
                  c.I, 1.0f);
}

// computeVisibilityFromHSM (:535-554)
float hsm_visibility(const Ctx& c, V4 n) {
    float lo[2], hi[2];
    bilinear(c.hsm_lo, c.lo_w, c.lo_h, 2, n.x, n.y, lo);
    bilinear(c.hsm_hi, c.hi_w, c.hi_h, 2, n.x, n.y, hi);
    const float f = c.hsm_frac;
    const float mn = (1.0f - f) * lo[0] + f * hi[0], mx = (1.0f - f) * lo[1] + f * hi[1];
    if (n.z <= mn) return 1.0f;
    if (n.z > mx) return c.I;
    return 0.555f;
}

float soft_moment_lookup(const Ctx& c, V4 n) {
    switch (c.p->technique) {
        case GI_TECH_SAVSM: {  // summedAreaVarianceShadowMapping (:565-572)
            const float avg = avg_blocker_grid(c, n);
            return soft_vsm(c, penumbra_width(c, avg, n.z), n);
        }
        case GI_TECH_VSSM: {  // varianceSoftShadowMapping (:574-585)
            const float v = hsm_visibility(c, n);
            if (v == c.I || v == 1.0f) return v;
            const float avg = vsm_blocker(c, n);
            return soft_vsm(c, penumbra_width(c, avg, n.z), n);
        }
        case GI_TECH_ESSM:  // exponentialSoftShadowMapping (:587-594)
            return soft_esm(c, penumbra_width(c, esm_blocker(c, n), n.z), n);
        default:  // momentSoftShadowMapping (:596-603)
            return soft_msm(c, penumbra_width(c, msm_blocker(c, n), n.z), n);
    }
}

float shade_pixel(const Ctx& c, V4 vertex, V4 normal, const float* poisson) {
    if (vertex.x == 0.0f) return 0.0f;  // discard: the target keeps its clear value 0
    const gi_vis_params* p = c.p;
    V4 sc = mat4_mul(p->light_mvp_biased, vertex);
    V4 n = {sc.x / sc.w, sc.y / sc.w, sc.z / sc.w, sc.w / sc.w};
    float shadow = pretest(c, vertex, normal);
    switch (p->technique) {
        case GI_TECH_HARD:
            if (sc.w > 0.0f && shadow == 1.0f) {
                float d = fetch(c, n.x, n.y);
                shadow = (n.z <= d) ? 1.0f : c.I;
            }
            return shadow;
        case GI_TECH_PCF:
            if (sc.w > 0.0f && shadow == 1.0f) shadow = pcf_bilinear(c, n);
            return shadow;
        case GI_TECH_PCF_TRICUBIC:
            if (sc.w > 0.0f && shadow == 1.0f) shadow = pcf_tricubic(c, n);
            return shadow;
        case GI_TECH_PCSS_GRID:
            if (sc.w > 0.0f && shadow == 1.0f) {
                float avg = avg_blocker_grid(c, n);
                float pw = penumbra_width(c, avg, n.z);
                shadow = pcss_filter_grid(c, pw, n);
            }
            return shadow;
        case GI_TECH_PCSS_POISSON:
            if (sc.w > 0.0f && shadow == 1.0f) {
                float avg = avg_blocker_poisson(c, n, poisson);
                float pw = penumbra_width(c, avg, n.z);
                shadow = pcss_filter_poisson(c, pw, n, poisson + 2 * p->poisson_blocker_taps);
            }
            return shadow;
        case GI_TECH_SMSR_NONCONSERVATIVE:
            if (shadow == 1.0f) shadow = nc_smsr(c, n);
            return shadow;
        case GI_TECH_RPCF_SMSR:
            if (shadow == 1.0f) shadow = nc_rpcf(c, n, false);
            return shadow;
        case GI_TECH_RSMSS:
            if (shadow == 1.0f) shadow = nc_rpcf(c, n, true);
            return shadow;
        case GI_TECH_SMSR_CONSERVATIVE:
            if (shadow == 1.0f) shadow = cs_smsr(c, n);
            return shadow;
        case GI_TECH_RPCF_CONSERVATIVE:
            if (shadow == 1.0f) shadow = cs_rpcf(c, n);
            return shadow;
        case GI_TECH_RBSSM:  // RBSSM.frag:1362-1376
            if (sc.w > 0.0f && shadow == 1.0f) shadow = rb_rbssm(c, n);
            return shadow;
        case GI_TECH_VSM:
        case GI_TECH_ESM:
        case GI_TECH_EVSM:
        case GI_TECH_MSM:
            if (sc.w > 0.0f && shadow == 1.0f) shadow = moment_lookup(c, n);
            return shadow;
        case GI_TECH_SAVSM:
        case GI_TECH_VSSM:
        case GI_TECH_ESSM:
        case GI_TECH_MSSM:
            if (sc.w > 0.0f && shadow == 1.0f) shadow = soft_moment_lookup(c, n);
            return shadow;
        case GI_TECH_HARD_SOFTAPP: {
            float r = shadow;
            if (sc.w > 0.0f && r == 1.0f) {
                float d = fetch(c, n.x, n.y);
                r = (n.z <= d) ? 1.0f : c.I;
            }
            if (pretest(c, vertex, normal) == c.I) r = 0.0f;
            return r;
        }
        default:
            return 0.0f;
    }
}

}  // namespace

extern "C" void or_visibility(const gi_vis_params* p, const float* depth, int map_w, int map_h,
                              const float* pos, const float* nrm, float* out, int W, int H,
                              const float* poisson_xy, int threads) {
    Ctx c;
    c.p = p;
    c.map = depth;
    c.W = map_w;
    c.H = map_h;
    c.sx = (float)(1.0 / map_w);  // glUniform2f(1.0/w, 1.0/h): double then float
    c.sy = (float)(1.0 / map_h);
    c.I = p->shadow_intensity;
    std::vector<float> moments;
    std::vector<std::vector<float>> hsm;
    if (p->technique >= GI_TECH_VSM && p->technique <= GI_TECH_MSM) {
        moments = moment_filtered(p->technique, depth, map_w, W);
        c.map = moments.data();
        c.W = c.H = W;
    }
    if (is_soft_moment(p->technique)) {
        moments = soft_moment_map(p->technique, depth, map_w, map_h);
        if (p->summed_area_table) summed_area_table(moments, map_w, map_h);
        c.mom = moments.data();
        if (p->technique == GI_TECH_VSSM) {
            const float lod = hsm_lod(map_w);
            const int lo = (int)std::floor(lod);
            hsm = hsm_levels(depth, map_w, map_h, p->hsm_alpha, p->hsm_beta, lo + 1);
            c.hsm_lo = hsm[lo].data();
            c.hsm_hi = hsm[lo + 1].data();
            c.lo_w = map_w >> lo;
            c.lo_h = map_h >> lo;
            c.hi_w = map_w >> (lo + 1);
            c.hi_h = map_h >> (lo + 1);
            c.hsm_frac = lod - (float)lo;
        }
    }
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads(threads))
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            size_t i = (size_t)y * W + x;
            V4 v = {pos[4 * i], pos[4 * i + 1], pos[4 * i + 2], pos[4 * i + 3]};
            V4 nn = {nrm[4 * i], nrm[4 * i + 1], nrm[4 * i + 2], nrm[4 * i + 3]};
            out[i] = shade_pixel(c, v, nn, poisson_xy);
        }
}

// The light-side maps of the moment soft shadows: the moment map (or its
// summed-area table) and one min-max level.
extern "C" void or_soft_moment_map(const gi_vis_params* p, const float* depth, int S, int T, float* out) {
    std::vector<float> m = soft_moment_map(p->technique, depth, S, T);
    if (p->summed_area_table) summed_area_table(m, S, T);
    std::memcpy(out, m.data(), m.size() * sizeof(float));
}

extern "C" void or_hierarchical_shadow_map(const gi_vis_params* p, const float* depth, int S, int T, int level,
                                           float* out) {
    const std::vector<std::vector<float>> lv = hsm_levels(depth, S, T, p->hsm_alpha, p->hsm_beta, level);
    std::memcpy(out, lv[level].data(), lv[level].size() * sizeof(float));
}

// shadeScene / PhongShading.frag:11-46: shadow * fragmentColor *
// (Idiff + Ispec + Iamb), normalize(x) = x * (1 / sqrt(dot(x, x))), E from
// the 4-component eye-space vertex, pow(x, 3) as x * x * x.
extern "C" void or_phong_shade(const gi_vis_params* p, const float* pos, const float* nrm, const float* vis,
                               const float* color, int W, int H, float* out) {
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        const float* pv = pos + 4 * i;
        float* o = out + 4 * i;
        if (pv[0] == 0.0f) {
            o[0] = 0.63f;
            o[1] = 0.82f;
            o[2] = 0.96f;
            o[3] = 1.0f;
            continue;
        }
        const float* nv = nrm + 4 * i;
        const float shadow = vis[i];
        const float spec_shadow = shadow - p->shadow_intensity;
        V4 v = mat4_mul(p->camera_mv, V4{pv[0], pv[1], pv[2], pv[3]});
        const float* nm = p->normal_matrix;
        float nx = nm[0] * nv[0] + nm[3] * nv[1] + nm[6] * nv[2];
        float ny = nm[1] * nv[0] + nm[4] * nv[1] + nm[7] * nv[2];
        float nz = nm[2] * nv[0] + nm[5] * nv[1] + nm[8] * nv[2];
        const float ninv = 1.0f / std::sqrt(nx * nx + ny * ny + nz * nz);
        nx = nx * ninv;
        ny = ny * ninv;
        nz = nz * ninv;
        float lx = p->light_position[0] - v.x, ly = p->light_position[1] - v.y, lz = p->light_position[2] - v.z;
        const float linv = 1.0f / std::sqrt(lx * lx + ly * ly + lz * lz);
        lx = lx * linv;
        ly = ly * linv;
        lz = lz * linv;
        const float ex0 = -v.x, ey0 = -v.y, ez0 = -v.z, ew0 = -v.w;
        const float einv = 1.0f / std::sqrt(ex0 * ex0 + ey0 * ey0 + ez0 * ez0 + ew0 * ew0);
        const float ex = ex0 * einv, ey = ey0 * einv, ez = ez0 * einv;
        const float ndl = nx * lx + ny * ly + nz * lz;
        float rx = -(lx - 2.0f * ndl * nx), ry = -(ly - 2.0f * ndl * ny), rz = -(lz - 2.0f * ndl * nz);
        const float rinv = 1.0f / std::sqrt(rx * rx + ry * ry + rz * rz);
        rx = rx * rinv;
        ry = ry * rinv;
        rz = rz * rinv;
        const float diff = gmax(ndl, 0.0f);
        const float re = gmax(rx * ex + ry * ey + rz * ez, 0.0f);
        const float spec = re * re * re;
        const float cc[4] = {color ? color[4 * i] : 1.0f, color ? color[4 * i + 1] : 1.0f,
                             color ? color[4 * i + 2] : 1.0f, color ? color[4 * i + 3] : 1.0f};
        const float amb[4] = {0.4f, 0.4f, 0.4f, 1.0f}, dif[4] = {0.5f, 0.5f, 0.5f, 1.0f};
        const float spc[4] = {0.25f, 0.25f, 0.25f, 1.0f};
        for (int k = 0; k < 4; ++k) {
            const float idiff = dif[k] * diff;
            const float ispec = (spec_shadow * spc[k]) * spec;
            o[k] = (shadow * cc[k]) * ((idiff + ispec) + amb[k]);
        }
    }
}

// renderMonteCarlo (SoftShadowMapping/src/main.cpp:756-811) + the uniform
// branch of AccurateSoftShadow.frag:52-133: one map per sample (mvps, the
// unbiased light MVPs), then per pixel commonShadowCoord from columns 0-2 of
// the last sample's biased MVP, shadowCoord = common + the sample's biased
// translation column, / w, one NEAREST fetch, accShadow += (z <= d ? 1 : I)
// * 1, shadow = accShadow / count.  No pre-test; background 0.
extern "C" void or_area_light_visibility(const float* points, const float* normals, int nv, const int* indices,
                                         int nt, const float* mvps, const float* biased, int n, int S,
                                         int bias_mode, float cbias, float factor, float units,
                                         const float camera_mvp[16], float I, int W, int H, float* out,
                                         int threads) {
    std::vector<float> pos((size_t)W * H * 4), nrm((size_t)W * H * 4), map((size_t)S * S);
    or_gbuffer(points, normals, nv, indices, nt, camera_mvp, W, H, pos.data(), nrm.data(), threads);
    std::vector<float> acc((size_t)W * H, 0.0f);
    const float* m = biased + (size_t)(n - 1) * 16;
    for (int i = 0; i < n; ++i) {
        or_shadow_map(points, nv, indices, nt, mvps + (size_t)i * 16, S, S, bias_mode, cbias, factor, units,
                      map.data(), threads);
        const float* t = biased + (size_t)i * 16 + 12;
        Ctx c;
        c.p = nullptr;
        c.map = map.data();
        c.W = S;
        c.H = S;
        c.sx = c.sy = 0.0f;
        c.I = I;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t q = (size_t)y * W + x;
                const float* v = &pos[4 * q];
                if (v[0] == 0.0f) continue;
                const float cx = m[0] * v[0] + m[4] * v[1] + m[8] * v[2];
                const float cy = m[1] * v[0] + m[5] * v[1] + m[9] * v[2];
                const float cz = m[2] * v[0] + m[6] * v[1] + m[10] * v[2];
                const float cw = m[3] * v[0] + m[7] * v[1] + m[11] * v[2];
                const float sx = cx + t[0], sy = cy + t[1], sz = cz + t[2], sw = cw + t[3];
                const float d = fetch(c, sx / sw, sy / sw);
                acc[q] += ((sz / sw <= d) ? 1.0f : I) * 1.0f;
            }
    }
    float count = 0.0f;
    for (int i = 0; i < n; ++i) count += 1.0f;
    for (size_t q = 0; q < (size_t)W * H; ++q) out[q] = pos[4 * q] == 0.0f ? 0.0f : acc[q] / count;
}

// Adaptive area-light sampling (SoftShadowMapping adaptiveSampling:
// main.cpp:423-690, 820-870; QuadTreeLightSource.cpp; Shaders/QuadTree/
// Reprojection.frag, Evaluation.frag; AccurateSoftShadow.frag adaptive
// branch), depth first as the reference runs it.  `view_mvp` returns the
// light MVP and biased MVP of a sample eye / at (the reference's
// glm::perspective * lookAt, computed by the caller).
namespace {

struct OrQt {
    const float *points, *normals;
    const int* indices;
    int nv, nt;
    or_view_mvp_fn view_mvp;
    void* user;
    float size;
    int max_level, S, bias_mode;
    float cbias, factor, units;
    int W, H, threads;
    int div;  // evaluation viewport divisor (4: lower-accuracy mode)
    const float* pos;
    int hash[17][17];
    std::vector<std::vector<float>> maps;
    std::vector<std::array<float, 16>> biased;
    std::vector<std::array<float, 6>> eyes;
    std::vector<float> level;
};

struct OrQtNode {
    int level;
    float eye[3], at[3];
    std::array<int, 4> kids;
};

void or_qt_offset(const float ref[3], float size, int div_pow, int index, float out[3]) {
    const int div = (int)std::pow(2.0f, (float)div_pow);
    const float step = size / (float)div;
    out[0] = ref[0];
    out[1] = ref[1];
    out[2] = ref[2];
    out[0] += -step + (2.0f * step * (float)(index % 2));
    out[1] += -step + (2.0f * step * (float)(index / 2));
}

int or_qt_map(OrQt& q, const OrQtNode& node, int index, int x, int y) {
    if (q.hash[x][y] >= 0) return q.hash[x][y];
    std::array<float, 6> e;
    or_qt_offset(node.eye, q.size, node.level + 1, index, &e[0]);
    or_qt_offset(node.at, q.size, node.level + 1, index, &e[3]);
    float mvp[16];
    std::array<float, 16> b;
    q.view_mvp(&e[0], &e[3], mvp, b.data(), q.user);
    std::vector<float> m((size_t)q.S * q.S);
    or_shadow_map(q.points, q.nv, q.indices, q.nt, mvp, q.S, q.S, q.bias_mode, q.cbias, q.factor, q.units, m.data(),
                  q.threads);
    const int idx = (int)q.maps.size();
    q.maps.push_back(std::move(m));
    q.biased.push_back(b);
    q.eyes.push_back(e);
    q.level.push_back(0.0f);
    q.hash[x][y] = idx;
    return idx;
}

void or_qt_corner(int level, int node, int index, int* x, int* y) {
    const int cf = (int)(16.0f / std::pow(2.0f, (float)level)), pf = (int)std::pow(2.0f, (float)level);
    *x = (index % 2) * cf + (node % pf) * cf;
    *y = (index / 2) * cf + (node / pf) * cf;
}

void or_qt_children(int level, int node, int child[4]) {
    const int div = (int)std::pow(2.0f, (float)level);
    const int x = node % div, y = node / div;
    const int base = 2 * x + (int)std::pow(2.0f, (float)(level + 2)) * y;
    const int row = (int)std::pow(2.0f, (float)(level + 1));
    child[0] = base;
    child[1] = base + 1;
    child[2] = base + row;
    child[3] = base + row + 1;
}

// Reprojection.frag + Evaluation.frag + the occlusion query's result
bool or_qt_subdivide(OrQt& q, const int idx[4]) {
    const int W = q.W, H = q.H;
    std::vector<float> sum((size_t)W * H);
    Ctx c;
    c.p = nullptr;
    c.W = q.S;
    c.H = q.S;
    c.sx = c.sy = 0.0f;
    c.I = 0.0f;
    for (size_t p = 0; p < (size_t)W * H; ++p) {
        const float* v = &q.pos[4 * p];
        if (v[0] == 0.0f) {
            sum[p] = 0.63f;  // the reprojection target's clear colour
            continue;
        }
        float s = 0.0f;
        for (int k = 0; k < 4; ++k) {
            const V4 sc = mat4_mul(q.biased[idx[k]].data(), V4{v[0], v[1], v[2], v[3]});
            c.map = q.maps[idx[k]].data();
            s += (sc.z / sc.w <= fetch(c, sc.x / sc.w, sc.y / sc.w)) ? 1.0f : 0.0f;
        }
        sum[p] = s;
    }
    // the evaluation viewport: Wq x Hq = (W / div) x (H / div), coarse pixel
    // i reading the count texel at its centre, floor((2 i + 1) W / (2 Wq))
    const int Wq = W / q.div, Hq = H / q.div;
    auto coarse = [&](int i, int j) {
        if (i < 0 || i >= Wq || j < 0 || j >= Hq) return 0.0f;  // border
        const int x = (int)(((long long)(2 * i + 1) * W) / (2LL * Wq));
        const int y = (int)(((long long)(2 * j + 1) * H) / (2LL * Hq));
        return sum[(size_t)y * W + x];
    };
    for (int y = 0; y < Hq; ++y)
        for (int x = 0; x < Wq; ++x) {
            const float s = coarse(x, y);
            if (s == 0.63f || s == 0.0f || s == 4.0f || s == 5.0f) continue;
            bool pass = true;
            for (int dy = -1; dy <= 1 && pass; ++dy)
                for (int dx = -1; dx <= 1; ++dx)
                    if (s != coarse(x + dx, y + dy)) {
                        pass = false;
                        break;
                    }
            if (pass) return true;
        }
    return false;
}

void or_qt_evaluate(OrQt& q, std::vector<OrQtNode>& nodes, int n, int node) {
    if (nodes[n].level == q.max_level) return;
    int child[4];
    or_qt_children(nodes[n].level, node, child);
    int idx[4];
    for (int index = 0; index < 4; ++index) {
        int x, y;
        or_qt_corner(nodes[n].level, node, index, &x, &y);
        idx[index] = or_qt_map(q, nodes[n], index, x, y);
    }
    if (!or_qt_subdivide(q, idx)) return;
    for (int c = 0; c < 4; ++c) {
        OrQtNode k;
        k.level = nodes[n].level + 1;
        or_qt_offset(nodes[n].eye, q.size, nodes[n].level + 2, c, k.eye);
        or_qt_offset(nodes[n].at, q.size, nodes[n].level + 2, c, k.at);
        k.kids = {-1, -1, -1, -1};
        nodes[n].kids[c] = (int)nodes.size();
        nodes.push_back(k);
    }
    for (int c = 0; c < 4; ++c) or_qt_evaluate(q, nodes, nodes[n].kids[c], child[c]);
}

void or_qt_render(OrQt& q, std::vector<OrQtNode>& nodes, int n, int node) {
    if (nodes[n].kids[0] >= 0) {
        int child[4];
        or_qt_children(nodes[n].level, node, child);
        for (int c = 0; c < 4; ++c) or_qt_render(q, nodes, nodes[n].kids[c], child[c]);
        return;
    }
    for (int index = 0; index < 4; ++index) {
        int x, y;
        or_qt_corner(nodes[n].level, node, index, &x, &y);
        q.level[or_qt_map(q, nodes[n], index, x, y)] = (float)nodes[n].level;
    }
}

}  // namespace

extern "C" int or_area_light_adaptive(const float* points, const float* normals, int nv, const int* indices, int nt,
                                      const float light_eye[3], const float light_at[3], float size, int max_level,
                                      int lower_accuracy, or_view_mvp_fn view_mvp, void* user, int S, int bias_mode,
                                      float cbias,
                                      float factor, float units, const float camera_mvp[16], float I, int W, int H,
                                      float* out, float* eyes_out, float* levels_out, int threads) {
    std::vector<float> pos((size_t)W * H * 4), nrm((size_t)W * H * 4);
    or_gbuffer(points, normals, nv, indices, nt, camera_mvp, W, H, pos.data(), nrm.data(), threads);
    OrQt q;
    q.points = points;
    q.normals = normals;
    q.indices = indices;
    q.nv = nv;
    q.nt = nt;
    q.view_mvp = view_mvp;
    q.user = user;
    q.size = size;
    q.max_level = max_level;
    q.S = S;
    q.bias_mode = bias_mode;
    q.cbias = cbias;
    q.factor = factor;
    q.units = units;
    q.W = W;
    q.H = H;
    q.threads = threads;
    q.div = lower_accuracy ? 4 : 1;
    q.pos = pos.data();
    for (auto& row : q.hash)
        for (int& h : row) h = -1;
    std::vector<OrQtNode> nodes(1);
    nodes[0].level = 0;
    for (int c = 0; c < 3; ++c) {
        nodes[0].eye[c] = light_eye[c];
        nodes[0].at[c] = light_at[c];
    }
    nodes[0].kids = {-1, -1, -1, -1};
    or_qt_evaluate(q, nodes, 0, 0);
    or_qt_render(q, nodes, 0, 0);
    const int n = (int)q.maps.size();
    // the final pass: weights from the level carried in each translation's w
    const float* m = q.biased[n - 1].data();
    std::vector<float> acc((size_t)W * H, 0.0f);
    float count = 0.0f;
    // the lower-accuracy branch's float loops (AccurateSoftShadow.frag:98-110)
    std::vector<float> offs;
    if (lower_accuracy) {
        const float offset = 1.0f, step = 2.0f * offset / 3.0f;
        for (float w = -offset; w <= offset; w += step) offs.push_back(w);
    }
    const float incr = 1.0f / (float)S;
    for (int i = 0; i < n; ++i) {
        const float* b = q.biased[i].data();
        const float w_enc = b[15] + q.level[i] * 10000.0f;
        int ql = (int)(w_enc / 10000.0f);
        if (ql > 4) ql = 4;
        const float wv = w_enc - (float)(ql * 10000);
        float f = 1.0f;
        for (int e = 1; e <= ql; ++e) f *= 2.0f;
        f = f + 1.0f;
        const float wt = 1.0f / (f * f);
        Ctx c;
        c.p = nullptr;
        c.map = q.maps[i].data();
        c.W = S;
        c.H = S;
        c.sx = c.sy = 0.0f;
        c.I = I;
        for (size_t p = 0; p < (size_t)W * H; ++p) {
            const float* v = &pos[4 * p];
            if (v[0] == 0.0f) continue;
            const float cx = m[0] * v[0] + m[4] * v[1] + m[8] * v[2];
            const float cy = m[1] * v[0] + m[5] * v[1] + m[9] * v[2];
            const float cz = m[2] * v[0] + m[6] * v[1] + m[10] * v[2];
            const float cw = m[3] * v[0] + m[7] * v[1] + m[11] * v[2];
            const float sx = cx + b[12], sy = cy + b[13], sz = cz + b[14], sw = cw + wv;
            if (!lower_accuracy) {
                const float d = fetch(c, sx / sw, sy / sw);
                acc[p] += ((sz / sw <= d) ? 1.0f : I) * wt;
            } else {
                const float ux = sx / sw, uy = sy / sw, uz = sz / sw;
                float illum = 0.0f;
                for (float ow : offs)
                    for (float oh : offs) {
                        if (uz <= fetch(c, ux + ow * incr, uy + oh * incr)) illum = illum + 1.0f;
                        else illum += I;
                    }
                acc[p] += (illum / (float)(offs.size() * offs.size())) * wt;
            }
        }
        count += wt;
        if (eyes_out)
            for (int k = 0; k < 6; ++k) eyes_out[6 * i + k] = q.eyes[i][k];
        if (levels_out) levels_out[i] = q.level[i];
    }
    for (size_t p = 0; p < (size_t)W * H; ++p) out[p] = pos[4 * p] == 0.0f ? 0.0f : acc[p] / count;
    return n;
}

extern "C" void or_rbssm_hits(unsigned long long* out4096, int reset) {
    for (int i = 0; i < 4096; ++i) {
        if (out4096) out4096[i] = g_rb_hits[i].load();
        if (reset) g_rb_hits[i].store(0);
    }
}

// ===========================================================================
// EDT-filtered hard shadows (ShadowMapping's EDTSM mode) and the exact
// Euclidean distance transform it runs: the parallel banding algorithm (PBA,
// Cao et al. 2010) as ShadowMapping/src/EDT/pba2DHost.cu:121-242 sequences
// the kernels of ShadowMapping/include/EDT/pba2DKernel.h.  Equidistant sites
// are resolved by the algorithm's own comparisons (flood and merge order,
// FP32 bisector intersections, the coloring walk of each group of m3
// threads), so the restatement keeps every band, merge and group of the
// reference; a site image is processed column by column (phase 1) and then
// row by row (phases 2-3), which is what the reference's transposes do.
// ===========================================================================
// PBA: Copyright (c) 2010, School of Computing, National University of
// Singapore.  All rights reserved.  Redistribution terms: the BSD notice
// reproduced at the top of globalillumination_gb300/csrc/edt.cu.
namespace {
namespace pba {

constexpr int kMarker = -32768;  // MARKER, pba2D.h:60

struct P {
    int x, y;
};

// Phase 1 on one column (pba2DPhase1, pba2DHost.cu:121-143): in[y] is the
// row of the site at (x, y) or kMarker; out[y] the row of the site chosen
// for (x, y) or kMarker.  Sites carry their own row as their y.
void column(const int* in, int H, int m1, int* out) {
    const int B = H / m1;
    std::vector<int> down(H), up(H), links(in, in + H);
    // kernelFloodDown (pba2DKernel.h:112-130): last site at or above, per band
    for (int b = 0; b < m1; ++b) {
        int cur = kMarker;
        for (int i = 0; i < B; ++i) {
            const int y = b * B + i;
            if (in[y] != kMarker) cur = in[y];
            down[y] = cur;
        }
    }
    // kernelFloodUp (:132-153): from the band's last row upwards, take this
    // row's flood value only when strictly closer than the carried one
    for (int b = 0; b < m1; ++b) {
        const int ty = (b + 1) * B - 1;
        int cur = kMarker;
        for (int i = 0; i < B; ++i) {
            const int y = ty - i;
            if (std::abs(down[y] - y) < std::abs(cur - y)) cur = down[y];
            up[y] = cur;
        }
    }
    // kernelPropagateInterband (:155-198): a band's first row looks at the last
    // row of the nearest non-empty band above, its last row at the first row
    // of the nearest non-empty band below; strictly closer sites are written
    // over the site input, which is where the next step reads them.
    for (int b = 0; b < m1; ++b) {
        int ty = b * B;
        int mine = std::abs(up[ty] - ty);
        for (int nb = b - 1; nb >= 0; --nb) {
            const int v = up[nb * B + B - 1];
            if (v != kMarker) {
                if (std::abs(v - ty) < mine) links[ty] = v;
                break;
            }
        }
        ty = b * B + B - 1;
        mine = std::abs(up[ty] - ty);
        for (int nb = b + 1; nb < m1; ++nb) {
            const int v = up[nb * B];
            if (v != kMarker) {
                if (std::abs(v - ty) < mine) links[ty] = v;
                break;
            }
        }
    }
    // kernelUpdateVertical (:200-225): each row compares its band value with
    // the band's first-row and last-row links, strictly closer wins
    for (int b = 0; b < m1; ++b) {
        const int ty = b * B;
        const int top = links[ty], bottom = links[ty + B - 1];
        for (int i = 0; i < B; ++i) {
            const int y = ty + i;
            int v = up[y], mine = std::abs(v - y);
            int d = std::abs(top - y);
            if (d < mine) {
                mine = d;
                v = top;
            }
            d = std::abs(bottom - y);
            if (d < mine) v = bottom;
            out[y] = v;
        }
    }
}

// interpoint (pba2DKernel.h:227-236): where the bisector of (x1, y1) and
// (x2, y2) crosses the line x = x0; FP32, each operation rounded once.
float interpoint(int x1, int y1, int x2, int y2, int x0) {
    const float xM = float(x1 + x2) / 2.0f;
    const float yM = float(y1 + y2) / 2.0f;
    const float nx = float(x2 - x1);
    const float ny = float(y2 - y1);
    return yM + nx * (xM - float(x0)) / ny;
}

// One line of phases 2-3 (pba2DPhase2 / pba2DPhase3, pba2DHost.cu:145-190).
// cand[p] is the row of column p's phase-1 site (kMarker for none), line
// the row being colored; out_x / out_y receive the site of every pixel.
// lk[] plays the reference's textures[0] line: (x, y) = stack value and back
// pointer after the proximate-points pass, (forward, back) pointers after
// the forward pointers are created.
struct Line {
    const int* cand;
    int W, line;
    std::vector<P> lk;

    P col(int p) const {  // textures[0] after kernelDoubleToSingleList; zero outside
        if (p < 0 || p >= W) return P{0, 0};
        return P{cand[p], lk[p].y};
    }

    // kernelProximatePoints (pba2DKernel.h:238-268)
    void proximate(int b0, int B) {
        int lasty = -1;
        P last1{0, -1}, last2{0, -1};
        for (int p = b0; p < b0 + B; ++p) {
            if (cand[p] == kMarker) continue;
            while (last2.y >= 0) {
                const float i1 = interpoint(last1.x, last2.y, last2.x, lasty, line);
                const float i2 = interpoint(last2.x, lasty, cand[p], p, line);
                if (i1 < i2) break;
                lasty = last2.y;
                last2 = last1;
                if (last1.y >= 0) last1 = lk[last1.y];
            }
            last1 = last2;
            last2 = P{cand[p], lasty};
            lasty = p;
            lk[p] = last2;
        }
        if (lasty != b0 + B - 1) lk[b0 + B - 1] = P{kMarker, lasty};
    }

    // kernelCreateForwardPointers (:270-296)
    void forward(int b0, int B) {
        const int ty = b0 + B - 1;
        int lasty = -1;
        P cur = lk[ty];
        int nexty = cur.x == kMarker ? cur.y : ty;
        int p = ty;
        for (int i = 0; i < B; ++i, --p)
            if (ty - i == nexty) {
                cur = P{lasty, lk[p].y};
                lk[p] = cur;
                lasty = nexty;
                nexty = cur.y;
            }
        if (lasty != ty - B + 1) lk[p + 1] = P{lasty, kMarker};
    }

    // kernelMergeBands (:298-435), bands band1 and band1 + 1 of size B
    void merge(int band1, int B) {
        const int band2 = band1 + 1;
        int lasty = band2 * B - 1;
        P last2{cand[lasty], lk[lasty].y}, last1{0, 0};
        if (last2.x == kMarker) {
            lasty = last2.y;
            last2 = lasty >= 0 ? P{cand[lasty], lk[lasty].y} : P{kMarker, kMarker};
        }
        if (last2.y >= 0) last1 = P{cand[last2.y], lk[last2.y].y};
        int firsty = band2 * B;
        P cur{lk[firsty].x, cand[firsty]};
        if (cur.y == kMarker) {
            firsty = cur.x;
            cur = firsty >= 0 ? P{lk[firsty].x, cand[firsty]} : P{kMarker, kMarker};
        }
        int top = 0;
        while (top < 2 && cur.y >= 0) {
            while (last2.y >= 0) {
                const float i1 = interpoint(last1.x, last2.y, last2.x, lasty, line);
                const float i2 = interpoint(last2.x, lasty, cur.y, firsty, line);
                if (i1 < i2) break;
                lasty = last2.y;
                last2 = last1;
                --top;
                if (last1.y >= 0) last1 = P{cand[last1.y], lk[last1.y].y};
            }
            lk[firsty] = P{cur.x, lasty};
            if (lasty >= 0) lk[lasty] = P{firsty, last2.y};
            last1 = last2;
            last2 = P{cur.y, lasty};
            lasty = firsty;
            firsty = cur.x;
            top = std::max(1, top + 1);
            cur = firsty >= 0 ? P{lk[firsty].x, cand[firsty]} : P{kMarker, kMarker};
        }
        // head and tail pointers of the merged band
        firsty = band1 * B;
        lasty = band2 * B;
        cur = lk[firsty];
        if (cur.y == kMarker && cur.x < 0) {
            const P l = lk[lasty];
            cur.x = l.y == kMarker ? l.x : lasty;
            lk[firsty] = cur;
        }
        firsty = band1 * B + B - 1;
        lasty = band2 * B + B - 1;
        cur = lk[lasty];
        if (cur.x == kMarker && cur.y < 0) {
            const P l = lk[firsty];
            cur.y = l.x == kMarker ? l.y : firsty;
            lk[lasty] = cur;
        }
    }

    // kernelColor (:437-497): groups of m3 pixels from the line's end; each
    // pixel walks the list from the state the group's last pixel left after
    // the previous group, moving on while the squared distance does not grow.
    void color(int m3, int16_t* out_xy) {
        struct S {
            P last1, last2;
            int lasty;
        } s;
        s.lasty = W - 1;
        s.last2 = col(s.lasty);
        if (s.last2.x == kMarker) {
            s.lasty = s.last2.y;
            s.last2 = col(s.lasty);
        }
        s.last1 = P{0, 0};
        if (s.last2.y >= 0) s.last1 = col(s.last2.y);
        for (int g0 = W - 1; g0 >= 0; g0 -= m3) {
            S next = s;
            for (int t = 0; t < m3; ++t) {
                const int ty = g0 - t;
                S w = s;
                int dx = w.last2.x - line, dy = w.lasty - ty;
                uint32_t best = (uint32_t)((int64_t)dx * dx + (int64_t)dy * dy);
                while (w.last2.y >= 0) {
                    dx = w.last1.x - line;
                    dy = w.last2.y - ty;
                    const uint32_t dist = (uint32_t)((int64_t)dx * dx + (int64_t)dy * dy);
                    if (dist > best) break;
                    best = dist;
                    w.lasty = w.last2.y;
                    w.last2 = w.last1;
                    if (w.last2.y >= 0) w.last1 = col(w.last2.y);
                }
                out_xy[2 * ty] = (int16_t)w.lasty;      // the final transpose swaps
                out_xy[2 * ty + 1] = (int16_t)w.last2.x;  // (row, column) back
                if (t == m3 - 1) next = w;
            }
            s = next;
        }
    }
};

bool shape_ok(int W, int H, int m1, int m2, int m3) {
    return W > 0 && H > 0 && W <= 32767 && H <= 32767 && m1 > 0 && H % m1 == 0 && m2 > 0 && W % m2 == 0 &&
           (m2 & (m2 - 1)) == 0 && m3 > 0 && W % m3 == 0;
}

// pba2DCompute on a site mask (site[y * W + x] != 0): nearest site per
// pixel as (x, y) pairs.
void voronoi(const uint8_t* site, int W, int H, int m1, int m2, int m3, int16_t* out, int threads) {
    std::vector<int> cols((size_t)W * H);  // [x][y]
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (int x = 0; x < W; ++x) {
        std::vector<int> in(H);
        for (int y = 0; y < H; ++y) in[y] = site[(size_t)y * W + x] ? y : kMarker;
        column(in.data(), H, m1, &cols[(size_t)x * H]);
    }
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (int y = 0; y < H; ++y) {
        std::vector<int> cand(W);
        for (int x = 0; x < W; ++x) cand[x] = cols[(size_t)x * H + y];
        Line L{cand.data(), W, y, std::vector<P>(W, P{0, 0})};
        const int B2 = W / m2;
        for (int b = 0; b < m2; ++b) L.proximate(b * B2, B2);
        for (int b = 0; b < m2; ++b) L.forward(b * B2, B2);
        for (int nb = m2; nb > 1; nb /= 2)
            for (int b = 0; b < nb; b += 2) L.merge(b, W / nb);
        L.color(m3, out + (size_t)2 * y * W);
    }
}

// linearize (pba2DKernel.h:499-506): n = 1, f = 1000; 2.0 * n is a double,
// so the division is a double one rounded to float.
float linearize(float depth) {
    const float n = 1.0f, f = 1000.0f;
    return (float)((2.0 * n) / (f + n - depth * (f - n)));
}

// initializeInput (pba2DKernel.h:509-528): (x, y) is a site when one of its
// 3 x 3 neighbours p in the image has p.x != x's, |linearize(depth)
// difference| <= 0.0025 and p.z == 1.
bool is_site(const float* img, int W, int H, int px, int py) {
    const float* c = img + 4 * ((size_t)py * W + px);
    for (int x = -1; x <= 1; ++x)
        for (int y = -1; y <= 1; ++y)
            if (px + x >= 0 && px + x < W && py + y >= 0 && py + y < H) {
                const float* p = img + 4 * ((size_t)(py + y) * W + (px + x));
                if (p[0] != c[0] && std::fabs(linearize(c[1]) - linearize(p[1])) <= 0.0025 && p[2] == 1.0f)
                    return true;
            }
    return false;
}

// tex2D with point sampling and clamp addressing at integer coordinates
const float* texel(const float* img, int W, int H, int x, int y) {
    x = x < 0 ? 0 : (x >= W ? W - 1 : x);
    y = y < 0 ? 0 : (y >= H ? H - 1 : y);
    return img + 4 * ((size_t)y * W + x);
}

float plerp(float v0, float v1, float t) { return (1 - t) * v0 + t * v1; }

// MeanFilter.frag's linearize: all-float GLSL (zNear 1, zFar 1000)
float gl_linearize_f(float depth) { return 2.0f / (1001.0f - depth * 999.0f); }

}  // namespace pba
}  // namespace

extern "C" void or_pba_voronoi(const int16_t* sites, int W, int H, int m1, int m2, int m3, int16_t* out,
                               int threads) {
    if (!pba::shape_ok(W, H, m1, m2, m3)) return;
    std::vector<uint8_t> site((size_t)W * H);
    for (size_t i = 0; i < site.size(); ++i) site[i] = sites[2 * i] != pba::kMarker;
    pba::voronoi(site.data(), W, H, m1, m2, m3, out, threads);
}

extern "C" void or_edt_sites(const float* image, int W, int H, int16_t* sites) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const bool s = pba::is_site(image, W, H, x, y);
            sites[2 * ((size_t)y * W + x)] = (int16_t)(s ? x : pba::kMarker);
            sites[2 * ((size_t)y * W + x) + 1] = (int16_t)(s ? y : pba::kMarker);
        }
}

// pbaNormalizeDistanceTransform (pba2DKernel.h:541-569): distance between
// the pixel's and its nearest site's positions; outside the penumbra (site
// not lit-facing, depths apart, or farther than penumbra / 2) the hard value
// stays, otherwise plerp(0.5 -/+ distance / penumbra, 1, intensity) for
// umbra / lit pixels.  Channels 0 and 1 of out4 are written.
extern "C" void or_edt_normalize(const int16_t* nearest, const float* image, const float* position, int W, int H,
                                 float penumbra, float intensity, float* out4) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t q = (size_t)y * W + x;
            const int sx = nearest[2 * q], sy = nearest[2 * q + 1];
            const float* ip = image + 4 * q;
            const float* sp = pba::texel(image, W, H, sx, sy);
            const float* p1 = position + 4 * q;
            const float* p2 = pba::texel(position, W, H, sx, sy);
            const float dist = std::sqrt((p1[0] - p2[0]) * (p1[0] - p2[0]) + (p1[1] - p2[1]) * (p1[1] - p2[1]) +
                                         (p1[2] - p2[2]) * (p1[2] - p2[2]));
            float r;
            if (sp[2] != 1.0f || std::fabs(pba::linearize(sp[1]) - pba::linearize(ip[1])) > 0.0005 ||
                dist > penumbra / 2)
                r = ip[0];
            else if (ip[0] == intensity)
                r = pba::plerp((float)(0.5 - dist / penumbra), 1.0f, intensity);
            else
                r = pba::plerp((float)(0.5 + dist / penumbra), 1.0f, intensity);
            out4[4 * q] = r;
            out4[4 * q + 1] = ip[1];
        }
}

// initializeInput + pba2DCompute(m1, m2, m3) + pbaNormalizeDistanceTransform
// (filterHardShadowsUsingEDT's CUDA part, ShadowMapping/src/main.cpp:
// 416-422).  sites / nearest may be NULL.
extern "C" void or_edt_soft_shadows(const float* image, const float* position, int W, int H, int m1, int m2,
                                    int m3, float penumbra, float intensity, int16_t* sites, int16_t* nearest,
                                    float* out4, int threads) {
    if (!pba::shape_ok(W, H, m1, m2, m3)) return;
    std::vector<int16_t> s((size_t)2 * W * H), nn((size_t)2 * W * H);
    or_edt_sites(image, W, H, s.data());
    or_pba_voronoi(s.data(), W, H, m1, m2, m3, nn.data(), threads);
    or_edt_normalize(nn.data(), image, position, W, H, penumbra, intensity, out4);
    if (sites) std::memcpy(sites, s.data(), s.size() * sizeof(int16_t));
    if (nearest) std::memcpy(nearest, nn.data(), nn.size() * sizeof(int16_t));
}

// The EDTSM output of the SMSR shaders (NonConservativeSMSR.frag:367-397,
// ConservativeSMSR.frag:215-245): image (shadow, depth, preEvaluatedShadow,
// 1) and position = MVP * vertex, with depth = position.z / position.w * 0.5
// + 0.5; background pixels keep the clear colour (0, 0, 0, 1) in both.
extern "C" void or_edt_inputs(const gi_vis_params* p, const float camera_mvp[16], const float* pos, const float* nrm,
                              const float* vis, int W, int H, float* image, float* position) {
    Ctx c;
    c.p = p;
    c.map = nullptr;
    c.W = c.H = 0;
    c.sx = c.sy = 0.0f;
    c.I = p->shadow_intensity;
    for (size_t q = 0; q < (size_t)W * H; ++q) {
        const float* v = pos + 4 * q;
        float* im = image + 4 * q;
        float* po = position + 4 * q;
        if (v[0] == 0.0f) {
            im[0] = im[1] = im[2] = 0.0f;
            im[3] = 1.0f;
            po[0] = po[1] = po[2] = 0.0f;
            po[3] = 1.0f;
            continue;
        }
        const V4 vertex{v[0], v[1], v[2], v[3]};
        const V4 normal{nrm[4 * q], nrm[4 * q + 1], nrm[4 * q + 2], nrm[4 * q + 3]};
        const float pre = pretest(c, vertex, normal);
        const V4 cp = mat4_mul(camera_mvp, vertex);
        float depth = cp.z / cp.w;
        depth = depth * 0.5f + 0.5f;
        im[0] = vis[q];
        im[1] = depth;
        im[2] = pre;
        im[3] = 1.0f;
        po[0] = cp.x;
        po[1] = cp.y;
        po[2] = cp.z;
        po[3] = cp.w;
    }
}

// MeanFilter.frag's x and y passes (ShadowMapping/src/main.cpp:424-447) with
// the same choices as the CUDA path: centre = (i + 0.5) / size, pass 1
// GL_NEAREST (texel floor(u * size)), pass 2 bilinear at level 0 along the
// filtered axis, zero border, at most 2049 samples, dscreen from tan(22.5)
// (GLSL's tan of the 45-degree fov uniform, taken as radians).
extern "C" void or_edt_mean_filter(const gi_vis_params* p, const float* image, const float* pos, int W, int H,
                                   int order, float* out) {
    const float dscreen = 1.0f / (2.0f * (float)std::tan((double)(45.0f / 2.0f)));
    const float* m = p->camera_mv;
    std::vector<float> xpass((size_t)W * H * 4);
    for (int pass = 0; pass < 2; ++pass) {
        const bool vertical = pass == 1;
        const float* in = vertical ? xpass.data() : image;
        float* dst = vertical ? out : xpass.data();
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t q = (size_t)y * W + x;
                const float* v = pos + 4 * q;
                float* o = dst + 4 * q;
                if (v[0] == 0.0f) {
                    o[0] = o[1] = o[2] = 0.0f;
                    o[3] = 1.0f;
                    continue;
                }
                const float* color = in + 4 * q;
                const float ez = m[2] * v[0] + m[6] * v[1] + m[10] * v[2] + m[14] * v[3];
                const float deye = -ez;
                const float kc = (dscreen * (float)order * 50.0f) / (deye * 2.0f);
                const float step = vertical ? 1.0f / (float)H : 1.0f / (float)W;
                const float cs = ((float)(vertical ? y : x) + 0.5f) / (float)(vertical ? H : W);
                const float Lc = pba::gl_linearize_f(color[1]);
                const float size = (float)(vertical ? H : W);
                float sum = 0.0f;
                int count = 0;
                for (float sample = -kc; sample <= kc && count < 2049; sample = sample + 1.0f) {
                    const float u = cs + sample * step;
                    float r = 0.0f, g = 0.0f;
                    if (!vertical) {
                        const float fi = std::floor(u * size);
                        if (fi >= 0.0f && fi < size) {
                            const float* t = in + 4 * ((size_t)y * W + (int)fi);
                            r = t[0];
                            g = t[1];
                        }
                    } else {
                        const float uu = u * size - 0.5f;
                        const float f0 = std::floor(uu), w1 = uu - f0, w0 = 1.0f - w1;
                        const int j0 = (int)f0;
                        float t0r = 0.0f, t0g = 0.0f, t1r = 0.0f, t1g = 0.0f;
                        if (j0 >= 0 && j0 < H) {
                            t0r = in[4 * ((size_t)j0 * W + x)];
                            t0g = in[4 * ((size_t)j0 * W + x) + 1];
                        }
                        if (j0 + 1 >= 0 && j0 + 1 < H) {
                            t1r = in[4 * ((size_t)(j0 + 1) * W + x)];
                            t1g = in[4 * ((size_t)(j0 + 1) * W + x) + 1];
                        }
                        r = w0 * t0r + w1 * t1r;
                        g = w0 * t0g + w1 * t1g;
                    }
                    if (r == 0.0f || std::fabs(pba::gl_linearize_f(g) - Lc) >= 0.0005f) r = color[0];
                    sum = sum + r;
                    ++count;
                }
                sum = sum / (float)count;
                o[0] = sum;
                o[1] = color[1];
                o[2] = 0.0f;
                o[3] = 0.0f;
            }
    }
}
