// raster.cu -- tiled software rasteriser for sm_103a.
//
// Replaces the OpenGL fixed-function work the reference gets from the GL
// driver in three passes:
//   * the light-view depth map (renderShadowMap / displaySceneFromLightPOV,
//     ShadowMapping/src/main.cpp:221-274, 350-361; glPolygonOffset(4, 20)
//     at main.cpp:246-247; depth texture setup MyGLTextureViewer.cpp:3-28);
//   * the camera G-buffer (renderGBuffer, main.cpp:363-372; GBuffer.vert /
//     GBuffer.frag:32-38);
//   * the shadow-volume stencil pass (ShadowVolumes/src/main.cpp:120-206,
//     volumes from ShadowVolume::update, ShadowVolume.cpp:116-194).
//
// Rasterisation rules (OpenGL 4.6 core spec 13.6, 14.6, 14.9; choices the
// spec leaves open are fixed as follows and shared with the CPU oracle):
//   clip c = MVP (x, y, z, 1) in glm's operation order; clipping against
//   z >= -w, z <= w and the guard band |x|, |y| <= 16 w (Sutherland-Hodgman,
//   intersection from the inside vertex, fan from vertex 0); window
//   x = x_ndc W/2 + W/2, z = z_ndc / 2 + 1/2; 8 sub-pixel bits rounded to
//   nearest even; integer edge functions at pixel centres with the top-left
//   rule of the counter-clockwise (y-up) triangle; gl_FrontFacing = CCW;
//   depth linear in window space from l_i = E_i * (1/area); polygon offset
//   m * factor + 2^(e-23) * units; depth clamped to [0, 1]; depth buffers
//   cleared to 1 with test LESS.
//
// GPU organisation (one pass = 4 launches, all stream-ordered and graph
// capturable):
//   1. clear the target;
//   2. k_setup: one thread per primitive transforms, clips and sets up its
//      triangle(s); triangles whose pixel bounding box is small are
//      rasterised by that thread, large ones are appended to a record list;
//   3. k_scan: one block turns the per-record tile counts (16x16 tiles)
//      into offsets;
//   4. k_tiles: a persistent grid of warps splits the implied tile list into
//      contiguous ranges, rejects tiles the triangle misses and covers each
//      16x16 tile with one warp (8 pixels per lane, incremental edges).
// Depth and the G-buffer's (depth, primitive) keys are resolved with
// atomicMin, which makes the result independent of the launch order; the
// stencil pass uses integer atomicAdd of +1 / -1 and wraps at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>

#include "internal.h"
#include "raster.h"
#include "raster_common.cuh"

namespace gi {
namespace dev {

constexpr int kTile = 16;

struct TriRec {
    int X[3];
    int Y[3];
    float z[3];
    float zoff;
    unsigned prim;
    unsigned short x0, x1, y0, y1;
    unsigned short tx0, ty0, ntx, nty;
    unsigned front;
    unsigned long long base;
};

enum { MODE_DEPTH = 0, MODE_VKEY = 1, MODE_STENCIL = 2 };

struct RasterArgs {
    const float* points;
    const float* normals;
    const int* indices;
    int num_prims;
    Mat4 mvp;
    int W, H;
    int bias_mode;
    float cbias, factor, units;
    int depth_func;
    float L[3];
    float infinity;
    unsigned* depth;
    unsigned long long* keys;
    int* counts;
    TriRec* recs;
    unsigned rec_cap;
    unsigned* counters;  // [0] records requested, [1] spilled to in-thread
    unsigned long long* tile_total;
    int small_px;
};

__device__ __forceinline__ void load_vertex(const float* p, int idx, float out[3]) {
    out[0] = __ldg(p + 3 * (size_t)idx + 0);
    out[1] = __ldg(p + 3 * (size_t)idx + 1);
    out[2] = __ldg(p + 3 * (size_t)idx + 2);
}

// Pattern of the six side triangles (ShadowVolume.cpp:61-110).
__constant__ int c_patA[6][3] = {{1, 0, 3}, {1, 3, 4}, {2, 1, 4}, {2, 4, 5}, {0, 2, 5}, {0, 5, 3}};
__constant__ int c_patB[6][3] = {{4, 3, 0}, {4, 0, 1}, {5, 4, 1}, {5, 1, 2}, {3, 5, 2}, {3, 2, 0}};

// Object-space vertices of primitive `prim` for the pass `MODE`.
template <int MODE>
__device__ __forceinline__ void prim_vertices(const RasterArgs& a, int prim, float v[3][3]) {
    if (MODE != MODE_STENCIL) {
        const int* tri = a.indices + 3 * (size_t)prim;
#pragma unroll
        for (int j = 0; j < 3; ++j) load_vertex(a.points, __ldg(tri + j), v[j]);
    } else {
        int t = prim / 6, k = prim - t * 6;
        const int* tri = a.indices + 3 * (size_t)t;
        int i0 = __ldg(tri), i1 = __ldg(tri + 1), i2 = __ldg(tri + 2);
        float n0[3], n1[3], n2[3];
        load_vertex(a.normals, i0, n0);
        load_vertex(a.normals, i1, n1);
        load_vertex(a.normals, i2, n2);
        float n[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) n[ax] = ((n0[ax] + n1[ax]) + n2[ax]) / 3.0f;
        float d = n[0] * a.L[0] + n[1] * a.L[1] + n[2] * a.L[2];
        int ids[3] = {i0, i1, i2};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            int q = d >= 0.0f ? c_patA[k][j] : c_patB[k][j];
            float p[3];
            load_vertex(a.points, ids[q % 3], p);
            if (q < 3) {
                v[j][0] = p[0];
                v[j][1] = p[1];
                v[j][2] = p[2];
            } else {
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) v[j][ax] = (p[ax] - a.L[ax]) * a.infinity;
            }
        }
    }
}

template <int MODE>
__device__ __forceinline__ void emit(const RasterArgs& a, int x, int y, float z, float zoff,
                                     unsigned prim, bool front) {
    size_t idx = (size_t)y * a.W + x;
    if (MODE == MODE_DEPTH) {
        z = clamp01(z + zoff);
        if (z < 1.0f) atomicMin(a.depth + idx, __float_as_uint(z));
    } else if (MODE == MODE_VKEY) {
        z = clamp01(z);
        if (z < 1.0f) {
            unsigned long long k = ((unsigned long long)__float_as_uint(z) << 32) | prim;
            atomicMin(a.keys + idx, k);
        }
    } else {
        z = clamp01(z);
        float d = __uint_as_float(__ldg(a.depth + idx));
        bool pass = a.depth_func == GI_DEPTH_LEQUAL ? (z <= d) : (z < d);
        if (pass) atomicAdd(a.counts + idx, front ? 1 : -1);
    }
}

// In-thread rasterisation of a small triangle over its pixel bounding box.
template <int MODE>
__device__ void raster_small(const RasterArgs& a, const Setup& s, const Edges& e, int x0, int x1,
                             int y0, int y1, float zoff, unsigned prim) {
    for (int y = y0; y <= y1; ++y) {
        int64_t py = (int64_t)y * kSub + kSub / 2;
        int64_t px = (int64_t)x0 * kSub + kSub / 2;
        int64_t E[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) E[i] = edge_at(e, i, px, py);
        for (int x = x0; x <= x1; ++x) {
            if (inside3(e, E)) emit<MODE>(a, x, y, depth_at(s, E), zoff, prim, s.front);
#pragma unroll
            for (int i = 0; i < 3; ++i) E[i] -= e.B[i] * kSub;
        }
    }
}

template <int MODE>
__device__ void process_sub(const RasterArgs& a, const float* c0, const float* c1, const float* c2,
                            const float* b0, const float* b1, const float* b2, unsigned prim) {
    Setup s;
    if (!setup_triangle(c0, c1, c2, b0, b1, b2, a.W, a.H, s)) return;
    int64_t minX = min(s.X[0], min(s.X[1], s.X[2])), maxX = max(s.X[0], max(s.X[1], s.X[2]));
    int64_t minY = min(s.Y[0], min(s.Y[1], s.Y[2])), maxY = max(s.Y[0], max(s.Y[1], s.Y[2]));
    int64_t bx0 = -((-(minX - kSub / 2)) >> kSubBits);
    int64_t bx1 = (maxX - kSub / 2) >> kSubBits;
    int64_t by0 = -((-(minY - kSub / 2)) >> kSubBits);
    int64_t by1 = (maxY - kSub / 2) >> kSubBits;
    int x0 = (int)max((int64_t)0, bx0), x1 = (int)min((int64_t)a.W - 1, bx1);
    int y0 = (int)max((int64_t)0, by0), y1 = (int)min((int64_t)a.H - 1, by1);
    if (x0 > x1 || y0 > y1) return;
    float zoff = 0.0f;
    if (MODE == MODE_DEPTH) {
        if (a.bias_mode == GI_BIAS_POLYGON_OFFSET) zoff = polygon_offset(s, a.factor, a.units);
        else if (a.bias_mode == GI_BIAS_CONSTANT) zoff = a.cbias;
    }
    int npx = (x1 - x0 + 1) * (y1 - y0 + 1);
    Edges e;
    make_edges(s, e);
    if (npx > a.small_px) {
        unsigned slot = atomicAdd(a.counters + 0, 1u);
        if (slot < a.rec_cap) {
            TriRec r;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                r.X[i] = (int)s.X[i];
                r.Y[i] = (int)s.Y[i];
                r.z[i] = s.z[i];
            }
            r.zoff = zoff;
            r.prim = prim;
            r.x0 = (unsigned short)x0;
            r.x1 = (unsigned short)x1;
            r.y0 = (unsigned short)y0;
            r.y1 = (unsigned short)y1;
            r.tx0 = (unsigned short)(x0 / kTile);
            r.ty0 = (unsigned short)(y0 / kTile);
            r.ntx = (unsigned short)(x1 / kTile - x0 / kTile + 1);
            r.nty = (unsigned short)(y1 / kTile - y0 / kTile + 1);
            r.front = s.front ? 1u : 0u;
            r.base = 0;
            a.recs[slot] = r;
            return;
        }
        atomicAdd(a.counters + 1, 1u);  // record list full: rasterise here
    }
    raster_small<MODE>(a, s, e, x0, x1, y0, y1, zoff, prim);
}

template <int MODE>
__global__ void __launch_bounds__(128) k_setup(RasterArgs a) {
    int prim = blockIdx.x * blockDim.x + threadIdx.x;
    if (prim >= a.num_prims) return;
    float v[3][3];
    prim_vertices<MODE>(a, prim, v);
    float c[3][4];
#pragma unroll
    for (int j = 0; j < 3; ++j) transform(a.mvp, v[j][0], v[j][1], v[j][2], c[j]);
    const float id[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
    unsigned base_id = MODE == MODE_VKEY ? ((unsigned)prim << 3) : (unsigned)prim;
    if (all_inside(c[0], c[1], c[2])) {
        process_sub<MODE>(a, c[0], c[1], c[2], id[0], id[1], id[2], base_id);
        return;
    }
    CV poly[9];
    int n = clip_polygon(c[0], c[1], c[2], poly);
    for (int i = 1; i + 1 < n; ++i)
        process_sub<MODE>(a, poly[0].c, poly[i].c, poly[i + 1].c, poly[0].b, poly[i].b,
                          poly[i + 1].b, MODE == MODE_VKEY ? (base_id | (unsigned)(i - 1)) : base_id);
}

// Exclusive scan of the records' tile counts (one block of 1024 threads).
__global__ void __launch_bounds__(1024) k_scan(TriRec* recs, const unsigned* counters,
                                               unsigned rec_cap, unsigned long long* total) {
    __shared__ unsigned long long warp_sums[32];
    __shared__ unsigned long long carry;
    const unsigned n = min(counters[0], rec_cap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (unsigned start = 0; start < n; start += 1024) {
        unsigned i = start + threadIdx.x;
        unsigned long long v = 0;
        if (i < n) v = (unsigned long long)recs[i].ntx * recs[i].nty;
        unsigned long long x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = warp_sums[lane];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                unsigned long long y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            warp_sums[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        unsigned long long warp_off = warp == 0 ? 0 : warp_sums[warp - 1];
        if (i < n) recs[i].base = carry + warp_off + x - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sums[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Warp-per-tile rasterisation of the recorded large triangles.
template <int MODE>
__global__ void __launch_bounds__(256) k_tiles(RasterArgs a) {
    const unsigned n = min(a.counters[0], a.rec_cap);
    if (n == 0) return;
    const unsigned long long total = *a.tile_total;
    const int lane = threadIdx.x & 31;
    const unsigned long long nwarps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long w = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    unsigned long long begin = total * w / nwarps, end = total * (w + 1) / nwarps;
    if (begin >= end) return;
    // first record whose range ends after `begin`
    unsigned lo = 0, hi = n - 1;
    while (lo < hi) {
        unsigned mid = (lo + hi) >> 1;
        const TriRec* r = a.recs + mid;
        if (r->base + (unsigned long long)r->ntx * r->nty <= begin) lo = mid + 1;
        else hi = mid;
    }
    unsigned ri = lo;
    TriRec r = a.recs[ri];
    Setup s;
    Edges e;
    auto load_setup = [&]() {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.X[i] = r.X[i];
            s.Y[i] = r.Y[i];
            s.z[i] = r.z[i];
        }
        s.area = (s.X[1] - s.X[0]) * (s.Y[2] - s.Y[0]) - (s.X[2] - s.X[0]) * (s.Y[1] - s.Y[0]);
        s.inv_area = 1.0f / (float)s.area;
        s.front = r.front != 0;
        make_edges(s, e);
    };
    load_setup();
    for (unsigned long long item = begin; item < end; ++item) {
        while (item >= r.base + (unsigned long long)r.ntx * r.nty) {
            ++ri;
            r = a.recs[ri];
            load_setup();
        }
        unsigned local = (unsigned)(item - r.base);
        int ty = r.ty0 + (int)(local / r.ntx);
        int tx = r.tx0 + (int)(local % r.ntx);
        int px0 = max(tx * kTile, (int)r.x0), px1 = min(tx * kTile + kTile - 1, (int)r.x1);
        int py0 = max(ty * kTile, (int)r.y0), py1 = min(ty * kTile + kTile - 1, (int)r.y1);
        // Reject the tile if some edge is negative at every pixel centre.
        bool miss = false;
        {
            int64_t cx0 = (int64_t)px0 * kSub + kSub / 2, cx1 = (int64_t)px1 * kSub + kSub / 2;
            int64_t cy0 = (int64_t)py0 * kSub + kSub / 2, cy1 = (int64_t)py1 * kSub + kSub / 2;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                int64_t ymax = e.A[i] > 0 ? cy1 : cy0;
                int64_t xmin = e.B[i] > 0 ? cx0 : cx1;
                int64_t emax = e.A[i] * (ymax - e.Ya[i]) - e.B[i] * (xmin - e.Xa[i]);
                miss |= emax < 0;
            }
        }
        if (miss) continue;
        int x = tx * kTile + (lane & 15);
        int y = ty * kTile + (lane >> 4);
        if (x < px0 || x > px1) continue;
        int64_t px = (int64_t)x * kSub + kSub / 2, py = (int64_t)y * kSub + kSub / 2;
        int64_t E[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) E[i] = edge_at(e, i, px, py);
#pragma unroll 2
        for (int k = 0; k < kTile / 2; ++k, y += 2) {
            if (y >= py0 && y <= py1 && inside3(e, E))
                emit<MODE>(a, x, y, depth_at(s, E), r.zoff, r.prim, s.front);
#pragma unroll
            for (int i = 0; i < 3; ++i) E[i] += e.A[i] * (2 * kSub);
        }
    }
}

__global__ void k_fill_u32(unsigned* p, size_t n, unsigned v) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    // 16-byte vector stores only when the base is 16-byte aligned.
    size_t n4 = (reinterpret_cast<uintptr_t>(p) & 15) ? 0 : n / 4;
    uint4 v4 = make_uint4(v, v, v, v);
    uint4* p4 = reinterpret_cast<uint4*>(p);
    for (size_t j = i; j < n4; j += stride) p4[j] = v4;
    for (size_t j = n4 * 4 + i; j < n; j += stride) p[j] = v;
}

__global__ void k_fill_u64(unsigned long long* p, size_t n, unsigned long long v) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t j = i; j < n; j += stride) p[j] = v;
}

// G-buffer resolve: re-derive the winning sub-triangle of each pixel and
// interpolate object position and normal perspective-correctly.
__global__ void __launch_bounds__(128) k_gbuffer_resolve(const unsigned long long* keys,
                                                         const float* points, const float* normals,
                                                         const int* indices, Mat4 mvp, int W,
                                                         int H, float4* pos, float4* nrm) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    size_t p = (size_t)y * W + x;
    const unsigned long long clear = ((unsigned long long)__float_as_uint(1.0f) << 32) | 0xFFFFFFFFull;
    unsigned long long k = __ldg(keys + p);
    float4 bg = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (k == clear) {
        pos[p] = bg;
        nrm[p] = bg;
        return;
    }
    unsigned prim = (unsigned)(k & 0xFFFFFFFFull);
    int t = (int)(prim >> 3), sub = (int)(prim & 7);
    const int* tri = indices + 3 * (size_t)t;
    int ids[3] = {__ldg(tri), __ldg(tri + 1), __ldg(tri + 2)};
    float c[3][4];
    for (int j = 0; j < 3; ++j) {
        float v[3];
        load_vertex(points, ids[j], v);
        transform(mvp, v[0], v[1], v[2], c[j]);
    }
    const float id[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
    Setup s;
    bool ok;
    if (all_inside(c[0], c[1], c[2])) {
        ok = sub == 0 && setup_triangle(c[0], c[1], c[2], id[0], id[1], id[2], W, H, s);
    } else {
        CV poly[9];
        int n = clip_polygon(c[0], c[1], c[2], poly);
        ok = (sub + 2 < n) && setup_triangle(poly[0].c, poly[sub + 1].c, poly[sub + 2].c, poly[0].b,
                                             poly[sub + 1].b, poly[sub + 2].b, W, H, s);
    }
    if (!ok) {
        pos[p] = bg;
        nrm[p] = bg;
        return;
    }
    Edges e;
    make_edges(s, e);
    int64_t px = (int64_t)x * kSub + kSub / 2, py = (int64_t)y * kSub + kSub / 2;
    float q[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        float l = (float)edge_at(e, j, px, py) * s.inv_area;
        q[j] = l * s.iw[j];
    }
    float sum = (q[0] + q[1]) + q[2];
    float pc[3] = {q[0] / sum, q[1] / sum, q[2] / sum};
    float B[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) B[j] = (pc[0] * s.b[0][j] + pc[1] * s.b[1][j]) + pc[2] * s.b[2][j];
    float P[3][3], N[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        load_vertex(points, ids[j], P[j]);
        load_vertex(normals, ids[j], N[j]);
    }
    float o[3], on[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o[j] = (B[0] * P[0][j] + B[1] * P[1][j]) + B[2] * P[2][j];
        on[j] = (B[0] * N[0][j] + B[1] * N[1][j]) + B[2] * N[2][j];
    }
    pos[p] = make_float4(o[0], o[1], o[2], 1.0f);
    nrm[p] = make_float4(on[0], on[1], on[2], s.front ? 1.0f : 0.0f);
}

__global__ void k_wrap_stencil(const int* counts, unsigned char* out, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (unsigned char)((unsigned)counts[i] & 0xFFu);
}

}  // namespace dev

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {

int sm_count(int device) {
    static int cached[64] = {0};
    if (device < 0 || device >= 64) return 152;
    if (!cached[device]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0)
            v = 152;
        cached[device] = v;
    }
    return cached[device];
}

unsigned grid_for(size_t n, unsigned block) {
    size_t g = (n + block - 1) / block;
    if (g > 1u << 30) g = 1u << 30;
    return (unsigned)std::max<size_t>(g, 1);
}

}  // namespace

gi_status launch_fill_u32(gi_context* ctx, unsigned* p, size_t n, unsigned v, cudaStream_t st) {
    unsigned grid = std::min<unsigned>(grid_for(n / 4 + 1, 256), (unsigned)sm_count(ctx->device) * 8);
    dev::k_fill_u32<<<grid, 256, 0, st>>>(p, n, v);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "fill kernel launch");
}

static gi_status ensure_records(gi_context* ctx) {
    // Start with room for 256K large triangles; grow 4x after a pass that
    // spilled (the spilled triangles were still rasterised, only slower).
    size_t want = ctx->cap_tri_records ? ctx->cap_tri_records / sizeof(dev::TriRec) : 0;
    if (want == 0) want = 256 * 1024;
    if (ctx->h_status && ctx->h_status[1] > 0 && ctx->h_status[0] > want) {
        while (want < ctx->h_status[0] && want < (size_t)1 << 26) want *= 4;
        ctx->h_status[1] = 0;
    }
    return ensure_buffer(&ctx->d_tri_records, &ctx->cap_tri_records, want * sizeof(dev::TriRec));
}

// One raster pass: setup, scan and tile kernels (the target is cleared by
// the caller).  `mode` selects the fragment operation.
static gi_status run_raster(gi_context* ctx, dev::RasterArgs& a, int mode, cudaStream_t st) {
    if (a.num_prims <= 0) return GI_OK;
    gi_status s = ensure_records(ctx);
    if (s != GI_OK) return s;
    a.recs = static_cast<dev::TriRec*>(ctx->d_tri_records);
    a.rec_cap = (unsigned)(ctx->cap_tri_records / sizeof(dev::TriRec));
    a.counters = ctx->d_status + 4;
    a.tile_total = reinterpret_cast<unsigned long long*>(ctx->d_status + 8);
    if (a.small_px <= 0) a.small_px = 128;
    cudaError_t e = cudaMemsetAsync(ctx->d_status + 4, 0, 8 * sizeof(unsigned), st);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemsetAsync(counters)");
    unsigned g = grid_for((size_t)a.num_prims, 128);
    const int blocks_tiles = sm_count(ctx->device) * 8;
    switch (mode) {
        case dev::MODE_DEPTH:
            dev::k_setup<dev::MODE_DEPTH><<<g, 128, 0, st>>>(a);
            dev::k_scan<<<1, 1024, 0, st>>>(a.recs, a.counters, a.rec_cap, a.tile_total);
            dev::k_tiles<dev::MODE_DEPTH><<<blocks_tiles, 256, 0, st>>>(a);
            break;
        case dev::MODE_VKEY:
            dev::k_setup<dev::MODE_VKEY><<<g, 128, 0, st>>>(a);
            dev::k_scan<<<1, 1024, 0, st>>>(a.recs, a.counters, a.rec_cap, a.tile_total);
            dev::k_tiles<dev::MODE_VKEY><<<blocks_tiles, 256, 0, st>>>(a);
            break;
        default:
            dev::k_setup<dev::MODE_STENCIL><<<g, 128, 0, st>>>(a);
            dev::k_scan<<<1, 1024, 0, st>>>(a.recs, a.counters, a.rec_cap, a.tile_total);
            dev::k_tiles<dev::MODE_STENCIL><<<blocks_tiles, 256, 0, st>>>(a);
            break;
    }
    ctx->launches += 3;
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "raster kernel launch");
    // Mirror the counters for the capacity heuristic (read on a later call).
    e = cudaMemcpyAsync(ctx->h_status, ctx->d_status + 4, 2 * sizeof(unsigned),
                        cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpyAsync(counters)");
    return GI_OK;
}

static dev::Mat4 mat_of(const float m[16]) {
    dev::Mat4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = m[i];
    return r;
}

gi_status raster_depth_map(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W,
                           int H, int bias_mode, float cbias, float factor, float units,
                           float* d_depth, int small_px, cudaStream_t st) {
    gi_status s = launch_fill_u32(ctx, reinterpret_cast<unsigned*>(d_depth), (size_t)W * H,
                                  0x3f800000u, st);
    if (s != GI_OK) return s;
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    a.num_prims = scene->dev_triangles;
    a.mvp = mat_of(mvp);
    a.W = W;
    a.H = H;
    a.bias_mode = bias_mode;
    a.cbias = cbias;
    a.factor = factor;
    a.units = units;
    a.depth = reinterpret_cast<unsigned*>(d_depth);
    a.small_px = small_px;
    return run_raster(ctx, a, dev::MODE_DEPTH, st);
}

gi_status raster_gbuffer(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W, int H,
                         float* d_pos, float* d_nrm, int small_px, cudaStream_t st) {
    const size_t npx = (size_t)W * H;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_vkeys), &ctx->cap_vkeys,
                                npx * sizeof(unsigned long long));
    if (s != GI_OK) return s;
    const unsigned long long clear = ((unsigned long long)0x3f800000u << 32) | 0xFFFFFFFFull;
    dev::k_fill_u64<<<std::min<unsigned>(grid_for(npx, 256), (unsigned)sm_count(ctx->device) * 8),
                      256, 0, st>>>(ctx->d_vkeys, npx, clear);
    ctx->launches++;
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    a.num_prims = scene->dev_triangles;
    a.mvp = mat_of(mvp);
    a.W = W;
    a.H = H;
    a.keys = ctx->d_vkeys;
    a.small_px = small_px;
    s = run_raster(ctx, a, dev::MODE_VKEY, st);
    if (s != GI_OK) return s;
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    dev::k_gbuffer_resolve<<<grid, 128, 0, st>>>(ctx->d_vkeys, scene->d_points, scene->d_normals,
                                                 scene->d_indices, a.mvp, W, H,
                                                 reinterpret_cast<float4*>(d_pos),
                                                 reinterpret_cast<float4*>(d_nrm));
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gbuffer resolve launch");
}

gi_status raster_shadow_volumes(gi_context* ctx, const gi_scene* scene, const float L[3],
                                float infinity, const float mvp[16], int W, int H, int depth_func,
                                unsigned char* d_stencil, float* d_depth_out, int small_px,
                                cudaStream_t st) {
    const size_t npx = (size_t)W * H;
    float* depth = d_depth_out;
    gi_status s;
    if (!depth) {
        s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_depth_tmp), &ctx->cap_depth_tmp,
                          npx * sizeof(float));
        if (s != GI_OK) return s;
        depth = ctx->d_depth_tmp;
    }
    s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_counts), &ctx->cap_counts, npx * sizeof(int));
    if (s != GI_OK) return s;
    s = raster_depth_map(ctx, scene, mvp, W, H, GI_BIAS_NONE, 0.0f, 0.0f, 0.0f, depth, small_px, st);
    if (s != GI_OK) return s;
    cudaError_t e = cudaMemsetAsync(ctx->d_counts, 0, npx * sizeof(int), st);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemsetAsync(counts)");
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    if ((long long)scene->dev_triangles * 6 > 0x7fffffffLL)
        return fail(GI_ERR_CAPACITY, "too many volume triangles");
    a.num_prims = scene->dev_triangles * 6;
    a.mvp = mat_of(mvp);
    a.W = W;
    a.H = H;
    a.depth_func = depth_func;
    a.L[0] = L[0];
    a.L[1] = L[1];
    a.L[2] = L[2];
    a.infinity = infinity;
    a.depth = reinterpret_cast<unsigned*>(depth);
    a.counts = ctx->d_counts;
    a.small_px = small_px;
    s = run_raster(ctx, a, dev::MODE_STENCIL, st);
    if (s != GI_OK) return s;
    dev::k_wrap_stencil<<<grid_for(npx, 256), 256, 0, st>>>(ctx->d_counts, d_stencil, npx);
    ctx->launches++;
    e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "stencil wrap launch");
}

// ---------------------------------------------------------------------------
// Allocation-free G-buffer (gi_gbuffer_noalloc)
//
// Some callers cannot allocate device memory: a real-time frame loop where
// cudaMalloc's implicit device synchronisation would stall the frame, or a
// host application whose device memory is all owned by its own pool.  This
// variant of the G-buffer pass takes every input and output from the caller
// and keeps its scratch (the per-pixel visibility keys, the large-triangle
// records and the pass counters) in the file-scope array below instead of
// in a gi_context.  The array is reserved on every GPU that loads the
// library, for the life of the process.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocMaxPixels = 1024 * 1024;  // width * height limit
constexpr unsigned kNoallocRecords = 16384;         // large triangles before spilling
constexpr size_t kNoallocKeysBytes = kNoallocMaxPixels * sizeof(unsigned long long);
constexpr size_t kNoallocRecsBytes = (size_t)kNoallocRecords * sizeof(dev::TriRec);
constexpr size_t kNoallocStatusBytes = 256;
constexpr size_t kNoallocBytes = kNoallocKeysBytes + kNoallocRecsBytes + kNoallocStatusBytes;
static_assert(kNoallocKeysBytes % 256 == 0 && kNoallocRecsBytes % 8 == 0, "scratch carving");

// keys | records | status words (counters[2], tile total)
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kNoallocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, resolved once
// per device.  The array's name in host code is only a host-side handle.
gi_status noalloc_scratch(unsigned char** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e, "gi_gbuffer_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kNoallocMaxDevices)
        return fail(GI_ERR_UNSUPPORTED, "gi_gbuffer_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail_cuda(e == cudaSuccess ? cudaErrorInvalidSymbol : e,
                             "gi_gbuffer_noalloc: cudaGetSymbolAddress");
        g_noalloc_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
    return GI_OK;
}

}  // namespace
}  // namespace gi

extern "C" gi_status gi_gbuffer_noalloc(const float* d_points, const float* d_normals,
                                        int num_vertices, const int* d_indices, int num_triangles,
                                        const float camera_mvp[16], int width, int height,
                                        float* d_pos, float* d_nrm, void* stream) {
    using namespace gi;
    if (num_vertices < 0 || num_triangles < 0 || !camera_mvp || !d_pos || !d_nrm ||
        (num_vertices > 0 && (!d_points || !d_normals)) || (num_triangles > 0 && !d_indices))
        return fail(GI_ERR_INVALID_ARG, "gi_gbuffer_noalloc: bad arguments");
    if (width <= 0 || height <= 0 || width > 16384 || height > 16384)
        return fail(GI_ERR_INVALID_ARG, "gi_gbuffer_noalloc: image size must be in [1, 16384]");
    const size_t npx = (size_t)width * height;
    if (npx > kNoallocMaxPixels)
        return fail(GI_ERR_CAPACITY,
                    "gi_gbuffer_noalloc: " + std::to_string(npx) +
                        " pixels exceed the allocation-free scratch (at most 1048576 = 1024 x 1024)");
    if ((size_t)num_triangles >= ((size_t)1 << 29))
        return fail(GI_ERR_CAPACITY, "gi_gbuffer_noalloc: more than 2^29 triangles");
    unsigned char* base = nullptr;
    gi_status st = noalloc_scratch(&base);
    if (st != GI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(base);
    dev::TriRec* recs = reinterpret_cast<dev::TriRec*>(base + kNoallocKeysBytes);
    unsigned* status = reinterpret_cast<unsigned*>(base + kNoallocKeysBytes + kNoallocRecsBytes);
    // The array keeps the previous call's contents: reset the counters and
    // the keys before use.
    cudaError_t e = cudaMemsetAsync(status, 0, kNoallocStatusBytes, cs);
    if (e != cudaSuccess) return fail_cuda(e, "gi_gbuffer_noalloc: cudaMemsetAsync");
    int device = 0;
    cudaGetDevice(&device);
    const unsigned fill_blocks = std::min<unsigned>(grid_for(npx, 256), (unsigned)sm_count(device) * 8);
    const unsigned long long clear = ((unsigned long long)0x3f800000u << 32) | 0xFFFFFFFFull;
    dev::k_fill_u64<<<fill_blocks, 256, 0, cs>>>(keys, npx, clear);
    dev::RasterArgs a = {};
    a.points = d_points;
    a.normals = d_normals;
    a.indices = d_indices;
    a.num_prims = num_triangles;
    a.mvp = mat_of(camera_mvp);
    a.W = width;
    a.H = height;
    a.keys = keys;
    a.recs = recs;
    a.rec_cap = kNoallocRecords;
    a.counters = status;
    a.tile_total = reinterpret_cast<unsigned long long*>(status + 4);
    a.small_px = 128;
    if (num_triangles > 0) {
        dev::k_setup<dev::MODE_VKEY><<<grid_for((size_t)num_triangles, 128), 128, 0, cs>>>(a);
        dev::k_scan<<<1, 1024, 0, cs>>>(a.recs, a.counters, a.rec_cap, a.tile_total);
        dev::k_tiles<dev::MODE_VKEY><<<sm_count(device) * 8, 256, 0, cs>>>(a);
    }
    dim3 grid((width + 31) / 32, (height + 3) / 4);
    dev::k_gbuffer_resolve<<<grid, 128, 0, cs>>>(keys, d_points, d_normals, d_indices, a.mvp, width,
                                                 height, reinterpret_cast<float4*>(d_pos),
                                                 reinterpret_cast<float4*>(d_nrm));
    e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_gbuffer_noalloc: kernel launch");
}
