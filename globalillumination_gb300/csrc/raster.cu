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
#include <atomic>
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
    const int* prim_list;  // stencil: the volume triangles to draw (nullptr: all 6T)
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
        if (a.prim_list) prim = __ldg(a.prim_list + prim);
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

// The volume triangles exactly as the stencil pass draws them: entry 6t + k
// holds side triangle k of input triangle t as three object-space vertices
// (ShadowVolume::build, ShadowVolume.cpp:15-114, resolved through its index
// buffer).
__global__ void __launch_bounds__(256) k_volume_geometry(RasterArgs a, float* out) {
    const int prim = blockIdx.x * blockDim.x + threadIdx.x;
    if (prim >= a.num_prims) return;
    float v[3][3];
    prim_vertices<MODE_STENCIL>(a, prim, v);
    float* o = out + (size_t)prim * 9;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) o[j * 3 + ax] = v[j][ax];
}

// Winding pattern ShadowVolume::build picks for triangle t: the sign of
// dot((n0 + n1 + n2) / 3, L) (ShadowVolume.cpp:55-61), computed as
// prim_vertices computes it.
__device__ __forceinline__ bool volume_pattern_a(const float* normals, const int* indices, int t, const float L[3]) {
    const int* tri = indices + 3 * (size_t)t;
    float n0[3], n1[3], n2[3];
    load_vertex(normals, __ldg(tri), n0);
    load_vertex(normals, __ldg(tri + 1), n1);
    load_vertex(normals, __ldg(tri + 2), n2);
    float n[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) n[ax] = ((n0[ax] + n1[ax]) + n2[ax]) / 3.0f;
    return n[0] * L[0] + n[1] * L[1] + n[2] * L[2] >= 0.0f;
}

// Silhouette extraction over the volume's quads.  Edge k of triangle t
// owns volume triangles 6t + 2k and 6t + 2k + 1 (one quad) in either
// pattern.  adj[3t + k] is the neighbouring triangle across that edge
// (value >> 1) and whether it runs the edge in the same direction
// (value & 1), or -1 for a boundary or non-manifold edge.  The two quads of
// a shared edge span the same four points; they have opposite orientations
// -- and would cancel -- when the triangles run the edge in opposite
// directions and pick the same pattern, or run it in the same direction and
// pick different ones.  Every other quad is a silhouette quad.  One thread
// per edge; each warp compacts its silhouette quads with one ballot and one
// atomic.
__global__ void __launch_bounds__(256) k_silhouette_prims(const float* __restrict__ normals,
                                                          const int* __restrict__ indices,
                                                          const int* __restrict__ adj, int num_tris, float Lx,
                                                          float Ly, float Lz, int* __restrict__ list,
                                                          unsigned* __restrict__ count) {
    const float L[3] = {Lx, Ly, Lz};
    const int lane = threadIdx.x & 31;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool emit_quad = false;
    int t = 0, k = 0;
    if (e < 3LL * num_tris) {
        t = (int)(e / 3);
        k = (int)(e - 3LL * t);
        const int nb = __ldg(adj + e);
        if (nb < 0) {
            emit_quad = true;
        } else {
            const bool pa = volume_pattern_a(normals, indices, t, L);
            const bool pb = volume_pattern_a(normals, indices, nb >> 1, L);
            const bool cancel = (nb & 1) ? (pa != pb) : (pa == pb);
            emit_quad = !cancel;
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, emit_quad);
    if (m == 0) return;
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, 2u * (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (emit_quad) {
        const unsigned off = base + 2u * (unsigned)__popc(m & ((1u << lane) - 1u));
        list[off] = 6 * t + 2 * k;
        list[off + 1] = 6 * t + 2 * k + 1;
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
                                                         int H, float4* pos, float4* nrm,
                                                         const unsigned* rec_of, const BRec* recs,
                                                         const uint4* rres) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    size_t p = (size_t)y * W + x;
    float4 o, on;
    resolve_pixel(__ldg(keys + p), points, normals, indices, mvp, W, H, x, y, rec_of, recs, rres, o, on);
    pos[p] = o;
    nrm[p] = on;
}

__global__ void k_wrap_stencil(const int* counts, unsigned char* out, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (unsigned char)((unsigned)counts[i] & 0xFFu);
}


// ===========================================================================
// Binned (sort-middle) rasteriser
//
// The image is cut into 32 x 32-pixel bins.  k_bin_setup turns every
// primitive into sub-triangle records (transform, clip, set up) and counts
// them into the bins their bounding box touches; records spanning more than
// four bins go through a second, exact bin-overlap expansion (k_big_scan /
// k_big_pairs).  After an exclusive scan of the bin counts, the record ids
// are scattered into per-bin lists, and k_bin_raster runs one CTA per bin:
// warp w owns rows 4w..4w+3 of the bin, lane l owns column l, so every
// pixel has a single owner thread that keeps its depth (or key, or stencil
// count) in registers while it walks the bin's list, and writes it once at
// the end: no global atomics, no clear pass.  Records that do not fit the
// scratch capacities are "spilled" and rasterised afterwards with the
// global-atomic path (k_spill), so every capacity overflow stays exact.
// ===========================================================================
constexpr int kBin = 32;
constexpr int kBinShift = 5;
constexpr int kDirectBins = 4;
constexpr unsigned kSeg = 256;        // records per bin work item
constexpr unsigned kItemBinBits = 18; // work item = bin | segment << 18
constexpr unsigned kFlagBig = 2u;


struct BinArgs {
    RasterArgs r;
    BRec* recs;
    unsigned rec_cap;
    unsigned* big_list;
    unsigned long long* big_base;
    unsigned big_cap;
    unsigned* spill;
    unsigned spill_cap;
    unsigned* bin_count;   // small-record entries per bin (setup)
    unsigned* big_count;   // big-record entries per bin (expansion)
    unsigned* bin_offset;  // nbins + 1
    unsigned* bin_cursor;  // big-record scatter cursors
    unsigned* ranks;       // per small record: its slot within each of its <= 4 bins
    unsigned* items;       // bin work items (bin | segment << 18)
    unsigned item_cap;
    unsigned* bin_list;
    unsigned long long list_cap;
    unsigned long long big_pair_cap;
    unsigned* ctr;  // [0] records [1] big records [2] spills [3] error bits [4,5] admitted big pairs
                    // [6] work items
    int nbx, nby;
};

__device__ __forceinline__ void spill_push(const BinArgs& a, unsigned id) {
    unsigned s = atomicAdd(a.ctr + 2, 1u);
    if (s < a.spill_cap) a.spill[s] = id;
    else atomicOr(a.ctr + 3, 1u);  // spill list full: results incomplete
}

template <int MODE>
__device__ void bin_sub(const BinArgs& a, const float* c0, const float* c1, const float* c2,
                        const float* b0, const float* b1, const float* b2, unsigned prim,
                        unsigned sub) {
    Setup s;
    if (!setup_triangle(c0, c1, c2, b0, b1, b2, a.r.W, a.r.H, s)) return;
    int64_t minX = min(s.X[0], min(s.X[1], s.X[2])), maxX = max(s.X[0], max(s.X[1], s.X[2]));
    int64_t minY = min(s.Y[0], min(s.Y[1], s.Y[2])), maxY = max(s.Y[0], max(s.Y[1], s.Y[2]));
    int64_t bx0 = -((-(minX - kSub / 2)) >> kSubBits);
    int64_t bx1 = (maxX - kSub / 2) >> kSubBits;
    int64_t by0 = -((-(minY - kSub / 2)) >> kSubBits);
    int64_t by1 = (maxY - kSub / 2) >> kSubBits;
    int x0 = (int)max((int64_t)0, bx0), x1 = (int)min((int64_t)a.r.W - 1, bx1);
    int y0 = (int)max((int64_t)0, by0), y1 = (int)min((int64_t)a.r.H - 1, by1);
    if (x0 > x1 || y0 > y1) return;
    const unsigned spill_id = (prim << 3) | sub;
    unsigned slot = atomicAdd(a.ctr + 0, 1u);
    if (slot >= a.rec_cap) {
        spill_push(a, spill_id);
        return;
    }
    float zoff = 0.0f;
    if (MODE == MODE_DEPTH) {
        if (a.r.bias_mode == GI_BIAS_POLYGON_OFFSET) zoff = polygon_offset(s, a.r.factor, a.r.units);
        else if (a.r.bias_mode == GI_BIAS_CONSTANT) zoff = a.r.cbias;
    }
    const int cx0 = x0 >> kBinShift, cx1 = x1 >> kBinShift, cy0 = y0 >> kBinShift, cy1 = y1 >> kBinShift;
    const int nb = (cx1 - cx0 + 1) * (cy1 - cy0 + 1);
    BRec r;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        r.X[i] = (int)s.X[i];
        r.Y[i] = (int)s.Y[i];
    }
    r.z0 = s.z[0];
    r.dz1 = s.z[1] - s.z[0];
    r.dz2 = s.z[2] - s.z[0];
    r.inv_area = s.inv_area;
    r.zoff = zoff;
    r.prim = MODE == MODE_VKEY ? spill_id : prim;
    r.x0 = (unsigned short)x0;
    r.x1 = (unsigned short)x1;
    r.y0 = (unsigned short)y0;
    r.y1 = (unsigned short)y1;
    r.flags = (s.front ? kFlagFront : 0u) | (nb > kDirectBins ? kFlagBig : 0u);
    r.spill_id = spill_id;
    a.recs[slot] = r;
    if (nb <= kDirectBins) {
        int k = 0;
        for (int by = cy0; by <= cy1; ++by)
            for (int bx = cx0; bx <= cx1; ++bx, ++k)
                a.ranks[4 * (size_t)slot + k] = atomicAdd(a.bin_count + by * a.nbx + bx, 1u);
    } else {
        unsigned bi = atomicAdd(a.ctr + 1, 1u);
        if (bi < a.big_cap) a.big_list[bi] = slot;
        else spill_push(a, spill_id);  // the record stays unreferenced
    }
}

template <int MODE>
__global__ void __launch_bounds__(128) k_bin_setup(BinArgs a) {
    int prim = blockIdx.x * blockDim.x + threadIdx.x;
    if (prim >= a.r.num_prims) return;
    float v[3][3];
    prim_vertices<MODE>(a.r, prim, v);
    float c[3][4];
#pragma unroll
    for (int j = 0; j < 3; ++j) transform(a.r.mvp, v[j][0], v[j][1], v[j][2], c[j]);
    const float id[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
    if (all_inside(c[0], c[1], c[2])) {
        bin_sub<MODE>(a, c[0], c[1], c[2], id[0], id[1], id[2], (unsigned)prim, 0u);
        return;
    }
    CV poly[9];
    int n = clip_polygon(c[0], c[1], c[2], poly);
    for (int i = 1; i + 1 < n; ++i)
        bin_sub<MODE>(a, poly[0].c, poly[i].c, poly[i + 1].c, poly[0].b, poly[i].b, poly[i + 1].b,
                      (unsigned)prim, (unsigned)(i - 1));
}

__device__ __forceinline__ int rec_bins(const BRec& r) {
    return ((r.x1 >> kBinShift) - (r.x0 >> kBinShift) + 1) * ((r.y1 >> kBinShift) - (r.y0 >> kBinShift) + 1);
}

// Block-wide exclusive scan helper (1024 threads); returns the exclusive
// prefix of v and writes the block total to *total.
__device__ __forceinline__ unsigned long long block_scan_1024(unsigned long long v,
                                                             unsigned long long* warp_sums,
                                                             unsigned long long* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
        warp_sums[lane] = w;
    }
    __syncthreads();
    unsigned long long r = (warp == 0 ? 0ull : warp_sums[warp - 1]) + x - v;
    *total = warp_sums[31];
    __syncthreads();
    return r;
}

// Offsets of the big records' bin ranges.  Admission is a prefix (bases
// grow): records whose range ends past the pair capacity are spilled.
__global__ void __launch_bounds__(1024) k_big_scan(BinArgs a) {
    __shared__ unsigned long long warp_sums[32];
    __shared__ unsigned long long admitted;
    const unsigned n = min(a.ctr[1], a.big_cap);
    if (threadIdx.x == 0) admitted = 0;
    unsigned long long carry = 0;
    for (unsigned start = 0; start < n; start += 1024) {
        unsigned i = start + threadIdx.x;
        unsigned long long v = 0;
        if (i < n) v = (unsigned long long)rec_bins(a.recs[a.big_list[i]]);
        unsigned long long tot;
        unsigned long long ex = block_scan_1024(v, warp_sums, &tot);
        if (i < n) {
            unsigned long long base = carry + ex;
            if (base + v <= a.big_pair_cap) {
                a.big_base[i] = base;
                atomicMax(&admitted, base + v);
            } else {
                a.big_base[i] = ~0ull;
                spill_push(a, a.recs[a.big_list[i]].spill_id);
            }
        }
        carry += tot;
    }
    __syncthreads();
    if (threadIdx.x == 0) *reinterpret_cast<unsigned long long*>(a.ctr + 4) = admitted;
}

// Smallest edge-function upper bound test: true if the record may cover a
// pixel centre of the rectangle [px0, px1] x [py0, py1].
__device__ __forceinline__ bool rect_may_cover(const BRec& r, int px0, int px1, int py0, int py1) {
    int64_t cx0 = (int64_t)px0 * kSub + kSub / 2, cx1 = (int64_t)px1 * kSub + kSub / 2;
    int64_t cy0 = (int64_t)py0 * kSub + kSub / 2, cy1 = (int64_t)py1 * kSub + kSub / 2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        int a = (i + 1) % 3, b = (i + 2) % 3;
        int64_t A = (int64_t)r.X[b] - r.X[a], B = (int64_t)r.Y[b] - r.Y[a];
        int64_t ymax = A > 0 ? cy1 : cy0;
        int64_t xmin = B > 0 ? cx0 : cx1;
        if (A * (ymax - r.Y[a]) - B * (xmin - r.X[a]) < 0) return false;
    }
    return true;
}

// Expansion of the admitted big records into (bin, record) pairs: counts
// (FILL = false) or list entries (FILL = true).  Warps take contiguous pair
// ranges and walk the record list.
template <bool FILL>
__global__ void __launch_bounds__(256) k_big_pairs(BinArgs a) {
    const unsigned n = min(a.ctr[1], a.big_cap);
    const unsigned long long total = *reinterpret_cast<const unsigned long long*>(a.ctr + 4);
    if (n == 0 || total == 0) return;
    const unsigned long long nthreads = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long begin = total * t / nthreads, end = total * (t + 1) / nthreads;
    if (begin >= end) return;
    unsigned lo = 0, hi = n - 1;
    while (lo < hi) {
        unsigned mid = (lo + hi + 1) >> 1;
        unsigned long long b = a.big_base[mid];
        if (b != ~0ull && b <= begin) lo = mid;
        else hi = mid - 1;
    }
    unsigned ri = lo;
    unsigned rec_id = a.big_list[ri];
    BRec r = a.recs[rec_id];
    unsigned long long base = a.big_base[ri];
    int cx0 = r.x0 >> kBinShift, cy0 = r.y0 >> kBinShift;
    int ncx = (r.x1 >> kBinShift) - cx0 + 1;
    unsigned long long nb = (unsigned long long)rec_bins(r);
    for (unsigned long long p = begin; p < end; ++p) {
        while (p >= base + nb) {
            ++ri;
            rec_id = a.big_list[ri];
            r = a.recs[rec_id];
            base = a.big_base[ri];
            cx0 = r.x0 >> kBinShift;
            cy0 = r.y0 >> kBinShift;
            ncx = (r.x1 >> kBinShift) - cx0 + 1;
            nb = (unsigned long long)rec_bins(r);
        }
        unsigned local = (unsigned)(p - base);
        int bx = cx0 + (int)(local % (unsigned)ncx), by = cy0 + (int)(local / (unsigned)ncx);
        int px0 = max(bx * kBin, (int)r.x0), px1 = min(bx * kBin + kBin - 1, (int)r.x1);
        int py0 = max(by * kBin, (int)r.y0), py1 = min(by * kBin + kBin - 1, (int)r.y1);
        if (!rect_may_cover(r, px0, px1, py0, py1)) continue;
        unsigned bin = (unsigned)(by * a.nbx + bx);
        if (!FILL) {
            atomicAdd(a.big_count + bin, 1u);
        } else {
            unsigned slot = atomicAdd(a.bin_cursor + bin, 1u);
            a.bin_list[slot] = rec_id;
        }
    }
}

// Exclusive scan of the bin counts into offsets and cursors, and of the
// bins' segment counts into the work-item list (one block).  Empty bins get
// no work item: the target was cleared before the raster.
__global__ void __launch_bounds__(1024) k_bin_scan(BinArgs a) {
    __shared__ unsigned long long warp_sums[32];
    const unsigned nbins = (unsigned)(a.nbx * a.nby);
    unsigned long long carry = 0, icarry = 0;
    for (unsigned start = 0; start < nbins; start += 1024) {
        unsigned i = start + threadIdx.x;
        unsigned small = i < nbins ? a.bin_count[i] : 0u;
        unsigned long long v = i < nbins ? (unsigned long long)small + a.big_count[i] : 0u;
        unsigned long long tot;
        unsigned long long ex = block_scan_1024(v, warp_sums, &tot);
        if (i < nbins) {
            a.bin_offset[i] = (unsigned)(carry + ex);
            a.bin_cursor[i] = (unsigned)(carry + ex) + small;
        }
        carry += tot;
        const unsigned long long nseg = (v + kSeg - 1) / kSeg;
        unsigned long long itot;
        unsigned long long iex = block_scan_1024(nseg, warp_sums, &itot);
        for (unsigned long long k = 0; k < nseg; ++k) {
            unsigned long long slot = icarry + iex + k;
            if (slot < a.item_cap) a.items[slot] = i | ((unsigned)k << kItemBinBits);
        }
        icarry += itot;
    }
    if (threadIdx.x == 0) {
        a.bin_offset[nbins] = (unsigned)carry;
        a.ctr[6] = (unsigned)min(icarry, (unsigned long long)a.item_cap);
        if (icarry > a.item_cap) atomicOr(a.ctr + 3, 2u);
    }
}

// Scatter of the small records into their (at most four) bins, at the
// ranks the setup kernel drew from the bin counters (no atomics here).
__global__ void __launch_bounds__(256) k_bin_fill_small(BinArgs a) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned n = min(a.ctr[0], a.rec_cap);
    if (i >= n) return;
    // the last 16 bytes of the record hold the bounding box and the flags
    const uint4 tail = __ldg(reinterpret_cast<const uint4*>(a.recs + i) + 3);
    const unsigned flags = tail.z;
    if (flags & kFlagBig) return;
    const int x0 = (int)(tail.x & 0xFFFFu), x1 = (int)(tail.x >> 16);
    const int y0 = (int)(tail.y & 0xFFFFu), y1 = (int)(tail.y >> 16);
    const int cx0 = x0 >> kBinShift, cx1 = x1 >> kBinShift;
    const int cy0 = y0 >> kBinShift, cy1 = y1 >> kBinShift;
    int k = 0;
    for (int by = cy0; by <= cy1; ++by)
        for (int bx = cx0; bx <= cx1; ++bx, ++k) {
            const unsigned bin = (unsigned)(by * a.nbx + bx);
            a.bin_list[a.bin_offset[bin] + a.ranks[4 * (size_t)i + k]] = i;
        }
}

template <int MODE>
struct BinVal;
template <>
struct BinVal<MODE_DEPTH> {
    typedef unsigned T;
};
template <>
struct BinVal<MODE_VKEY> {
    typedef unsigned long long T;
};
template <>
struct BinVal<MODE_STENCIL> {
    typedef int T;
};

// Fragment update of one bin pixel (index t in the 32 x 32 tile).
template <int MODE, typename V>
__device__ __forceinline__ void bin_frag(const BinArgs& a, V* tile, const float* dtile, int t,
                                         const BRec& r, float fe1, float fe2) {
    const float l1 = fe1 * r.inv_area;
    const float l2 = fe2 * r.inv_area;
    float z = r.z0 + (l1 * r.dz1 + l2 * r.dz2);
    if (MODE == MODE_DEPTH) {
        z = clamp01(z + r.zoff);
        if (z < 1.0f) atomicMin(reinterpret_cast<unsigned*>(&tile[t]), __float_as_uint(z));
    } else if (MODE == MODE_VKEY) {
        z = clamp01(z);
        if (z < 1.0f)
            atomicMin(reinterpret_cast<unsigned long long*>(&tile[t]),
                      ((unsigned long long)__float_as_uint(z) << 32) | r.prim);
    } else {
        z = clamp01(z);
        const float d = dtile[t];
        const bool pass = a.r.depth_func == GI_DEPTH_LEQUAL ? (z <= d) : (z < d);
        if (pass) atomicAdd(reinterpret_cast<int*>(&tile[t]), (r.flags & kFlagFront) ? 1 : -1);
    }
}

// One CTA per work item (a bin, or a 256-record segment of a heavy bin).
// The bin's 32 x 32 values live in shared memory.  Records are staged and
// sorted by their coverage of the bin: those covering more than 256 pixels
// are swept by the whole CTA (thread = column, 4 rows apart by 8,
// incremental edge values), the others one record per warp with the lanes
// over the record's bounding box clipped to the bin.  Shared-memory
// atomicMin / atomicAdd merge overlaps, so the order does not matter.  A
// single-segment bin stores its tile; the segments of a heavy bin merge
// theirs into the cleared target with global atomics.
template <int MODE>
__global__ void __launch_bounds__(256) k_bin_raster(BinArgs a) {
    typedef typename BinVal<MODE>::T V;
    __shared__ BRec srec[kSeg];
    __shared__ V tile[kBin * kBin];
    __shared__ float dtile[MODE == MODE_STENCIL ? kBin * kBin : 1];
    __shared__ float recip[kBin + 1];
    __shared__ unsigned short s_small[kSeg], s_big[kSeg];
    __shared__ int n_small, n_big;
    if (blockIdx.x >= a.ctr[6]) return;
    const unsigned item = a.items[blockIdx.x];
    const int bin = (int)(item & ((1u << kItemBinBits) - 1));
    const unsigned seg = item >> kItemBinBits;
    const int bx = bin % a.nbx, by = bin / a.nbx;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ox = bx * kBin, oy = by * kBin;
    const unsigned bbegin = a.bin_offset[bin], bend = a.bin_offset[bin + 1];
    const bool multi = bend - bbegin > kSeg;
    const unsigned begin = bbegin + seg * kSeg, end = min(bend, begin + kSeg);
    if (threadIdx.x <= kBin) recip[threadIdx.x] = threadIdx.x ? 1.0f / (float)threadIdx.x : 0.0f;
    if (threadIdx.x == 0) {
        n_small = 0;
        n_big = 0;
    }
    const V clearv = MODE == MODE_DEPTH ? (V)0x3f800000u
                     : MODE == MODE_VKEY ? (V)(((unsigned long long)0x3f800000u << 32) | 0xFFFFFFFFull)
                                         : (V)0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = threadIdx.x + 256 * k;
        tile[i] = clearv;
        if (MODE == MODE_STENCIL) {
            const int x = ox + (i & (kBin - 1)), y = oy + (i >> kBinShift);
            dtile[i] = (x < a.r.W && y < a.r.H) ? __uint_as_float(__ldg(a.r.depth + (size_t)y * a.r.W + x))
                                                 : 1.0f;
        }
    }
    __syncthreads();
    const unsigned cnt = end - begin;
    if (threadIdx.x < cnt) {
        const uint4* src = reinterpret_cast<const uint4*>(a.recs + a.bin_list[begin + threadIdx.x]);
        uint4* dst = reinterpret_cast<uint4*>(srec + threadIdx.x);
        uint4 q3 = __ldg(src + 3);
        dst[0] = __ldg(src + 0);
        dst[1] = __ldg(src + 1);
        dst[2] = __ldg(src + 2);
        dst[3] = q3;
        const int x0 = max((int)(q3.x & 0xFFFFu), ox), x1 = min((int)(q3.x >> 16), ox + kBin - 1);
        const int y0 = max((int)(q3.y & 0xFFFFu), oy), y1 = min((int)(q3.y >> 16), oy + kBin - 1);
        if (x0 <= x1 && y0 <= y1) {
            const int n = (x1 - x0 + 1) * (y1 - y0 + 1);
            if (n > 256) s_big[atomicAdd(&n_big, 1)] = (unsigned short)threadIdx.x;
            else s_small[atomicAdd(&n_small, 1)] = (unsigned short)threadIdx.x;
        }
    }
    __syncthreads();
    // -- records covering most of the bin: the whole CTA, one column each
    const int col = threadIdx.x & (kBin - 1), row0 = threadIdx.x >> kBinShift;  // rows row0 + 8k
    const int x = ox + col;
    const int64_t px = (int64_t)x * kSub + kSub / 2;
    for (int b = 0; b < n_big; ++b) {
        const BRec& r = srec[s_big[b]];
        int64_t A[3], E[3];
        bool tl[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int ia = (i + 1) % 3, ib = (i + 2) % 3;
            A[i] = (int64_t)r.X[ib] - r.X[ia];
            const int64_t B = (int64_t)r.Y[ib] - r.Y[ia];
            tl[i] = (B < 0) || (B == 0 && A[i] < 0);
            const int64_t py = (int64_t)(oy + row0) * kSub + kSub / 2;
            E[i] = A[i] * (py - r.Y[ia]) - B * (px - r.X[ia]) - tl_bias(tl[i]);
        }
        const bool colin = x >= (int)r.x0 && x <= (int)r.x1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int y = oy + row0 + 8 * k;
            const bool in = colin && y >= (int)r.y0 && y <= (int)r.y1 && inside_biased(E);
            if (in)
                bin_frag<MODE>(a, tile, dtile, (row0 + 8 * k) * kBin + col, r, i2f(E[1] + tl_bias(tl[1])),
                               i2f(E[2] + tl_bias(tl[2])));
#pragma unroll
            for (int i = 0; i < 3; ++i) E[i] += A[i] * (8 * kSub);
        }
    }
    // -- the other records: one per warp
    for (int j = warp; j < n_small; j += 8) {
        const BRec& r = srec[s_small[j]];
        const int x0 = max((int)r.x0, ox), x1 = min((int)r.x1, ox + kBin - 1);
        const int y0 = max((int)r.y0, oy), y1 = min((int)r.y1, oy + kBin - 1);
        const int w = x1 - x0 + 1, n = w * (y1 - y0 + 1);
        const float inv_w = recip[w];
        const int64_t cx = (int64_t)x0 * kSub + kSub / 2, cy = (int64_t)y0 * kSub + kSub / 2;
        int64_t A[3], B[3], E0[3];
        bool tl[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int ia = (i + 1) % 3, ib = (i + 2) % 3;
            A[i] = (int64_t)r.X[ib] - r.X[ia];
            B[i] = (int64_t)r.Y[ib] - r.Y[ia];
            tl[i] = (B[i] < 0) || (B[i] == 0 && A[i] < 0);
            E0[i] = A[i] * (cy - r.Y[ia]) - B[i] * (cx - r.X[ia]);
        }
        // Small triangles: every edge value over the bin fits in 32 bits
        // (|A|, |B| <= 2^13 and the bin spans 2^13 sub-pixels), so the same
        // integers are formed with 32-bit arithmetic.
        const bool small = max(max(abs(A[0]), abs(A[1])), abs(A[2])) <= 8192 &&
                           max(max(abs(B[0]), abs(B[1])), abs(B[2])) <= 8192 &&
                           abs(E0[0]) < (1LL << 28) && abs(E0[1]) < (1LL << 28) && abs(E0[2]) < (1LL << 28);
        for (int p = lane; p < n; p += 32) {
            // p / w by a reciprocal: exact because (p + 1/2) / w is never
            // within 2^-11 of an integer for p < 1024, w <= 32.
            const int dy = (int)(((float)p + 0.5f) * inv_w);
            const int dx = p - dy * w;
            bool in;
            float fe1, fe2;
            if (small) {
                int e[3];
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    e[i] = (int)E0[i] + (int)A[i] * (dy << kSubBits) - (int)B[i] * (dx << kSubBits) - tl_bias(tl[i]);
                in = (e[0] | e[1] | e[2]) >= 0;
                fe1 = (float)(e[1] + tl_bias(tl[1]));
                fe2 = (float)(e[2] + tl_bias(tl[2]));
            } else {
                int64_t E[3];
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    E[i] = E0[i] + A[i] * (int64_t)(dy << kSubBits) - B[i] * (int64_t)(dx << kSubBits) - tl_bias(tl[i]);
                in = inside_biased(E);
                fe1 = i2f(E[1] + tl_bias(tl[1]));
                fe2 = i2f(E[2] + tl_bias(tl[2]));
            }
            if (in) bin_frag<MODE>(a, tile, dtile, (y0 + dy - oy) * kBin + (x0 + dx - ox), r, fe1, fe2);
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = threadIdx.x + 256 * k;
        const int xx = ox + (i & (kBin - 1)), y = oy + (i >> kBinShift);
        if (xx >= a.r.W || y >= a.r.H) continue;
        const size_t idx = (size_t)y * a.r.W + xx;
        const V v = tile[i];
        if (!multi) {
            if (MODE == MODE_DEPTH) a.r.depth[idx] = (unsigned)v;
            else if (MODE == MODE_VKEY) a.r.keys[idx] = (unsigned long long)v;
            else a.r.counts[idx] = (int)v;
        } else if (v != clearv) {
            if (MODE == MODE_DEPTH) atomicMin(a.r.depth + idx, (unsigned)v);
            else if (MODE == MODE_VKEY) atomicMin(a.r.keys + idx, (unsigned long long)v);
            else atomicAdd(a.r.counts + idx, (int)v);
        }
    }
}

// ---- stencil slivers ------------------------------------------------------
// Extruded shadow-volume sides are long, thin triangles whose bounding boxes
// cover most of the screen.  Every stencil record spanning more than four
// bins is drawn here instead of through bin pairs: one warp per triangle,
// lanes over rows.  On a row the covered pixel centres form one interval;
// each edge bounds it by floor((K - c) / (B * 256)), tracked exactly from
// row to row with an integer quotient / remainder step, so the interval is
// the set of pixels the per-pixel inside test accepts (each pixel is still
// tested before its update).  Counts are added with global atomics after
// k_bin_raster (sums commute with its stores and atomics).
struct FloorTrack {
    int64_t q, rem, den, dq, dr;
    __device__ __forceinline__ static int64_t fdiv(int64_t a, int64_t b) {  // b > 0
        int64_t q = a / b;
        if (a % b != 0 && a < 0) --q;
        return q;
    }
    // floor(v / d) for 0 <= v < 64 d (a small quotient): float estimate,
    // then exact integer correction
    __device__ __forceinline__ static int64_t small_quot(int64_t v, int64_t d) {
        int64_t c = (int64_t)((float)v / (float)d);
        if (c < 0) c = 0;
        for (int it = 0; it < 4 && c * d > v; ++it) --c;
        for (int it = 0; it < 4 && (c + 1) * d <= v; ++it) ++c;
        return c;
    }
    __device__ __forceinline__ void step() {
        q += dq;
        rem += dr;
        if (rem >= den) {
            rem -= den;
            ++q;
        }
    }
};

__global__ void __launch_bounds__(256) k_sliver(BinArgs a) {
    const unsigned n = min(a.ctr[1], a.big_cap);
    const int lane = threadIdx.x & 31;
    const unsigned nwarps = gridDim.x * (blockDim.x >> 5);
    for (unsigned i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nwarps) {
        const BRec r = a.recs[a.big_list[i]];
        int64_t A[3], B[3], XA[3], YA[3];
        bool tl[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int ia = (k + 1) % 3, ib = (k + 2) % 3;
            A[k] = (int64_t)r.X[ib] - r.X[ia];
            B[k] = (int64_t)r.Y[ib] - r.Y[ia];
            tl[k] = (B[k] < 0) || (B[k] == 0 && A[k] < 0);
            XA[k] = r.X[ia];
            YA[k] = r.Y[ia];
        }
        // every lane takes part in the shuffles below; lanes past the last
        // row simply run no row iterations
        const int y_first = (int)r.y0 + lane;
        // edge k at row y: E(x) = K - B * (x * 256 + 128), K = A * (py - Ya) + B * Xa.
        // The bound of edge k is floor(num / den) with num linear in the row;
        // the warp computes the row-y0 quotients and the one-row steps with
        // one 64-bit division per lane (lanes 0-5), shares them, and each
        // lane derives its own first row (y0 + lane) and its 32-row step
        // with small exact quotients.
        FloorTrack f[3];
        int64_t K0[3];
        const int64_t py0 = (int64_t)y_first * kSub + kSub / 2;
        int64_t num_b[3], den[3], step1[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int64_t base_py = (int64_t)r.y0 * kSub + kSub / 2;
            const int64_t Kb = A[k] * (base_py - YA[k]) + B[k] * XA[k];
            const int64_t dK = A[k] * (int64_t)kSub;
            K0[k] = A[k] * (py0 - YA[k]) + B[k] * XA[k];
            if (B[k] > 0) {
                num_b[k] = Kb - B[k] * (kSub / 2) - tl_bias(tl[k]);
                den[k] = B[k] * kSub;
                step1[k] = dK;
            } else if (B[k] < 0) {
                const int64_t Bp = -B[k];
                den[k] = Bp * kSub;
                num_b[k] = tl[k] ? Kb + Bp * (kSub / 2) : -Kb - Bp * (kSub / 2);
                step1[k] = tl[k] ? dK : -dK;
            } else {
                num_b[k] = 0;
                den[k] = 1;
                step1[k] = 0;
            }
        }
        // lanes 0-2: floor(num_b / den); lanes 3-5: floor(step1 / den)
        int64_t mine = 0;
        if (lane < 6) {
            const int k = lane % 3;
            mine = FloorTrack::fdiv(lane < 3 ? num_b[k] : step1[k], den[k]);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int64_t q0 = __shfl_sync(0xffffffffu, mine, k);
            const int64_t dq1 = __shfl_sync(0xffffffffu, mine, 3 + k);
            if (B[k] == 0) continue;
            const int64_t rem0 = num_b[k] - q0 * den[k];
            const int64_t dr1 = step1[k] - dq1 * den[k];
            // row y0 + lane
            const int64_t v = rem0 + (int64_t)lane * dr1;
            const int64_t c = FloorTrack::small_quot(v, den[k]);
            f[k].den = den[k];
            f[k].q = q0 + (int64_t)lane * dq1 + c;
            f[k].rem = v - c * den[k];
            // 32-row step
            const int64_t v32 = 32 * dr1;
            const int64_t c32 = FloorTrack::small_quot(v32, den[k]);
            f[k].dq = 32 * dq1 + c32;
            f[k].dr = v32 - c32 * den[k];
        }
        const float sgn_front = (r.flags & kFlagFront) ? 1.0f : -1.0f;
        const int inc = sgn_front > 0.0f ? 1 : -1;
        for (int y = y_first, it = 0; y <= (int)r.y1; y += 32, ++it) {
            if (it > 0) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    K0[k] += A[k] * (int64_t)(32 * kSub);
                    if (B[k] != 0) f[k].step();
                }
            }
            int lo = r.x0, hi = r.x1;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (B[k] == 0) {
                    if (!(K0[k] > 0 || (K0[k] == 0 && tl[k]))) hi = lo - 1;
                } else if (B[k] > 0) {
                    if (f[k].q < (int64_t)hi) hi = (int)max(f[k].q, (int64_t)lo - 1);
                } else {
                    const int64_t xm = tl[k] ? -f[k].q : f[k].q + 1;
                    if (xm > (int64_t)lo) lo = (int)min(xm, (int64_t)hi + 1);
                }
            }
            const int64_t py = (int64_t)y * kSub + kSub / 2;
            for (int x = lo; x <= hi; ++x) {
                const int64_t px = (int64_t)x * kSub + kSub / 2;
                int64_t E[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) E[k] = A[k] * (py - YA[k]) - B[k] * (px - XA[k]) - tl_bias(tl[k]);
                if (!inside_biased(E)) continue;
                const float l1 = i2f(E[1] + tl_bias(tl[1])) * r.inv_area, l2 = i2f(E[2] + tl_bias(tl[2])) * r.inv_area;
                const float z = clamp01(r.z0 + (l1 * r.dz1 + l2 * r.dz2));
                const size_t idx = (size_t)y * a.r.W + x;
                const float d = __uint_as_float(__ldg(a.r.depth + idx));
                const bool pass = a.r.depth_func == GI_DEPTH_LEQUAL ? (z <= d) : (z < d);
                if (pass) atomicAdd(a.r.counts + idx, inc);
            }
        }
    }
}

// Spilled sub-triangles: re-derived from (primitive, sub) and rasterised by
// one thread each with global atomics after k_bin_raster.
template <int MODE>
__global__ void __launch_bounds__(128) k_spill(BinArgs a) {
    const unsigned n = min(a.ctr[2], a.spill_cap);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned id = a.spill[i];
        const int prim = (int)(id >> 3), sub = (int)(id & 7);
        float v[3][3];
        prim_vertices<MODE>(a.r, prim, v);
        float c[3][4];
#pragma unroll
        for (int j = 0; j < 3; ++j) transform(a.r.mvp, v[j][0], v[j][1], v[j][2], c[j]);
        const float idm[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
        Setup s;
        bool ok;
        if (all_inside(c[0], c[1], c[2])) {
            ok = sub == 0 && setup_triangle(c[0], c[1], c[2], idm[0], idm[1], idm[2], a.r.W, a.r.H, s);
        } else {
            CV poly[9];
            int np = clip_polygon(c[0], c[1], c[2], poly);
            ok = (sub + 2 < np) && setup_triangle(poly[0].c, poly[sub + 1].c, poly[sub + 2].c, poly[0].b,
                                                  poly[sub + 1].b, poly[sub + 2].b, a.r.W, a.r.H, s);
        }
        if (!ok) continue;
        int64_t minX = min(s.X[0], min(s.X[1], s.X[2])), maxX = max(s.X[0], max(s.X[1], s.X[2]));
        int64_t minY = min(s.Y[0], min(s.Y[1], s.Y[2])), maxY = max(s.Y[0], max(s.Y[1], s.Y[2]));
        int x0 = (int)max((int64_t)0, -((-(minX - kSub / 2)) >> kSubBits));
        int x1 = (int)min((int64_t)a.r.W - 1, (maxX - kSub / 2) >> kSubBits);
        int y0 = (int)max((int64_t)0, -((-(minY - kSub / 2)) >> kSubBits));
        int y1 = (int)min((int64_t)a.r.H - 1, (maxY - kSub / 2) >> kSubBits);
        if (x0 > x1 || y0 > y1) continue;
        float zoff = 0.0f;
        if (MODE == MODE_DEPTH) {
            if (a.r.bias_mode == GI_BIAS_POLYGON_OFFSET) zoff = polygon_offset(s, a.r.factor, a.r.units);
            else if (a.r.bias_mode == GI_BIAS_CONSTANT) zoff = a.r.cbias;
        }
        Edges e;
        make_edges(s, e);
        raster_small<MODE>(a.r, s, e, x0, x1, y0, y1, zoff, MODE == MODE_VKEY ? id : (unsigned)prim);
    }
}


// ===========================================================================
// Tiered rasteriser (light map and G-buffer)
//
// k_tier_setup turns every primitive into sub-triangle records and sorts
// them by pixel bounding box: tiny (<= 16 pixels), warp-sized (<= 1024) and
// large.  k_large_scan picks up to eight "huge" records (bounding box of at
// least an eighth of the image, e.g. a ground plane) and scans the 16 x 16
// tile counts of the other large ones.  k_base then evaluates the huge
// records at every pixel and writes the target with plain stores (this is
// also the clear).  Last, tiny records (one thread each), warp-sized records
// (one warp each, lanes over the bounding box) and large records (one warp
// per 16 x 16 tile) merge into the target with global atomicMin; the result
// is the same in any order.
// ===========================================================================
constexpr int kHugeMax = 8;

struct TierArgs {
    RasterArgs r;
    BRec* recs;
    unsigned rec_cap;
    unsigned* tiny;
    unsigned* coop;
    unsigned* large;
    unsigned long long* large_base;
    unsigned* spill;
    unsigned spill_cap;
    unsigned long long huge_px;  // bounding-box pixels that make a record huge
    int tiny_px, coop_px;        // tier thresholds (bounding-box pixels; coop_px <= 1024)
    unsigned* rec_of;            // G-buffer: triangle -> record of its unclipped triangle (~0: none)
    uint4* rres;                 // G-buffer: per record (1/w0, 1/w1, 1/w2 bits, swapped)
    unsigned* ctr;  // [0] records [1] tiny [2] coop [3] large [4] spills [5] error bits
                    // [6] huge count [8,9] tile total (u64) [16..23] huge record ids
};

__device__ __forceinline__ void tier_spill(const TierArgs& a, unsigned id) {
    unsigned s = atomicAdd(a.ctr + 4, 1u);
    if (s < a.spill_cap) a.spill[s] = id;
    else atomicOr(a.ctr + 5, 1u);
}

template <int MODE>
__device__ void tier_sub(const TierArgs& a, const float* c0, const float* c1, const float* c2,
                         const float* b0, const float* b1, const float* b2, unsigned prim,
                         unsigned sub, bool unclipped) {
    Setup s;
    if (!setup_triangle(c0, c1, c2, b0, b1, b2, a.r.W, a.r.H, s)) return;
    int64_t minX = min(s.X[0], min(s.X[1], s.X[2])), maxX = max(s.X[0], max(s.X[1], s.X[2]));
    int64_t minY = min(s.Y[0], min(s.Y[1], s.Y[2])), maxY = max(s.Y[0], max(s.Y[1], s.Y[2]));
    int x0 = (int)max((int64_t)0, -((-(minX - kSub / 2)) >> kSubBits));
    int x1 = (int)min((int64_t)a.r.W - 1, (maxX - kSub / 2) >> kSubBits);
    int y0 = (int)max((int64_t)0, -((-(minY - kSub / 2)) >> kSubBits));
    int y1 = (int)min((int64_t)a.r.H - 1, (maxY - kSub / 2) >> kSubBits);
    if (x0 > x1 || y0 > y1) return;
    const unsigned spill_id = (prim << 3) | sub;
    unsigned slot = atomicAdd(a.ctr + 0, 1u);
    if (slot >= a.rec_cap) {
        tier_spill(a, spill_id);
        return;
    }
    float zoff = 0.0f;
    if (MODE == MODE_DEPTH) {
        if (a.r.bias_mode == GI_BIAS_POLYGON_OFFSET) zoff = polygon_offset(s, a.r.factor, a.r.units);
        else if (a.r.bias_mode == GI_BIAS_CONSTANT) zoff = a.r.cbias;
    }
    BRec r;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        r.X[i] = (int)s.X[i];
        r.Y[i] = (int)s.Y[i];
    }
    r.z0 = s.z[0];
    r.dz1 = s.z[1] - s.z[0];
    r.dz2 = s.z[2] - s.z[0];
    r.inv_area = s.inv_area;
    r.zoff = zoff;
    r.prim = MODE == MODE_VKEY ? spill_id : prim;
    r.x0 = (unsigned short)x0;
    r.x1 = (unsigned short)x1;
    r.y0 = (unsigned short)y0;
    r.y1 = (unsigned short)y1;
    r.flags = s.front ? kFlagFront : 0u;
    r.spill_id = spill_id;
    a.recs[slot] = r;
    if (MODE == MODE_VKEY && a.rec_of) {
        a.rres[slot] = make_uint4(__float_as_uint(s.iw[0]), __float_as_uint(s.iw[1]),
                                  __float_as_uint(s.iw[2]), s.swapped ? 1u : 0u);
        if (unclipped) a.rec_of[prim] = slot;
    }
    const long long npx = (long long)(x1 - x0 + 1) * (y1 - y0 + 1);
    if (npx <= a.tiny_px) a.tiny[atomicAdd(a.ctr + 1, 1u)] = slot;
    else if (npx <= a.coop_px) a.coop[atomicAdd(a.ctr + 2, 1u)] = slot;
    else a.large[atomicAdd(a.ctr + 3, 1u)] = slot;
}

template <int MODE>
__global__ void __launch_bounds__(128) k_tier_setup(TierArgs a) {
    pdl_enter();
    int prim = blockIdx.x * blockDim.x + threadIdx.x;
    if (prim >= a.r.num_prims) return;
    float v[3][3];
    prim_vertices<MODE>(a.r, prim, v);
    float c[3][4];
#pragma unroll
    for (int j = 0; j < 3; ++j) transform(a.r.mvp, v[j][0], v[j][1], v[j][2], c[j]);
    const float id[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
    // The G-buffer resolve reads an unclipped triangle's record through
    // rec_of; every other triangle is marked and resolved from scratch.
    if (MODE == MODE_VKEY && a.rec_of) a.rec_of[prim] = ~0u;
    if (all_inside(c[0], c[1], c[2])) {
        tier_sub<MODE>(a, c[0], c[1], c[2], id[0], id[1], id[2], (unsigned)prim, 0u, true);
        return;
    }
    CV poly[9];
    int n = clip_polygon(c[0], c[1], c[2], poly);
    for (int i = 1; i + 1 < n; ++i)
        tier_sub<MODE>(a, poly[0].c, poly[i].c, poly[i + 1].c, poly[0].b, poly[i].b, poly[i + 1].b,
                       (unsigned)prim, (unsigned)(i - 1), false);
}

constexpr unsigned kFlagHuge = 4u;

// 16 x 16 tiles of a large record's bounding box (0 for the huge ones,
// which k_base draws).
__device__ __forceinline__ unsigned long long rec_tiles(const BRec& r) {
    if (r.flags & kFlagHuge) return 0;
    return (unsigned long long)((r.x1 / kTile) - (r.x0 / kTile) + 1) * ((r.y1 / kTile) - (r.y0 / kTile) + 1);
}

// Picks the huge records and scans the 16 x 16 tile counts of the others
// (bases are non-decreasing; huge records get an empty range).
__global__ void __launch_bounds__(1024) k_large_scan(TierArgs a) {
    __shared__ unsigned long long warp_sums[32];
    __shared__ int nhuge;
    pdl_enter();
    const unsigned n = a.ctr[3];
    if (threadIdx.x == 0) nhuge = 0;
    __syncthreads();
    unsigned long long carry = 0;
    for (unsigned start = 0; start < n; start += 1024) {
        unsigned i = start + threadIdx.x;
        unsigned long long v = 0;
        if (i < n) {
            BRec* rp = a.recs + a.large[i];
            const BRec r = *rp;
            const unsigned long long npx = (unsigned long long)(r.x1 - r.x0 + 1) * (r.y1 - r.y0 + 1);
            bool huge = false;
            if (npx >= a.huge_px) {
                const int h = atomicAdd(&nhuge, 1);
                if (h < kHugeMax) {
                    a.ctr[16 + h] = a.large[i];
                    rp->flags = r.flags | kFlagHuge;
                    huge = true;
                }
            }
            if (!huge) v = (unsigned long long)((r.x1 / kTile) - (r.x0 / kTile) + 1) * ((r.y1 / kTile) - (r.y0 / kTile) + 1);
        }
        unsigned long long tot;
        unsigned long long ex = block_scan_1024(v, warp_sums, &tot);
        if (i < n) a.large_base[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        a.ctr[6] = (unsigned)min(nhuge, kHugeMax);
        *reinterpret_cast<unsigned long long*>(a.ctr + 8) = carry;
    }
}

// Huge records at every pixel; writes the target (and so clears it).  A
// thread owns kBaseRows rows of one column, so a record's 64-bit edge set-up
// is shared by that many texels; the rows after the first step the edges by
// exact integer adds.  Measured on the pcss_1080p frame (2048^2 map, 1920 x
// 1080 keys; depth / key rows per thread): 4 / 4 -> 8 / 8 took the light-map
// pass 0.071 -> 0.066 ms; 16 / 8, 16 / 16 and 32 / 8 were slower (more
// registers, fewer resident blocks).
constexpr int kBaseRows = 8;

template <int MODE>
__global__ void __launch_bounds__(256) k_base(TierArgs a) {
    typedef typename BinVal<MODE>::T V;
    __shared__ BRec hr[kHugeMax];
    pdl_enter();
    const int nh = (int)a.ctr[6];
    if (threadIdx.x < nh) hr[threadIdx.x] = a.recs[a.ctr[16 + threadIdx.x]];
    __syncthreads();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int yb = (blockIdx.y * 8 + (threadIdx.x >> 5)) * kBaseRows;
    if (x >= a.r.W) return;
    const V clearv = MODE == MODE_DEPTH ? (V)0x3f800000u
                                        : (V)(((unsigned long long)0x3f800000u << 32) | 0xFFFFFFFFull);
    V val[kBaseRows];
#pragma unroll
    for (int k = 0; k < kBaseRows; ++k) val[k] = clearv;
    const int64_t px = (int64_t)x * kSub + kSub / 2;
    for (int h = 0; h < nh; ++h) {
        const BRec& r = hr[h];
        if (x < (int)r.x0 || x > (int)r.x1) continue;
        // Edge values carry the top-left bias (-1 where the edge does not
        // own its boundary): inside exactly when no high word is negative.
        int64_t A[3], E[3];
        int bias[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int ia = (i + 1) % 3, ib = (i + 2) % 3;
            A[i] = (int64_t)r.X[ib] - r.X[ia];
            const int64_t B = (int64_t)r.Y[ib] - r.Y[ia];
            bias[i] = tl_bias((B < 0) || (B == 0 && A[i] < 0));
            E[i] = A[i] * ((int64_t)yb * kSub + kSub / 2 - r.Y[ia]) - B * (px - r.X[ia]) - bias[i];
        }
#pragma unroll
        for (int k = 0; k < kBaseRows; ++k) {
            const int y = yb + k;
            const bool in = y >= (int)r.y0 && y <= (int)r.y1 && inside_biased(E);
            if (in) {
                const float l1 = i2f(E[1] + bias[1]) * r.inv_area, l2 = i2f(E[2] + bias[2]) * r.inv_area;
                float z = r.z0 + (l1 * r.dz1 + l2 * r.dz2);
                if (MODE == MODE_DEPTH) {
                    z = clamp01(z + r.zoff);
                    if (z < 1.0f && __float_as_uint(z) < (unsigned)val[k]) val[k] = __float_as_uint(z);
                } else {
                    z = clamp01(z);
                    if (z < 1.0f) {
                        const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | r.prim;
                        if (key < (unsigned long long)val[k]) val[k] = key;
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) E[i] += A[i] * kSub;
        }
    }
#pragma unroll
    for (int k = 0; k < kBaseRows; ++k) {
        const int y = yb + k;
        if (y >= a.r.H) break;
        const size_t idx = (size_t)y * a.r.W + x;
        if (MODE == MODE_DEPTH) a.r.depth[idx] = (unsigned)val[k];
        else a.r.keys[idx] = (unsigned long long)val[k];
    }
}

__device__ __forceinline__ void rec_edges(const BRec& r, int64_t A[3], int64_t B[3], bool tl[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int ia = (i + 1) % 3, ib = (i + 2) % 3;
        A[i] = (int64_t)r.X[ib] - r.X[ia];
        B[i] = (int64_t)r.Y[ib] - r.Y[ia];
        tl[i] = (B[i] < 0) || (B[i] == 0 && A[i] < 0);
    }
}

template <int MODE>
__device__ __forceinline__ void rec_emit(const TierArgs& a, const BRec& r, int x, int y, float fe1, float fe2) {
    const float l1 = fe1 * r.inv_area, l2 = fe2 * r.inv_area;
    const float z = r.z0 + (l1 * r.dz1 + l2 * r.dz2);
    emit<MODE>(a.r, x, y, z, r.zoff, r.prim, (r.flags & kFlagFront) != 0);
}

// Tiny records: one thread each over the bounding box.
template <int MODE>
__device__ __forceinline__ void tiny_record(const TierArgs& a, unsigned i) {
    const BRec r = a.recs[a.tiny[i]];
    int64_t A[3], B[3];
    bool tl[3];
    rec_edges(r, A, B, tl);
    // When every edge value over the box fits 32 bits (the usual case: a
    // vertex far in the guard band is what breaks it), step the edges
    // incrementally in int32: +A kSub per row, -B kSub per column.  The
    // values are the same integers, so the tests and conversions are too.
    {
        const int w = r.x1 - r.x0 + 1, h = r.y1 - r.y0 + 1;
        const int64_t cx = (int64_t)r.x0 * kSub + kSub / 2, cy = (int64_t)r.y0 * kSub + kSub / 2;
        int64_t E0[3];
        bool fits32 = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int ia = (k + 1) % 3;
            E0[k] = A[k] * (cy - r.Y[ia]) - B[k] * (cx - r.X[ia]);
            const int64_t bound =
                abs(E0[k]) + abs(A[k]) * (int64_t)(h - 1) * kSub + abs(B[k]) * (int64_t)(w - 1) * kSub;
            fits32 &= bound < (1LL << 31);
        }
        if (fits32) {
            // the steps are only added when the box has a next row / column,
            // and then they are bounded by `bound` too
            // The edges carry the top-left bias (-1 on an edge that does not
            // own its boundary), so a pixel is inside exactly when no biased
            // value is negative: one OR of the three and a sign test.
            int er[3], sa[3], sb[3];
            const int b1 = tl[1] ? 0 : 1, b2 = tl[2] ? 0 : 1;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                er[k] = (int)E0[k] - tl_bias(tl[k]);
                sa[k] = h > 1 ? (int)(A[k] * kSub) : 0;
                sb[k] = w > 1 ? (int)(B[k] * kSub) : 0;
            }
            for (int y = r.y0;; ++y) {
                int e0 = er[0], e1 = er[1], e2 = er[2];
                for (int x = r.x0;; ++x) {
                    if ((e0 | e1 | e2) >= 0) rec_emit<MODE>(a, r, x, y, (float)(e1 + b1), (float)(e2 + b2));
                    if (x == (int)r.x1) break;  // no step past the box: it could leave 32 bits
                    e0 -= sb[0];
                    e1 -= sb[1];
                    e2 -= sb[2];
                }
                if (y == (int)r.y1) break;
                er[0] += sa[0];
                er[1] += sa[1];
                er[2] += sa[2];
            }
            return;
        }
    }
    for (int y = r.y0; y <= (int)r.y1; ++y) {
        const int64_t py = (int64_t)y * kSub + kSub / 2;
        for (int x = r.x0; x <= (int)r.x1; ++x) {
            const int64_t px = (int64_t)x * kSub + kSub / 2;
            int64_t E[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int ia = (k + 1) % 3;
                E[k] = A[k] * (py - r.Y[ia]) - B[k] * (px - r.X[ia]);
            }
            const bool in = (E[0] > 0 || (E[0] == 0 && tl[0])) && (E[1] > 0 || (E[1] == 0 && tl[1])) &&
                            (E[2] > 0 || (E[2] == 0 && tl[2]));
            if (in) rec_emit<MODE>(a, r, x, y, i2f(E[1]), i2f(E[2]));
        }
    }
}

// Warp-sized records: one warp per record, lanes over the bounding box.
template <int MODE>
__device__ __forceinline__ void coop_record(const TierArgs& a, unsigned i, int lane) {
    const BRec r = a.recs[a.coop[i]];
    const int w = r.x1 - r.x0 + 1, h = r.y1 - r.y0 + 1, npx = w * h;
    // p / w by a reciprocal: (p + 1/2) / w stays at least 1/(2w) >= 2^-11
    // from an integer and the product errs by under 2^-13 for p < 1024.
    const float inv_w = 1.0f / (float)w;
    int64_t A[3], B[3], E0[3];
    bool tl[3];
    rec_edges(r, A, B, tl);
    const int64_t cx = (int64_t)r.x0 * kSub + kSub / 2, cy = (int64_t)r.y0 * kSub + kSub / 2;
    bool fits32 = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int ia = (k + 1) % 3;
        E0[k] = A[k] * (cy - r.Y[ia]) - B[k] * (cx - r.X[ia]);
        const int64_t bound = abs(E0[k]) + abs(A[k]) * (int64_t)(h - 1) * kSub + abs(B[k]) * (int64_t)(w - 1) * kSub;
        fits32 &= bound < (1LL << 31);
    }
    for (int p = lane; p < npx; p += 32) {
        const int dy = (int)(((float)p + 0.5f) * inv_w);
        const int dx = p - dy * w;
        bool in;
        float fe1, fe2;
        if (fits32) {
            // biased edges as in tiny_record: inside when none is negative
            int e[3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                e[k] = (int)E0[k] + (int)A[k] * (dy << kSubBits) - (int)B[k] * (dx << kSubBits) - tl_bias(tl[k]);
            in = (e[0] | e[1] | e[2]) >= 0;
            fe1 = (float)(e[1] + tl_bias(tl[1]));
            fe2 = (float)(e[2] + tl_bias(tl[2]));
        } else {
            int64_t E[3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                E[k] = E0[k] + A[k] * (int64_t)(dy << kSubBits) - B[k] * (int64_t)(dx << kSubBits);
            in = (E[0] > 0 || (E[0] == 0 && tl[0])) && (E[1] > 0 || (E[1] == 0 && tl[1])) &&
                 (E[2] > 0 || (E[2] == 0 && tl[2]));
            fe1 = i2f(E[1]);
            fe2 = i2f(E[2]);
        }
        if (in) rec_emit<MODE>(a, r, r.x0 + dx, r.y0 + dy, fe1, fe2);
    }
}

// The warp-sized and tiny records in one launch, so both tiers share the
// SMs instead of running one after the other: warps stride over a joint
// list of units, first the warp records (one unit each, the larger and
// more uneven work), then the tiny records in units of 32 (one per lane).
// Their atomic updates commute, so the order does not change the result.
template <int MODE>
__global__ void __launch_bounds__(256) k_tiny_coop(TierArgs a) {
    pdl_enter();
    const unsigned ncoop = a.ctr[2], ntiny = a.ctr[1];
    const unsigned units = ncoop + (ntiny + 31) / 32;
    const int lane = threadIdx.x & 31;
    const unsigned nwarps = gridDim.x * (blockDim.x >> 5);
    for (unsigned u = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < units; u += nwarps) {
        if (u < ncoop) {
            coop_record<MODE>(a, u, lane);
        } else {
            const unsigned i = (u - ncoop) * 32 + lane;
            if (i < ntiny) tiny_record<MODE>(a, i);
        }
    }
}

// Large (non-huge) records: warps take contiguous ranges of the implied
// 16 x 16 tile list, reject tiles the triangle misses, 8 pixels per lane.
template <int MODE>
__global__ void __launch_bounds__(256) k_large_tiles(TierArgs a) {
    pdl_enter();
    const unsigned n = a.ctr[3];
    const unsigned long long total = *reinterpret_cast<const unsigned long long*>(a.ctr + 8);
    if (n == 0 || total == 0) return;
    const int lane = threadIdx.x & 31;
    const unsigned long long nwarps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long w = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const unsigned long long begin = total * w / nwarps, end = total * (w + 1) / nwarps;
    if (begin >= end) return;
    // last record whose base is <= begin
    unsigned lo = 0, hi = n - 1;
    while (lo < hi) {
        const unsigned mid = (lo + hi + 1) >> 1;
        if (a.large_base[mid] <= begin) lo = mid;
        else hi = mid - 1;
    }
    unsigned ri = lo;
    BRec r = a.recs[a.large[ri]];
    unsigned long long base = a.large_base[ri], nt = rec_tiles(r);
    int64_t A[3], B[3];
    bool tl[3];
    rec_edges(r, A, B, tl);
    for (unsigned long long item = begin; item < end; ++item) {
        while (item >= base + nt) {
            ++ri;
            r = a.recs[a.large[ri]];
            base = a.large_base[ri];
            nt = rec_tiles(r);
            rec_edges(r, A, B, tl);
        }
        const unsigned local = (unsigned)(item - base);
        const int ntx = (r.x1 / kTile) - (r.x0 / kTile) + 1;
        const int ty = (r.y0 / kTile) + (int)(local / (unsigned)ntx);
        const int tx = (r.x0 / kTile) + (int)(local % (unsigned)ntx);
        const int px0 = max(tx * kTile, (int)r.x0), px1 = min(tx * kTile + kTile - 1, (int)r.x1);
        const int py0 = max(ty * kTile, (int)r.y0), py1 = min(ty * kTile + kTile - 1, (int)r.y1);
        bool miss = false;
        {
            const int64_t cx0 = (int64_t)px0 * kSub + kSub / 2, cx1 = (int64_t)px1 * kSub + kSub / 2;
            const int64_t cy0 = (int64_t)py0 * kSub + kSub / 2, cy1 = (int64_t)py1 * kSub + kSub / 2;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int ia = (i + 1) % 3;
                const int64_t ymax = A[i] > 0 ? cy1 : cy0, xmin = B[i] > 0 ? cx0 : cx1;
                miss |= A[i] * (ymax - r.Y[ia]) - B[i] * (xmin - r.X[ia]) < 0;
            }
        }
        if (miss) continue;
        const int x = tx * kTile + (lane & 15);
        int y = ty * kTile + (lane >> 4);
        if (x < px0 || x > px1) continue;
        const int64_t px = (int64_t)x * kSub + kSub / 2, py = (int64_t)y * kSub + kSub / 2;
        int64_t E[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int ia = (i + 1) % 3;
            E[i] = A[i] * (py - r.Y[ia]) - B[i] * (px - r.X[ia]) - tl_bias(tl[i]);
        }
#pragma unroll 2
        for (int k = 0; k < kTile / 2; ++k, y += 2) {
            const bool in = y >= py0 && y <= py1 && inside_biased(E);
            if (in) rec_emit<MODE>(a, r, x, y, i2f(E[1] + tl_bias(tl[1])), i2f(E[2] + tl_bias(tl[2])));
#pragma unroll
            for (int i = 0; i < 3; ++i) E[i] += A[i] * (2 * kSub);
        }
    }
}

// Spilled sub-triangles of the tiered passes (one thread each, atomics).
template <int MODE>
__global__ void __launch_bounds__(128) k_tier_spill(TierArgs a) {
    pdl_enter();
    const unsigned n = min(a.ctr[4], a.spill_cap);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned id = a.spill[i];
        const int prim = (int)(id >> 3), sub = (int)(id & 7);
        float v[3][3];
        prim_vertices<MODE>(a.r, prim, v);
        float c[3][4];
#pragma unroll
        for (int j = 0; j < 3; ++j) transform(a.r.mvp, v[j][0], v[j][1], v[j][2], c[j]);
        const float idm[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
        Setup s;
        bool ok;
        if (all_inside(c[0], c[1], c[2])) {
            ok = sub == 0 && setup_triangle(c[0], c[1], c[2], idm[0], idm[1], idm[2], a.r.W, a.r.H, s);
        } else {
            CV poly[9];
            int np = clip_polygon(c[0], c[1], c[2], poly);
            ok = (sub + 2 < np) && setup_triangle(poly[0].c, poly[sub + 1].c, poly[sub + 2].c, poly[0].b,
                                                  poly[sub + 1].b, poly[sub + 2].b, a.r.W, a.r.H, s);
        }
        if (!ok) continue;
        int64_t minX = min(s.X[0], min(s.X[1], s.X[2])), maxX = max(s.X[0], max(s.X[1], s.X[2]));
        int64_t minY = min(s.Y[0], min(s.Y[1], s.Y[2])), maxY = max(s.Y[0], max(s.Y[1], s.Y[2]));
        int x0 = (int)max((int64_t)0, -((-(minX - kSub / 2)) >> kSubBits));
        int x1 = (int)min((int64_t)a.r.W - 1, (maxX - kSub / 2) >> kSubBits);
        int y0 = (int)max((int64_t)0, -((-(minY - kSub / 2)) >> kSubBits));
        int y1 = (int)min((int64_t)a.r.H - 1, (maxY - kSub / 2) >> kSubBits);
        if (x0 > x1 || y0 > y1) continue;
        float zoff = 0.0f;
        if (MODE == MODE_DEPTH) {
            if (a.r.bias_mode == GI_BIAS_POLYGON_OFFSET) zoff = polygon_offset(s, a.r.factor, a.r.units);
            else if (a.r.bias_mode == GI_BIAS_CONSTANT) zoff = a.r.cbias;
        }
        Edges e;
        make_edges(s, e);
        raster_small<MODE>(a.r, s, e, x0, x1, y0, y1, zoff, MODE == MODE_VKEY ? id : (unsigned)prim);
    }
}

}  // namespace dev

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {

// SM count per device, queried once; callers on several threads may race to
// fill a slot, which is harmless since they all store the same value.
int sm_count(int device) {
    static std::atomic<int> cached[64];
    if (device < 0 || device >= 64) return 152;
    int v = cached[device].load(std::memory_order_relaxed);
    if (!v) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0)
            v = 152;
        cached[device].store(v, std::memory_order_relaxed);
    }
    return v;
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



static dev::Mat4 mat_of(const float m[16]) {
    dev::Mat4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = m[i];
    return r;
}

// Binned pass: setup, big-record expansion, bin scan, scatter, per-bin
// raster and the spill pass (8 launches + 2 memsets, stream-ordered).
static gi_status run_binned(gi_context* ctx, dev::RasterArgs& r, int mode, cudaStream_t st) {
    const int nbx = (r.W + dev::kBin - 1) / dev::kBin, nby = (r.H + dev::kBin - 1) / dev::kBin;
    const size_t nbins = (size_t)nbx * nby;
    const size_t prims = (size_t)std::max(r.num_prims, 0);
    const size_t rec_cap = 2 * prims + 4096;
    const size_t big_pair_cap = 16 * nbins + 4 * rec_cap;
    const size_t list_cap = 4 * rec_cap + big_pair_cap;
    const size_t item_cap = nbins + list_cap / dev::kSeg + 1;
    const size_t need[8] = {rec_cap * sizeof(dev::BRec), rec_cap * sizeof(unsigned),
                            rec_cap * sizeof(unsigned long long), rec_cap * sizeof(unsigned),
                            4 * (nbins + 1) * sizeof(unsigned), list_cap * sizeof(unsigned),
                            4 * rec_cap * sizeof(unsigned), item_cap * sizeof(unsigned)};
    for (int i = 0; i < 8; ++i) {
        gi_status s = ensure_buffer(&ctx->bin_buf[i], &ctx->bin_cap[i], need[i]);
        if (s != GI_OK) return s;
    }
    dev::BinArgs a;
    a.r = r;
    a.recs = static_cast<dev::BRec*>(ctx->bin_buf[0]);
    a.rec_cap = (unsigned)rec_cap;
    a.big_list = static_cast<unsigned*>(ctx->bin_buf[1]);
    a.big_base = static_cast<unsigned long long*>(ctx->bin_buf[2]);
    a.big_cap = (unsigned)rec_cap;
    a.spill = static_cast<unsigned*>(ctx->bin_buf[3]);
    a.spill_cap = (unsigned)rec_cap;
    unsigned* bins = static_cast<unsigned*>(ctx->bin_buf[4]);
    a.bin_count = bins;
    a.big_count = bins + (nbins + 1);
    a.bin_offset = bins + 2 * (nbins + 1);
    a.bin_cursor = bins + 3 * (nbins + 1);
    a.bin_list = static_cast<unsigned*>(ctx->bin_buf[5]);
    a.ranks = static_cast<unsigned*>(ctx->bin_buf[6]);
    a.items = static_cast<unsigned*>(ctx->bin_buf[7]);
    a.item_cap = (unsigned)item_cap;
    a.list_cap = list_cap;
    a.big_pair_cap = big_pair_cap;
    a.ctr = ctx->d_status + 4;  // [0..3] counters, [4..5] admitted pairs (u64)
    a.nbx = nbx;
    a.nby = nby;
    cudaError_t e = cudaMemsetAsync(a.bin_count, 0, 2 * (nbins + 1) * sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.ctr, 0, 8 * sizeof(unsigned), st);
    if (e != cudaSuccess) return fail_cuda(e, "binned raster memset");
    const unsigned sms = (unsigned)sm_count(ctx->device);
    const unsigned gsetup = grid_for(prims ? prims : 1, 128);
    const unsigned gfill = grid_for(rec_cap, 256);
    switch (mode) {
        case dev::MODE_DEPTH:
            if (prims) dev::k_bin_setup<dev::MODE_DEPTH><<<gsetup, 128, 0, st>>>(a);
            break;
        case dev::MODE_VKEY:
            if (prims) dev::k_bin_setup<dev::MODE_VKEY><<<gsetup, 128, 0, st>>>(a);
            break;
        default:
            if (prims) dev::k_bin_setup<dev::MODE_STENCIL><<<gsetup, 128, 0, st>>>(a);
            break;
    }
    // stencil records spanning more than four bins go to k_sliver instead of
    // the bin-pair expansion (big_count stays zero)
    const bool pairs = mode != dev::MODE_STENCIL;
    if (pairs) {
        dev::k_big_scan<<<1, 1024, 0, st>>>(a);
        dev::k_big_pairs<false><<<sms * 4, 256, 0, st>>>(a);
    }
    dev::k_bin_scan<<<1, 1024, 0, st>>>(a);
    dev::k_bin_fill_small<<<gfill, 256, 0, st>>>(a);
    if (pairs) dev::k_big_pairs<true><<<sms * 4, 256, 0, st>>>(a);
    // the raster leaves empty bins alone: clear the target first
    const size_t npx = (size_t)r.W * r.H;
    const unsigned gclear = std::min<unsigned>(grid_for(npx / 4 + 1, 256), sms * 8);
    if (mode == dev::MODE_DEPTH) {
        dev::k_fill_u32<<<gclear, 256, 0, st>>>(r.depth, npx, 0x3f800000u);
    } else if (mode == dev::MODE_VKEY) {
        dev::k_fill_u64<<<std::min<unsigned>(grid_for(npx, 256), sms * 8), 256, 0, st>>>(
            r.keys, npx, ((unsigned long long)0x3f800000u << 32) | 0xFFFFFFFFull);
    } else {
        e = cudaMemsetAsync(r.counts, 0, npx * sizeof(int), st);
        if (e != cudaSuccess) return fail_cuda(e, "binned raster memset(counts)");
    }
    const unsigned graster = (unsigned)item_cap;
    switch (mode) {
        case dev::MODE_DEPTH:
            dev::k_bin_raster<dev::MODE_DEPTH><<<graster, 256, 0, st>>>(a);
            dev::k_spill<dev::MODE_DEPTH><<<sms * 2, 128, 0, st>>>(a);
            break;
        case dev::MODE_VKEY:
            dev::k_bin_raster<dev::MODE_VKEY><<<graster, 256, 0, st>>>(a);
            dev::k_spill<dev::MODE_VKEY><<<sms * 2, 128, 0, st>>>(a);
            break;
        default:
            dev::k_bin_raster<dev::MODE_STENCIL><<<graster, 256, 0, st>>>(a);
            dev::k_sliver<<<sms * 8, 256, 0, st>>>(a);
            dev::k_spill<dev::MODE_STENCIL><<<sms * 2, 128, 0, st>>>(a);
            break;
    }
    ctx->launches += (prims ? 8 : 7) + (mode == dev::MODE_STENCIL ? -2 : 1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "binned raster launch");
    return GI_OK;
}

// Tiered pass (light map, G-buffer keys): setup, large-record scan, base
// layer (huge records + clear), tiny and warp records in one launch, tile
// rasterisation, spill; atomics after the base layer (6 launches + 1
// memset, stream-ordered).
static gi_status run_tiered(gi_context* ctx, dev::RasterArgs& r, int mode, cudaStream_t st) {
    const size_t prims = (size_t)std::max(r.num_prims, 0);
    const size_t rec_cap = 2 * prims + 4096;
    const bool keys = mode == dev::MODE_VKEY;
    const size_t need[8] = {rec_cap * sizeof(dev::BRec), rec_cap * sizeof(unsigned),
                            rec_cap * sizeof(unsigned), rec_cap * sizeof(unsigned),
                            rec_cap * sizeof(unsigned long long), rec_cap * sizeof(unsigned),
                            keys ? std::max<size_t>(prims, 1) * sizeof(unsigned) : 0,
                            keys ? rec_cap * sizeof(uint4) : 0};
    void** buf = ctx->tier_buf[keys ? 1 : 0];
    size_t* cap = ctx->tier_cap[keys ? 1 : 0];
    for (int i = 0; i < 8; ++i) {
        if (!need[i]) continue;
        gi_status s = ensure_buffer(&buf[i], &cap[i], need[i]);
        if (s != GI_OK) return s;
    }
    dev::TierArgs a;
    a.r = r;
    a.recs = static_cast<dev::BRec*>(buf[0]);
    a.rec_cap = (unsigned)rec_cap;
    a.tiny = static_cast<unsigned*>(buf[1]);
    a.coop = static_cast<unsigned*>(buf[2]);
    a.large = static_cast<unsigned*>(buf[3]);
    a.large_base = static_cast<unsigned long long*>(buf[4]);
    a.spill = static_cast<unsigned*>(buf[5]);
    a.spill_cap = (unsigned)rec_cap;
    a.huge_px = std::max<unsigned long long>(65536ull, (unsigned long long)r.W * r.H / 8);
    a.tiny_px = ctx->tiny_px;
    a.coop_px = ctx->coop_px;
    a.rec_of = keys ? static_cast<unsigned*>(buf[6]) : nullptr;
    a.rres = keys ? static_cast<uint4*>(buf[7]) : nullptr;
    a.ctr = ctx->d_status + (keys ? 64 : 32);  // 24 words per set
    cudaError_t e = cudaMemsetAsync(a.ctr, 0, 24 * sizeof(unsigned), st);
    if (e != cudaSuccess) return fail_cuda(e, "tiered raster memset");
    const unsigned sms = (unsigned)sm_count(ctx->device);
    const unsigned gsetup = grid_for(prims ? prims : 1, 128);
    const int base_rows = 8 * dev::kBaseRows;  // rows per block of k_base (8 warps)
    const dim3 gbase((r.W + 31) / 32, (r.H + base_rows - 1) / base_rows);
    // Each kernel after the first is a programmatic dependent of the one
    // before it (launch_dependent, pdl_enter): launched directly, the
    // pcss_1080p frame went 8,700 -> 9,400 frames/s; under stream capture
    // (frame graphs, batches) the launches are ordinary (with the dependents
    // inside frame graphs, graph-mode end to end fell 11,100 -> 10,600).
    auto chain = [&](auto kernel, dim3 grid, int threads) {
        cudaError_t le = launch_dependent(kernel, grid, dim3((unsigned)threads), 0, st, a);
        if (le != cudaSuccess && e == cudaSuccess) e = le;
    };
    if (mode == dev::MODE_DEPTH) {
        if (prims) dev::k_tier_setup<dev::MODE_DEPTH><<<gsetup, 128, 0, st>>>(a);
        chain(dev::k_large_scan, dim3(1), 1024);
        chain(dev::k_base<dev::MODE_DEPTH>, gbase, 256);
        chain(dev::k_tiny_coop<dev::MODE_DEPTH>, dim3(sms * 8), 256);
        chain(dev::k_large_tiles<dev::MODE_DEPTH>, dim3(sms * 8), 256);
        chain(dev::k_tier_spill<dev::MODE_DEPTH>, dim3(sms * 2), 128);
    } else {
        if (prims) dev::k_tier_setup<dev::MODE_VKEY><<<gsetup, 128, 0, st>>>(a);
        chain(dev::k_large_scan, dim3(1), 1024);
        chain(dev::k_base<dev::MODE_VKEY>, gbase, 256);
        chain(dev::k_tiny_coop<dev::MODE_VKEY>, dim3(sms * 8), 256);
        chain(dev::k_large_tiles<dev::MODE_VKEY>, dim3(sms * 8), 256);
        chain(dev::k_tier_spill<dev::MODE_VKEY>, dim3(sms * 2), 128);
    }
    ctx->launches += prims ? 6 : 5;
    if (e != cudaSuccess) return fail_cuda(e, "tiered raster launch");
    e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "tiered raster launch");
}

gi_status raster_depth_map(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W,
                           int H, int bias_mode, float cbias, float factor, float units,
                           float* d_depth, int small_px, cudaStream_t st) {
    (void)small_px;
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
    return run_tiered(ctx, a, dev::MODE_DEPTH, st);
}

gi_status raster_gbuffer(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W, int H,
                         float* d_pos, float* d_nrm, int small_px, cudaStream_t st) {
    (void)small_px;
    const size_t npx = (size_t)W * H;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_vkeys), &ctx->cap_vkeys,
                                npx * sizeof(unsigned long long));
    if (s != GI_OK) return s;
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    a.num_prims = scene->dev_triangles;
    a.mvp = mat_of(mvp);
    a.W = W;
    a.H = H;
    a.keys = ctx->d_vkeys;
    s = run_tiered(ctx, a, dev::MODE_VKEY, st);
    if (s != GI_OK) return s;
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    dev::k_gbuffer_resolve<<<grid, 128, 0, st>>>(
        ctx->d_vkeys, scene->d_points, scene->d_normals, scene->d_indices, a.mvp, W, H,
        reinterpret_cast<float4*>(d_pos), reinterpret_cast<float4*>(d_nrm),
        static_cast<const unsigned*>(ctx->tier_buf[1][6]), static_cast<const dev::BRec*>(ctx->tier_buf[1][0]),
        static_cast<const uint4*>(ctx->tier_buf[1][7]));
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gbuffer resolve launch");
}

gi_status raster_gbuffer_keys(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W,
                              int H, cudaStream_t st) {
    const size_t npx = (size_t)W * H;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_vkeys), &ctx->cap_vkeys,
                                npx * sizeof(unsigned long long));
    if (s != GI_OK) return s;
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    a.num_prims = scene->dev_triangles;
    a.mvp = mat_of(mvp);
    a.W = W;
    a.H = H;
    a.keys = ctx->d_vkeys;
    return run_tiered(ctx, a, dev::MODE_VKEY, st);
}

gi_status raster_volume_geometry(gi_context* ctx, const gi_scene* scene, const float L[3],
                                 float infinity, float* d_out, cudaStream_t st) {
    if ((long long)scene->dev_triangles * 6 >= (1LL << 29))
        return fail(GI_ERR_CAPACITY, "too many volume triangles (6 T must stay below 2^29)");
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    a.num_prims = scene->dev_triangles * 6;
    a.L[0] = L[0];
    a.L[1] = L[1];
    a.L[2] = L[2];
    a.infinity = infinity;
    if (a.num_prims == 0) return GI_OK;
    dev::k_volume_geometry<<<grid_for((size_t)a.num_prims, 256), 256, 0, st>>>(a, d_out);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "volume geometry launch");
}

// Adjacency of the scene's triangles for the silhouette mode, built on the
// host from the uploaded indices and cached until the next upload:
// adj[3t + k] = (u << 1) | same for the triangle u sharing edge k of t
// (vertices k, k + 1 mod 3), same = 1 when u runs the edge in the same
// direction; -1 for an edge with one triangle or more than two.
static gi_status ensure_adjacency(gi_scene* scene, cudaStream_t st) {
    if (scene->adj_serial == scene->upload_serial && scene->d_adj) return GI_OK;
    const int T = scene->dev_triangles;
    std::vector<int> idx(3 * (size_t)T);
    cudaError_t e = cudaSuccess;
    if (T) e = cudaMemcpyAsync(idx.data(), scene->d_indices, idx.size() * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, "silhouette adjacency: index read-back");
    struct HalfEdge {
        unsigned long long key;  // (min vertex << 32) | max vertex
        int slot;                // 3t + k
    };
    std::vector<HalfEdge> he(3 * (size_t)T);
    for (int t = 0; t < T; ++t)
        for (int k = 0; k < 3; ++k) {
            const unsigned a = (unsigned)idx[3 * (size_t)t + k], b = (unsigned)idx[3 * (size_t)t + (k + 1) % 3];
            const unsigned lo = a < b ? a : b, hi = a < b ? b : a;
            he[3 * (size_t)t + k] = {((unsigned long long)lo << 32) | hi, 3 * t + k};
        }
    std::sort(he.begin(), he.end(), [](const HalfEdge& x, const HalfEdge& y) {
        return x.key < y.key || (x.key == y.key && x.slot < y.slot);
    });
    std::vector<int> adj(3 * (size_t)T, -1);
    for (size_t i = 0; i < he.size();) {
        size_t j = i + 1;
        while (j < he.size() && he[j].key == he[i].key) ++j;
        if (j - i == 2 && (he[i].key >> 32) != (he[i].key & 0xffffffffull)) {
            const int s0 = he[i].slot, s1 = he[i + 1].slot;
            const int t0 = s0 / 3, k0 = s0 % 3, t1 = s1 / 3, k1 = s1 % 3;
            const bool fwd0 = idx[3 * (size_t)t0 + k0] < idx[3 * (size_t)t0 + (k0 + 1) % 3];
            const bool fwd1 = idx[3 * (size_t)t1 + k1] < idx[3 * (size_t)t1 + (k1 + 1) % 3];
            const int same = fwd0 == fwd1 ? 1 : 0;
            adj[s0] = (t1 << 1) | same;
            adj[s1] = (t0 << 1) | same;
        }
        i = j;
    }
    size_t cap = scene->cap_adj;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&scene->d_adj), &cap, std::max<size_t>(adj.size(), 1) * sizeof(int));
    if (s != GI_OK) return s;
    scene->cap_adj = cap;
    if (T) e = cudaMemcpyAsync(scene->d_adj, adj.data(), adj.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // adj is a local vector
    if (e != cudaSuccess) return fail_cuda(e, "silhouette adjacency: upload");
    scene->adj_serial = scene->upload_serial;
    return GI_OK;
}

gi_status raster_shadow_volumes(gi_context* ctx, const gi_scene* scene, const float L[3],
                                float infinity, const float mvp[16], int W, int H, int depth_func,
                                unsigned char* d_stencil, float* d_depth_out, int small_px,
                                cudaStream_t st, bool silhouette, int* drawn) {
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
    dev::RasterArgs a = {};
    a.points = scene->d_points;
    a.normals = scene->d_normals;
    a.indices = scene->d_indices;
    if ((long long)scene->dev_triangles * 6 >= (1LL << 29))
        return fail(GI_ERR_CAPACITY, "too many volume triangles (6 T must stay below 2^29)");
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
    if (silhouette) {
        // Only the silhouette quads are drawn (k_silhouette_prims); their
        // number is read back to size the binned pass.
        s = ensure_adjacency(const_cast<gi_scene*>(scene), st);
        if (s != GI_OK) return s;
        s = ensure_buffer(&ctx->d_sil_list, &ctx->cap_sil_list,
                          std::max<size_t>((size_t)a.num_prims, 1) * sizeof(int));
        if (s != GI_OK) return s;
        unsigned* count = ctx->d_status + 101;
        cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned), st);
        if (e != cudaSuccess) return fail_cuda(e, "silhouette count reset");
        const long long edges = 3LL * scene->dev_triangles;
        if (edges > 0) {
            dev::k_silhouette_prims<<<grid_for((size_t)edges, 256), 256, 0, st>>>(
                scene->d_normals, scene->d_indices, scene->d_adj, scene->dev_triangles, L[0], L[1], L[2],
                static_cast<int*>(ctx->d_sil_list), count);
            ctx->launches++;
        }
        e = cudaMemcpyAsync(ctx->h_status + 101, count, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail_cuda(e, "silhouette count read-back");
        a.num_prims = (int)ctx->h_status[101];
        a.prim_list = static_cast<const int*>(ctx->d_sil_list);
    }
    if (drawn) *drawn = a.num_prims;
    s = run_binned(ctx, a, dev::MODE_STENCIL, st);
    if (s != GI_OK) return s;
    dev::k_wrap_stencil<<<grid_for(npx, 256), 256, 0, st>>>(ctx->d_counts, d_stencil, npx);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
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
// Per device: the scratch address under which the pass's kernels were last
// loaded.  A new CUDA context on the same device (after cudaDeviceReset, or
// a caller's own driver-API context) has its own copy of the module and so
// a different address; the kernels are then loaded again.
void* g_noalloc_loaded[kNoallocMaxDevices] = {};

// Device address of g_noalloc_scratch in the current context.  The array's
// name in host code is only a host-side handle; the address is looked up on
// every call (cheap once the module is loaded) and never cached across
// contexts.  The first call in a context loads the library's module and,
// here, every kernel the pass launches (cudaFuncGetAttributes), so that no
// later call, whatever its triangle count, triggers lazy loading.
gi_status noalloc_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kNoallocMaxDevices)
        return fail(GI_ERR_UNSUPPORTED, "gi_gbuffer_noalloc: device index out of range");
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return fail_cuda(e == cudaSuccess ? cudaErrorInvalidSymbol : e,
                         "gi_gbuffer_noalloc: cudaGetSymbolAddress");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_loaded[dev] != p) {
        const void* kernels[] = {
            reinterpret_cast<const void*>(&dev::k_fill_u64),
            reinterpret_cast<const void*>(&dev::k_setup<dev::MODE_VKEY>),
            reinterpret_cast<const void*>(&dev::k_scan),
            reinterpret_cast<const void*>(&dev::k_tiles<dev::MODE_VKEY>),
            reinterpret_cast<const void*>(&dev::k_gbuffer_resolve),
        };
        for (const void* k : kernels) {
            cudaFuncAttributes fa;
            e = cudaFuncGetAttributes(&fa, k);
            if (e != cudaSuccess) return fail_cuda(e, "gi_gbuffer_noalloc: loading the pass's kernels");
        }
        g_noalloc_loaded[dev] = p;
    }
    *out = static_cast<unsigned char*>(p);
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
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail_cuda(e, "gi_gbuffer_noalloc: cudaGetDevice");
    unsigned char* base = nullptr;
    gi_status st = noalloc_scratch(device, &base);
    if (st != GI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(base);
    dev::TriRec* recs = reinterpret_cast<dev::TriRec*>(base + kNoallocKeysBytes);
    unsigned* status = reinterpret_cast<unsigned*>(base + kNoallocKeysBytes + kNoallocRecsBytes);
    // The array keeps the previous call's contents: reset the counters and
    // the keys before use.
    e = cudaMemsetAsync(status, 0, kNoallocStatusBytes, cs);
    if (e != cudaSuccess) return fail_cuda(e, "gi_gbuffer_noalloc: cudaMemsetAsync");
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
                                                 reinterpret_cast<float4*>(d_nrm), nullptr, nullptr, nullptr);
    e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_gbuffer_noalloc: kernel launch");
}
