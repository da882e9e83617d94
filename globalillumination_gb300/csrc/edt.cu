// edt.cu -- exact Euclidean distance transform and EDT-filtered hard shadows
// for sm_103a.
//
// The band stacks, the merges and the coloring walk below restate PBA, the
// parallel banding algorithm of Cao Thanh Tung (2010), whose code carries
// this notice:
//
//   Copyright (c) 2010, School of Computing, National University of Singapore.
//   All rights reserved.
//
//   Project homepage: http://www.comp.nus.edu.sg/~tants/pba.html
//
//   If you use PBA and you like it or have comments on its usefulness etc., we
//   would love to hear from you at <tants@comp.nus.edu.sg>. You may share with us
//   your experience and any possibilities that we may improve the work/code.
//
//   ===============================================================================
//
//   Redistribution and use in source and binary forms, with or without modification,
//   are permitted provided that the following conditions are met:
//
//   Redistributions of source code must retain the above copyright notice, this list of
//   conditions and the following disclaimer. Redistributions in binary form must reproduce
//   the above copyright notice, this list of conditions and the following disclaimer
//   in the documentation and/or other materials provided with the distribution.
//
//   Neither the name of the National University of University nor the names of its contributors
//   may be used to endorse or promote products derived from this software without specific
//   prior written permission from the National University of Singapore.
//
//   THIS SOFTWARE IS PROVIDED BY THE COPYRIGHT HOLDERS AND CONTRIBUTORS "AS IS" AND ANY
//   EXPRESS OR IMPLIED WARRANTIES, INCLUDING, BUT NOT LIMITED TO THE IMPLIED WARRANTIES
//   OF MERCHANTABILITY AND FITNESS FOR A PARTICULAR PURPOSE ARE DISCLAIMED. IN NO EVENT
//   SHALL THE COPYRIGHT OWNER OR CONTRIBUTORS BE LIABLE FOR ANY DIRECT, INDIRECT,
//   INCIDENTAL, SPECIAL, EXEMPLARY, OR CONSEQUENTIAL DAMAGES (INCLUDING, BUT NOT LIMITED
//   TO, PROCUREMENT OF SUBSTITUTE  GOODS OR SERVICES; LOSS OF USE, DATA, OR PROFITS; OR
//   BUSINESS INTERRUPTION) HOWEVER CAUSED AND ON ANY THEORY OF LIABILITY, WHETHER IN
//   CONTRACT, STRICT LIABILITY, OR TORT (INCLUDING NEGLIGENCE OR OTHERWISE) ARISING IN
//   ANY WAY OUT OF THE USE OF THIS SOFTWARE, EVEN IF ADVISED OF THE POSSIBILITY OF SUCH
//   DAMAGE.
//
//
// Restates on device buffers the reference's only CUDA code: the parallel
// banding algorithm (PBA, Cao et al. 2010) of ShadowMapping/include/EDT/
// pba2DKernel.h as ShadowMapping/src/EDT/pba2DHost.cu:121-242 sequences it,
// together with the site detection (initializeInput, pba2DKernel.h:509-528)
// and the normalisation (pbaNormalizeDistanceTransform, :541-569) of
// ShadowMapping's EDTSM mode (src/main.cpp:416-422).  Which of two
// equidistant sites a pixel receives depends on PBA's bands (m1, m2, m3), its
// merge order and its FP32 bisector tests, so every result equals the
// reference's for the same bands.  The kernels are organised for this GPU:
//
//   k_pba_columns  phase 1 in one pass.  For band height B = H / m1 >= 2
//                  the reference's flood / propagate / update kernels give
//                  each pixel the nearest site of its column, an equidistant
//                  pair resolved to the site below when that site lies in the
//                  pixel's band and to the site above otherwise.  A CTA owns 8
//                  columns x 128 row segments (one thread each): it tests its
//                  pixels for sites, keeps them as a 64-bit mask, and two warp
//                  scans over the CTA's segments give every segment its
//                  nearest sites above and below.  Output: the chosen site's
//                  row per pixel (int16, row-major, MARKER for an empty
//                  column) -- no transposes are needed.
//   k_pba_rows     phases 2-3, one image row per warp, in shared memory: the
//                  per-band proximate-point stacks and forward links (one
//                  lane per band), the pairwise band merges level by level
//                  (one lane per pair), then the coloring.  A row whose list
//                  is a strict lower envelope is colored by a binary search
//                  over its exact crossing points, which gives every pixel
//                  the site the reference's group walks reach; other rows
//                  replay the groups' chain of states.  Writes each pixel's
//                  nearest site.
//   k_edt_normalize  the penumbra normalisation, one thread per pixel.
//
// Compiled like every pass with -fmad=false and IEEE division / square root,
// so each FP32 operation rounds once in the order written (the CPU oracle
// and the reference's kernels run on the CPU round the same way).
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>

#include "internal.h"
#include "raster.h"

namespace gi {
namespace edt {

constexpr int kMarker = -32768;  // MARKER (ShadowMapping/include/EDT/pba2D.h:60)
constexpr unsigned kFull = 0xffffffffu;
constexpr int kColW = 8;                 // columns per CTA in the column pass
constexpr int kSegs = 128;               // row segments per CTA
constexpr int kColThreads = kColW * kSegs;
constexpr int kMaxSegRows = 64;          // one 64-bit site mask per thread
constexpr int kRowThreads = 256;         // 8 rows per CTA in the row pass

enum : int { kFromSites = 0, kFromImage = 1 };

// linearize (pba2DKernel.h:499-506) with n = 1, f = 1000: 2.0 * n is a
// double, so the reference divides in double and rounds to float.  For a
// quotient in float's normal range that equals the IEEE float division
// (double carries more than 2 x 24 + 2 bits, so the second rounding is
// innocuous); tiny quotients take the double path.
__device__ __forceinline__ float linearize(float depth) {
    const float d = 1001.0f - depth * 999.0f;
    float q = 2.0f / d;
    if (!(fabsf(q) >= 2.3509887e-38f)) q = (float)(2.0 / (double)d);
    return q;
}

// ---- phase 1 ---------------------------------------------------------------

struct ColArgs {
    const short2* sites;   // kFromSites: (x, y) at a site, x == MARKER elsewhere
    const float4* image;   // kFromImage: (shadow, depth, preEvaluatedShadow, 1)
    int16_t* cols;         // [H][W]: row of the chosen column site, or MARKER
    int W, H, S, band;     // S rows per segment; band = H / m1
    float thr;             // the largest float <= 0.0025
};

struct Px {
    float s, L;  // shadow value, linearised depth
    int f;       // bit 0: inside the image, bit 1: p.z == 1
};

__device__ __forceinline__ Px px_load(const ColArgs& a, int x, int y) {
    Px p{0.0f, 0.0f, 0};
    if (x < 0 || x >= a.W || y < 0 || y >= a.H) return p;
    const float4 v = __ldg(a.image + (size_t)y * a.W + x);
    p.s = v.x;
    p.L = linearize(v.y);
    p.f = 1 | (v.z == 1.0f ? 2 : 0);
    return p;
}

// initializeInput's test of neighbour p against centre c (pba2DKernel.h:520)
__device__ __forceinline__ bool triggers(const Px& c, const Px& p, float thr) {
    return p.f == 3 && p.s != c.s && fabsf(c.L - p.L) <= thr;
}

// (x - 1, x, x + 1) of row y: the centre is loaded, its neighbours come from
// the adjacent lanes of the 8-lane column group, the group's edge lanes load
// their outer neighbour themselves.
__device__ __forceinline__ void load_row(const ColArgs& a, int x, int col, int y, Px* r) {
    const Px m = px_load(a, x, y);
    Px l, rr;
    l.s = __shfl_up_sync(kFull, m.s, 1, kColW);
    l.L = __shfl_up_sync(kFull, m.L, 1, kColW);
    l.f = __shfl_up_sync(kFull, m.f, 1, kColW);
    rr.s = __shfl_down_sync(kFull, m.s, 1, kColW);
    rr.L = __shfl_down_sync(kFull, m.L, 1, kColW);
    rr.f = __shfl_down_sync(kFull, m.f, 1, kColW);
    if (col == 0) l = px_load(a, x - 1, y);
    if (col == kColW - 1) rr = px_load(a, x + 1, y);
    r[0] = l;
    r[1] = m;
    r[2] = rr;
}

template <int kMode>
__global__ void __launch_bounds__(kColThreads) k_pba_columns(const ColArgs a) {
    __shared__ int s_first[kSegs][kColW], s_last[kSegs][kColW];
    __shared__ int s_above[kSegs][kColW], s_below[kSegs][kColW];
    const int col = threadIdx.x & (kColW - 1), seg = threadIdx.x / kColW;
    const int x = blockIdx.x * kColW + col;
    const int y0 = seg * a.S;
    unsigned long long mask = 0;
    if (kMode == kFromSites) {
        if (x < a.W)
            for (int i = 0; i < a.S; ++i) {
                const int y = y0 + i;
                if (y < a.H && a.sites[(size_t)y * a.W + x].x != kMarker) mask |= 1ull << i;
            }
    } else {
        Px u[3], c[3], d[3];
        load_row(a, x, col, y0 - 1, u);
        load_row(a, x, col, y0, c);
        for (int i = 0; i < a.S; ++i) {
            load_row(a, x, col, y0 + i + 1, d);
            if (x < a.W && y0 + i < a.H) {
                const Px& ctr = c[1];
                bool s = false;
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    s = s || triggers(ctr, u[k], a.thr) || triggers(ctr, c[k], a.thr) || triggers(ctr, d[k], a.thr);
                if (s) mask |= 1ull << i;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                u[k] = c[k];
                c[k] = d[k];
            }
        }
    }
    s_first[seg][col] = mask ? y0 + __ffsll((long long)mask) - 1 : INT_MAX;
    s_last[seg][col] = mask ? y0 + 63 - __clzll((long long)mask) : -1;
    __syncthreads();
    // warp w < 8 scans column w: lane l holds segments 4l .. 4l + 3
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < kColW) {
        int lv[4], fv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            lv[k] = s_last[4 * lane + k][warp];
            fv[k] = s_first[4 * lane + k][warp];
        }
        int incl = max(max(lv[0], lv[1]), max(lv[2], lv[3]));
        int inclf = min(min(fv[0], fv[1]), min(fv[2], fv[3]));
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            const int tf = __shfl_down_sync(kFull, inclf, o);
            if (lane >= o) incl = max(incl, t);
            if (lane + o < 32) inclf = min(inclf, tf);
        }
        int run = __shfl_up_sync(kFull, incl, 1);
        int runf = __shfl_down_sync(kFull, inclf, 1);
        if (lane == 0) run = -1;
        if (lane == 31) runf = INT_MAX;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s_above[4 * lane + k][warp] = run;
            run = max(run, lv[k]);
        }
#pragma unroll
        for (int k = 3; k >= 0; --k) {
            s_below[4 * lane + k][warp] = runf;
            runf = min(runf, fv[k]);
        }
    }
    __syncthreads();
    if (x >= a.W) return;
    const int above = s_above[seg][col], below = s_below[seg][col];
    for (int i = 0; i < a.S; ++i) {
        const int y = y0 + i;
        if (y >= a.H) break;
        const unsigned long long le = mask & ((2ull << i) - 1);  // sites at rows <= y
        const unsigned long long ge = mask >> i;                  // sites at rows >= y
        const int up = le ? y0 + 63 - __clzll((long long)le) : above;
        const int dn = ge ? y + __ffsll((long long)ge) - 1 : below;
        int v;
        if (up < 0) {
            v = dn == INT_MAX ? kMarker : dn;
        } else if (dn == INT_MAX) {
            v = up;
        } else {
            const int da = y - up, db = dn - y;
            v = db < da ? dn : (da < db ? up : (dn / a.band == y / a.band ? dn : up));
        }
        a.cols[(size_t)y * a.W + x] = (int16_t)v;
    }
}

// ---- phases 2 and 3 ----------------------------------------------------------

struct RowArgs {
    const int16_t* cols;
    int W, H, m2, m3, wpb, per_warp;  // per_warp: shared bytes per row
    short2* nearest;                  // (site x, site y) per pixel
    unsigned* status;                 // [0] += rows colored by the exact chain
};

// One row's state in shared memory.  cand[p] = row of column p's phase-1
// site (the reference's transposed texture); lk[p] = its textures[0] line
// (stack value and back pointer, later forward and back pointers); alive[p]
// = p is on the list; ic[p] = interpoint(predecessor, p) of a stack entry
// (phase 2), then site[p] = x of pixel p's site and ex[i] = i-th list
// position (coloring); st[k] = the list position group k starts from.
struct RowLayout {
    int cand, lk, ic, site, ex, alive, st, cm, bytes;
};

__host__ __device__ __forceinline__ int up16(int b) { return (b + 15) & ~15; }

__host__ __device__ __forceinline__ RowLayout row_layout(int W, int m3) {
    RowLayout l;
    l.cand = 0;
    l.lk = up16(2 * W);
    l.ic = l.lk + 4 * W;
    l.site = l.ic;  // over ic once phase 2 is done
    l.ex = l.ic + up16(2 * W);
    l.alive = l.ic + 4 * W;
    l.st = l.alive + up16(W);
    l.cm = l.st + up16(4 * (W / m3));
    l.bytes = l.cm + up16(4 * ((W + 31) / 32));
    return l;
}

struct Row {
    int16_t* cand;
    short2* lk;
    uint8_t* alive;
    float* ic;
    int16_t* site;
    int16_t* ex;
    int* st;
    unsigned* cm;  // bit p & 31 of word p >> 5: column p has a site
    int W, line;

    __device__ __forceinline__ int C(int p) const { return cand[p]; }
    __device__ __forceinline__ short2& L(int p) const { return lk[p]; }
    __device__ __forceinline__ float& I(int p) const { return ic[p]; }
    __device__ __forceinline__ uint8_t& A(int p) const { return alive[p]; }
    __device__ __forceinline__ int16_t& S(int p) const { return site[p]; }
    __device__ __forceinline__ int16_t& E(int i) const { return ex[i]; }

    // textures[0] after kernelDoubleToSingleList; tex1Dfetch reads zero
    // outside the texture
    __device__ __forceinline__ short2 col(int p) const {
        if (p < 0 || p >= W) return make_short2(0, 0);
        return make_short2((short)C(p), L(p).y);
    }
};

// interpoint (pba2DKernel.h:227-236).  A zero numerator (two sites in one
// row, or the bisector's midpoint on the line) gives yM + (+-0) = yM, as yM
// >= 0.5 here (y1 < y2 are list positions); answering it directly keeps the
// division's special-case path out of the common case.
__device__ __forceinline__ float interpoint(int x1, int y1, int x2, int y2, int x0) {
    const float xM = (float)(x1 + x2) / 2.0f;
    const float yM = (float)(y1 + y2) / 2.0f;
    if (x1 == x2 || x1 + x2 == 2 * x0) return yM;
    const float nx = (float)(x2 - x1);
    const float ny = (float)(y2 - y1);
    return yM + nx * (xM - (float)x0) / ny;
}

// Next position after p (before end) whose column has a site, from the
// row's candidate bit words.
__device__ __forceinline__ int next_cand(const unsigned* cm, int p, int end) {
    int q = p + 1;
    while (q < end) {
        const unsigned w = cm[q >> 5] >> (q & 31);
        if (w) {
            q += __ffs(w) - 1;
            return q < end ? q : end;
        }
        q = (q | 31) + 1;
    }
    return end;
}

// kernelProximatePoints (pba2DKernel.h:238-268) for the band [b0, b0 + B).
// The reference's i1 = interpoint(last1, last2) is the intersection of the
// top entry with the entry below it, fixed since the top was pushed, so it
// is computed once, at the push, and read back from ic[] (same operands,
// same float).  The nested push / pop loops run as one loop of single steps
// -- a test that pops, or a push -- whose updates are selects, so the 16
// lanes of a warp, each on its own band, stay converged.
__device__ void proximate(const Row& r, int b0, int B) {
    const int end = b0 + B;
    int lasty = -1;
    short2 last1 = make_short2(0, -1), last2 = make_short2(0, -1);
    int p = next_cand(r.cm, b0 - 1, end);
    int g = p < end ? r.C(p) : 0;
    while (p < end) {
        float i2 = 0.0f;
        bool pop = false;
        if (lasty >= 0) {
            i2 = interpoint(last2.x, lasty, g, p, r.line);
            pop = last2.y >= 0 && !(r.I(lasty) < i2);
        }
        const short2 below = r.L(last1.y >= 0 ? last1.y : 0);  // used only by a pop
        if (pop) {
            r.A(lasty) = 0;
        } else {
            if (lasty >= 0) r.I(p) = i2;
            r.L(p) = make_short2((short)g, (short)lasty);
            r.A(p) = 1;
        }
        const short2 n1 = pop ? (last1.y >= 0 ? below : last1) : last2;
        const short2 n2 = pop ? last1 : make_short2((short)g, (short)lasty);
        lasty = pop ? last2.y : p;
        last1 = n1;
        last2 = n2;
        if (!pop) {
            p = next_cand(r.cm, p, end);
            if (p < end) g = r.C(p);
        }
    }
    if (lasty != end - 1) r.L(end - 1) = make_short2((short)kMarker, (short)lasty);
}

// kernelCreateForwardPointers (:270-296)
__device__ void forward(const Row& r, int b0, int B) {
    const int ty = b0 + B - 1;
    int lasty = -1;
    short2 cur = r.L(ty);
    int nexty = cur.x == kMarker ? cur.y : ty;
    int p = ty;
    for (int i = 0; i < B; ++i, --p)
        if (ty - i == nexty) {
            cur = make_short2((short)lasty, r.L(p).y);
            r.L(p) = cur;
            lasty = nexty;
            nexty = cur.y;
        }
    if (lasty != ty - B + 1) r.L(p + 1) = make_short2((short)lasty, (short)kMarker);
}

// kernelMergeBands (:298-435) for bands band1 and band1 + 1 of size B
__device__ void merge(const Row& r, int band1, int B) {
    const int band2 = band1 + 1;
    int lasty = band2 * B - 1;
    short2 last2 = make_short2(r.C(lasty), r.L(lasty).y), last1 = make_short2(0, 0);
    if (last2.x == kMarker) {
        lasty = last2.y;
        last2 = lasty >= 0 ? make_short2(r.C(lasty), r.L(lasty).y) : make_short2(kMarker, kMarker);
    }
    if (last2.y >= 0) last1 = make_short2(r.C(last2.y), r.L(last2.y).y);
    int firsty = band2 * B;
    short2 cur = make_short2(r.L(firsty).x, r.C(firsty));
    if (cur.y == kMarker) {
        firsty = cur.x;
        cur = firsty >= 0 ? make_short2(r.L(firsty).x, r.C(firsty)) : make_short2(kMarker, kMarker);
    }
    int top = 0;
    while (top < 2 && cur.y >= 0) {
        while (last2.y >= 0) {
            const float i1 = interpoint(last1.x, last2.y, last2.x, lasty, r.line);
            const float i2 = interpoint(last2.x, lasty, cur.y, firsty, r.line);
            if (i1 < i2) break;
            r.A(lasty) = 0;
            lasty = last2.y;
            last2 = last1;
            --top;
            if (last1.y >= 0) last1 = make_short2(r.C(last1.y), r.L(last1.y).y);
        }
        r.L(firsty) = make_short2(cur.x, (short)lasty);
        if (lasty >= 0) r.L(lasty) = make_short2((short)firsty, last2.y);
        last1 = last2;
        last2 = make_short2(cur.y, (short)lasty);
        lasty = firsty;
        firsty = cur.x;
        top = max(1, top + 1);
        cur = firsty >= 0 ? make_short2(r.L(firsty).x, r.C(firsty)) : make_short2(kMarker, kMarker);
    }
    // head and tail pointers of the merged band
    firsty = band1 * B;
    lasty = band2 * B;
    cur = r.L(firsty);
    if (cur.y == kMarker && cur.x < 0) {
        const short2 l = r.L(lasty);
        cur.x = l.y == kMarker ? l.x : (short)lasty;
        r.L(firsty) = cur;
    }
    firsty = band1 * B + B - 1;
    lasty = band2 * B + B - 1;
    cur = r.L(lasty);
    if (cur.x == kMarker && cur.y < 0) {
        const short2 l = r.L(firsty);
        cur.y = l.x == kMarker ? l.y : (short)firsty;
        r.L(lasty) = cur;
    }
}

// kernelColor's walk (:467-486) from the list position lasty for pixel ty:
// move on towards the head while the squared distance does not grow.
// Returns the final list position (the site's x); its row is col(x).x.
__device__ __forceinline__ int walk(const Row& r, int lasty, int ty) {
    short2 last2 = r.col(lasty), last1 = make_short2(0, 0);
    if (last2.y >= 0) last1 = r.col(last2.y);
    int dx = last2.x - r.line, dy = lasty - ty;
    unsigned best = (unsigned)(dx * dx + dy * dy);
    while (last2.y >= 0) {
        dx = last1.x - r.line;
        dy = last2.y - ty;
        const unsigned dist = (unsigned)(dx * dx + dy * dy);
        if (dist > best) break;
        best = dist;
        lasty = last2.y;
        last2 = last1;
        if (last2.y >= 0) last1 = r.col(last2.y);
    }
    return lasty;
}

// 2 x (x_b - x_a) c, where c is the position at which list entries a < b
// (positions) are equally far: entry a is at least as near as b for pixel
// p exactly when 2 (x_b - x_a) p <= num(a, b).
__device__ __forceinline__ long long crossing_num(const Row& r, int xa, int xb) {
    const long long ha = r.C(xa) - r.line, hb = r.C(xb) - r.line;
    return (long long)xb * xb - (long long)xa * xa + hb * hb - ha * ha;
}

// Coloring (kernelColor).  The reference's groups of m3 pixels each start
// from the state the previous group's last pixel reached.  When the list's
// exact crossing points increase strictly, the squared distances along the
// list fall and then rise for every pixel, with at most two equal minima
// next to each other, so every walk that starts on the tail side of the
// minimum -- as each group's does -- stops at the head-most nearest entry:
// a binary search over the crossing points finds it.  Rows whose list
// breaks that order (entries kept by the FP32 bisector tests that are
// nowhere strictly nearest) replay the groups' chain of states exactly.
__device__ void color(const Row& r, int m3, int lane, unsigned* status) {
    const int W = r.W;
    // list entries in position order (the list's order)
    int n = 0;
    for (int c0 = 0; c0 < W; c0 += 32) {
        const bool on = c0 + lane < W && r.A(c0 + lane) != 0;
        const unsigned m = __ballot_sync(kFull, on);
        if (on) r.E(n + __popc(m & ((1u << lane) - 1))) = (int16_t)(c0 + lane);
        n += __popc(m);
    }
    __syncwarp();
    bool ordered = true;
    for (int i = lane; i + 2 < n; i += 32) {
        const int x0 = r.E(i), x1 = r.E(i + 1), x2 = r.E(i + 2);
        // num01 / (2 (x1 - x0)) < num12 / (2 (x2 - x1))
        if (!(crossing_num(r, x0, x1) * (x2 - x1) < crossing_num(r, x1, x2) * (x1 - x0))) ordered = false;
    }
    ordered = __all_sync(kFull, ordered);
    if (n == 0) {
        // no site on the row (only when the image has none): the reference
        // reads its list head outside the texture and colors every pixel
        // with (x, y) = (-1, 0)
        for (int p = lane; p < W; p += 32) r.S(p) = -1;
    } else if (ordered) {
        const int chunk = (W + 31) / 32;
        const int p0 = lane * chunk, p1 = min(p0 + chunk, W);
        // first entry i with 2 (x_{i+1} - x_i) p0 <= num(i, i+1)
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const int xa = r.E(mid), xb = r.E(mid + 1);
            if (2ll * (xb - xa) * p0 <= crossing_num(r, xa, xb))
                hi = mid;
            else
                lo = mid + 1;
        }
        int i = lo;
        for (int p = p0; p < p1; ++p) {
            while (i < n - 1) {
                const int xa = r.E(i), xb = r.E(i + 1);
                if (2ll * (xb - xa) * p <= crossing_num(r, xa, xb)) break;
                ++i;
            }
            r.S(p) = r.E(i);
        }
    } else {
        if (lane == 0) {
            atomicAdd(status, 1u);
            int lasty = W - 1;
            const short2 tail = r.col(lasty);
            if (tail.x == kMarker) lasty = tail.y;
            for (int k = 0; k < W / m3; ++k) {
                r.st[k] = lasty;
                lasty = walk(r, lasty, W - (k + 1) * m3);
            }
        }
        __syncwarp();
        for (int p = lane; p < W; p += 32) r.S(p) = (int16_t)walk(r, r.st[(W - 1 - p) / m3], p);
    }
    __syncwarp();
}

__device__ __forceinline__ float plerp1(float v0, float t) { return (1.0f - t) * v0 + t * 1.0f; }

__global__ void __launch_bounds__(kRowThreads) k_pba_rows(const RowArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int line = blockIdx.x * a.wpb + warp;
    if (line >= a.H) return;  // whole warps only; the kernel has no block barrier
    const int W = a.W;
    unsigned char* base = smem + (size_t)warp * a.per_warp;
    const RowLayout lay = row_layout(W, a.m3);
    Row r;
    r.W = W;
    r.line = line;
    r.cand = reinterpret_cast<int16_t*>(base + lay.cand);
    r.lk = reinterpret_cast<short2*>(base + lay.lk);
    r.ic = reinterpret_cast<float*>(base + lay.ic);
    r.site = reinterpret_cast<int16_t*>(base + lay.site);
    r.ex = reinterpret_cast<int16_t*>(base + lay.ex);
    r.alive = base + lay.alive;
    r.st = reinterpret_cast<int*>(base + lay.st);
    r.cm = reinterpret_cast<unsigned*>(base + lay.cm);
    const uint4* src = reinterpret_cast<const uint4*>(a.cols + (size_t)line * W);
    for (int i = lane; i < W / 8; i += 32) reinterpret_cast<uint4*>(r.cand)[i] = src[i];
    for (int i = lane; i < (lay.st - lay.alive) / 4; i += 32) reinterpret_cast<unsigned*>(r.alive)[i] = 0u;
    __syncwarp();
    for (int c0 = 0; c0 < W; c0 += 32) {
        const unsigned m = __ballot_sync(kFull, c0 + lane < W && r.C(c0 + lane) != kMarker);
        if (lane == 0) r.cm[c0 >> 5] = m;
    }
    __syncwarp();
    // pba2DPhase2: band stacks and links, then the merges
    const int B2 = W / a.m2;
    for (int b = lane; b < a.m2; b += 32) {
        proximate(r, b * B2, B2);
        forward(r, b * B2, B2);
    }
    __syncwarp();
    for (int nb = a.m2; nb > 1; nb /= 2) {
        const int B = W / nb;
        for (int pr = lane; pr < nb / 2; pr += 32) merge(r, 2 * pr, B);
        __syncwarp();
    }
    // pba2DPhase3
    color(r, a.m3, lane, a.status);
    const size_t row = (size_t)line * W;
    for (int p = lane; p < W; p += 32) {
        const int sx = r.S(p);
        a.nearest[row + p] = make_short2((short)sx, (short)r.col(sx).x);
    }
}

struct NormArgs {
    const short2* nearest;
    const float4* image;
    const float4* position;
    float* out4;
    int W, H;
    float penumbra, intensity, thr;  // thr: the largest float <= 0.0005
};

// pbaNormalizeDistanceTransform (pba2DKernel.h:541-569), one thread per
// pixel: the distance between the pixel's and its site's positions; outside
// the penumbra (site not lit-facing, depths apart, farther than penumbra / 2)
// the hard value stays, otherwise plerp(0.5 -/+ distance / penumbra, 1,
// intensity) for umbra / lit pixels.  tex2D clamps the site's coordinates.
__global__ void __launch_bounds__(256) k_edt_normalize(const NormArgs a) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= a.W || y >= a.H) return;
    const size_t q = (size_t)y * a.W + x;
    const short2 n = a.nearest[q];
    const int cx = min(max((int)n.x, 0), a.W - 1), cy = min(max((int)n.y, 0), a.H - 1);
    const size_t qs = (size_t)cy * a.W + cx;
    const float4 ip = __ldg(a.image + q), sp = __ldg(a.image + qs);
    const float4 p1 = __ldg(a.position + q), p2 = __ldg(a.position + qs);
    const float dx = p1.x - p2.x, dy = p1.y - p2.y, dz = p1.z - p2.z;
    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    float v;
    if (sp.z != 1.0f || fabsf(linearize(sp.y) - linearize(ip.y)) > a.thr || dist > a.penumbra / 2.0f)
        v = ip.x;
    else if (ip.x == a.intensity)
        v = plerp1(0.5f - dist / a.penumbra, a.intensity);
    else
        v = plerp1(0.5f + dist / a.penumbra, a.intensity);
    *reinterpret_cast<float2*>(a.out4 + 4 * q) = make_float2(v, ip.y);
}

// ---- the screen-space mean filter of filterHardShadowsUsingEDT --------------
// MeanFilter.frag, one pass per launch (main.cpp:424-447: x into a scratch
// target, then y).  Per geometry pixel: kernelCenter = dscreen * order * 50
// / (deye * 2) with deye = -(MV * vertex).z and dscreen = 1 / (2 tan(fov /
// 2)) (fov = 45 passed to GLSL's tan, i.e. 45 radians, computed once on the
// host); samples from -kernelCenter in steps of 1 while <= kernelCenter, each
// read at centre + dir * sample / size and replaced by the centre value when
// it is 0 or its linearised depth differs by >= 0.0005; the mean of the
// samples in channel 0, the centre's depth in channel 1.  Pass 1 reads the
// EDT image GL_NEAREST (texel floor(u * size)), pass 2 reads the x pass
// bilinearly at level 0 along the filtered axis (its GL_LINEAR_MIPMAP_LINEAR
// level is the driver's choice), each at the pixel's own row or column on
// the other axis; both with a zero border.  A window is cut at 2049 samples,
// which only a vertex at eye depth < 0.16 (nearer than the camera's near
// plane at 1) could reach.
struct MeanArgs {
    const float4* image;  // pass 1: the EDT image; pass 2: the x pass
    const float4* pos;    // G-buffer vertex (x == 0: background)
    float4* out;
    int W, H, order;
    float dscreen;
    float mv[16];
};

__device__ __forceinline__ float gl_lin(float depth) { return 2.0f / (1001.0f - depth * 999.0f); }

template <bool VERTICAL>
__global__ void __launch_bounds__(256) k_edt_mean_filter(const MeanArgs a) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= a.W || y >= a.H) return;
    const size_t q = (size_t)y * a.W + x;
    const float4 v = __ldg(a.pos + q);
    if (v.x == 0.0f) {  // discard: the target keeps its clear colour
        a.out[q] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        return;
    }
    const float4 color = __ldg(a.image + q);  // the centre texel (exact in both passes)
    const float* m = a.mv;
    const float ez = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    const float deye = -ez;
    const float kc = (a.dscreen * (float)a.order * 50.0f) / (deye * 2.0f);
    const float step = VERTICAL ? 1.0f / (float)a.H : 1.0f / (float)a.W;
    const float cs = ((float)(VERTICAL ? y : x) + 0.5f) / (float)(VERTICAL ? a.H : a.W);
    const float Lc = gl_lin(color.y);
    const float size = (float)(VERTICAL ? a.H : a.W);
    float sum = 0.0f;
    int count = 0;
    const float lo = -kc;
    for (float sample = lo; sample <= kc && count < 2049; sample = sample + 1.0f) {
        const float u = cs + sample * step;
        float r = 0.0f, g = 0.0f;
        if (!VERTICAL) {
            const float fi = floorf(u * size);
            if (fi >= 0.0f && fi < size) {
                const float4 t = __ldg(a.image + (size_t)y * a.W + (int)fi);
                r = t.x;
                g = t.y;
            }
        } else {
            const float uu = u * size - 0.5f;
            const float f0 = floorf(uu), w1 = uu - f0, w0 = 1.0f - w1;
            const int j0 = (int)f0;
            float4 t0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), t1 = t0;
            if (j0 >= 0 && j0 < a.H) t0 = __ldg(a.image + (size_t)j0 * a.W + x);
            if (j0 + 1 >= 0 && j0 + 1 < a.H) t1 = __ldg(a.image + (size_t)(j0 + 1) * a.W + x);
            r = w0 * t0.x + w1 * t1.x;
            g = w0 * t0.y + w1 * t1.y;
        }
        // adjustColor (MeanFilter.frag:27-36)
        if (r == 0.0f || fabsf(gl_lin(g) - Lc) >= 0.0005f) r = color.x;
        sum = sum + r;
        ++count;
    }
    sum = sum / (float)count;
    a.out[q] = make_float4(sum, color.y, 0.0f, 0.0f);
}

// largest float not above c
float float_at_most(double c) {
    float t = (float)c;
    if ((double)t > c) t = nextafterf(t, -INFINITY);
    return t;
}

template <class K>
gi_status set_smem(K kernel, int bytes) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "pba rows shared memory");
}

}  // namespace edt

gi_status launch_edt_mean_filter(gi_context* ctx, const float camera_mv[16], const float* d_image,
                                 const float* d_pos, int W, int H, int order, float* d_out, cudaStream_t st) {
    using namespace edt;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_edt_meanx), &ctx->cap_edt_meanx,
                                (size_t)W * H * sizeof(float4));
    if (s != GI_OK) return s;
    MeanArgs a;
    a.pos = reinterpret_cast<const float4*>(d_pos);
    a.W = W;
    a.H = H;
    a.order = order;
    // dscreen = 1 / (2 tan(fov / 2)) with the float uniform fov = 45 read by
    // GLSL's tan as radians (MyGLGeometryViewer.cpp:6,119-120)
    a.dscreen = 1.0f / (2.0f * (float)std::tan((double)(45.0f / 2.0f)));
    for (int k = 0; k < 16; ++k) a.mv[k] = camera_mv[k];
    const dim3 grid((W + 31) / 32, (H + 7) / 8);
    a.image = reinterpret_cast<const float4*>(d_image);
    a.out = reinterpret_cast<float4*>(ctx->d_edt_meanx);
    k_edt_mean_filter<false><<<grid, 256, 0, st>>>(a);
    a.image = a.out;
    a.out = reinterpret_cast<float4*>(d_out);
    k_edt_mean_filter<true><<<grid, 256, 0, st>>>(a);
    ctx->launches += 2;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "EDT mean filter launch");
}

gi_status pba_check_shape(int W, int H, int m1, int m2, int m3, const char* who) {
    const std::string w(who);
    if (W < 8 || H < 2 || W > 8192 || H > edt::kSegs * edt::kMaxSegRows || W % 8 != 0)
        return fail(GI_ERR_INVALID_ARG, w + ": width must be a multiple of 8 in [8, 8192], height in [2, 8192]");
    if (m1 < 1 || H % m1 != 0 || H / m1 < 2)
        return fail(GI_ERR_INVALID_ARG, w + ": phase-1 bands must divide the height into bands of >= 2 rows");
    if (m2 < 1 || (m2 & (m2 - 1)) != 0 || W % m2 != 0 || W / m2 < 2)
        return fail(GI_ERR_INVALID_ARG,
                    w + ": phase-2 bands must be a power of two dividing the width into bands of >= 2 pixels");
    if (m3 < 1 || W % m3 != 0) return fail(GI_ERR_INVALID_ARG, w + ": phase-3 groups must divide the width");
    return GI_OK;
}

gi_status launch_pba(gi_context* ctx, const int16_t* d_sites, const float* d_image, const float* d_position,
                     int W, int H, int m1, int m2, int m3, float penumbra, float intensity, int16_t* d_nearest,
                     float* d_out4, cudaStream_t st) {
    using namespace edt;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_pba_cols), &ctx->cap_pba_cols,
                                (size_t)W * H * sizeof(int16_t));
    if (s != GI_OK) return s;
    ColArgs ca;
    ca.sites = reinterpret_cast<const short2*>(d_sites);
    ca.image = reinterpret_cast<const float4*>(d_image);
    ca.cols = ctx->d_pba_cols;
    ca.W = W;
    ca.H = H;
    ca.S = (H + kSegs - 1) / kSegs;
    ca.band = H / m1;
    ca.thr = float_at_most(0.0025);
    const dim3 cgrid((W + kColW - 1) / kColW);
    if (d_sites)
        k_pba_columns<kFromSites><<<cgrid, kColThreads, 0, st>>>(ca);
    else
        k_pba_columns<kFromImage><<<cgrid, kColThreads, 0, st>>>(ca);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "pba columns launch");

    short2* near = reinterpret_cast<short2*>(d_nearest);
    if (!near) {
        s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_pba_near), &ctx->cap_pba_near,
                          (size_t)W * H * sizeof(short2));
        if (s != GI_OK) return s;
        near = reinterpret_cast<short2*>(ctx->d_pba_near);
    }
    RowArgs ra;
    ra.cols = ctx->d_pba_cols;
    ra.W = W;
    ra.H = H;
    ra.m2 = m2;
    ra.m3 = m3;
    ra.per_warp = row_layout(W, m3).bytes;
    // two rows per CTA spread the rows over every SM
    ra.wpb = max(1, min(2, (200 * 1024) / ra.per_warp));
    ra.nearest = near;
    ra.status = ctx->d_status + 96;
    const int smem = ra.per_warp * ra.wpb;
    s = set_smem(k_pba_rows, smem);
    if (s != GI_OK) return s;
    k_pba_rows<<<dim3((H + ra.wpb - 1) / ra.wpb), ra.wpb * 32, smem, st>>>(ra);
    ctx->launches++;
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "pba rows launch");
    if (!d_out4) return GI_OK;
    NormArgs na;
    na.nearest = near;
    na.image = reinterpret_cast<const float4*>(d_image);
    na.position = reinterpret_cast<const float4*>(d_position);
    na.out4 = d_out4;
    na.W = W;
    na.H = H;
    na.penumbra = penumbra;
    na.intensity = intensity;
    na.thr = float_at_most(0.0005);
    k_edt_normalize<<<dim3((W + 31) / 32, (H + 7) / 8), 256, 0, st>>>(na);
    ctx->launches++;
    e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "EDT normalise launch");
}

}  // namespace gi
