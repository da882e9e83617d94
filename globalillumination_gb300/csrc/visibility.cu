// visibility.cu -- per-pixel shadow visibility kernels for sm_103a.
//
// One thread per camera pixel reads the G-buffer (object position and
// normal+frontFacing, float4 each) and the light-view depth map, and writes
// the r channel of the visibility target.  Each technique restates a
// fragment shader of the reference (paths relative to the reference root):
//   HARD            ShadowMapping/Shaders/Shadow.frag:240-272 (naive == 1)
//   PCF             Shadow.frag:86-116 (bilinearPCF: NEAREST taps)
//   PCF_TRICUBIC    Shadow.frag:41-116 (textureBicubic over NEAREST taps)
//   PCSS_GRID       SoftShadowMapping/Shaders/SoftShadow/PlausibleSoftShadow.frag
//                   :166-194, 365-398, 556-563, 605-633
//   PCSS_POISSON    the same blocker / penumbra / filter structure with
//                   Poisson-disk taps (no reference counterpart)
//   SMSR_*, RPCF_*, RSMSS
//                   ShadowMapping/Shaders/RBSM/{Conservative,NonConservative}SMSR.frag,
//                   FilteredRBSM.frag
//   HARD_SOFTAPP    SoftShadowMapping/Shaders/HardShadow/HardShadow.frag:35-58
//   RBSSM           SoftShadowMapping/Shaders/SoftShadow/RBSSM.frag:25-35,
//                   193-1117, 1202-1376 (PCSS blocker search, then K x K
//                   taps filled by the discontinuity-space smoothing)
// plus the normal-orientation pre-test every one of them runs
// (Shadow.frag:222-238).  The file is compiled with -fmad=false and IEEE
// division / square root so each FP32 operation rounds once, in the order
// written, exactly as the CPU oracle does.
//
// Texture fetches are GL_NEAREST with CLAMP_TO_BORDER and border depth 0
// (MyGLTextureViewer.cpp:3-28): texel (floor(s W), floor(t H)), outside the
// map (or NaN) reads 0.  Blocks are 32 x 4 pixels so a warp reads one
// coalesced row segment of the G-buffer and its taps land on neighbouring
// texels of the map (L1 / L2 hits: a 2048^2 map is 16 MiB and stays in L2).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "internal.h"
#include "minmax.h"
#include "raster.h"
#include "raster_common.cuh"

namespace gi {

const float kPoissonDisk[64][2] = {
#include "poisson_table.inc"
};

namespace vis {

__constant__ float2 c_poisson[64] = {
#include "poisson_table.inc"
};

struct V4 {
    float x, y, z, w;
};
struct V2 {
    float x, y;
};

__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ float gfract(float x) { return x - floorf(x); }

struct PoissonOffsets;

struct Ctx {
    const float* __restrict__ map;
    int W, H;
    float fW, fH;
    float sx, sy;
    float I;
    SoftMaps sm;  // moment soft shadows only
    // PCSS_POISSON: the blocker taps' offsets c_poisson[i] * bsw, rounded as
    // the multiplication rounds them, computed once per launch (nullptr:
    // multiply per tap)
    const float2* boff = nullptr;
    // the launch's offset table and pyramid (nullptr: run every tap)
    const PoissonOffsets* tab = nullptr;
};

// The blocker-search offsets of one launch, a kernel parameter read in place,
// with the extreme offsets of the blocker and filter taps (componentwise
// minimum and maximum: the blocker offsets as rounded products, the filter's
// Poisson points before their scale by the penumbra width) and the light
// map's min-max pyramid (levels 0: none).
struct PoissonOffsets {
    float2 b[64];
    float2 bmin, bmax, fmin, fmax;
    // PCF: the first and last offsets of the tap loop (in texels) and the
    // number of taps (0: no skipping)
    float pcf_lo, pcf_hi;
    int pcf_count;
    Pyramid pyr;
};

__device__ __forceinline__ float fetch(const Ctx& c, float s, float t) {
    float fi = floorf(s * c.fW);
    float fj = floorf(t * c.fH);
    if (!(fi >= 0.0f && fi < c.fW && fj >= 0.0f && fj < c.fH)) return 0.0f;
    return __ldg(c.map + (size_t)(int)fj * c.W + (int)fi);
}

__device__ __forceinline__ V4 mat4_mul(const float* m, V4 v) {
    V4 r;
    r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return r;
}

__device__ __forceinline__ float pretest(const gi_vis_params& p, const Ctx& c, V4 vertex, V4 normal) {
    if (p.pretest == GI_PRETEST_OFF) return 1.0f;
    V4 ev = mat4_mul(p.camera_mv, vertex);
    const float* nm = p.normal_matrix;
    float nx = nm[0] * normal.x + nm[3] * normal.y + nm[6] * normal.z;
    float ny = nm[1] * normal.x + nm[4] * normal.y + nm[7] * normal.z;
    float nz = nm[2] * normal.x + nm[5] * normal.y + nm[8] * normal.z;
    float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
    nx = nx * inv;
    ny = ny * inv;
    nz = nz * inv;
    float lx = p.light_position[0] - ev.x;
    float ly = p.light_position[1] - ev.y;
    float lz = p.light_position[2] - ev.z;
    float linv = 1.0f / sqrtf(lx * lx + ly * ly + lz * lz);
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

// Same texel as fetch() when s * W and t * H are not NaN: floor-convert
// (out-of-range values saturate and fail the unsigned range check, -0
// becomes 0 as floorf(-0) >= 0 does).  Callers use it only when every
// input of the tap coordinates is finite, so no coordinate can be NaN.
__device__ __forceinline__ float fetch_finite(const Ctx& c, float s, float t) {
    const int ix = __float2int_rd(s * c.fW);
    const int iy = __float2int_rd(t * c.fH);
    if ((unsigned)ix >= (unsigned)c.W || (unsigned)iy >= (unsigned)c.H) return 0.0f;
    return __ldg(c.map + (iy * c.W + ix));
}

// Exact tap skipping.  The taps at (sx, sy) = (n.x + o.x, n.y + o.y) for
// offsets o in [lo, hi] (componentwise) read texels inside the box
// [floor(sx0 W), floor(sx1 W)] x [floor(sy0 H), floor(sy1 H)], where sx0 /
// sx1 are the coordinates of the smallest / largest offset computed with the
// taps' own operations: float addition, multiplication by a positive scale
// and floor are monotone, so no tap leaves the box.  Gives the minimum and
// maximum of the map over the box from the pyramid (at the level where the
// box spans at most 2 x 2 cells); false when the box leaves the map (border
// texels read 0) or is wider than the pyramid's top level.  Boxes of at
// most 3 x 3 texels are read from the map itself, so they need no pyramid.
__device__ __forceinline__ bool tap_box_minmax(const Ctx& c, float sx0, float sx1, float sy0, float sy1, float& mn,
                                               float& mx) {
    const int x0 = __float2int_rd(sx0 * c.fW), x1 = __float2int_rd(sx1 * c.fW);
    const int y0 = __float2int_rd(sy0 * c.fH), y1 = __float2int_rd(sy1 * c.fH);
    if (x0 < 0 || y0 < 0 || x1 >= c.W || y1 >= c.H) return false;
    if (x1 - x0 <= 2 && y1 - y0 <= 2) {
        // at most 3 x 3 texels (the blocker box of PCSS up to 2048^2 maps,
        // 5 x 5 PCF): read them from the map
        mn = __int_as_float(0x7f800000);
        mx = -mn;
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const float v = __ldg(c.map + (y * c.W + x));
                mn = fminf(mn, v);
                mx = fmaxf(mx, v);
            }
        return true;
    }
    const int span = max(x1 - x0, y1 - y0);
    const int L = 32 - __clz(span);  // 2^L > span: at most two cells per axis
    if (L > c.tab->pyr.levels) return false;
    const float2* lv = c.tab->pyr.lv[L];
    const int w = c.W >> L;
    const int cx0 = x0 >> L, cx1 = x1 >> L, cy0 = y0 >> L, cy1 = y1 >> L;
    const float2 a = __ldg(lv + (cy0 * w + cx0)), b = __ldg(lv + (cy0 * w + cx1));
    const float2 d = __ldg(lv + (cy1 * w + cx0)), e = __ldg(lv + (cy1 * w + cx1));
    mn = fminf(fminf(a.x, b.x), fminf(d.x, e.x));
    mx = fmaxf(fmaxf(a.y, b.y), fmaxf(d.y, e.y));
    return true;
}

__device__ __forceinline__ bool finite3(float a, float b, float d) {
    return isfinite(a) && isfinite(b) && isfinite(d);
}

// ---- Shadow.frag -------------------------------------------------------------
template <bool FAST>
__device__ float pcf_bilinear_t(const gi_vis_params& p, const Ctx& c, V4 n) {
    float incrW = 1.0f / c.fW, incrH = 1.0f / c.fH;
    float illum = 0.0f;
    if (FAST && c.tab && c.tab->pcf_count > 0) {
        // the loop's offsets increase from pcf_lo to pcf_hi; incr > 0
        const float lo = c.tab->pcf_lo, hi = c.tab->pcf_hi;
        float mn, mx;
        if (tap_box_minmax(c, n.x + lo * incrW, n.x + hi * incrW, n.y + lo * incrH, n.y + hi * incrH, mn, mx)) {
            const int count = c.tab->pcf_count;
            if (n.z <= mn) return 1.0f;  // every tap lit: count additions of 1, over count
            if (n.z > mx) {              // every tap shadowed
                for (int k = 0; k < count; ++k) illum += c.I;
                return illum / (float)count;
            }
        }
    }
    float offset = (float)p.penumbra_size;
    float step = 2.0f * offset / (float)p.kernel_order;
    int count = 0;
    for (float w = -offset; w < offset; w += step)
        for (float h = -offset; h < offset; h += step) {
            const float s = n.x + w * incrW, t = n.y + h * incrH;
            float d = FAST ? fetch_finite(c, s, t) : fetch(c, s, t);
            if (n.z <= d) illum = illum + 1.0f;
            else illum += c.I;
            count++;
        }
    return illum / (float)count;
}

__device__ float pcf_bilinear(const gi_vis_params& p, const Ctx& c, V4 n) {
    // offsets are finite (kernel_order, penumbra_size >= 1), so finite n.x,
    // n.y give finite tap coordinates
    return (isfinite(n.x) && isfinite(n.y)) ? pcf_bilinear_t<true>(p, c, n) : pcf_bilinear_t<false>(p, c, n);
}

__device__ __forceinline__ void cubic(float v, float out[4]) {
    float nn[4] = {1.0f - v, 2.0f - v, 3.0f - v, 4.0f - v};
    float s[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) s[i] = nn[i] * nn[i] * nn[i];
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

__device__ float texture_bicubic(const Ctx& c, float u, float v) {
    float tsx = c.fW, tsy = c.fH;
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
#pragma unroll
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

__device__ float pcf_tricubic(const gi_vis_params& p, const Ctx& c, V4 n) {
    float incrW = 1.0f / c.fW, incrH = 1.0f / c.fH;
    float illum = 0.0f;
    float offset = (float)p.penumbra_size;
    float step = 2.0f * offset / (float)p.kernel_order;
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

// ---- PlausibleSoftShadow.frag --------------------------------------------------
__device__ __forceinline__ float blocker_search_width(const gi_vis_params& p, const Ctx& c) {
    float R = p.light_radius;
    if (c.fW <= 1024.0f) return R / c.fW;
    return R / 1024.0f;
}

// The tap offsets of the reference's grid loops, for (int k = (int)(-fw);
// (float)k <= fw; k++) ... ((float)k * width) / fw: each depends on k alone,
// so they are computed once (at most 63: grid sizes are capped at 63) and
// both axes read them; the taps get the same numbers as when every tap
// divided for itself.
struct GridTaps {
    float o[64];
    int n;
};

__device__ __forceinline__ void grid_taps(float width, float fw, GridTaps& g) {
    g.n = 0;
    for (int k = (int)(-fw); (float)k <= fw && g.n < 64; k++) g.o[g.n++] = ((float)k * width) / fw;
}

__device__ float avg_blocker_grid(const gi_vis_params& p, const Ctx& c, V4 n) {
    float avg = 0.0f;
    int nb = 0;
    float bsw = blocker_search_width(p, c);
    float fw = ((float)p.blocker_search_size - 1.0f) * 0.5f;
    GridTaps g;
    grid_taps(bsw, fw, g);
    for (int hi = 0; hi < g.n; hi++)
        for (int wi = 0; wi < g.n; wi++) {
            float d = fetch(c, n.x + g.o[wi], n.y + g.o[hi]);
            if (n.z > d) {
                avg += d;
                nb++;
            }
        }
    return nb == 0 ? 1.0f : avg / (float)nb;
}

template <bool FAST>
__device__ float avg_blocker_poisson_t(const gi_vis_params& p, const Ctx& c, V4 n, float bsw) {
    const float2* bo = c.boff;
    if (FAST && bo && c.tab) {
        // no texel the taps can reach is below z: no tap finds a blocker
        const float2 lo = c.tab->bmin, hi = c.tab->bmax;
        float mn, mx;
        if (tap_box_minmax(c, n.x + lo.x, n.x + hi.x, n.y + lo.y, n.y + hi.y, mn, mx) && n.z <= mn) return 1.0f;
    }
    float avg = 0.0f;
    int nb = 0;
    for (int i = 0; i < p.poisson_blocker_taps; ++i) {
        float s, t;
        if (bo) {
            const float2 ob = bo[i];
            s = n.x + ob.x;
            t = n.y + ob.y;
        } else {
            const float2 o = c_poisson[i];
            s = n.x + o.x * bsw;
            t = n.y + o.y * bsw;
        }
        float d = FAST ? fetch_finite(c, s, t) : fetch(c, s, t);
        if (n.z > d) {
            avg += d;
            nb++;
        }
    }
    return nb == 0 ? 1.0f : avg / (float)nb;
}

template <bool FAST>
__device__ float pcss_filter_poisson_t(const gi_vis_params& p, const Ctx& c, float pw, V4 n) {
    float illum = 0.0f;
    const int nf = p.poisson_filter_taps;
    if (FAST && c.tab) {
        // pw > 0 here (the caller checked the step), so o.x * pw is monotone in o.x
        const float2 lo = c.tab->fmin, hi = c.tab->fmax;
        float mn, mx;
        if (tap_box_minmax(c, n.x + lo.x * pw, n.x + hi.x * pw, n.y + lo.y * pw, n.y + hi.y * pw, mn, mx)) {
            if (n.z <= mn) return 1.0f;  // every tap lit: nf additions of 1, over nf
            if (n.z > mx) {              // every tap shadowed: the same additions of I
                for (int j = 0; j < nf; ++j) illum += c.I;
                return illum / (float)nf;
            }
        }
    }
    for (int j = 0; j < nf; ++j) {
        float2 o = c_poisson[j];
        const float s = n.x + o.x * pw, t = n.y + o.y * pw;
        float d = FAST ? fetch_finite(c, s, t) : fetch(c, s, t);
        if (n.z <= d) illum = illum + 1.0f;
        else illum += c.I;
    }
    return illum / (float)nf;
}

__device__ __forceinline__ float penumbra_width(const gi_vis_params& p, float avg, float z) {
    if (avg < p.pcss_min_blocker_depth) return 0.0f;
    float pw = ((z - avg) / avg) * p.light_radius;
    return (p.znear * pw) / z;
}

__device__ float pcss_filter_grid(const gi_vis_params& p, const Ctx& c, float pw, V4 n) {
    float illum = 0.0f;
    int K = p.kernel_size;
    float step = 2.0f * pw / (float)K;
    float fw = ((float)K - 1.0f) * 0.5f;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    GridTaps g;
    grid_taps(pw, fw, g);
    for (int hi = 0; hi < g.n; hi++)
        for (int wi = 0; wi < g.n; wi++) {
            float d = fetch(c, n.x + g.o[wi], n.y + g.o[hi]);
            if (n.z <= d) illum = illum + 1.0f;
            else illum += c.I;
        }
    return illum / (float)(K * K);
}


// ---- RBSM/NonConservativeSMSR.frag and FilteredRBSM.frag -----------------------
__device__ V4 nc_get_disc_all(const Ctx& c, V4 n) {
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

__device__ bool nc_get_disc_type(const Ctx& c, V4 n, V2 dir, float disc_type) {
    if (dir.x == 0.0f) {
        n.x -= c.sx;
        float left = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (fabsf(left - disc_type) == 0.0f) return true;
        n.x += 2.0f * c.sx;
        float right = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (fabsf(right - disc_type) == 0.0f) return true;
        n.x -= c.sx;
    }
    if (dir.y == 0.0f) {
        n.y += c.sy;
        float bottom = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (fabsf(bottom - disc_type) == 0.0f) return true;
        n.y -= 2.0f * c.sy;
        float top = (n.z <= fetch(c, n.x, n.y)) ? 1.0f : 0.0f;
        if (fabsf(top - disc_type) == 0.0f) return true;
    }
    return false;
}

__device__ __forceinline__ bool nc_probe(const Ctx& c, float thr, V4& n, V4 dt, float& new_depth,
                                         float s, float t) {
    float d = fetch(c, s, t);
    if (dt.z == 1.0f) {
        if (fabsf(n.z - d) < thr) {
            n.z -= thr;
            new_depth = n.z;
        }
    }
    float v = (n.z <= d) ? 1.0f : 0.0f;
    return fabsf(v - dt.z) == 0.0f;
}

__device__ bool nc_get_disc_vec(const Ctx& c, float thr, V4 n, V2 dir, V4 dt, float& new_depth) {
    V4 rel = n;
    new_depth = n.z;
    if (dir.x == 0.0f) {
        if (dt.x == 0.5f || dt.x == 0.75f) {
            rel.x = n.x - c.sx;
            if (nc_probe(c, thr, n, dt, new_depth, rel.x, rel.y)) return true;
        }
        if (dt.x == 0.75f || dt.x == 0.25f) {
            rel.x = n.x + c.sx;
            if (nc_probe(c, thr, n, dt, new_depth, rel.x, rel.y)) return true;
        }
    }
    if (dir.y == 0.0f) {
        if (dt.y == 0.5f || dt.y == 0.75f) {
            rel.y = n.y + c.sy;
            if (nc_probe(c, thr, n, dt, new_depth, rel.x, rel.y)) return true;
        }
        if (dt.y == 0.75f || dt.y == 0.25f) {
            rel.y = n.y - c.sy;
            if (nc_probe(c, thr, n, dt, new_depth, rel.x, rel.y)) return true;
        }
    }
    return false;
}

__device__ float nc_disc_length(const gi_vis_params& p, const Ctx& c, V4 in_disc, V4 lc, V2 dir,
                                float sub) {
    V4 cc = lc;
    float found = 0.0f;
    float dist = 0.0f;
    float new_depth = 0.0f;
    V2 st = {dir.x * c.sx, dir.y * c.sy};
    cc.x += st.x;
    cc.y += st.y;
    const float thr = p.depth_threshold;
    for (int it = 0; it < p.max_search; it++) {
        float d = fetch(c, cc.x, cc.y);
        if (in_disc.z == 0.0f)
            if (fabsf(cc.z - d) < thr) cc.z -= thr;
        float center = (cc.z <= d) ? 1.0f : 0.0f;
        if (fabsf(center - in_disc.z) == 0.0f) {
            bool has = nc_get_disc_type(c, cc, V2{0.0f, 0.0f}, in_disc.z);
            found = has ? 1.0f : 0.0f;
            break;
        } else {
            bool has = nc_get_disc_vec(c, thr, cc, dir, in_disc, new_depth);
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

__device__ __forceinline__ float nc_rel_pos(const gi_vis_params& p, V2 dir, float shadow,
                                            bool filtered) {
    float T = 1.0f;
    if (dir.x < 0.0f && dir.y < 0.0f) T = 0.0f;
    if (dir.x > 0.0f && dir.y > 0.0f) T = -2.0f;
    float edge_len = gmin(fabsf(dir.x) + fabsf(dir.y), (float)p.max_search);
    if (filtered) return (T * fabsf(gmax(T * dir.x, T * dir.y))) / edge_len;
    return (gmax(T, 2.0f * shadow - 1.0f) * fabsf(gmax(T * dir.x, T * dir.y))) / edge_len;
}

__device__ __forceinline__ float nc_revectorize(V2 r, float shadow, bool filtered) {
    if (filtered) {
        if (r.x * r.y < 0.0f) return (1.0f - shadow) + (2.0f * shadow - 1.0f) * gmax(r.x, r.y);
        else if (r.x * r.y == 0.0f) return shadow;
        return gclamp((1.0f - shadow) + (2.0f * shadow - 1.0f) * (r.x + r.y), 0.0f, 1.0f);
    }
    if ((r.x * r.y == 2.0f * shadow) ||
        ((fabsf(r.x) * fabsf(r.y) > 0.0f) &&
         ((1.0f - shadow) + (2.0f * shadow - 1.0f) * (fabsf(r.x) + fabsf(r.y)) < 0.5f)))
        return 0.0f;
    return 1.0f;
}

__device__ __forceinline__ V4 nc_compute_disc(const Ctx& c, V4 n, float dist) {
    float center = (n.z <= dist) ? 1.0f : 0.0f;
    float disc_type = 1.0f - center;
    V4 dir = nc_get_disc_all(c, n);
    float dx = fabsf(dir.x - center), dy = fabsf(dir.y - center);
    float dz = fabsf(dir.z - center), dw = fabsf(dir.w - center);
    return V4{(2.0f * dx + dy) / 4.0f, (2.0f * dz + dw) / 4.0f, disc_type, 1.0f};
}

__device__ float nc_revectorized_tap(const gi_vis_params& p, const Ctx& c, V4 n, V4 disc,
                                     float shadow, bool filtered) {
    V2 sub = {gfract(n.x * c.fW), gfract(n.y * c.fH)};
    float l = nc_disc_length(p, c, disc, n, V2{-1.0f, 0.0f}, 1.0f - sub.x);
    float r = nc_disc_length(p, c, disc, n, V2{1.0f, 0.0f}, sub.x);
    float d = nc_disc_length(p, c, disc, n, V2{0.0f, -1.0f}, 1.0f - sub.y);
    float u = nc_disc_length(p, c, disc, n, V2{0.0f, 1.0f}, sub.y);
    V2 rr = {nc_rel_pos(p, V2{l, r}, shadow, filtered), nc_rel_pos(p, V2{d, u}, shadow, filtered)};
    return gmix(nc_revectorize(rr, shadow, filtered), 1.0f, c.I);
}

__device__ float nc_smsr(const gi_vis_params& p, const Ctx& c, V4 n) {
    float dist = fetch(c, n.x, n.y);
    V4 disc = nc_compute_disc(c, n, dist);
    float shadow = (n.z <= dist) ? 1.0f : 0.0f;
    if (disc.x > 0.0f || disc.y > 0.0f) {
        if (disc.x == 0.75f && disc.y == 0.75f) return gmix(1.0f - shadow, 1.0f, c.I);
        return nc_revectorized_tap(p, c, n, disc, shadow, false);
    }
    return gmix(shadow, 1.0f, c.I);
}

__device__ float nc_rpcf(const gi_vis_params& p, const Ctx& c, V4 n, bool filtered) {
    float incrW = 1.0f / c.fW, incrH = 1.0f / c.fH;
    float illum = 0.0f;
    float offset = (float)p.penumbra_size;
    float step = 2.0f * offset / (float)p.kernel_order;
    int count = 0;
    for (float w = -offset; w <= offset; w += step)
        for (float h = -offset; h <= offset; h += step) {
            V4 s = {n.x + w * incrW, n.y + h * incrH, n.z, n.w};
            float d = fetch(c, s.x, s.y);
            float shadow = (s.z <= d) ? 1.0f : 0.0f;
            V4 disc = nc_compute_disc(c, s, d);
            if (disc.x > 0.0f || disc.y > 0.0f) {
                illum += nc_revectorized_tap(p, c, s, disc, shadow, filtered);
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
__device__ __forceinline__ float gstep(float edge, float x) { return x < edge ? 0.0f : 1.0f; }

// compressPositiveDiscontinuity / decompressPositiveDiscontinuity
// (RBSSM.frag:25-35).
__device__ __forceinline__ float rb_compress(float nd) { return -2.0f - ((0.5f - nd) * 2.0f); }
__device__ __forceinline__ float rb_decompress(float nd) { return 0.5f - ((nd + 2.0f) * -1.0f) / 2.0f; }

__device__ __forceinline__ bool rb_disc_t(const Ctx& c, V4 n, float dx, float dy, float type) {
    return nc_get_disc_type(c, n, V2{dx, dy}, type);
}
__device__ __forceinline__ bool rb_disc_v(const gi_vis_params& p, const Ctx& c, V4 n, float dx, float dy,
                                          V4 type) {
    float unused = 0.0f;
    return nc_get_disc_vec(c, p.depth_threshold, n, V2{dx, dy}, type, unused);
}

// computeDiscontinuityLength (RBSSM.frag:193-253).
__device__ float rb_disc_length(const gi_vis_params& p, const Ctx& c, V4 in_disc, V4 lc, V2 dir) {
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
    const float thr = p.depth_threshold;
    for (int it = 0; it < p.max_search; it++) {
        float d = fetch(c, cc.x, cc.y);
        if (in_disc.z == 0.0f)
            if (fabsf(cc.z - d) < thr) cc.z -= thr;
        float center = (cc.z <= d) ? 1.0f : 0.0f;
        if (fabsf(center - in_disc.z) == 0.0f) {
            bool has = nc_get_disc_type(c, cc, V2{0.0f, 0.0f}, in_disc.z);
            found = has ? 1.0f : 0.0f;
            break;
        } else {
            bool has = nc_get_disc_vec(c, thr, cc, dir, in_disc, new_depth);
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
__device__ __forceinline__ float rb_normalize_space(const gi_vis_params& p, V2 dir, float sub) {
    if (dir.x < 0.0f && dir.y < 0.0f) return -1.0f;
    float edge = gmin(fabsf(dir.x) + fabsf(dir.y) - 1.0f, (float)p.max_search);
    float nd = 1.0f - gmax(dir.x, dir.y) / edge;
    if (dir.x == dir.y) nd += gmix(sub / edge, (1.0f - sub) / edge, gstep(0.5f, sub));
    else if (dir.x == gmax(dir.x, dir.y)) nd += (1.0f - sub) / edge;
    else nd += sub / edge;
    if (dir.x > 0.0f && dir.y > 0.0f) return rb_compress(nd);
    return nd;
}

// smoothONDS (RBSSM.frag:311-1117): the fill of one discontinuity tap.
// lc, nd and disc are by-value copies that the cases modify in place, as
// the shader does; a case that does not return leaves its changes for the
// cases below it.
__device__ __noinline__ float rb_smooth_onds(const gi_vis_params& p, const Ctx& c, V4 lc, V4 nd, V4 disc, V2 sub) {
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
                    if (top && bottom) return 0.0f;
                    lc.y += gmix(-sy, sy, gstep(1.0f, top ? 1.0f : 0.0f));
                    left = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, 0.0f});
                    right = !left;
                } else {
                    if (disc.y == 0.5f) top = false;
                    else if (disc.y == 0.25f) bottom = false;
                    lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
                    left = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    right = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                    if (left && right) {
                        if (nd.y <= -2.0f) nd.y = rb_decompress(nd.y) + 0.5f;
                        float a = gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f);
                        float b = gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f);
                        float cc = gmix(1.0f - sub.y, sub.y, gstep(disc.y, 1.0f));
                        return gmin(gmin(a, b), cc);
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
                    if (left && right) return 0.0f;
                    lc.x += gmix(sx, -sx, gstep(1.0f, left ? 1.0f : 0.0f));
                    bottom = rb_disc_v(p, c, lc, 0.0f, 0.25f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    top = !bottom;
                } else {
                    if (disc.x == 0.5f) right = false;
                    else if (disc.x == 0.25f) left = false;
                    lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                    bottom = rb_disc_v(p, c, lc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                    top = rb_disc_v(p, c, lc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                    if (bottom && top) {
                        if (nd.x <= -2.0f) nd.x = rb_decompress(nd.x) + 0.5f;
                        float a = gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f);
                        float b = gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f);
                        float cc = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 1.0f));
                        return gmin(gmin(a, b), cc);
                    }
                }
            }
            if (!left && !bottom) return gclamp((1.0f - sub.x) - (1.0f - sub.y), 0.0f, 1.0f);
            else if (!right && !bottom) return gclamp(sub.x - (1.0f - sub.y), 0.0f, 1.0f);
            else if (!left && !top) return gclamp((1.0f - sub.y) - sub.x, 0.0f, 1.0f);
            else if (!right && !top) return gclamp((1.0f - sub.y) - (1.0f - sub.x), 0.0f, 1.0f);
        }
        if (disc.x == 0.75f || disc.y == 0.75f) {
            // entering left and right, plus top or bottom
            if (disc.x == 0.75f && disc.y != 0.0f) {
                lc.y += ((disc.y - 0.75f) * 4.0f) * sy;
                bool left = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                bool right = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                if (!left && !right) return gclamp(1.0f - nd.y, 0.0f, 1.0f);
                float s = gmix(1.0f - sub.y, sub.y, gstep(1.0f, disc.y));
                float a = gmix(s, gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f),
                               gstep(1.0f, right ? 1.0f : 0.0f));
                float b = gmix(s, gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f),
                               gstep(1.0f, left ? 1.0f : 0.0f));
                return gmin(a, b);
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
                    topLeft = rb_disc_v(p, c, tlc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    topRight = rb_disc_v(p, c, tlc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                }
                if (!bottomCenter) {
                    blc.y -= sy;
                    float center = (blc.z <= fetch(c, blc.x, blc.y)) ? 1.0f : 0.0f;
                    bottomCenter = !(center != 0.0f);
                    bottomLeft = rb_disc_v(p, c, blc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                    bottomRight = rb_disc_v(p, c, blc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
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
                    if (!bottomRight || !topRight) return a;
                    else if (!bottomLeft || !topLeft) return b;
                    else return gmin(a, b);
                }
                if ((!bottomRight && !bottomLeft) || (!topRight && !topLeft))
                    return gclamp(1.0f - nd.y, 0.0f, 1.0f);
                else if (!bottomRight || !topRight)
                    return gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f);
                else
                    return gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f);
            }
            // entering top and bottom, plus left or right
            if (disc.x != 0.0f && disc.y == 0.75f) {
                lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                bool bottom = rb_disc_v(p, c, lc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                bool top = rb_disc_v(p, c, lc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                if (!bottom && !top) return gclamp(1.0f - nd.x, 0.0f, 1.0f);
                float s = gmix(sub.x, 1.0f - sub.x, gstep(disc.x, 0.25f));
                float a = gmix(s, gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f), gstep(1.0f, top ? 1.0f : 0.0f));
                float b = gmix(s, gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f),
                               gstep(1.0f, bottom ? 1.0f : 0.0f));
                return gmin(a, b);
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
                    bottomRight = rb_disc_v(p, c, rlc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                    topRight = rb_disc_v(p, c, rlc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                }
                if (!leftCenter) {
                    llc.x -= sx;
                    float center = (llc.z <= fetch(c, llc.x, llc.y)) ? 1.0f : 0.0f;
                    leftCenter = !(center != 0.0f);
                    bottomLeft = rb_disc_v(p, c, llc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                    topLeft = rb_disc_v(p, c, llc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
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
                    if (!bottomRight || !bottomLeft) return a;
                    else if (!topRight || !topLeft) return b;
                    else return gmin(a, b);
                }
                if ((!bottomRight && !topRight) || (!bottomLeft && !topLeft))
                    return gclamp(1.0f - nd.x, 0.0f, 1.0f);
                else if (!bottomRight || !bottomLeft)
                    return gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f);
                else
                    return gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f);
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
                if (disc.y == 0.5f) return gclamp((1.0f - nd.x) - (sub.y - 1.0f), 0.0f, 1.0f);
                else if (disc.y == 0.25f) return gclamp((1.0f - nd.x) + sub.y, 0.0f, 1.0f);
            } else {
                float a, b;
                if (disc.x == 0.5f && disc.y == 0.5f) {
                    a = gmix(1.0f - sub.y, gclamp(1.0f - (nd.x - (1.0f - sub.y)), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(1.0f - (nd.y - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmin(a, b);
                } else if (disc.x == 0.5f && disc.y == 0.25f) {
                    a = gmix(sub.y, gclamp(1.0f - (nd.x - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(1.0f - (nd.y - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmin(a, b);
                } else if (disc.x == 0.25f && disc.y == 0.5f) {
                    a = gmix(1.0f - sub.y, gclamp(1.0f - (nd.x - (1.0f - sub.y)), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(1.0f - (nd.y - (1.0f - sub.x)), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmin(a, b);
                } else if (disc.x == 0.25f && disc.y == 0.25f) {
                    a = gmix(sub.y, gclamp(1.0f - (nd.x - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(1.0f - (nd.y - (1.0f - sub.x)), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmin(a, b);
                }
            }
        }
        if (nd.x <= -2.0f) return gmix(1.0f - sub.y, sub.y, gstep(disc.y, 0.25f));
        if (nd.y <= -2.0f) return gmix(sub.x, 1.0f - sub.x, gstep(disc.x, 0.25f));
        if (disc.y > 0.0f) {
            if (disc.y == 0.5f) return gclamp((1.0f - sub.y) - (nd.x - 1.0f), 0.0f, 1.0f);
            else return gclamp(sub.y - (nd.x - 1.0f), 0.0f, 1.0f);
        }
        if (disc.x > 0.0f) {
            if (disc.x == 0.5f) return gclamp(sub.x - (nd.y - 1.0f), 0.0f, 1.0f);
            else return gclamp((1.0f - sub.x) - (nd.y - 1.0f), 0.0f, 1.0f);
        }
    } else {
        // exiting discontinuity
        if (disc.x == 0.75f || disc.y == 0.75f) {
            // exiting left and right only
            if (disc.x == 0.75f && disc.y == 0.0f) {
                V4 ref = lc;
                ref.x = lc.x - sx;
                bool left = rb_disc_v(p, c, ref, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                ref.x = lc.x + sx;
                bool right = rb_disc_v(p, c, ref, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                if (left && right) {
                    return gclamp(nd.y, 0.0f, 1.0f);
                } else if (left || right) {
                    if (!left) return gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    else return gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                } else {
                    // one pass of the commented-out while loop: count = 0, mult = 1
                    const int count = 0;
                    const int mult = (count / 2) + 1;
                    if (fmodf((float)count, 2.0f) == 0.0f) ref.y = lc.y + (float)mult * sy;
                    else ref.y = lc.y - (float)mult * sy;
                    ref.x = lc.x - sx;
                    left = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    ref.x = lc.x + sx;
                    right = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    if (left && right) {
                        return gclamp(nd.y, 0.0f, 1.0f);
                    } else {
                        if (!left) return gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                        else return gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    }
                }
            }
            // exiting left and right, plus top or bottom
            if (disc.x == 0.75f && disc.y != 0.0f) {
                lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
                bool left = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.5f, 0.0f, 0.0f, disc.z});
                bool right = rb_disc_v(p, c, lc, 0.0f, 1.0f, V4{0.25f, 0.0f, 0.0f, disc.z});
                float a = 0.0f, b = 0.0f;
                if (left && right) {
                    return gclamp(nd.y, 0.0f, 1.0f);
                } else if (left || right) {
                    if (left) a = gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
                    else a = gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    if (right) b = gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
                    else b = gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmax(a, b);
                } else {
                    if (disc.y == 0.75f) return 0.0f;
                    V4 ref = lc;
                    ref.x = lc.x - sx;
                    left = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    ref.x = lc.x + sx;
                    right = rb_disc_t(c, ref, 1.0f, 0.0f, 0.0f);
                    lc.y += ((0.5f - disc.y) * 8.0f - 1.0f) * sy;
                    if (left && right) {
                        return gclamp(nd.y, 0.0f, 1.0f);
                    } else {
                        a = gmix(1.0f - sub.x, sub.x, gstep(1.0f, left ? 1.0f : 0.0f));
                        b = gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
                        return gmax(a, b);
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
                    return gclamp(nd.x, 0.0f, 1.0f);
                } else if (bottom || top) {
                    if (!top) return gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    else return gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                } else {
                    const int count = 0;
                    const int mult = (count / 2) + 1;
                    if (fmodf((float)count, 2.0f) == 0.0f) ref.x = lc.x + (float)mult * sx;
                    else ref.x = lc.x - (float)mult * sx;
                    ref.y = lc.y - sy;
                    top = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    ref.y = lc.y + sy;
                    bottom = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    if (top && bottom) {
                        return gclamp(nd.x, 0.0f, 1.0f);
                    } else {
                        if (!top) return gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                        else return gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    }
                }
            }
            // exiting top and bottom, plus left or right
            if (disc.x != 0.0f && disc.y == 0.75f) {
                lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                bool bottom = rb_disc_v(p, c, lc, 1.0f, 0.0f, V4{0.0f, 0.5f, 0.0f, disc.z});
                bool top = rb_disc_v(p, c, lc, 1.0f, 0.0f, V4{0.0f, 0.25f, 0.0f, disc.z});
                float a = 0.0f, b = 0.0f;
                if (bottom && top) {
                    return gclamp(nd.x, 0.0f, 1.0f);
                } else if (bottom || top) {
                    if (top) a = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
                    else a = gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    if (bottom) b = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
                    else b = gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    return gmax(a, b);
                } else {
                    if (disc.x == 0.75f) return 0.0f;
                    V4 ref = lc;
                    ref.y = lc.y - sy;
                    top = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    ref.y = lc.y + sy;
                    bottom = rb_disc_t(c, ref, 0.0f, 1.0f, 0.0f);
                    lc.x -= ((0.5f - disc.x) * 8.0f - 1.0f) * sx;
                    if (top && bottom) {
                        return gclamp(nd.x, 0.0f, 1.0f);
                    } else {
                        a = gmix(1.0f - sub.y, sub.y, gstep(1.0f, top ? 1.0f : 0.0f));
                        b = gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
                        return gmax(a, b);
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
                if (disc.y == 0.5f) return gclamp(sub.y - (1.0f - nd.x), 0.0f, 1.0f);
                else if (disc.y == 0.25f) return gclamp((1.0f - sub.y) - (1.0f - nd.x), 0.0f, 1.0f);
            } else {
                float a, b;
                if (disc.x == 0.5f && disc.y == 0.5f) {
                    a = gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmax(a, b);
                } else if (disc.x == 0.5f && disc.y == 0.25f) {
                    a = gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(1.0f - sub.x, gclamp(nd.y - sub.x, 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmax(a, b);
                } else if (disc.x == 0.25f && disc.y == 0.5f) {
                    a = gmix(sub.y, gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmax(a, b);
                } else if (disc.x == 0.25f && disc.y == 0.25f) {
                    a = gmix(1.0f - sub.y, gclamp(nd.x - sub.y, 0.0f, 1.0f), gstep(-2.0f, nd.x));
                    b = gmix(sub.x, gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f), gstep(-2.0f, nd.y));
                    return gmax(a, b);
                }
            }
        }
        if (nd.x <= -2.0f) return gmix(sub.y, 1.0f - sub.y, gstep(disc.y, 0.25f));
        if (nd.y <= -2.0f) return gmix(1.0f - sub.x, sub.x, gstep(disc.x, 0.25f));
        if (disc.y > 0.0f) {
            if (disc.y == 0.5f) return gclamp(nd.x - (1.0f - sub.y), 0.0f, 1.0f);
            else return gclamp(nd.x - sub.y, 0.0f, 1.0f);
        }
        if (disc.x > 0.0f) {
            if (disc.x == 0.5f) return gclamp(nd.y - sub.x, 0.0f, 1.0f);
            else return gclamp(nd.y - (1.0f - sub.x), 0.0f, 1.0f);
        }
    }
    return 1.0f - disc.z;
}

// RBSSM (RBSSM.frag:1202-1339, the commented-out branches left out): K x K
// taps over the penumbra; a discontinuity tap is filled by smoothONDS.
__device__ float rb_filter(const gi_vis_params& p, const Ctx& c, float pw, V4 n) {
    float illum = 0.0f;
    const int K = p.kernel_size;
    float fw = ((float)K - 1.0f) * 0.5f;
    GridTaps g;
    grid_taps(pw, fw, g);
    for (int hi = 0; hi < g.n; hi++)
        for (int wi = 0; wi < g.n; wi++) {
            V4 lc = {n.x + g.o[wi], n.y + g.o[hi], n.z, n.w};
            V2 sub = {gfract(lc.x * c.fW), gfract(lc.y * c.fH)};
            float d = fetch(c, lc.x, lc.y);
            V4 disc = nc_compute_disc(c, lc, d);
            if (disc.x > 0.0f || disc.y > 0.0f) {
                V4 ds;
                ds.x = rb_disc_length(p, c, disc, lc, V2{-1.0f, 0.0f});
                ds.y = rb_disc_length(p, c, disc, lc, V2{1.0f, 0.0f});
                ds.z = rb_disc_length(p, c, disc, lc, V2{0.0f, -1.0f});
                ds.w = rb_disc_length(p, c, disc, lc, V2{0.0f, 1.0f});
                V4 nd = {rb_normalize_space(p, V2{ds.x, ds.y}, sub.x),
                         rb_normalize_space(p, V2{ds.z, ds.w}, sub.y), 0.0f, 0.0f};
                float fill = rb_smooth_onds(p, c, lc, nd, disc, sub);
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
__device__ float rb_rbssm(const gi_vis_params& p, const Ctx& c, V4 n) {
    float avg = avg_blocker_grid(p, c, n);
    float pw = penumbra_width(p, avg, n.z);
    float step = 2.0f * pw / (float)p.kernel_size;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    return rb_filter(p, c, pw, n);
}

// ---- RBSM/ConservativeSMSR.frag ---------------------------------------------------
__device__ __forceinline__ V4 cs_compute_disc(const Ctx& c, V4 s) {
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
    return V4{fabsf(dir.x - 1.0f), fabsf(dir.y - 1.0f), fabsf(dir.z - 1.0f), fabsf(dir.w - 1.0f)};
}

__device__ float cs_rel_dist(const gi_vis_params& p, const Ctx& c, V4 s, V2 dir, float cc) {
    V4 t = s;
    float found = 0.0f, distance = 0.0f;
    V2 st = {dir.x * c.sx, dir.y * c.sy};
    t.x += st.x;
    t.y += st.y;
    const float thr = p.depth_threshold;
    for (int it = 0; it < p.max_search; it++) {
        float d = fetch(c, t.x, t.y);
        if (fabsf(t.z - d) < thr) t.z -= thr;
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

__device__ __forceinline__ float cs_normalize(const gi_vis_params& p, V2 d) {
    float T = 1.0f;
    if (d.x < 0.0f && d.y < 0.0f) T = 0.0f;
    if (d.x > 0.0f && d.y > 0.0f) T = -2.0f;
    float len = gmin(fabsf(d.x) + fabsf(d.y), (float)p.max_search);
    return fabsf(gmax(T * d.x, T * d.y)) / len;
}

__device__ float cs_revectorized(const gi_vis_params& p, const Ctx& c, V4 s) {
    V2 sub = {gfract(s.x * c.fW), gfract(s.y * c.fH)};
    float dl = cs_rel_dist(p, c, s, V2{-1.0f, 0.0f}, 1.0f - sub.x);
    float dr = cs_rel_dist(p, c, s, V2{1.0f, 0.0f}, sub.x);
    float db = cs_rel_dist(p, c, s, V2{0.0f, -1.0f}, 1.0f - sub.y);
    float dt = cs_rel_dist(p, c, s, V2{0.0f, 1.0f}, sub.y);
    V2 r = {cs_normalize(p, V2{dl, dr}), cs_normalize(p, V2{db, dt})};
    if ((r.x * r.y > 0.0f) && (1.0f - r.x > r.y)) return c.I;
    return 1.0f;
}

__device__ float cs_smsr(const gi_vis_params& p, const Ctx& c, V4 s) {
    float d = fetch(c, s.x, s.y);
    float shadow = (s.z <= d) ? 1.0f : 0.0f;
    if (shadow == 0.0f) return c.I;
    V4 dd = cs_compute_disc(c, s);
    if ((dd.x + dd.y + dd.z + dd.w) == 0.0f) return 1.0f;
    else if ((dd.x + dd.y) == 2.0f || (dd.z + dd.w) == 2.0f) return c.I;
    return cs_revectorized(p, c, s);
}

__device__ float cs_rpcf(const gi_vis_params& p, const Ctx& c, V4 n) {
    float incrW = 1.0f / c.fW, incrH = 1.0f / c.fH;
    float illum = 0.0f;
    float offset = (float)p.penumbra_size;
    float step = 2.0f * offset / (float)p.kernel_order;
    int count = 0;
    for (float w = -offset; w <= offset; w += step)
        for (float h = -offset; h <= offset; h += step) {
            float d = fetch(c, n.x + w * incrW, n.y + h * incrH);
            float shadow = (n.z <= d) ? 1.0f : c.I;
            if (shadow == 1.0f) {
                V4 s = {n.x + w * incrW, n.y + h * incrH, n.z, n.w};
                V4 dd = cs_compute_disc(c, s);
                if (dd.x == 0.0f && dd.y == 0.0f) illum = illum + 1.0f;
                else illum += cs_revectorized(p, c, s);
            } else {
                illum += c.I;
            }
            count++;
        }
    return illum / (float)count;
}

// ---- filtered moment maps (Shadow.frag:118-220) -------------------------------
// c.map holds the blurred moment map (float4 per texel, c.W x c.H); the
// MSM inverse quantisation and its offset come from c_msm.
__constant__ float c_msm[20];

__device__ __forceinline__ float gl_linearize(float depth) { return 2.0f / (1001.0f - depth * 999.0f); }

// texture2D on the blurred map: bilinear at level 0, FP32 weights, zero
// border; coordinates that are not finite read the border.
__device__ __forceinline__ V4 moment_fetch(const Ctx& c, float s, float t) {
    const float4* m = reinterpret_cast<const float4*>(c.map);
    const float u = s * c.fW - 0.5f, v = t * c.fH - 0.5f;
    V4 r{0.0f, 0.0f, 0.0f, 0.0f};
    if (!(u > -2.0f && u < c.fW + 1.0f && v > -2.0f && v < c.fH + 1.0f)) return r;
    const float fu = floorf(u), fv = floorf(v);
    const int i0 = (int)fu, j0 = (int)fv;
    const float a = u - fu, b = v - fv;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float4 T[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = i0 + (k & 1), j = j0 + (k >> 1);
        T[k] = (i >= 0 && i < c.W && j >= 0 && j < c.H) ? __ldg(m + (size_t)j * c.W + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    r.x = ((w00 * T[0].x + w10 * T[1].x) + w01 * T[2].x) + w11 * T[3].x;
    r.y = ((w00 * T[0].y + w10 * T[1].y) + w01 * T[2].y) + w11 * T[3].y;
    r.z = ((w00 * T[0].z + w10 * T[1].z) + w01 * T[2].z) + w11 * T[3].z;
    r.w = ((w00 * T[0].w + w10 * T[1].w) + w01 * T[2].w) + w11 * T[3].w;
    return r;
}

// chebyshevUpperBound (Shadow.frag:118-131)
__device__ __forceinline__ float chebyshev(float mx, float my, float z, float I) {
    if (z <= mx) return 1.0f;
    const float variance = my - mx * mx;
    const float d = z - mx;
    float p_max = variance / (variance + d * d);
    const float p = z <= mx ? 1.0f : 0.0f;
    p_max = gmax(p, p_max);
    return gmix(p_max, 1.0f, I);
}

// varianceShadowMapping (:133-141)
__device__ __forceinline__ float vsm(const Ctx& c, V4 n) {
    const V4 m = moment_fetch(c, n.x, n.y);
    return chebyshev(m.x, m.y, gl_linearize(n.z), c.I);
}

// exponentialShadowMapping (:144-157)
__device__ __forceinline__ float esm(const Ctx& c, V4 n) {
    const float k = 80.0f;
    float e2 = moment_fetch(c, n.x, n.y).x;
    e2 = expf(k * e2);
    const float z = gl_linearize(n.z);
    const float e1 = expf(-k * z);
    return gclamp(e1 * e2, c.I, 1.0f);
}

// exponentialVarianceShadowMapping (:160-176)
__device__ __forceinline__ float evsm(const Ctx& c, V4 n) {
    const float z = gl_linearize(n.z);
    const V4 m = moment_fetch(c, n.x, n.y);
    const float variance = chebyshev(m.x, m.y, z, c.I);
    const float k = 60.0f;
    const float e1 = expf(-k * z);
    const float e2 = expf(k * m.z);
    const float exponential = gclamp(e1 * e2, c.I, 1.0f);
    return gmin(variance, exponential);
}

// hamburger4MSM (:178-220)
__device__ __forceinline__ float msm(const Ctx& c, V4 n) {
    V4 b = moment_fetch(c, n.x, n.y);
    b = V4{b.x - c_msm[16], b.y - c_msm[17], b.z - c_msm[18], b.w - c_msm[19]};
    b = mat4_mul(c_msm, b);
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
    const float r = sqrtf(D);
    const float zy = -(p / 2.0f) - r, zz = -(p / 2.0f) + r;
    if (z0 <= zy) return 1.0f;
    if (z0 <= zz)
        return gclamp(1.0f - gclamp((z0 * zz - b.x * (z0 + zz) + b.y) / ((zz - zy) * (z0 - zy)), 0.0f, 1.0f), c.I,
                      1.0f);
    return gclamp(1.0f - gclamp(1.0f - (zy * zz - b.x * (zy + zz) + b.y) / ((z0 - zy) * (z0 - zz)), 0.0f, 1.0f),
                  c.I, 1.0f);
}

// ---- moment soft shadows (SoftShadowMapping PlausibleSoftShadow.frag) --------
// c.sm.mom holds the moment map or its summed-area table (c.W x c.H float4),
// c.sm.hsm_* the two min-max levels VSSM's lookup blends.  Every read is
// bilinear at its level with FP32 weights and a zero border.
template <class F>
__device__ __forceinline__ float2 bilinear2(const F& tex, int w, int h, float s, float t) {
    const float u = s * (float)w - 0.5f, v = t * (float)h - 0.5f;
    if (!(u > -2.0f && u < (float)w + 1.0f && v > -2.0f && v < (float)h + 1.0f)) return make_float2(0.0f, 0.0f);
    const float fu = floorf(u), fv = floorf(v);
    const int i0 = (int)fu, j0 = (int)fv;
    const float a = u - fu, b = v - fv;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    const float2 T0 = tex(i0, j0), T1 = tex(i0 + 1, j0), T2 = tex(i0, j0 + 1), T3 = tex(i0 + 1, j0 + 1);
    return make_float2(((w00 * T0.x + w10 * T1.x) + w01 * T2.x) + w11 * T3.x,
                       ((w00 * T0.y + w10 * T1.y) + w01 * T2.y) + w11 * T3.y);
}

__device__ __forceinline__ V4 mom_at(const Ctx& c, float s, float t) {
    const float4* m = c.sm.mom;
    const float u = s * c.fW - 0.5f, v = t * c.fH - 0.5f;
    V4 r{0.0f, 0.0f, 0.0f, 0.0f};
    if (!(u > -2.0f && u < c.fW + 1.0f && v > -2.0f && v < c.fH + 1.0f)) return r;
    const float fu = floorf(u), fv = floorf(v);
    const int i0 = (int)fu, j0 = (int)fv;
    const float a = u - fu, b = v - fv;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float4 T[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = i0 + (k & 1), j = j0 + (k >> 1);
        T[k] = (i >= 0 && i < c.W && j >= 0 && j < c.H) ? __ldg(m + (size_t)j * c.W + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    r.x = ((w00 * T[0].x + w10 * T[1].x) + w01 * T[2].x) + w11 * T[3].x;
    r.y = ((w00 * T[0].y + w10 * T[1].y) + w01 * T[2].y) + w11 * T[3].y;
    r.z = ((w00 * T[0].z + w10 * T[1].z) + w01 * T[2].z) + w11 * T[3].z;
    r.w = ((w00 * T[0].w + w10 * T[1].w) + w01 * T[2].w) + w11 * T[3].w;
    return r;
}

__device__ __forceinline__ float nonlinearize(float d) { return -(2.0f - d * 1001.0f) / (d * 999.0f); }

// chebyshevUpperBound (PlausibleSoftShadow.frag:78-91)
__device__ __forceinline__ float chebyshev_soft(float mx, float my, float z) {
    if (z <= mx) return 1.0f;
    const float variance = my - mx * mx;
    const float d = z - mx;
    const float p_max = variance / (variance + d * d);
    const float p = z <= mx ? 1.0f : 0.0f;
    return gmax(p, p_max);
}

// the SAT branch: four corner reads, (D + A - B - C) / SATFilterSize^2
__device__ __forceinline__ V4 sat_box(const Ctx& c, V4 n, float width, float step) {
    const float div = 2.0f * width / step;
    const float size = div / 2.0f;
    const float xmax = n.x + div * step, xmin = n.x - (div + 1.0f) * step;
    const float ymax = n.y + div * step, ymin = n.y - (div + 1.0f) * step;
    const V4 A = mom_at(c, xmin, ymin), B = mom_at(c, xmax, ymin), C = mom_at(c, xmin, ymax), D = mom_at(c, xmax, ymax);
    const float den = size * size;
    return V4{(((D.x + A.x) - B.x) - C.x) / den, (((D.y + A.y) - B.y) - C.y) / den, (((D.z + A.z) - B.z) - C.z) / den,
              (((D.w + A.w) - B.w) - C.w) / den};
}

// the tap loop: bilinear reads at n.xy + (w, h) * width / fw summed in
// (h, w) order, then / float(count^2)
__device__ V4 loop_box(const Ctx& c, V4 n, float width, int count) {
    const float fw = ((float)count - 1.0f) * 0.5f;
    V4 acc{0.0f, 0.0f, 0.0f, 0.0f};
    GridTaps g;
    grid_taps(width, fw, g);
    for (int hi = 0; hi < g.n; hi++)
        for (int wi = 0; wi < g.n; wi++) {
            const V4 t = mom_at(c, n.x + g.o[wi], n.y + g.o[hi]);
            acc = V4{acc.x + t.x, acc.y + t.y, acc.z + t.z, acc.w + t.w};
        }
    const float den = (float)(count * count);
    return V4{acc.x / den, acc.y / den, acc.z / den, acc.w / den};
}

__device__ __forceinline__ V4 soft_box(const gi_vis_params& p, const Ctx& c, V4 n, float width, float step,
                                       int count) {
    return p.summed_area_table ? sat_box(c, n, width, step) : loop_box(c, n, width, count);
}

// VSM (:400-440)
__device__ float soft_vsm(const gi_vis_params& p, const Ctx& c, float pw, V4 n) {
    const int K = p.kernel_size;
    const float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const V4 m = soft_box(p, c, n, pw, step, K);
    const float mx = m.x + 0.5f, my = m.y + 0.5f;
    return gclamp(gmix(chebyshev_soft(mx, my, gl_linearize(n.z)), 1.0f, c.I), 0.0f, 1.0f);
}

// computeAverageBlockerDepthBasedOnVSM (:196-244)
__device__ float vsm_blocker(const gi_vis_params& p, const Ctx& c, V4 n) {
    const float bsw = blocker_search_width(p, c);
    const int B = p.blocker_search_size;
    const float step = 2.0f * bsw / (float)B;
    const float zun = gl_linearize(n.z);
    const V4 m = soft_box(p, c, n, bsw, step, B);
    const float mx = m.x + 0.5f, my = m.y + 0.5f;
    const float prob = chebyshev_soft(mx, my, zun);
    float zocc = nonlinearize((mx - prob * zun) / (1.0f - prob));
    if (prob > 0.99f) zocc = 1.0f;
    return zocc;
}

// computeAverageBlockerDepthBasedOnESM (:246-301)
__device__ float esm_blocker(const gi_vis_params& p, const Ctx& c, V4 n) {
    const float bsw = blocker_search_width(p, c);
    const int B = p.blocker_search_size;
    const float step = 2.0f * bsw / (float)B;
    const V4 s = soft_box(p, c, n, bsw, step, B);
    const float lz = gl_linearize(n.z);
    const float prob = expf(-80.0f * lz) * s.y;
    if (prob > 0.91f) return 1.0f;
    const float zocc = (s.x - expf(-80.0f * lz) * s.z) / (1.0f - prob);
    return nonlinearize(zocc);
}

// ESM (:442-490)
__device__ float soft_esm(const gi_vis_params& p, const Ctx& c, float pw, V4 n) {
    const int K = p.kernel_size;
    const float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const float avg = soft_box(p, c, n, pw, step, K).y;
    const float dist = mom_at(c, n.x, n.y).x + 0.0001f;
    const float lz = gl_linearize(n.z);
    float v = expf(-80.0f * lz) * avg;
    v = gclamp(v, c.I, 1.0f);
    if (dist > lz && v == c.I) return 1.0f;
    return v;
}

// computeMomentDepthsFromMSM (:93-132): b and the three depths
struct MsmSolve {
    V4 b;
    float zx, zy, zz;
};

__device__ __forceinline__ MsmSolve msm_solve(V4 b, float lz) {
    b = V4{b.x - c_msm[16], b.y - c_msm[17], b.z - c_msm[18], b.w - c_msm[19]};
    b = mat4_mul(c_msm, b);
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
    const float pp = cy / cz, q = cx / cz;
    const float D = ((pp * pp) / 4.0f) - q;
    const float r = sqrtf(D);
    return MsmSolve{b, lz, -(pp / 2.0f) - r, -(pp / 2.0f) + r};
}

// computeAverageBlockerDepthBasedOnMSM (:303-363) with computeWeightsFromMSM
__device__ float msm_blocker(const gi_vis_params& p, const Ctx& c, V4 n) {
    const float bias = 0.01f;
    const float bsw = p.light_radius / c.fW;
    const int B = p.blocker_search_size;
    const float step = 2.0f * bsw / (float)B;
    const MsmSolve z = msm_solve(soft_box(p, c, n, bsw, step, B), gl_linearize(n.z));
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

// MSM (:492-533) with computeShadowIntensityFromMSM (:149-164)
__device__ float soft_msm(const gi_vis_params& p, const Ctx& c, float pw, V4 n) {
    const int K = p.kernel_size;
    const float step = 2.0f * pw / (float)K;
    if (step <= 0.0f || step >= 1.0f) return 1.0f;
    const MsmSolve z = msm_solve(soft_box(p, c, n, pw, step, K), gl_linearize(n.z));
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

// computeVisibilityFromHSM (:535-554): levels floor(lod) and floor(lod) + 1
// blended (1 - f) t1 + f t2; level 0 is read from the light map
__device__ float hsm_visibility(const gi_vis_params& p, const Ctx& c, V4 n) {
    const float2* hi = c.sm.hsm_hi;
    const auto tex_hi = [&](int i, int j) {
        return (i >= 0 && i < c.sm.hi_w && j >= 0 && j < c.sm.hi_h) ? __ldg(hi + (size_t)j * c.sm.hi_w + i)
                                                                    : make_float2(0.0f, 0.0f);
    };
    float2 lo;
    if (c.sm.hsm_lo) {
        const float2* l = c.sm.hsm_lo;
        const auto tex_lo = [&](int i, int j) {
            return (i >= 0 && i < c.sm.lo_w && j >= 0 && j < c.sm.lo_h) ? __ldg(l + (size_t)j * c.sm.lo_w + i)
                                                                        : make_float2(0.0f, 0.0f);
        };
        lo = bilinear2(tex_lo, c.sm.lo_w, c.sm.lo_h, n.x, n.y);
    } else {
        const auto tex0 = [&](int i, int j) {
            if (i < 0 || i >= c.W || j < 0 || j >= c.H) return make_float2(0.0f, 0.0f);
            const float d = __ldg(c.map + (size_t)j * c.W + i);
            return make_float2((d == 0.0f ? 1.0f : d) + p.hsm_alpha, d + p.hsm_beta);
        };
        lo = bilinear2(tex0, c.W, c.H, n.x, n.y);
    }
    const float2 up = bilinear2(tex_hi, c.sm.hi_w, c.sm.hi_h, n.x, n.y);
    const float f = c.sm.hsm_frac;
    const float mn = (1.0f - f) * lo.x + f * up.x, mx = (1.0f - f) * lo.y + f * up.y;
    if (n.z <= mn) return 1.0f;
    if (n.z > mx) return c.I;
    return 0.555f;
}

template <int TECH>
__device__ __forceinline__ float shade(const gi_vis_params& p, const Ctx& c, V4 vertex, V4 normal) {
    if (vertex.x == 0.0f) return 0.0f;
    V4 sc = mat4_mul(p.light_mvp_biased, vertex);
    V4 n = {sc.x / sc.w, sc.y / sc.w, sc.z / sc.w, sc.w / sc.w};
    float shadow = pretest(p, c, vertex, normal);
    if (TECH == GI_TECH_HARD) {
        if (sc.w > 0.0f && shadow == 1.0f) {
            float d = fetch(c, n.x, n.y);
            shadow = (n.z <= d) ? 1.0f : c.I;
        }
    } else if (TECH == GI_TECH_PCF) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = pcf_bilinear(p, c, n);
    } else if (TECH == GI_TECH_PCF_TRICUBIC) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = pcf_tricubic(p, c, n);
    } else if (TECH == GI_TECH_PCSS_GRID) {
        if (sc.w > 0.0f && shadow == 1.0f) {
            float avg = avg_blocker_grid(p, c, n);
            float pw = penumbra_width(p, avg, n.z);
            shadow = pcss_filter_grid(p, c, pw, n);
        }
    } else if (TECH == GI_TECH_PCSS_POISSON) {
        if (sc.w > 0.0f && shadow == 1.0f) {
            const float bsw = blocker_search_width(p, c);
            float avg = finite3(n.x, n.y, bsw) ? avg_blocker_poisson_t<true>(p, c, n, bsw)
                                               : avg_blocker_poisson_t<false>(p, c, n, bsw);
            float pw = penumbra_width(p, avg, n.z);
            const float step = 2.0f * pw / (float)p.kernel_size;
            if (step <= 0.0f || step >= 1.0f) shadow = 1.0f;
            else if (finite3(n.x, n.y, pw)) shadow = pcss_filter_poisson_t<true>(p, c, pw, n);
            else shadow = pcss_filter_poisson_t<false>(p, c, pw, n);
        }
    } else if (TECH == GI_TECH_SMSR_NONCONSERVATIVE) {
        if (shadow == 1.0f) shadow = nc_smsr(p, c, n);
    } else if (TECH == GI_TECH_RPCF_SMSR) {
        if (shadow == 1.0f) shadow = nc_rpcf(p, c, n, false);
    } else if (TECH == GI_TECH_RSMSS) {
        if (shadow == 1.0f) shadow = nc_rpcf(p, c, n, true);
    } else if (TECH == GI_TECH_SMSR_CONSERVATIVE) {
        if (shadow == 1.0f) shadow = cs_smsr(p, c, n);
    } else if (TECH == GI_TECH_RPCF_CONSERVATIVE) {
        if (shadow == 1.0f) shadow = cs_rpcf(p, c, n);
    } else if (TECH == GI_TECH_RBSSM) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = rb_rbssm(p, c, n);
    } else if (TECH == GI_TECH_VSM) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = vsm(c, n);
    } else if (TECH == GI_TECH_ESM) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = esm(c, n);
    } else if (TECH == GI_TECH_EVSM) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = evsm(c, n);
    } else if (TECH == GI_TECH_MSM) {
        if (sc.w > 0.0f && shadow == 1.0f) shadow = msm(c, n);
    } else if (TECH == GI_TECH_SAVSM) {  // summedAreaVarianceShadowMapping (:565-572)
        if (sc.w > 0.0f && shadow == 1.0f) {
            const float avg = avg_blocker_grid(p, c, n);
            shadow = soft_vsm(p, c, penumbra_width(p, avg, n.z), n);
        }
    } else if (TECH == GI_TECH_VSSM) {  // varianceSoftShadowMapping (:574-585)
        if (sc.w > 0.0f && shadow == 1.0f) {
            const float v = hsm_visibility(p, c, n);
            if (v == c.I || v == 1.0f) shadow = v;
            else shadow = soft_vsm(p, c, penumbra_width(p, vsm_blocker(p, c, n), n.z), n);
        }
    } else if (TECH == GI_TECH_ESSM) {  // exponentialSoftShadowMapping (:587-594)
        if (sc.w > 0.0f && shadow == 1.0f) shadow = soft_esm(p, c, penumbra_width(p, esm_blocker(p, c, n), n.z), n);
    } else if (TECH == GI_TECH_MSSM) {  // momentSoftShadowMapping (:596-603)
        if (sc.w > 0.0f && shadow == 1.0f) shadow = soft_msm(p, c, penumbra_width(p, msm_blocker(p, c, n), n.z), n);
    } else if (TECH == GI_TECH_HARD_SOFTAPP) {
        float r = shadow;
        if (sc.w > 0.0f && r == 1.0f) {
            float d = fetch(c, n.x, n.y);
            r = (n.z <= d) ? 1.0f : c.I;
        }
        if (pretest(p, c, vertex, normal) == c.I) r = 0.0f;
        shadow = r;
    }
    return shadow;
}

template <int TECH>
__global__ void __launch_bounds__(128) k_visibility(const gi_vis_params p,
                                                    const float* __restrict__ map, int map_w,
                                                    int map_h, float sx, float sy,
                                                    const float4* __restrict__ pos,
                                                    const float4* __restrict__ nrm,
                                                    float* __restrict__ out, int W, int H,
                                                    const SoftMaps sm,
                                                    const __grid_constant__ PoissonOffsets po) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    Ctx c;
    c.map = map;
    c.W = map_w;
    c.H = map_h;
    c.fW = (float)map_w;
    c.fH = (float)map_h;
    c.sx = sx;
    c.sy = sy;
    c.I = p.shadow_intensity;
    c.sm = sm;
    c.boff = TECH == GI_TECH_PCSS_POISSON ? po.b : nullptr;
    c.tab = (TECH == GI_TECH_PCSS_POISSON || TECH == GI_TECH_PCF) ? &po : nullptr;
    size_t i = (size_t)y * W + x;
    float4 pv = __ldcs(pos + i);
    float4 nv = __ldcs(nrm + i);
    V4 vertex = {pv.x, pv.y, pv.z, pv.w};
    V4 normal = {nv.x, nv.y, nv.z, nv.w};
    __stcs(out + i, shade<TECH>(p, c, vertex, normal));
}

// Persistent visibility pass of a batch: one launch shades every tile of
// every light-frame.  The light maps and the frames' G-buffers are complete
// when it starts (stream order), so nothing waits on another kernel: each
// CTA takes the next tile from a global counter (one atomic per tile), finds
// its light-frame by binary search over the tiles' prefix sums, stages that
// light-frame's parameters in shared memory, and shades the tile's pixels
// with the same shade<TECH> as the per-frame kernels.  Tiles of tile_w x
// tile_h pixels (tile_w a multiple of 32) are walked row by row, 128
// pixels per step.
template <int TECH>
__global__ void __launch_bounds__(128) k_batch_visibility(const BatchLightFrame* __restrict__ lf, int n_lf,
                                                          unsigned total_tiles, unsigned* __restrict__ queue,
                                                          int tile_w, int tile_h) {
    __shared__ BatchLightFrame s_lf;
    __shared__ unsigned s_tile;
    __shared__ int s_idx;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) {
            const unsigned t = atomicAdd(queue, 1u);
            s_tile = t;
            int lo = 0, hi = n_lf - 1;  // last light-frame whose first tile <= t
            if (t < total_tiles) {
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (lf[mid].tile_begin <= t) lo = mid;
                    else hi = mid - 1;
                }
            }
            s_idx = lo;
        }
        __syncthreads();
        const unsigned t = s_tile;
        if (t >= total_tiles) break;
        {
            const int* src = reinterpret_cast<const int*>(lf + s_idx);
            int* dst = reinterpret_cast<int*>(&s_lf);
            for (int k = tid; k < (int)(sizeof(BatchLightFrame) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        const BatchLightFrame& f = s_lf;
        const unsigned local = t - f.tile_begin;
        const int x0 = (int)(local % (unsigned)f.tiles_x) * tile_w;
        const int y0 = (int)(local / (unsigned)f.tiles_x) * tile_h;
        Ctx c;
        c.map = f.map;
        c.W = f.map_w;
        c.H = f.map_h;
        c.fW = (float)f.map_w;
        c.fH = (float)f.map_h;
        c.sx = f.sx;
        c.sy = f.sy;
        c.I = f.p.shadow_intensity;
        for (int k = tid; k < tile_w * tile_h; k += blockDim.x) {
            const int x = x0 + k % tile_w, y = y0 + k / tile_w;
            if (x >= f.W || y >= f.H) continue;
            const size_t i = (size_t)y * f.W + x;
            const float4 pv = __ldcs(f.pos + i);
            const float4 nv = __ldcs(f.nrm + i);
            V4 vertex = {pv.x, pv.y, pv.z, pv.w};
            V4 normal = {nv.x, nv.y, nv.z, nv.w};
            __stcs(f.out + i, shade<TECH>(f.p, c, vertex, normal));
        }
        __syncthreads();  // s_lf and s_tile are rewritten by the next take
    }
}

// Fused G-buffer resolve and visibility: the G-buffer texel of each pixel
// is interpolated from the visibility key in registers and shaded at once,
// so the frame never writes / reads the 32-byte-per-pixel G-buffer (it is
// stored only when the caller asks for it).  Same values as
// k_gbuffer_resolve followed by k_visibility.
// Occupancy: the kernel waits on memory (the key's record and vertices,
// the map taps) more than it computes, so extra resident warps pay for a
// few spilled words.  PCSS-Poisson: (128, 12), 40 registers, 48 warps per
// SM (resolve + visibility on pcss_1080p: (128, 8) 40.1 us, (128, 10)
// 37.0 us, (128, 12) 36.7 us, (128, 14) 39.6 us); the other techniques
// keep (128, 10), 48 registers.
template <int TECH>
__global__ void __launch_bounds__(128, TECH == GI_TECH_PCSS_POISSON ? 12 : 10) k_frame_visibility(
    const gi_vis_params p, const float* __restrict__ map, int map_w, int map_h, float sx, float sy,
    const unsigned long long* __restrict__ keys, const float* __restrict__ points,
    const float* __restrict__ normals, const int* __restrict__ indices, const dev::Mat4 mvp,
    const unsigned* __restrict__ rec_of, const dev::BRec* __restrict__ recs, const uint4* __restrict__ rres,
    float* __restrict__ out, int W, int H, float4* __restrict__ pos_out, float4* __restrict__ nrm_out,
    const SoftMaps sm, const __grid_constant__ PoissonOffsets po) {
    // A warp shades an 8 x 4 patch of the block's 32 x 4 pixels, so its
    // lanes more often share a triangle, a lit / shadowed state and map
    // texels (pcss_1080p resolve + visibility: 36.6 us as 32 x 1 rows,
    // 36.3 as 16 x 2, 36.0 as 8 x 4).
    constexpr int kWarpW = 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = blockIdx.x * 32 + (warp * kWarpW) % 32 + lane % kWarpW;
    int y = blockIdx.y * 4 + (warp * kWarpW) / 32 * (32 / kWarpW) + lane / kWarpW;
    if (x >= W || y >= H) return;
    Ctx c;
    c.sm = sm;
    c.boff = TECH == GI_TECH_PCSS_POISSON ? po.b : nullptr;
    c.tab = (TECH == GI_TECH_PCSS_POISSON || TECH == GI_TECH_PCF) ? &po : nullptr;
    c.map = map;
    c.W = map_w;
    c.H = map_h;
    c.fW = (float)map_w;
    c.fH = (float)map_h;
    c.sx = sx;
    c.sy = sy;
    c.I = p.shadow_intensity;
    const size_t i = (size_t)y * W + x;
    float4 pv, nv;
    dev::resolve_pixel(__ldcs(keys + i), points, normals, indices, mvp, W, H, x, y, rec_of, recs, rres, pv, nv);
    if (pos_out) {
        pos_out[i] = pv;
        nrm_out[i] = nv;
    }
    V4 vertex = {pv.x, pv.y, pv.z, pv.w};
    V4 normal = {nv.x, nv.y, nv.z, nv.w};
    __stcs(out + i, shade<TECH>(p, c, vertex, normal));
}

// ---- learned surrogate: per-pixel features and the final visibility -----------
// Features (BF16, 16 channels per pixel, 4 used):
//   0  hard visibility with the pre-test (shade<HARD>): 1, intensity or 0
//   1  (z - d) * 64 clamped to [-1, 4]: receiver depth minus the map depth
//      at the pixel's texel (window units)
//   2  penumbra estimate in map texels / 8 (<= 4) from four diagonal
//      blocker taps at the PCSS blocker-search radius
//   3  1 if the pre-test passed, 0.5 if it failed, 0 for background
__device__ __forceinline__ uint16_t f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

__global__ void __launch_bounds__(128) k_surrogate_features(
    const gi_vis_params p, const float* __restrict__ map, int map_w, int map_h, float sx, float sy,
    const unsigned long long* __restrict__ keys, const float* __restrict__ points,
    const float* __restrict__ normals, const int* __restrict__ indices, const dev::Mat4 mvp,
    const unsigned* __restrict__ rec_of, const dev::BRec* __restrict__ recs, const uint4* __restrict__ rres,
    int W, int H, uint4* __restrict__ feat) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    Ctx c;
    c.map = map;
    c.W = map_w;
    c.H = map_h;
    c.fW = (float)map_w;
    c.fH = (float)map_h;
    c.sx = sx;
    c.sy = sy;
    c.I = p.shadow_intensity;
    const size_t i = (size_t)y * W + x;
    float4 pv, nv;
    dev::resolve_pixel(__ldcs(keys + i), points, normals, indices, mvp, W, H, x, y, rec_of, recs, rres, pv, nv);
    float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, f3 = 0.0f;
    V4 vertex = {pv.x, pv.y, pv.z, pv.w};
    if (vertex.x != 0.0f) {
        V4 normal = {nv.x, nv.y, nv.z, nv.w};
        V4 sc = mat4_mul(p.light_mvp_biased, vertex);
        V4 n = {sc.x / sc.w, sc.y / sc.w, sc.z / sc.w, 1.0f};
        const float pre = pretest(p, c, vertex, normal);
        f3 = pre == 1.0f ? 1.0f : 0.5f;
        f0 = pre;
        const float d = fetch(c, n.x, n.y);
        if (sc.w > 0.0f && pre == 1.0f) f0 = (n.z <= d) ? 1.0f : c.I;
        f1 = fminf(fmaxf((n.z - d) * 64.0f, -1.0f), 4.0f);
        const float r = blocker_search_width(p, c) * 0.70710678f;
        float avg = 0.0f;
        int nb = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float dd = fetch(c, n.x + ((k & 1) ? r : -r), n.y + ((k & 2) ? r : -r));
            if (n.z > dd) {
                avg += dd;
                nb++;
            }
        }
        if (nb > 0) {
            avg /= (float)nb;
            const float pw = penumbra_width(p, avg, n.z);
            f2 = fminf(fmaxf(pw * c.fW * 0.125f, 0.0f), 4.0f);
        }
    }
    const uint32_t w0 = (uint32_t)f2bf(f0) | ((uint32_t)f2bf(f1) << 16);
    const uint32_t w1 = (uint32_t)f2bf(f2) | ((uint32_t)f2bf(f3) << 16);
    feat[2 * i] = make_uint4(w0, w1, 0u, 0u);
    feat[2 * i + 1] = make_uint4(0u, 0u, 0u, 0u);
}

// Visibility from the network head (FP32, head_stride channels per pixel: 0
// the visibility, 1 the predicted absolute error): background 0, failed
// pre-test the intensity, otherwise the prediction clamped to
// [intensity, 1], or the exact PCSS (Poisson) value where the predicted
// error exceeds `thr`.
__global__ void __launch_bounds__(128) k_surrogate_finish(
    const gi_vis_params p, const float* __restrict__ map, int map_w, int map_h, float sx, float sy,
    const unsigned long long* __restrict__ keys, const float* __restrict__ points,
    const float* __restrict__ normals, const int* __restrict__ indices, const dev::Mat4 mvp,
    const unsigned* __restrict__ rec_of, const dev::BRec* __restrict__ recs, const uint4* __restrict__ rres,
    const float* __restrict__ head, int head_stride, const uint4* __restrict__ feat, float thr,
    float* __restrict__ out, int W, int H, unsigned* __restrict__ n_fallback) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const uint4 f = __ldg(feat + 2 * i);
    const float f3 = __uint_as_float(f.y & 0xFFFF0000u);
    const float I = p.shadow_intensity;
    float v;
    if (f3 == 0.0f) {
        v = 0.0f;
    } else if (f3 != 1.0f) {
        v = I;
    } else {
        const float2 h = *reinterpret_cast<const float2*>(head + i * head_stride);
        if (h.y > thr) {
            Ctx c;
            c.map = map;
            c.W = map_w;
            c.H = map_h;
            c.fW = (float)map_w;
            c.fH = (float)map_h;
            c.sx = sx;
            c.sy = sy;
            c.I = I;
            float4 pv, nv;
            dev::resolve_pixel(keys[i], points, normals, indices, mvp, W, H, x, y, rec_of, recs, rres, pv, nv);
            V4 vertex = {pv.x, pv.y, pv.z, pv.w};
            V4 normal = {nv.x, nv.y, nv.z, nv.w};
            v = shade<GI_TECH_PCSS_POISSON>(p, c, vertex, normal);
            if (n_fallback) atomicAdd(n_fallback, 1u);
        } else {
            v = fminf(fmaxf(h.x, I), 1.0f);
        }
    }
    __stcs(out + i, v);
}

// ---- area-light ground truth (AccurateSoftShadow.frag:52-133, uniform samples) --
// Per pixel: commonShadowCoord from columns 0-2 of the light MVP uniform,
// then per sample shadowCoord = common + translation, divided by w, one
// NEAREST fetch from that sample's map and accShadow += (z <= d ? 1 : I) *
// accFactor (1); shadow = accShadow / count.  The pre-test is commented out
// in the shader; background pixels are discarded (0).
__global__ void __launch_bounds__(128) k_area_accumulate(
    const float* __restrict__ maps, int map_s, int nw, const AreaWave wave, float I,
    const unsigned long long* __restrict__ keys, const float* __restrict__ points,
    const float* __restrict__ normals, const int* __restrict__ indices, const dev::Mat4 mvp,
    const unsigned* __restrict__ rec_of, const dev::BRec* __restrict__ recs, const uint4* __restrict__ rres,
    float* __restrict__ acc, int first, int last, float count, float* __restrict__ out, int W, int H) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    float4 pv, nv;
    dev::resolve_pixel(__ldcs(keys + i), points, normals, indices, mvp, W, H, x, y, rec_of, recs, rres, pv, nv);
    if (pv.x == 0.0f) {
        if (last) out[i] = 0.0f;
        return;
    }
    const float* m = wave.common;
    const float cx = m[0] * pv.x + m[4] * pv.y + m[8] * pv.z;
    const float cy = m[1] * pv.x + m[5] * pv.y + m[9] * pv.z;
    const float cz = m[2] * pv.x + m[6] * pv.y + m[10] * pv.z;
    const float cw = m[3] * pv.x + m[7] * pv.y + m[11] * pv.z;
    Ctx c;
    c.W = map_s;
    c.H = map_s;
    c.fW = (float)map_s;
    c.fH = (float)map_s;
    float a = first ? 0.0f : acc[i];
    for (int k = 0; k < nw; ++k) {
        const float sx = cx + wave.trans[k][0], sy = cy + wave.trans[k][1];
        const float sz = cz + wave.trans[k][2], sw = cw + wave.trans[k][3];
        c.map = maps + (size_t)k * map_s * map_s;
        if (wave.pcf_n == 0) {
            const float d = fetch(c, sx / sw, sy / sw);
            a += ((sz / sw <= d) ? 1.0f : I) * wave.weight[k];
        } else {
            // AccurateSoftShadow.frag's lower-accuracy branch: the float
            // loops' offsets (w outer, h inner) in texels of 1 / map width
            const float ux = sx / sw, uy = sy / sw, uz = sz / sw;
            float illum = 0.0f;
            for (int wi = 0; wi < wave.pcf_n; ++wi)
                for (int hi = 0; hi < wave.pcf_n; ++hi) {
                    const float d = fetch(c, ux + wave.pcf_off[wi] * wave.pcf_incr_w,
                                          uy + wave.pcf_off[hi] * wave.pcf_incr_h);
                    if (uz <= d) illum = illum + 1.0f;
                    else illum += I;
                }
            a += (illum / (float)(wave.pcf_n * wave.pcf_n)) * wave.weight[k];
        }
    }
    if (last) out[i] = a / count;
    else acc[i] = a;
}

// ---- adaptive area-light sampling (SoftShadowMapping Shaders/QuadTree) ------
// Reprojection.frag: how many of a quad-tree node's four corner lights see
// the pixel (hard tests through each corner's biased MVP, GL_NEAREST with a
// zero border); background pixels keep the target's clear colour (0.63,
// stored as 255).
__global__ void __launch_bounds__(128) k_qt_reproject(const float4* __restrict__ pos, int W, int H,
                                                      const QuadCorners q, int map_s,
                                                      unsigned char* __restrict__ sums) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const float4 pv = pos[i];
    if (pv.x == 0.0f) {
        sums[i] = 255;
        return;
    }
    Ctx c;
    c.W = map_s;
    c.H = map_s;
    c.fW = (float)map_s;
    c.fH = (float)map_s;
    const V4 v = {pv.x, pv.y, pv.z, pv.w};
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const V4 sc = mat4_mul(q.mvp[k], v);
        c.map = q.maps[k];
        const float d = fetch(c, sc.x / sc.w, sc.y / sc.w);
        sum += (sc.z / sc.w <= d) ? 1.0f : 0.0f;
    }
    sums[i] = (unsigned char)sum;
}

// Evaluation.frag under an occlusion query: a pixel passes when its count
// is 1, 2 or 3 and all eight neighbours have the same count (a neighbour
// outside the image reads the border 0, a background one 0.63); any
// passing pixel asks for the node to be subdivided.
// The evaluation pass runs over a Wq x Hq viewport (W / div, H / div;
// div = 4 in the lower-accuracy mode): coarse pixel i reads the count image
// at its centre, texel floor((2 i + 1) W / (2 Wq)), and its neighbours one
// coarse pixel away (outside the viewport: the border).
__device__ __forceinline__ unsigned qt_coarse(const unsigned char* sums, int W, int H, int Wq, int Hq, int i, int j) {
    if (i < 0 || i >= Wq || j < 0 || j >= Hq) return 0u;
    const int x = (int)(((long long)(2 * i + 1) * W) / (2LL * Wq));
    const int y = (int)(((long long)(2 * j + 1) * H) / (2LL * Hq));
    return sums[(size_t)y * W + x];
}

__global__ void __launch_bounds__(128) k_qt_evaluate(const unsigned char* __restrict__ sums, int W, int H, int Wq,
                                                     int Hq, unsigned* __restrict__ passed) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= Wq || y >= Hq) return;
    const unsigned s = qt_coarse(sums, W, H, Wq, Hq, x, y);
    if (s == 255 || s == 0 || s == 4) return;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx)
            if (qt_coarse(sums, W, H, Wq, Hq, x + dx, y + dy) != s) return;
    atomicOr(passed, 1u);
}

// ---- deferred Phong shading (ShadowMapping/Shaders/GBuffer/PhongShading.frag:11-46)
// color = shadow * fragmentColor * (Idiff + Ispec + Iamb) with the light
// in eye space as the pre-test uses it; E = normalize(-vertex) normalises
// the 4-component eye-space vertex (w = 1) before the vec3 truncation, as
// the shader's implicit conversion does.  pow(x, 0.3 * 10) is evaluated as
// x * x * x.  Background pixels keep the clear colour (0.63, 0.82, 0.96, 1).
__global__ void __launch_bounds__(128) k_phong(const gi_vis_params p, const float4* __restrict__ pos,
                                               const float4* __restrict__ nrm, const float* __restrict__ vis,
                                               const float4* __restrict__ color, float4* __restrict__ out, int W,
                                               int H) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const float4 pv = pos[i];
    if (pv.x == 0.0f) {
        out[i] = make_float4(0.63f, 0.82f, 0.96f, 1.0f);
        return;
    }
    const float4 nv = nrm[i];
    const float shadow = vis[i];
    const float spec_shadow = shadow - p.shadow_intensity;
    V4 v = mat4_mul(p.camera_mv, V4{pv.x, pv.y, pv.z, pv.w});
    const float* nm = p.normal_matrix;
    float nx = nm[0] * nv.x + nm[3] * nv.y + nm[6] * nv.z;
    float ny = nm[1] * nv.x + nm[4] * nv.y + nm[7] * nv.z;
    float nz = nm[2] * nv.x + nm[5] * nv.y + nm[8] * nv.z;
    const float ninv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
    nx = nx * ninv;
    ny = ny * ninv;
    nz = nz * ninv;
    float lx = p.light_position[0] - v.x, ly = p.light_position[1] - v.y, lz = p.light_position[2] - v.z;
    const float linv = 1.0f / sqrtf(lx * lx + ly * ly + lz * lz);
    lx = lx * linv;
    ly = ly * linv;
    lz = lz * linv;
    const float ex0 = -v.x, ey0 = -v.y, ez0 = -v.z, ew0 = -v.w;
    const float einv = 1.0f / sqrtf(ex0 * ex0 + ey0 * ey0 + ez0 * ez0 + ew0 * ew0);
    const float ex = ex0 * einv, ey = ey0 * einv, ez = ez0 * einv;
    // reflect(L, N) = L - 2 * dot(N, L) * N; R = normalize(-reflect)
    const float ndl = nx * lx + ny * ly + nz * lz;
    float rx = -(lx - 2.0f * ndl * nx), ry = -(ly - 2.0f * ndl * ny), rz = -(lz - 2.0f * ndl * nz);
    const float rinv = 1.0f / sqrtf(rx * rx + ry * ry + rz * rz);
    rx = rx * rinv;
    ry = ry * rinv;
    rz = rz * rinv;
    const float diff = gmax(ndl, 0.0f);
    const float re = gmax(rx * ex + ry * ey + rz * ez, 0.0f);
    const float spec = re * re * re;
    const float4 c = color ? color[i] : make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    const float amb[4] = {0.4f, 0.4f, 0.4f, 1.0f}, dif[4] = {0.5f, 0.5f, 0.5f, 1.0f};
    const float spc[4] = {0.25f, 0.25f, 0.25f, 1.0f};
    const float cc[4] = {c.x, c.y, c.z, c.w};
    float o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float idiff = dif[k] * diff;
        const float ispec = (spec_shadow * spc[k]) * spec;
        o[k] = (shadow * cc[k]) * ((idiff + ispec) + amb[k]);
    }
    out[i] = make_float4(o[0], o[1], o[2], o[3]);
}

// The EDTSM branch of the SMSR shaders (NonConservativeSMSR.frag:367-397,
// ConservativeSMSR.frag:215-245): FragData[0] = (shadow, depth,
// preEvaluatedShadow, 1) with depth = position.z / position.w * 0.5 + 0.5,
// FragData[1] = position = MVP * vertex; discarded background pixels keep the
// clear colour (0, 0, 0, 1) in both.  shadow is the visibility target.
__global__ void __launch_bounds__(128) k_edt_inputs(const gi_vis_params p, const dev::Mat4 mvp,
                                                    const float4* __restrict__ pos, const float4* __restrict__ nrm,
                                                    const float* __restrict__ vis, float4* __restrict__ image,
                                                    float4* __restrict__ position, int W, int H) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const float4 pv = pos[i];
    if (pv.x == 0.0f) {
        image[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        position[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        return;
    }
    const float4 nv = nrm[i];
    Ctx c{};
    c.I = p.shadow_intensity;
    const V4 vertex{pv.x, pv.y, pv.z, pv.w};
    const float pre = pretest(p, c, vertex, V4{nv.x, nv.y, nv.z, nv.w});
    const V4 cp = mat4_mul(mvp.m, vertex);
    float depth = cp.z / cp.w;
    depth = depth * 0.5f + 0.5f;
    image[i] = make_float4(vis[i], depth, pre, 1.0f);
    position[i] = make_float4(cp.x, cp.y, cp.z, cp.w);
}

}  // namespace vis

gi_status launch_surrogate_features(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int map_w,
                                    int map_h, const gi_scene* scene, const float camera_mvp[16], int W, int H,
                                    void* d_feat, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    const float sx = (float)(1.0 / (double)map_w), sy = (float)(1.0 / (double)map_h);
    dev::Mat4 m;
    for (int k = 0; k < 16; ++k) m.m[k] = camera_mvp[k];
    vis::k_surrogate_features<<<grid, 128, 0, st>>>(
        *p, d_depth, map_w, map_h, sx, sy, ctx->d_vkeys, scene->d_points, scene->d_normals, scene->d_indices, m,
        static_cast<const unsigned*>(ctx->tier_buf[1][6]), static_cast<const dev::BRec*>(ctx->tier_buf[1][0]),
        static_cast<const uint4*>(ctx->tier_buf[1][7]), W, H, static_cast<uint4*>(d_feat));
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "surrogate features launch");
}

gi_status launch_surrogate_finish(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int map_w,
                                  int map_h, const gi_scene* scene, const float camera_mvp[16], int W, int H,
                                  const float* d_head, int head_stride, const void* d_feat, float thr,
                                  float* d_vis, unsigned* d_fallback, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    const float sx = (float)(1.0 / (double)map_w), sy = (float)(1.0 / (double)map_h);
    dev::Mat4 m;
    for (int k = 0; k < 16; ++k) m.m[k] = camera_mvp[k];
    vis::k_surrogate_finish<<<grid, 128, 0, st>>>(
        *p, d_depth, map_w, map_h, sx, sy, ctx->d_vkeys, scene->d_points, scene->d_normals, scene->d_indices, m,
        static_cast<const unsigned*>(ctx->tier_buf[1][6]), static_cast<const dev::BRec*>(ctx->tier_buf[1][0]),
        static_cast<const uint4*>(ctx->tier_buf[1][7]), d_head, head_stride, static_cast<const uint4*>(d_feat), thr,
        d_vis, W, H, d_fallback);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "surrogate finish launch");
}

gi_status launch_edt_inputs(gi_context* ctx, const gi_vis_params* p, const float camera_mvp[16], const float* d_pos,
                            const float* d_nrm, const float* d_vis, float* d_image, float* d_position, int W, int H,
                            cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    dev::Mat4 m;
    for (int k = 0; k < 16; ++k) m.m[k] = camera_mvp[k];
    vis::k_edt_inputs<<<grid, 128, 0, st>>>(*p, m, reinterpret_cast<const float4*>(d_pos),
                                            reinterpret_cast<const float4*>(d_nrm), d_vis,
                                            reinterpret_cast<float4*>(d_image), reinterpret_cast<float4*>(d_position),
                                            W, H);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "EDT inputs launch");
}

gi_status launch_phong(gi_context* ctx, const gi_vis_params* p, const float* d_pos, const float* d_nrm,
                       const float* d_vis, const float* d_color, float* d_out, int W, int H, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    vis::k_phong<<<grid, 128, 0, st>>>(*p, reinterpret_cast<const float4*>(d_pos),
                                      reinterpret_cast<const float4*>(d_nrm), d_vis,
                                      reinterpret_cast<const float4*>(d_color), reinterpret_cast<float4*>(d_out), W, H);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "phong launch");
}

gi_status launch_qt_evaluate(gi_context* ctx, const float* d_pos, int W, int H, int div, const QuadCorners& q,
                            int map_s, unsigned char* d_sums, unsigned* d_passed, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    vis::k_qt_reproject<<<grid, 128, 0, st>>>(reinterpret_cast<const float4*>(d_pos), W, H, q, map_s, d_sums);
    const int Wq = W / div, Hq = H / div;
    vis::k_qt_evaluate<<<dim3((Wq + 31) / 32, (Hq + 3) / 4), 128, 0, st>>>(d_sums, W, H, Wq, Hq, d_passed);
    ctx->launches += 2;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "quad-tree evaluation launch");
}

gi_status launch_area_accumulate(gi_context* ctx, const gi_scene* scene, const float camera_mvp[16], int W, int H,
                                 const float* maps, int map_s, int nw, const AreaWave& wave, float intensity,
                                 bool first, bool last, float count, float* d_vis, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    dev::Mat4 m;
    for (int k = 0; k < 16; ++k) m.m[k] = camera_mvp[k];
    vis::k_area_accumulate<<<grid, 128, 0, st>>>(
        maps, map_s, nw, wave, intensity, ctx->d_vkeys, scene->d_points, scene->d_normals, scene->d_indices, m,
        static_cast<const unsigned*>(ctx->tier_buf[1][6]), static_cast<const dev::BRec*>(ctx->tier_buf[1][0]),
        static_cast<const uint4*>(ctx->tier_buf[1][7]), ctx->d_area_acc, first ? 1 : 0, last ? 1 : 0, count, d_vis, W, H);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "area-light accumulate launch");
}

// c_poisson[i] * bsw for the PCSS_POISSON blocker taps (blocker_search_width:
// lightSourceRadius / min(map width, 1024)), each product rounded once as
// the kernel's multiplication would round it.
static vis::PoissonOffsets poisson_offsets(const gi_vis_params* p, int map_w) {
    vis::PoissonOffsets po{};
    if (p->technique == GI_TECH_PCF) {
        // the offsets of Shadow.frag's float loop (:86-116), as the kernel's
        // loop produces them
        const float offset = (float)p->penumbra_size;
        const float step = 2.0f * offset / (float)p->kernel_order;
        int n = 0;
        float last = -offset;
        if (step > 0.0f)
            for (float w = -offset; w < offset && n <= 64; w += step) {
                last = w;
                ++n;
            }
        if (n >= 1 && n <= 64) {
            po.pcf_lo = -offset;
            po.pcf_hi = last;
            po.pcf_count = n * n;
        }
        return po;
    }
    if (p->technique != GI_TECH_PCSS_POISSON) return po;
    const float fw = (float)map_w;
    const float bsw = fw <= 1024.0f ? p->light_radius / fw : p->light_radius / 1024.0f;
    po.bmin = po.fmin = make_float2(INFINITY, INFINITY);
    po.bmax = po.fmax = make_float2(-INFINITY, -INFINITY);
    for (int i = 0; i < 64 && i < p->poisson_blocker_taps; ++i) {
        po.b[i] = make_float2(kPoissonDisk[i][0] * bsw, kPoissonDisk[i][1] * bsw);
        po.bmin = make_float2(std::min(po.bmin.x, po.b[i].x), std::min(po.bmin.y, po.b[i].y));
        po.bmax = make_float2(std::max(po.bmax.x, po.b[i].x), std::max(po.bmax.y, po.b[i].y));
    }
    for (int j = 0; j < 64 && j < p->poisson_filter_taps; ++j) {
        po.fmin = make_float2(std::min(po.fmin.x, kPoissonDisk[j][0]), std::min(po.fmin.y, kPoissonDisk[j][1]));
        po.fmax = make_float2(std::max(po.fmax.x, kPoissonDisk[j][0]), std::max(po.fmax.y, kPoissonDisk[j][1]));
    }
    return po;
}

// PCSS_POISSON and PCF read the light map's min-max pyramid to skip taps
// exactly (maps with sides that are multiples of 64; others run every tap).
static gi_status prepare_pyramid(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int map_w,
                                 int map_h, cudaStream_t st, vis::PoissonOffsets* po) {
    if (!ctx->tap_pyramid) return GI_OK;  // boxes of up to 3 x 3 texels are still skipped
    const bool pcss = p->technique == GI_TECH_PCSS_POISSON && p->poisson_blocker_taps >= 1 &&
                      p->poisson_filter_taps >= 1;
    const bool pcf = p->technique == GI_TECH_PCF && po->pcf_count > 0;
    if (!pcss && !pcf) return GI_OK;
    return launch_minmax_pyramid(ctx, d_depth, map_w, map_h, st, &po->pyr);
}

// The maps the moment techniques read instead of (VSM..MSM) or beside
// (SAVSM..MSSM) the light map, and the MSM constants.
static gi_status prepare_maps(gi_context* ctx, const gi_vis_params* p, const float** d_depth, int* map_w,
                              int* map_h, int W, cudaStream_t st, SoftMaps* sm) {
    const int t = p->technique;
    gi_status s = GI_OK;
    if (is_moment_technique(t)) {
        s = launch_moments(ctx, t, *d_depth, *map_w, W, st, d_depth);
        *map_w = *map_h = W;
    } else if (is_soft_moment_technique(t)) {
        s = soft_moment_prepare(ctx, p, *d_depth, *map_w, *map_h, st, sm);
    }
    if (s != GI_OK || (t != GI_TECH_MSM && t != GI_TECH_MSSM)) return s;
    float mq[16], h[20];
    moment_quantization(mq, h, &h[16]);
    h[17] = h[18] = h[19] = 0.0f;
    const cudaError_t e = cudaMemcpyToSymbolAsync(vis::c_msm, h, sizeof h, 0, cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "MSM constants");
}

gi_status launch_visibility(gi_context* ctx, const gi_vis_params* p, const float* d_depth,
                            int map_w, int map_h, const float* d_pos, const float* d_nrm,
                            float* d_vis, int W, int H, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    SoftMaps sm;
    gi_status ps = prepare_maps(ctx, p, &d_depth, &map_w, &map_h, W, st, &sm);
    if (ps != GI_OK) return ps;
    // shadowMapStep = (1.0 / w, 1.0 / h) in double, stored as float
    // (glUniform2f at MyGLGeometryViewer.cpp:237-238)
    const float sx = (float)(1.0 / (double)map_w), sy = (float)(1.0 / (double)map_h);
    const float4* pos = reinterpret_cast<const float4*>(d_pos);
    const float4* nrm = reinterpret_cast<const float4*>(d_nrm);
    vis::PoissonOffsets po = poisson_offsets(p, map_w);
    ps = prepare_pyramid(ctx, p, d_depth, map_w, map_h, st, &po);
    if (ps != GI_OK) return ps;
#define GI_VIS_CASE(T)                                                                     \
    case T:                                                                                \
        vis::k_visibility<T><<<grid, 128, 0, st>>>(*p, d_depth, map_w, map_h, sx, sy, pos, nrm, d_vis, W, H, sm, po); \
        break;
    switch (p->technique) {
        GI_VIS_CASE(GI_TECH_HARD)
        GI_VIS_CASE(GI_TECH_PCF)
        GI_VIS_CASE(GI_TECH_PCF_TRICUBIC)
        GI_VIS_CASE(GI_TECH_PCSS_GRID)
        GI_VIS_CASE(GI_TECH_PCSS_POISSON)
        GI_VIS_CASE(GI_TECH_SMSR_CONSERVATIVE)
        GI_VIS_CASE(GI_TECH_SMSR_NONCONSERVATIVE)
        GI_VIS_CASE(GI_TECH_RPCF_CONSERVATIVE)
        GI_VIS_CASE(GI_TECH_RPCF_SMSR)
        GI_VIS_CASE(GI_TECH_RSMSS)
        GI_VIS_CASE(GI_TECH_HARD_SOFTAPP)
        GI_VIS_CASE(GI_TECH_RBSSM)
        GI_VIS_CASE(GI_TECH_VSM)
        GI_VIS_CASE(GI_TECH_ESM)
        GI_VIS_CASE(GI_TECH_EVSM)
        GI_VIS_CASE(GI_TECH_MSM)
        GI_VIS_CASE(GI_TECH_SAVSM)
        GI_VIS_CASE(GI_TECH_VSSM)
        GI_VIS_CASE(GI_TECH_ESSM)
        GI_VIS_CASE(GI_TECH_MSSM)
        default:
            return fail(GI_ERR_INVALID_ARG, "gi_visibility: unknown technique");
    }
#undef GI_VIS_CASE
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "visibility kernel launch");
}

gi_status launch_frame_visibility(gi_context* ctx, const gi_vis_params* p, const float* d_depth,
                                  int map_w, int map_h, const gi_scene* scene, const float camera_mvp[16],
                                  float* d_vis, int W, int H, float* d_pos, float* d_nrm,
                                  cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 3) / 4);
    SoftMaps sm;
    gi_status ps = prepare_maps(ctx, p, &d_depth, &map_w, &map_h, W, st, &sm);
    if (ps != GI_OK) return ps;
    const float sx = (float)(1.0 / (double)map_w), sy = (float)(1.0 / (double)map_h);
    const unsigned* rec_of = static_cast<const unsigned*>(ctx->tier_buf[1][6]);
    const dev::BRec* recs = static_cast<const dev::BRec*>(ctx->tier_buf[1][0]);
    const uint4* rres = static_cast<const uint4*>(ctx->tier_buf[1][7]);
    dev::Mat4 m;
    for (int k = 0; k < 16; ++k) m.m[k] = camera_mvp[k];
    float4* po = reinterpret_cast<float4*>(d_pos);
    float4* no = reinterpret_cast<float4*>(d_nrm);
    vis::PoissonOffsets boff = poisson_offsets(p, map_w);
    ps = prepare_pyramid(ctx, p, d_depth, map_w, map_h, st, &boff);
    if (ps != GI_OK) return ps;
#define GI_FRAME_CASE(T)                                                                          \
    case T:                                                                                       \
        vis::k_frame_visibility<T><<<grid, 128, 0, st>>>(*p, d_depth, map_w, map_h, sx, sy,         \
                                                          ctx->d_vkeys, scene->d_points,          \
                                                          scene->d_normals, scene->d_indices, m,  \
                                                          rec_of, recs, rres, d_vis, W, H, po, no, sm, boff); \
        break;
    switch (p->technique) {
        GI_FRAME_CASE(GI_TECH_HARD)
        GI_FRAME_CASE(GI_TECH_PCF)
        GI_FRAME_CASE(GI_TECH_PCF_TRICUBIC)
        GI_FRAME_CASE(GI_TECH_PCSS_GRID)
        GI_FRAME_CASE(GI_TECH_PCSS_POISSON)
        GI_FRAME_CASE(GI_TECH_SMSR_CONSERVATIVE)
        GI_FRAME_CASE(GI_TECH_SMSR_NONCONSERVATIVE)
        GI_FRAME_CASE(GI_TECH_RPCF_CONSERVATIVE)
        GI_FRAME_CASE(GI_TECH_RPCF_SMSR)
        GI_FRAME_CASE(GI_TECH_RSMSS)
        GI_FRAME_CASE(GI_TECH_HARD_SOFTAPP)
        GI_FRAME_CASE(GI_TECH_RBSSM)
        GI_FRAME_CASE(GI_TECH_VSM)
        GI_FRAME_CASE(GI_TECH_ESM)
        GI_FRAME_CASE(GI_TECH_EVSM)
        GI_FRAME_CASE(GI_TECH_MSM)
        GI_FRAME_CASE(GI_TECH_SAVSM)
        GI_FRAME_CASE(GI_TECH_VSSM)
        GI_FRAME_CASE(GI_TECH_ESSM)
        GI_FRAME_CASE(GI_TECH_MSSM)
        default:
            return fail(GI_ERR_INVALID_ARG, "gi_render_frame: unknown technique");
    }
#undef GI_FRAME_CASE
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "frame visibility kernel launch");
}

bool batch_visibility_supported(int technique) {
    switch (technique) {
        case GI_TECH_HARD:
        case GI_TECH_PCF:
        case GI_TECH_PCF_TRICUBIC:
        case GI_TECH_PCSS_GRID:
        case GI_TECH_PCSS_POISSON:
        case GI_TECH_SMSR_CONSERVATIVE:
        case GI_TECH_SMSR_NONCONSERVATIVE:
        case GI_TECH_RPCF_CONSERVATIVE:
        case GI_TECH_RPCF_SMSR:
        case GI_TECH_RSMSS:
        case GI_TECH_HARD_SOFTAPP:
        case GI_TECH_RBSSM:
            return true;
        default:
            return false;  // the moment techniques need per-light prepared maps
    }
}

gi_status launch_batch_visibility(int technique, const BatchLightFrame* d_lf, int n_lf, unsigned total_tiles,
                                  unsigned* d_queue, int tile_w, int tile_h, int grid, cudaStream_t st) {
#define GI_BATCH_CASE(T)                                                                                 \
    case T:                                                                                              \
        vis::k_batch_visibility<T><<<grid, 128, 0, st>>>(d_lf, n_lf, total_tiles, d_queue, tile_w, tile_h); \
        break;
    switch (technique) {
        GI_BATCH_CASE(GI_TECH_HARD)
        GI_BATCH_CASE(GI_TECH_PCF)
        GI_BATCH_CASE(GI_TECH_PCF_TRICUBIC)
        GI_BATCH_CASE(GI_TECH_PCSS_GRID)
        GI_BATCH_CASE(GI_TECH_PCSS_POISSON)
        GI_BATCH_CASE(GI_TECH_SMSR_CONSERVATIVE)
        GI_BATCH_CASE(GI_TECH_SMSR_NONCONSERVATIVE)
        GI_BATCH_CASE(GI_TECH_RPCF_CONSERVATIVE)
        GI_BATCH_CASE(GI_TECH_RPCF_SMSR)
        GI_BATCH_CASE(GI_TECH_RSMSS)
        GI_BATCH_CASE(GI_TECH_HARD_SOFTAPP)
        GI_BATCH_CASE(GI_TECH_RBSSM)
        default:
            return fail(GI_ERR_UNSUPPORTED, "persistent batch visibility: technique needs prepared maps");
    }
#undef GI_BATCH_CASE
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "persistent batch visibility launch");
}

}  // namespace gi
