// moments.cu -- moment shadow maps for sm_103a: ShadowMapping's filtered
// maps (VSM, ESM, EVSM, MSM) and SoftShadowMapping's moment soft shadows
// (SAVSM, VSSM, ESSM, MSSM: moment map, summed-area table, min-max levels).
//
// The reference renders a moment map instead of a depth map for these
// techniques, blurs it into a window-size target and samples the blurred
// map in Shadow.frag (ShadowMapping/src/main.cpp:220-240, 374-396).  Its GL
// path leaves several choices to the driver; each is fixed here, and the CPU
// oracle makes the same ones:
//
//   * moments come from the light map's depth (the value the depth test
//     kept, polygon offset included) rather than from the interpolated clip
//     position; a texel no fragment reached keeps the clear colour (0,0,0,1);
//   * dFdx / dFdy are the differences inside each 2 x 2 texel quad (right
//     minus left, top minus bottom), 0 where the quad partner is empty;
//   * the map is reduced to the window size by 2 x 2 box averages, one mip
//     level at a time ((a + b) + (c + d)) * 0.25, which is what the filter's
//     texture2D reads at lod log2(map / window) when that is an integer;
//   * the 7 Gaussian taps (Filter::buildGaussianKernel(7): binomial / 64)
//     land on texel centres, outside the target they read the border (0);
//     products and sums round separately, in tap order;
//   * Shadow.frag reads the blurred map bilinearly at level 0 with FP32
//     weights and a zero border.
//
//   k_moments       Moments.frag / Exponential.frag / ExponentialMoments.frag
//                   per light-map texel (+ MSM's quantisation)
//   k_moments_box   the same fused with the first box level: one thread per
//                   2 x 2 quad, so the full-size moment map is never stored
//   k_mip_box       one further 2 x 2 box level
//   k_moment_blur   GaussianFilter.frag (VSM, EVSM, MSM) or
//                   LogGaussianFilter.frag (ESM), one direction per launch
//   k_soft_moments  SoftShadowMapping's Moments.frag / Exponential.frag
//   k_sat_level     one horizontal + vertical SAT iteration (float4, or
//   k_sat_level2    .xy only for SAVSM / VSSM)
//   k_hsm_first / k_hsm_next / k_hsm_level0
//                   PrepareMinMax.frag and MinMax.frag levels
#include <cuda_runtime.h>

#include <cmath>

#include "internal.h"
#include "raster.h"
#include "launch.cuh"

namespace gi {
namespace mom {

__constant__ float kWeights[7] = {1.0f / 64.0f, 6.0f / 64.0f, 15.0f / 64.0f, 20.0f / 64.0f,
                               15.0f / 64.0f, 6.0f / 64.0f, 1.0f / 64.0f};

// linearize of the moment shaders and Shadow.frag (zNear = 1, zFar = 1000
// int uniforms, MyGLGeometryViewer.cpp:7-8,98-105): all-float GLSL.
__device__ __forceinline__ float gl_linearize(float depth) { return 2.0f / (1001.0f - depth * 999.0f); }

struct MomArgs {
    const float* depth;  // S x S light map
    float4* out;         // S x S moment map
    int S, tech;
    float mq[16], tq0;   // MSM quantisation (column-major) and tQuantization.x
};

__device__ __forceinline__ float lin_at(const MomArgs& a, int x, int y, bool& empty) {
    const float d = __ldg(a.depth + (size_t)y * a.S + x);
    empty = !(d < 1.0f);
    return gl_linearize(d);
}

// Moments.frag / Exponential.frag / ExponentialMoments.frag for texel
// (x, y); l, r, b, t are the linearised depths of its 2 x 2 quad partners
// (left / right of its row, bottom / top of its column).
__device__ __forceinline__ float4 moment_of(const MomArgs& a, float d, bool empty, float l, bool el, float r, bool er,
                                            float b, bool eb, float t, bool et) {
    if (empty) return make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (a.tech == GI_TECH_ESM) return make_float4(d, 0.0f, 0.0f, 1.0f);
    if (a.tech == GI_TECH_MSM) {
        const float d2 = d * d, d3 = d2 * d, d4 = d3 * d;
        const float* q = a.mq;
        return make_float4(q[0] * d + q[4] * d2 + q[8] * d3 + q[12] * d4 + a.tq0,
                           q[1] * d + q[5] * d2 + q[9] * d3 + q[13] * d4 + 0.0f,
                           q[2] * d + q[6] * d2 + q[10] * d3 + q[14] * d4 + 0.0f,
                           q[3] * d + q[7] * d2 + q[11] * d3 + q[15] * d4 + 0.0f);
    }
    // VSM / EVSM: moment.y += 0.25 * (dFdx^2 + dFdy^2) over the 2 x 2 quad
    const float dx = (el || er) ? 0.0f : r - l;
    const float dy = (eb || et) ? 0.0f : t - b;
    float m2 = d * d;
    m2 = m2 + 0.25f * (dx * dx + dy * dy);
    return a.tech == GI_TECH_EVSM ? make_float4(d, m2, d, 1.0f) : make_float4(d, m2, 0.0f, 0.0f);
}

// The moment map at the light map's own size (map side == window side).
__global__ void __launch_bounds__(256) k_moments(const MomArgs a) {
    pdl_enter();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= a.S || y >= a.S) return;
    bool e, el, er, eb, et;
    const int xr = (x | 1) < a.S ? (x | 1) : x, yt = (y | 1) < a.S ? (y | 1) : y;
    const float d = lin_at(a, x, y, e);
    const float l = lin_at(a, x & ~1, y, el), r = lin_at(a, xr, y, er);
    const float b = lin_at(a, x, y & ~1, eb), t = lin_at(a, x, yt, et);
    a.out[(size_t)y * a.S + x] = moment_of(a, d, e, l, el, r, er, b, eb, t, et);
}

// The moment map's first box level directly (map side == 2 x the output
// side): each thread reads one 2 x 2 quad of depths, forms the four texels'
// moments (the quad is also where dFdx / dFdy come from) and writes their
// box average ((q00 + q10) + (q01 + q11)) * 0.25, so the full-size moment
// map is never stored.
__global__ void __launch_bounds__(256) k_moments_box(const MomArgs a) {
    pdl_enter();
    const int h = a.S / 2;
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= h || y >= h) return;
    bool e00, e10, e01, e11;
    const float d00 = lin_at(a, 2 * x, 2 * y, e00), d10 = lin_at(a, 2 * x + 1, 2 * y, e10);
    const float d01 = lin_at(a, 2 * x, 2 * y + 1, e01), d11 = lin_at(a, 2 * x + 1, 2 * y + 1, e11);
    // per texel: row partners (left, right) and column partners (bottom, top)
    const float4 q00 = moment_of(a, d00, e00, d00, e00, d10, e10, d00, e00, d01, e01);
    const float4 q10 = moment_of(a, d10, e10, d00, e00, d10, e10, d10, e10, d11, e11);
    const float4 q01 = moment_of(a, d01, e01, d01, e01, d11, e11, d00, e00, d01, e01);
    const float4 q11 = moment_of(a, d11, e11, d01, e01, d11, e11, d10, e10, d11, e11);
    const float4 s = make_float4((q00.x + q10.x) + (q01.x + q11.x), (q00.y + q10.y) + (q01.y + q11.y),
                                 (q00.z + q10.z) + (q01.z + q11.z), (q00.w + q10.w) + (q01.w + q11.w));
    a.out[(size_t)y * h + x] = make_float4(s.x * 0.25f, s.y * 0.25f, s.z * 0.25f, s.w * 0.25f);
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

// One mip level of glGenerateMipmap as a 2 x 2 box: ((a + b) + (c + d)) * 0.25.
__global__ void __launch_bounds__(256) k_mip_box(const float4* __restrict__ in, int S, float4* __restrict__ out) {
    pdl_enter();
    const int h = S / 2;
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= h || y >= h) return;
    const float4 a = in[(size_t)(2 * y) * S + 2 * x], b = in[(size_t)(2 * y) * S + 2 * x + 1];
    const float4 c = in[(size_t)(2 * y + 1) * S + 2 * x], d = in[(size_t)(2 * y + 1) * S + 2 * x + 1];
    const float4 s = add4(add4(a, b), add4(c, d));
    out[(size_t)y * h + x] = make_float4(s.x * 0.25f, s.y * 0.25f, s.z * 0.25f, s.w * 0.25f);
}

// GaussianFilter.frag: sum += texture2D(image, centre + dir * k * step) *
// kernel[3 + k] for k = -3..3; LogGaussianFilter.frag: the log-space chain
// log_conv(x0, X, y0, Y) = X + log(x0 + y0 * exp(Y - X)) over the .x taps.
template <bool LOG>
__global__ void __launch_bounds__(256) k_moment_blur(const float4* __restrict__ in, int N, int dx, int dy,
                                                     float4* __restrict__ out) {
    pdl_enter();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= N || y >= N) return;
    auto tap = [&](int k) {
        const int xx = x + dx * k, yy = y + dy * k;
        if (xx < 0 || xx >= N || yy < 0 || yy >= N) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return in[(size_t)yy * N + xx];
    };
    float4 r;
    if (!LOG) {
        r = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int k = -3; k <= 3; ++k) {
            const float4 t = tap(k);
            const float w = kWeights[3 + k];
            r = make_float4(r.x + t.x * w, r.y + t.y * w, r.z + t.z * w, r.w + t.w * w);
        }
    } else {
        const float s0 = tap(-3).x, s1 = tap(-2).x;
        float sum = s0 + logf(kWeights[0] + kWeights[1] * expf(s1 - s0));
#pragma unroll
        for (int i = 2; i < 7; ++i) sum = sum + logf(1.0f + kWeights[i] * expf(tap(i - 3).x - sum));
        r = make_float4(sum, sum, sum, sum);
    }
    out[(size_t)y * N + x] = r;
}

// ---- moment soft shadows (SoftShadowMapping) ---------------------------------
// The light pass writes Moments.frag (SAVSM, VSSM, MSSM) or Exponential.frag
// (ESSM) into an S x T colour target cleared to 0, read unblurred at the
// map's size.  Same driver choices as above (moments from the light map's
// depth, quad differences for dFdx / dFdy).
struct SoftMomArgs {
    const float* depth;  // S x T light map
    float4* out;         // S x T moment map
    float2* out2;        // or its .xy only (SAVSM / VSSM, whose .zw are 0)
    int S, T, tech;
    float mq[16], tq0;
};

__device__ __forceinline__ float soft_lin_at(const SoftMomArgs& a, int x, int y, bool& empty) {
    const float d = __ldg(a.depth + (size_t)y * a.S + x);
    empty = !(d < 1.0f);
    return gl_linearize(d);
}

template <bool TWO, bool DEP>
__global__ void __launch_bounds__(256) k_soft_moments(const SoftMomArgs a) {
    if (DEP) pdl_enter();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= a.S || y >= a.T) return;
    bool e;
    const float d = soft_lin_at(a, x, y, e);
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!e) {
        if (a.tech == GI_TECH_ESSM) {
            const float ex = expf(80.0f * d);
            o = make_float4(d, ex, ex * d, 0.0f);
        } else if (a.tech == GI_TECH_MSSM) {
            const float d2 = d * d, d3 = d2 * d, d4 = d3 * d;
            const float* q = a.mq;
            o = make_float4(q[0] * d + q[4] * d2 + q[8] * d3 + q[12] * d4 + a.tq0,
                            q[1] * d + q[5] * d2 + q[9] * d3 + q[13] * d4 + 0.0f,
                            q[2] * d + q[6] * d2 + q[10] * d3 + q[14] * d4 + 0.0f,
                            q[3] * d + q[7] * d2 + q[11] * d3 + q[15] * d4 + 0.0f);
        } else {
            bool el, er, eb, et;
            const int xr = (x | 1) < a.S ? (x | 1) : x, yt = (y | 1) < a.T ? (y | 1) : y;
            const float l = soft_lin_at(a, x & ~1, y, el), r = soft_lin_at(a, xr, y, er);
            const float b = soft_lin_at(a, x, y & ~1, eb), t = soft_lin_at(a, x, yt, et);
            const float dx = (el || er) ? 0.0f : r - l;
            const float dy = (eb || et) ? 0.0f : t - b;
            o = make_float4(d - 0.5f, d * d + (0.25f * (dx * dx + dy * dy) - 0.5f), 0.0f, 0.0f);
        }
    }
    if (TWO) a.out2[(size_t)y * a.S + x] = make_float2(o.x, o.y);
    else a.out[(size_t)y * a.S + x] = o;
}

// One iteration i of the summed-area table (SATHorizontalPass.frag then
// SATVerticalPass.frag at offset d = 2^i, main.cpp:943-971):
//   t(x, y) = s(x, y) + s(x - d, y),  s'(x, y) = t(x, y) + t(x, y - d),
// i.e. s' = (s(x, y) + s(x - d, y)) + (s(x, y - d) + s(x - d, y - d)), reads
// outside the map being 0 (CLAMP_TO_BORDER), each sum rounded as written.
template <bool DEP>  // DEP: launched as a programmatic dependent (launch_dependent_if)
__global__ void __launch_bounds__(256) k_sat_level(const float4* __restrict__ in, int S, int T, int d,
                                                   float4* __restrict__ out) {
    if (DEP) pdl_enter();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= S || y >= T) return;
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const bool l = x >= d, u = y >= d;
    const float4 a = in[(size_t)y * S + x];
    const float4 b = l ? in[(size_t)y * S + x - d] : z;
    const float4 c = u ? in[(size_t)(y - d) * S + x] : z;
    const float4 e = (l && u) ? in[(size_t)(y - d) * S + x - d] : z;
    out[(size_t)y * S + x] = add4(add4(a, b), add4(c, e));
}

// The same over the .xy of SAVSM / VSSM tables, whose .zw stay +0 (sums of
// +0): half the traffic; the last iteration writes the float4 table.
template <bool LAST, bool DEP>
__global__ void __launch_bounds__(256) k_sat_level2(const float2* __restrict__ in, int S, int T, int d,
                                                    float2* __restrict__ out2, float4* __restrict__ out4) {
    if (DEP) pdl_enter();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= S || y >= T) return;
    const float2 z = make_float2(0.0f, 0.0f);
    const bool l = x >= d, u = y >= d;
    const float2 a = in[(size_t)y * S + x];
    const float2 b = l ? in[(size_t)y * S + x - d] : z;
    const float2 c = u ? in[(size_t)(y - d) * S + x] : z;
    const float2 e = (l && u) ? in[(size_t)(y - d) * S + x - d] : z;
    const float sx = (a.x + b.x) + (c.x + e.x), sy = (a.y + b.y) + (c.y + e.y);
    if (LAST) out4[(size_t)y * S + x] = make_float4(sx, sy, 0.0f, 0.0f);
    else out2[(size_t)y * S + x] = make_float2(sx, sy);
}

// renderHSM (main.cpp:696-751).  Level 0 (PrepareMinMax.frag) is
// ((d == 0 ? 1 : d) + alpha, d + beta) per light-map texel; level k
// (MinMax.frag) reads level k - 1 at the output texel's centre +- one output
// texel in x and y: two input texels, i.e. half-texel positions, so each
// read is the 0.25-weighted bilinear average of a 2 x 2 block, and the
// texel keeps the min of the .x and the max of the .y of the four reads.
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }

__device__ __forceinline__ float2 hsm0_texel(const float* __restrict__ depth, int S, int T, int i, int j,
                                             float alpha, float beta) {
    if (i < 0 || i >= S || j < 0 || j >= T) return make_float2(0.0f, 0.0f);
    const float d = __ldg(depth + (size_t)j * S + i);
    return make_float2((d == 0.0f ? 1.0f : d) + alpha, d + beta);
}

template <class F>
__device__ __forceinline__ float2 hsm_quad(const F& tex, int i0, int j0) {
    const float2 a = tex(i0, j0), b = tex(i0 + 1, j0), c = tex(i0, j0 + 1), d = tex(i0 + 1, j0 + 1);
    return make_float2(((0.25f * a.x + 0.25f * b.x) + 0.25f * c.x) + 0.25f * d.x,
                       ((0.25f * a.y + 0.25f * b.y) + 0.25f * c.y) + 0.25f * d.y);
}

template <class F>
__device__ __forceinline__ float2 hsm_minmax(const F& tex, int i, int j) {
    const int xa = 2 * i - 2, xb = 2 * i + 2, ya = 2 * j - 2, yb = 2 * j + 2;
    const float2 v0 = hsm_quad(tex, xa, ya), v1 = hsm_quad(tex, xa, yb);
    const float2 v2 = hsm_quad(tex, xb, ya), v3 = hsm_quad(tex, xb, yb);
    return make_float2(gmin(v0.x, gmin(v1.x, gmin(v2.x, v3.x))), gmax(v0.y, gmax(v1.y, gmax(v2.y, v3.y))));
}

__global__ void __launch_bounds__(256) k_hsm_level0(const float* __restrict__ depth, int S, int T, float alpha,
                                                    float beta, float2* __restrict__ out) {
    pdl_enter();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= S || y >= T) return;
    out[(size_t)y * S + x] = hsm0_texel(depth, S, T, x, y, alpha, beta);
}

// level 1 straight from the light map (level 0 is never stored)
__global__ void __launch_bounds__(256) k_hsm_first(const float* __restrict__ depth, int S, int T, float alpha,
                                                   float beta, float2* __restrict__ out) {
    pdl_enter();
    const int w = S / 2, h = T / 2;
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= w || y >= h) return;
    const auto tex = [&](int i, int j) { return hsm0_texel(depth, S, T, i, j, alpha, beta); };
    out[(size_t)y * w + x] = hsm_minmax(tex, x, y);
}

__global__ void __launch_bounds__(256) k_hsm_next(const float2* __restrict__ in, int pw, int ph,
                                                  float2* __restrict__ out) {
    pdl_enter();
    const int w = pw / 2, h = ph / 2;
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= w || y >= h) return;
    const auto tex = [&](int i, int j) {
        return (i >= 0 && i < pw && j >= 0 && j < ph) ? __ldg(in + (size_t)j * pw + i) : make_float2(0.0f, 0.0f);
    };
    out[(size_t)y * w + x] = hsm_minmax(tex, x, y);
}

}  // namespace mom

bool is_moment_technique(int t) { return t >= GI_TECH_VSM && t <= GI_TECH_MSM; }

bool is_soft_moment_technique(int t) { return t >= GI_TECH_SAVSM && t <= GI_TECH_MSSM; }

static bool power_of_two(int v) { return v > 0 && (v & (v - 1)) == 0; }

gi_status soft_moment_check_shape(int tech, int map_w, int map_h, const char* who) {
    if (tech == GI_TECH_VSSM && !(map_w == map_h && power_of_two(map_w) && map_w >= 8))
        return fail(GI_ERR_UNSUPPORTED, std::string(who) + ": VSSM needs a square power-of-two map of side >= 8");
    return GI_OK;
}

// main.cpp:943: int m = std::logf(shadowMapWidth) / std::logf(2), in float
static int sat_iterations(int S) { return (int)(logf((float)S) / logf(2.0f)); }

gi_status launch_soft_moment_map(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T,
                                 cudaStream_t st, float4* dst, const float4** out) {
    using namespace mom;
    const size_t n = (size_t)S * T;
    const bool sat = p->summed_area_table != 0;
    const int m = sat ? sat_iterations(S) : 0;
    const bool two = m > 0 && (p->technique == GI_TECH_SAVSM || p->technique == GI_TECH_VSSM);
    SoftMomArgs a;
    a.depth = d_depth;
    a.S = S;
    a.T = T;
    a.tech = p->technique;
    float mqi[16];
    moment_quantization(a.mq, mqi, &a.tq0);
    const dim3 grid((S + 31) / 32, (T + 7) / 8);
    // the chain of log2(S) dependent passes as programmatic dependent
    // launches up to 1024^2 (SAVSM 0.073 -> 0.062 ms, MSSM 0.083 -> 0.062
    // ms); ordinary launches above (the 2048^2 two-channel table lost 18 %)
    const bool small = (size_t)S * T <= (size_t)1024 * 1024;
    if (two) {
        // .xy planes ping-pong in the scratch, the last iteration writes the
        // float4 table into dst (or the scratch's first part)
        const size_t fin = dst ? 0 : n * sizeof(float4);
        gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_mom), &ctx->cap_mom, fin + 2 * n * sizeof(float2));
        if (s != GI_OK) return s;
        float4* last = dst ? dst : reinterpret_cast<float4*>(ctx->d_mom);
        float2* pa = reinterpret_cast<float2*>(static_cast<char*>(ctx->d_mom) + fin);
        float2* pb = pa + n;
        a.out = nullptr;
        a.out2 = pa;
        if (small) launch_dependent_if(true, k_soft_moments<true, true>, grid, dim3(256), 0, st, a);
        else k_soft_moments<true, false><<<grid, 256, 0, st>>>(a);
        ctx->launches++;
        const float2* cur = pa;
        for (int i = 0; i < m; ++i) {
            float2* nxt = (cur == pa) ? pb : pa;
            float2* o2 = i == m - 1 ? nullptr : nxt;
            float4* o4 = i == m - 1 ? last : nullptr;
            if (small) {
                if (i == m - 1) launch_dependent_if(true, k_sat_level2<true, true>, grid, dim3(256), 0, st, cur, S, T, 1 << i, o2, o4);
                else launch_dependent_if(true, k_sat_level2<false, true>, grid, dim3(256), 0, st, cur, S, T, 1 << i, o2, o4);
            } else {
                if (i == m - 1) k_sat_level2<true, false><<<grid, 256, 0, st>>>(cur, S, T, 1 << i, o2, o4);
                else k_sat_level2<false, false><<<grid, 256, 0, st>>>(cur, S, T, 1 << i, o2, o4);
            }
            ctx->launches++;
            cur = nxt;
        }
        *out = last;
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? GI_OK : fail_cuda(e, "soft moment map launch");
    }
    // m + 1 writes (the moment map, then one per SAT iteration) alternate
    // between two buffers so that the last lands in dst (or in the scratch)
    const size_t scratch = dst ? (m > 0 ? 1 : 0) : (m > 0 ? 2 : 1);
    gi_status s = GI_OK;
    if (scratch) s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_mom), &ctx->cap_mom, scratch * n * sizeof(float4));
    if (s != GI_OK) return s;
    float4* last = dst ? dst : reinterpret_cast<float4*>(ctx->d_mom);
    float4* spare = dst ? reinterpret_cast<float4*>(ctx->d_mom) : last + n;
    a.out = (m % 2 == 0) ? last : spare;
    a.out2 = nullptr;
    if (small) launch_dependent_if(true, k_soft_moments<false, true>, grid, dim3(256), 0, st, a);
    else k_soft_moments<false, false><<<grid, 256, 0, st>>>(a);
    ctx->launches++;
    float4* cur = a.out;
    for (int i = 0; i < m; ++i) {
        float4* nxt = (cur == last) ? spare : last;
        if (small) launch_dependent_if(true, k_sat_level<true>, grid, dim3(256), 0, st, cur, S, T, 1 << i, nxt);
        else k_sat_level<false><<<grid, 256, 0, st>>>(cur, S, T, 1 << i, nxt);
        ctx->launches++;
        cur = nxt;
    }
    *out = cur;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "soft moment map launch");
}

// Levels 1..L stored one after the other in ctx->d_hsm.
static gi_status hsm_levels(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T, int L,
                            cudaStream_t st, float2** levels) {
    using namespace mom;
    size_t need = 0;
    for (int k = 1; k <= L; ++k) need += (size_t)(S >> k) * (T >> k);
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_hsm), &ctx->cap_hsm, need * sizeof(float2));
    if (s != GI_OK) return s;
    float2* lv = reinterpret_cast<float2*>(ctx->d_hsm);
    for (int k = 1; k <= L; ++k) {
        levels[k] = lv;
        const int w = S >> k, h = T >> k;
        const dim3 grid((w + 31) / 32, (h + 7) / 8);
        if (k == 1)
            launch_dependent(k_hsm_first, grid, dim3(256), 0, st, d_depth, S, T, p->hsm_alpha, p->hsm_beta, lv);
        else
            launch_dependent(k_hsm_next, grid, dim3(256), 0, st, (const float2*)levels[k - 1], S >> (k - 1), T >> (k - 1), lv);
        ctx->launches++;
        lv += (size_t)w * h;
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "min-max shadow map launch");
}

gi_status launch_hsm(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T, int level,
                     cudaStream_t st, const float2** out) {
    using namespace mom;
    if (level == 0) {
        gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_hsm), &ctx->cap_hsm, (size_t)S * T * sizeof(float2));
        if (s != GI_OK) return s;
        float2* lv = reinterpret_cast<float2*>(ctx->d_hsm);
        launch_dependent(k_hsm_level0, dim3((S + 31) / 32, (T + 7) / 8), dim3(256), 0, st, d_depth, S, T, p->hsm_alpha, p->hsm_beta, lv);
        ctx->launches++;
        *out = lv;
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? GI_OK : fail_cuda(e, "min-max shadow map launch");
    }
    float2* levels[32] = {};
    gi_status s = hsm_levels(ctx, p, d_depth, S, T, level, st, levels);
    if (s == GI_OK) *out = levels[level];
    return s;
}

gi_status soft_moment_prepare(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T,
                              cudaStream_t st, SoftMaps* out) {
    *out = SoftMaps{};
    gi_status s = launch_soft_moment_map(ctx, p, d_depth, S, T, st, nullptr, &out->mom);
    if (s != GI_OK || p->technique != GI_TECH_VSSM) return s;
    // computeVisibilityFromHSM (PlausibleSoftShadow.frag:538-539) reads at
    // lod W / 1024 + 0.5 (1.75 above 1024): levels floor(lod) and the next
    const float lod = S > 1024 ? 1.75f : (float)S / 1024.0f + 0.5f;
    const int lo = (int)floorf(lod);
    float2* levels[32] = {};
    s = hsm_levels(ctx, p, d_depth, S, T, lo + 1, st, levels);
    if (s != GI_OK) return s;
    out->hsm_lo = lo == 0 ? nullptr : levels[lo];
    out->hsm_hi = levels[lo + 1];
    out->lo_w = S >> lo;
    out->lo_h = T >> lo;
    out->hi_w = S >> (lo + 1);
    out->hi_h = T >> (lo + 1);
    out->hsm_frac = lod - (float)lo;
    return GI_OK;
}

gi_status moment_check_shape(int map_w, int map_h, int W, int H, const char* who) {
    const std::string w(who);
    if (W != H || map_w != map_h)
        return fail(GI_ERR_UNSUPPORTED, w + ": moment techniques need a square window and a square map");
    for (int k = 0; k <= 4; ++k)
        if (map_w == (W << k)) return GI_OK;
    return fail(GI_ERR_UNSUPPORTED, w + ": moment techniques need map side = window side x 2^k, k = 0..4");
}

void moment_quantization(float mq[16], float mqi[16], float* tq0) {
    // MyGLGeometryViewer::configureMoments (ShadowMapping/src/Viewers/
    // MyGLGeometryViewer.cpp:186-215): rows of the optimised 4MSM
    // quantisation (moment_out = Q * (d, d^2, d^3, d^4) + t), stored
    // column-major as the shader receives it, and its inverse.
    const double Q[4][4] = {{-2.07224649, 32.2370378, -68.5710746, 39.3703274},
                            {13.7948857, -59.4683976, 82.035975, -35.3649032},
                            {0.105877704, -1.90774663, 9.34965551, -6.65434907},
                            {9.79240621, -33.76521106, 47.9456097, -23.9728048}};
    float qf[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            qf[r][c] = (float)Q[r][c];
            mq[c * 4 + r] = qf[r][c];
        }
    // inverse in double (Gauss-Jordan with partial pivoting) of the float
    // matrix, rounded to float
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? (double)qf[r][c] : (c - 4 == r ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if ((a[r][c] < 0 ? -a[r][c] : a[r][c]) > (a[piv][c] < 0 ? -a[piv][c] : a[piv][c])) piv = r;
        for (int k = 0; k < 8; ++k) {
            const double tmp = a[c][k];
            a[c][k] = a[piv][k];
            a[piv][k] = tmp;
        }
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
    *tq0 = 0.0359558848f;
}

gi_status launch_moments(gi_context* ctx, int tech, const float* d_depth, int S, int W, cudaStream_t st,
                         const float** filtered) {
    using namespace mom;
    const size_t big = (size_t)S * S * sizeof(float4), small = (size_t)W * W * sizeof(float4);
    // the moment map at the map's size when no box level is needed, else
    // its first box level (S^2 / 4) plus room for the next one
    const size_t need = S > W ? big / 4 + big / 16 : big;
    gi_status s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_mom), &ctx->cap_mom, need);
    if (s == GI_OK) s = ensure_buffer(reinterpret_cast<void**>(&ctx->d_mom_blur), &ctx->cap_mom_blur, 2 * small);
    if (s != GI_OK) return s;
    MomArgs ma;
    ma.depth = d_depth;
    ma.out = reinterpret_cast<float4*>(ctx->d_mom);
    ma.S = S;
    ma.tech = tech;
    float mqi[16];
    moment_quantization(ma.mq, mqi, &ma.tq0);
    float4* lvl = ma.out;
    int side = S;
    if (S > W) {
        // the first box level straight from the depths, at the scratch's start
        launch_dependent(k_moments_box, dim3((S / 2 + 31) / 32, (S / 2 + 7) / 8), dim3(256), 0, st, ma);
        side = S / 2;
    } else {
        launch_dependent(k_moments, dim3((S + 31) / 32, (S + 7) / 8), dim3(256), 0, st, ma);
    }
    ctx->launches++;
    // further box levels, ping-ponging between the two parts of the scratch
    float4* first = lvl;
    float4* other = lvl + (size_t)side * side;
    for (; side > W; side /= 2) {
        float4* dst = (lvl == first) ? other : first;
        launch_dependent(k_mip_box, dim3((side / 2 + 31) / 32, (side / 2 + 7) / 8), dim3(256), 0, st, (const float4*)lvl, side, dst);
        ctx->launches++;
        lvl = dst;
    }
    float4* bx = reinterpret_cast<float4*>(ctx->d_mom_blur);
    float4* by = bx + (size_t)W * W;
    const dim3 grid((W + 31) / 32, (W + 7) / 8);
    if (tech == GI_TECH_ESM) {
        launch_dependent(k_moment_blur<true>, grid, dim3(256), 0, st, (const float4*)lvl, W, 1, 0, bx);
        launch_dependent(k_moment_blur<true>, grid, dim3(256), 0, st, (const float4*)bx, W, 0, 1, by);
    } else {
        launch_dependent(k_moment_blur<false>, grid, dim3(256), 0, st, (const float4*)lvl, W, 1, 0, bx);
        launch_dependent(k_moment_blur<false>, grid, dim3(256), 0, st, (const float4*)bx, W, 0, 1, by);
    }
    ctx->launches += 2;
    *filtered = reinterpret_cast<const float*>(by);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "moment map launch");
}

}  // namespace gi
