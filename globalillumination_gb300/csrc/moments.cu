// moments.cu -- filtered moment shadow maps (VSM, ESM, EVSM, MSM) for sm_103a.
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
#include <cuda_runtime.h>

#include "internal.h"
#include "raster.h"

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

}  // namespace mom

bool is_moment_technique(int t) { return t >= GI_TECH_VSM && t <= GI_TECH_MSM; }

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
        k_moments_box<<<dim3((S / 2 + 31) / 32, (S / 2 + 7) / 8), 256, 0, st>>>(ma);
        side = S / 2;
    } else {
        k_moments<<<dim3((S + 31) / 32, (S + 7) / 8), 256, 0, st>>>(ma);
    }
    ctx->launches++;
    // further box levels, ping-ponging between the two parts of the scratch
    float4* first = lvl;
    float4* other = lvl + (size_t)side * side;
    for (; side > W; side /= 2) {
        float4* dst = (lvl == first) ? other : first;
        k_mip_box<<<dim3((side / 2 + 31) / 32, (side / 2 + 7) / 8), 256, 0, st>>>(lvl, side, dst);
        ctx->launches++;
        lvl = dst;
    }
    float4* bx = reinterpret_cast<float4*>(ctx->d_mom_blur);
    float4* by = bx + (size_t)W * W;
    const dim3 grid((W + 31) / 32, (W + 7) / 8);
    if (tech == GI_TECH_ESM) {
        k_moment_blur<true><<<grid, 256, 0, st>>>(lvl, W, 1, 0, bx);
        k_moment_blur<true><<<grid, 256, 0, st>>>(bx, W, 0, 1, by);
    } else {
        k_moment_blur<false><<<grid, 256, 0, st>>>(lvl, W, 1, 0, bx);
        k_moment_blur<false><<<grid, 256, 0, st>>>(bx, W, 0, 1, by);
    }
    ctx->launches += 2;
    *filtered = reinterpret_cast<const float*>(by);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "moment map launch");
}

}  // namespace gi
