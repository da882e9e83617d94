// minmax.cu -- min-max pyramid of a light map, staged tile by tile through
// shared memory with bulk-async (TMA) copies, for exact tap skipping in the
// visibility pass.
//
// The soft-shadow filters of the reference (PlausibleSoftShadow.frag:166-194
// blocker search, :376-398 filtering) compare the receiver depth z with the
// map at every tap.  When every texel a pixel's taps can reach is >= z, no
// tap finds a blocker (and every filter tap is lit); when every texel is
// < z, every filter tap is shadowed.  Both outcomes give the same float
// result as running the taps (the sums are built in the same order), so the
// visibility kernels test the taps' texel box against this pyramid first
// and run the taps only when the box mixes both sides.
//
// Level L (1..6) holds, for every 2^L x 2^L block of texels, float2(min,
// max), row-major over (W >> L) x (H >> L) cells.  One CTA of 256 threads
// owns a 64 x 64 texel tile: one warp issues 64 bulk copies (one 256-byte
// row each) onto one mbarrier, every thread reduces a 4 x 4 texel block
// (levels 1 and 2, thread t holding level-2 cell t in Morton order), warp
// shuffles give levels 3 and 4, and shared memory levels 5 and 6.  Maps
// whose sides are not multiples of 64 get no pyramid (the visibility
// kernels then run every tap).  If the copy's bounded wait runs out, the
// tile's cells are written as (-inf, +inf), which no skip test accepts, and
// bit 0 of the context's status word 100 is set.
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"
#include "minmax.h"

namespace gi {
namespace mm {

constexpr int kTile = 64;
constexpr unsigned kSpin = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    for (unsigned it = 0; it < kSpin; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ float2 mm2(float2 a, float2 b) { return make_float2(fminf(a.x, b.x), fmaxf(a.y, b.y)); }

__device__ __forceinline__ float2 shfl_xor2(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// even / odd bits of a Morton index
__device__ __forceinline__ int morton_x(int t) {
    return (t & 1) | ((t >> 1) & 2) | ((t >> 2) & 4) | ((t >> 3) & 8);
}
__device__ __forceinline__ int morton_y(int t) { return morton_x(t >> 1); }

__global__ void __launch_bounds__(256) k_minmax_pyramid(const float* __restrict__ map, int W, int H, Pyramid pyr,
                                                        unsigned* __restrict__ status) {
    __shared__ __align__(128) float tile[kTile * kTile];
    __shared__ uint64_t bar;
    __shared__ float2 l4[16];
    const int tid = threadIdx.x, lane = tid & 31;
    const int tx = blockIdx.x, ty = blockIdx.y;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid < 32) {
        if (lane == 0)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar)),
                         "r"((unsigned)(kTile * kTile * 4))
                         : "memory");
        __syncwarp();
        for (int r = lane; r < kTile; r += 32) {
            const float* src = map + (size_t)(ty * kTile + r) * W + (size_t)tx * kTile;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(tile + r * kTile)),
                "l"(src), "r"((unsigned)(kTile * 4)), "r"(smem_u32(&bar))
                : "memory");
        }
    }
    bool ok = mbar_wait(&bar, 0);
    const bool all_ok = __syncthreads_and(ok);
    // level-2 cell t (Morton order in the tile's 16 x 16 level-2 cells)
    const int x2 = morton_x(tid), y2 = morton_y(tid);
    float2 l1[4];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float4 r0 = *reinterpret_cast<const float4*>(tile + (4 * y2 + 2 * j) * kTile + 4 * x2);
        const float4 r1 = *reinterpret_cast<const float4*>(tile + (4 * y2 + 2 * j + 1) * kTile + 4 * x2);
        l1[2 * j] = make_float2(fminf(fminf(r0.x, r0.y), fminf(r1.x, r1.y)), fmaxf(fmaxf(r0.x, r0.y), fmaxf(r1.x, r1.y)));
        l1[2 * j + 1] =
            make_float2(fminf(fminf(r0.z, r0.w), fminf(r1.z, r1.w)), fmaxf(fmaxf(r0.z, r0.w), fmaxf(r1.z, r1.w)));
    }
    const float2 bad = make_float2(-__int_as_float(0x7f800000), __int_as_float(0x7f800000));
    if (!all_ok) {
#pragma unroll
        for (int k = 0; k < 4; ++k) l1[k] = bad;
    }
    {
        const int w1 = W >> 1;
        float2* o = pyr.lv[1] + (size_t)(ty * 32 + 2 * y2) * w1 + tx * 32 + 2 * x2;
        o[0] = l1[0];
        o[1] = l1[1];
        o[w1] = l1[2];
        o[w1 + 1] = l1[3];
    }
    float2 v = mm2(mm2(l1[0], l1[1]), mm2(l1[2], l1[3]));
    pyr.lv[2][(size_t)(ty * 16 + y2) * (W >> 2) + tx * 16 + x2] = v;
    v = mm2(v, shfl_xor2(v, 1));
    v = mm2(v, shfl_xor2(v, 2));
    if ((tid & 3) == 0) pyr.lv[3][(size_t)(ty * 8 + (y2 >> 1)) * (W >> 3) + tx * 8 + (x2 >> 1)] = v;
    v = mm2(v, shfl_xor2(v, 4));
    v = mm2(v, shfl_xor2(v, 8));
    if ((tid & 15) == 0) {
        pyr.lv[4][(size_t)(ty * 4 + (y2 >> 2)) * (W >> 4) + tx * 4 + (x2 >> 2)] = v;
        l4[tid >> 4] = v;
    }
    __syncthreads();
    if (tid < 4) {
        const float2 a = mm2(mm2(l4[4 * tid], l4[4 * tid + 1]), mm2(l4[4 * tid + 2], l4[4 * tid + 3]));
        pyr.lv[5][(size_t)(ty * 2 + (tid >> 1)) * (W >> 5) + tx * 2 + (tid & 1)] = a;
    }
    if (tid == 0) {
        float2 a = l4[0];
        for (int k = 1; k < 16; ++k) a = mm2(a, l4[k]);
        pyr.lv[6][(size_t)ty * (W >> 6) + tx] = a;
    }
    if (!all_ok) {
        // let the copies still in flight land before the shared memory goes
        // away (bounded as well), and report the timeout
        if (!ok) mbar_wait(&bar, 0);
        if (tid == 0 && status) atomicOr(status, 1u);
    }
    (void)H;
}

}  // namespace mm

bool pyramid_supported(int W, int H) { return W >= mm::kTile && H >= mm::kTile && W % mm::kTile == 0 && H % mm::kTile == 0; }

gi_status launch_minmax_pyramid(gi_context* ctx, const float* d_map, int W, int H, cudaStream_t st, Pyramid* out) {
    *out = Pyramid{};
    // the bulk copies need 16-byte aligned rows
    if (!pyramid_supported(W, H) || reinterpret_cast<uintptr_t>(d_map) % 16 != 0) return GI_OK;
    size_t cells = 0;
    for (int L = 1; L <= kPyramidLevels; ++L) cells += (size_t)(W >> L) * (H >> L);
    gi_status s = ensure_buffer(&ctx->d_pyr, &ctx->cap_pyr, cells * sizeof(float2));
    if (s != GI_OK) return s;
    float2* base = static_cast<float2*>(ctx->d_pyr);
    size_t off = 0;
    for (int L = 1; L <= kPyramidLevels; ++L) {
        out->lv[L] = base + off;
        off += (size_t)(W >> L) * (H >> L);
    }
    out->levels = kPyramidLevels;
    dim3 grid(W / mm::kTile, H / mm::kTile);
    mm::k_minmax_pyramid<<<grid, 256, 0, st>>>(d_map, W, H, *out, ctx->d_status + 100);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "min-max pyramid launch");
}

}  // namespace gi

extern "C" gi_status gi_light_map_minmax(gi_context* ctx, const float* d_map, int width, int height, float* d_levels,
                                         void* stream) {
    using namespace gi;
    if (!ctx || !d_map || !d_levels) return fail(GI_ERR_INVALID_ARG, "gi_light_map_minmax: NULL argument");
    if (!pyramid_supported(width, height))
        return fail(GI_ERR_UNSUPPORTED, "gi_light_map_minmax: map sides must be positive multiples of 64");
    if (reinterpret_cast<uintptr_t>(d_map) % 16 != 0)
        return fail(GI_ERR_INVALID_ARG, "gi_light_map_minmax: d_map must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Pyramid pyr;
    gi_status s = launch_minmax_pyramid(ctx, d_map, width, height, st, &pyr);
    if (s != GI_OK) return s;
    size_t cells = 0;
    for (int L = 1; L <= kPyramidLevels; ++L) cells += (size_t)(width >> L) * (height >> L);
    const cudaError_t e = cudaMemcpyAsync(d_levels, pyr.lv[1], cells * sizeof(float2), cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_light_map_minmax: copy");
}
