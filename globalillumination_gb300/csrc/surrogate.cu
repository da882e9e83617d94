// surrogate.cu -- tcgen05 (5th-generation tensor core) kernels of the
// learned soft-shadow surrogate: implicit-GEMM convolution forward / data
// gradient / weight gradient on NHWC BF16 tensors with FP32 accumulation in
// tensor memory, plus the memory-bound pieces of the U-Net (pooling,
// upsampling, channel slices, Adam).
//
// Convolution as GEMM: D[pixel, co] = sum_k A[pixel, k] * B[co, k] with
// k = (tap, ci) in K-blocks of 8 channels.  One CTA of 128 threads owns 128
// output pixels (M = 128) and all cout columns (N = cout <= 256).  Each
// pipeline stage holds 4 K-blocks (32 K elements) of A (gathered with
// zero padding by cp.async) and of B (packed weights) in shared memory, in
// the canonical no-swizzle K-major layout: 8 x 16-byte core matrices, the
// K-adjacent ones 128 B apart (LBO), the 8-row groups 512 B apart (SBO).
// Thread 0 issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) into a TMEM
// accumulator and commits each stage to an mbarrier, which the loaders
// wait on before refilling that stage.  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e.
// pixels), applies bias / ReLU / ReLU-derivative mask and stores BF16
// (and optionally FP32).
//
// Every wait on an mbarrier is bounded (gi_tc_set_wait_limit, default 2^20
// polls).  When a wait runs out, the kernel stops issuing loads and MMAs,
// skips its tensor-memory reads, waits (again bounded) for the copies and
// MMAs it already issued, frees its tensor memory, sets bit 0 of the
// caller's error word and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>

#include <algorithm>
#include <cstdint>

#include "../../include/gi_surrogate.h"
#include "internal.h"

namespace gi {
namespace tc {

constexpr int kThreads = 128;
constexpr int kNS = 4;          // pipeline stages
constexpr int kBKB = 4;         // K-blocks (8 elements) per stage
constexpr int kCore = 128;      // bytes per core matrix (8 rows x 16 B)
constexpr int kSBO = kBKB * kCore;
constexpr int kStageA = 16 * kSBO;  // 128 rows
constexpr unsigned kSpinLimit = 1u << 20;  // default polls per mbarrier wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start address, leading (K)
// and stride (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B,
// both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit) {
    const uint32_t a = smem_u32(bar);
    for (unsigned it = 0; it < limit; ++it) {
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

__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// One 32-byte store (the address 32-byte aligned): a whole sector per lane.
__device__ __forceinline__ void st_global_v8(void* ptr, const uint32_t (&v)[8]) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(ptr), "r"(v[0]), "r"(v[1]),
                 "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane, without the
// wait: the registers are valid after tmem_wait_ld().
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint32_t tmem_cols(int n) { return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u; }

__device__ __forceinline__ float bf16_to_f(uint16_t v) { return __uint_as_float((uint32_t)v << 16); }
__device__ __forceinline__ uint16_t f_to_bf16(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

struct ConvArgs {
    const uint16_t* x;
    int n, h, w, cin;
    const uint16_t* wt;
    int cout, nkb, nkb_pad, ksize;
    const float* bias;
    int act;
    const uint16_t* mask;
    uint16_t* y;
    int y_c, y_off;
    float* y32;
    uint32_t* err;
    unsigned spin;   // polls per mbarrier wait
    int withhold;    // test switch: the first asynchronous stage is not issued
    long long P;
    // optional fused 1x1 head on the activated BF16-rounded output:
    // hout[p][j] = hb[j] + sum_c hw[j][c] * bf16(v[c]), j < 2
    const float* hw;
    const float* hb;
    float* hout;
    // slab kernel only: pool (BF16, [n][h / 2][w / 2][cout]) also receives
    // the 2 x 2 max-pooled output; up2 writes y upsampled 2x (nearest) into
    // a [n][2 h][2 w][y_c] tensor
    uint16_t* pool;
    int up2;
};

__global__ void __launch_bounds__(kThreads) k_conv_fwd(ConvArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bars[kNS];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = a.cout;
    const int stage_bytes = kStageA + (N / 8) * kSBO;
    const uint32_t ncols = tmem_cols(N);
    if (warp == 0) tmem_alloc(&tmem_slot, ncols);
    if (tid == 0) {
        for (int s = 0; s < kNS; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const long long tile0 = (long long)blockIdx.x * 128;
    const int nk = a.nkb_pad / kBKB;
    const int cg = a.cin / 8;
    bool ok = true;

    auto load_stage = [&](int chunk, int s) {
        uint8_t* sa = smem + s * stage_bytes;
        uint8_t* sb = sa + kStageA;
        const int kb0 = chunk * kBKB;
        for (int c = tid; c < 128 * kBKB; c += kThreads) {
            const int m = c & 127, kl = c >> 7, kb = kb0 + kl;
            const long long p = tile0 + m;
            const uint16_t* src = a.x;
            int bytes = 0;
            if (p < a.P && kb < a.nkb) {
                const int tap = kb / cg, g = kb - tap * cg;
                const int dy = a.ksize == 3 ? tap / 3 - 1 : 0, dx = a.ksize == 3 ? tap % 3 - 1 : 0;
                const int xx = (int)(p % a.w);
                const long long t = p / a.w;
                const int yy = (int)(t % a.h);
                const long long img = t / a.h;
                const int x2 = xx + dx, y2 = yy + dy;
                if (x2 >= 0 && x2 < a.w && y2 >= 0 && y2 < a.h) {
                    src = a.x + ((img * a.h + y2) * a.w + x2) * a.cin + g * 8;
                    bytes = 16;
                }
            }
            cp_async16(smem_u32(sa + kl * kCore + (m >> 3) * kSBO + (m & 7) * 16), src, bytes);
        }
        for (int c = tid; c < N * kBKB; c += kThreads) {
            const int r = c % N, kl = c / N;
            const uint16_t* src = a.wt + ((long long)r * a.nkb_pad + kb0 + kl) * 8;
            cp_async16(smem_u32(sb + kl * kCore + (r >> 3) * kSBO + (r & 7) * 16), src, 16);
        }
    };

    const uint32_t idesc = idesc_bf16(128, N);
    for (int s = 0; s < kNS - 1; ++s) {
        if (s < nk) load_stage(s, s);
        cp_async_commit();
    }
    // Iteration i: wait for chunk i's copies, issue its MMAs, then refill
    // the stage chunk i - 1 used (its MMAs overlap with those just issued).
    // A wait that runs out stops the loop for the whole CTA at the next
    // iteration; `issued` is the last chunk whose MMAs were committed.
    int issued = -1;
    for (int i = 0; i < nk; ++i) {
        const int s = i % kNS;
        cp_async_wait<kNS - 2>();
        fence_proxy_async();
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        if (tid == 0 && !a.withhold) {
            fence_after();
            const uint8_t* sa = smem + s * stage_bytes;
            const uint8_t* sb = sa + kStageA;
#pragma unroll
            for (int kk = 0; kk < kBKB / 2; ++kk) {
                const uint64_t ad = smem_desc(smem_u32(sa + kk * 2 * kCore), kCore, kSBO);
                const uint64_t bd = smem_desc(smem_u32(sb + kk * 2 * kCore), kCore, kSBO);
                mma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&bars[s]);
        }
        if (!a.withhold) issued = i;
        const int j = i + kNS - 1;
        if (j < nk) {
            const int sj = j % kNS;
            if (i >= 1) ok = mbar_wait(&bars[sj], (unsigned)((i - 1) / kNS) & 1u, a.spin);
            if (ok) load_stage(j, sj);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (ok && nk > 0) {
        const int last = nk - 1;
        ok = mbar_wait(&bars[last % kNS], (unsigned)(last / kNS) & 1u, a.spin);
    } else if (issued >= 0) {
        // Stopped early: the committed MMAs (every chunk up to `issued`;
        // those before issued - 1 were already waited for) must land before
        // the tensor memory is freed.  The wait is bounded too.
        mbar_wait(&bars[issued % kNS], (unsigned)(issued / kNS) & 1u, a.spin);
    }
    const bool all_ok = __syncthreads_and(ok);
    fence_after();

    const long long p = tile0 + warp * 32 + lane;
    const bool live = p < a.P;
    for (int c0 = 0; all_ok && c0 < N; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (!live) continue;
        if (a.bias) {
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] += __ldg(a.bias + c0 + q);
        }
        if (a.act == GI_ACT_RELU) {
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = fmaxf(v[q], 0.0f);
        }
        const long long o = p * a.y_c + a.y_off + c0;
        if (a.mask) {
            const uint4* mp = reinterpret_cast<const uint4*>(a.mask + o);
            uint4 m0 = __ldg(mp), m1 = __ldg(mp + 1);
            const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const uint16_t mv = (uint16_t)(mw[q >> 1] >> ((q & 1) * 16));
                if (!(bf16_to_f(mv) > 0.0f)) v[q] = 0.0f;
            }
        }
        if (a.y32) {
            float4* yp = reinterpret_cast<float4*>(a.y32 + p * N + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) yp[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
        if (a.y) {
            uint32_t pk[8];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                pk[q] = (uint32_t)f_to_bf16(v[2 * q]) | ((uint32_t)f_to_bf16(v[2 * q + 1]) << 16);
            uint4* yp = reinterpret_cast<uint4*>(a.y + o);
            yp[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            yp[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
    }
    ok = all_ok;
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
    if (!ok && tid == 0 && a.err) atomicOr(a.err, 1u);
}

// ---- 3x3 convolution from halo slabs (cin % 16 == 0) ---------------------------
// A CTA computes R output rows x 128 pixels (R accumulators of 128 x N in
// TMEM).  A stage holds 16 channels of the R + 2 input rows y0-1 .. y0+R
// over x0-1 .. x0+128 ("slab": 130 pixels x 32 B per row), fetched by one
// 4-D TMA box load in the 32-byte swizzled layout (the halo outside the
// image is zero-filled by TMA), and the weights of all 9 taps for those
// channels, fetched by one bulk copy from the stage-ordered packing
// [chunk][tap][group][cout][8].  The MMA of tap (dy, dx) for output row r
// reads A at slab row r + dy, shifted by dx pixels (32 B): each pixel's 16
// channels are one 32-byte row of the K-major swizzled layout (8-pixel
// groups 256 B apart), and the swizzle is a function of the shared-memory
// address, which TMA and the MMA compute alike, so any pixel can start the
// operand.  Each input pixel is loaded (R + 2) / R times instead of 9, in
// boxes whose rows are 32 bytes (a 16-byte box row costs the TMA engine
// as much as a 32-byte one).
constexpr int kSlabPx = 130;
constexpr int kSlabRow = kSlabPx * 32;  // 4160 B

struct SlabGeom {
    int R, NS, ncols, a_box, a_bytes, b_bytes, stage_bytes;
};

// tcgen05 shared-memory descriptor of a K-major operand in the 32-byte
// swizzled layout that TMA writes with CU_TENSOR_MAP_SWIZZLE_32B: rows of
// 32 B (16 BF16 = one MMA's K), 8-row groups 256 B apart (SBO), layout
// type 6; the leading-dimension offset is unused because K fits the
// swizzle width.
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t addr) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(256u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)6 << 61;
    return d;
}

__host__ __device__ inline bool slab_layout(int kin, int ks) { return ks == 3 && kin % 16 == 0; }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Persistent CTAs (one per SM) of ten warps: warp 0 issues the TMA loads,
// warp 1 the MMAs, warps 2-9 drain the accumulators (warp w reads TMEM
// lanes 32 (w % 4) ..; the two warps of a lane quarter take alternate rows,
// or alternate row pairs when pooling).  Two TMEM accumulator sets
// alternate between tiles, so the epilogue of tile t overlaps the MMAs of
// tile t + 1.  Barriers: full / empty per smem stage, acc_full / acc_empty
// per accumulator set.
constexpr int kPersistThreads = 320;
constexpr int kEpilogueThreads = kPersistThreads - 64;

__host__ __device__ inline SlabGeom persist_geom(int N, int nk) {
    SlabGeom g;
    g.ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
    g.R = 256 / g.ncols;  // two accumulator sets of R x ncols columns
    if (g.R > 8) g.R = 8;
    g.a_box = (g.R + 2) * kSlabRow;
    g.a_bytes = (g.a_box + 1023) / 1024 * 1024;  // swizzled TMA destinations: 1024-byte aligned
    g.b_bytes = 9 * 2 * N * 16;
    g.stage_bytes = (g.a_bytes + g.b_bytes + 1023) / 1024 * 1024;
    g.NS = 4;
    while (g.NS > 2 && g.NS * g.stage_bytes > 200 * 1024) --g.NS;
    (void)nk;
    return g;
}

// R (output rows per tile, 256 / accumulator columns) is a template
// parameter so that the MMA warp's issue loop is fully unrolled: one
// 64-bit add per descriptor and the MMA itself per instruction.
template <int R>
__global__ void __launch_bounds__(kPersistThreads) k_conv3_slab(ConvArgs a, const __grid_constant__ CUtensorMap xmap,
                                                                int tiles_x, int tiles_y, int tiles) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[4], empty[4], acc_full[2], acc_empty[2];
    __shared__ uint32_t tmem_slot;
    // Stop flag (a wait ran out somewhere in the CTA) and the progress the
    // drain after a stop needs: stages loaded by the producer, stages the
    // MMA warp took (waited full), stages whose MMAs it committed, and
    // commits of `empty` the producer saw land.
    __shared__ int s_fail, s_loaded, s_taken, s_committed, s_freed;
    // the epilogue's per-channel constants, read once per CTA: bias and the
    // fused head's weights (the L1 cache is small next to the slab ring)
    __shared__ __align__(16) float s_bias[256];
    __shared__ __align__(16) float s_hw[512];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = a.cout;
    const int nk = a.cin / 16;
    const SlabGeom G = persist_geom(N, nk);
    const int NS = G.NS;
    constexpr int kCols = 256 / R;  // accumulator columns of one output row
    const uint32_t set_cols = (uint32_t)(R * kCols);
    const uint32_t tcols = 2 * set_cols;
    if (warp == 0) tmem_alloc(&tmem_slot, tcols);
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], kEpilogueThreads);
        }
        s_fail = 0;
        s_loaded = s_taken = s_committed = s_freed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // Launched as a programmatic dependent of the previous kernel in the
    // stream: everything above touches only shared and tensor memory, so it
    // overlaps that kernel's tail; no global memory is read or written
    // before the previous grid has completed and its writes are visible.
    // The next kernel may then be scheduled onto SMs as this grid's CTAs
    // finish.  (Both are no-ops for an ordinary launch.)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    for (int i = tid; i < N; i += kPersistThreads) s_bias[i] = a.bias ? __ldg(a.bias + i) : 0.0f;
    if (a.hw)
        for (int i = tid; i < 2 * N; i += kPersistThreads) s_hw[i] = __ldg(a.hw + i);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    volatile int* fail = &s_fail;
    const int ntiles_mine = tiles > (int)blockIdx.x ? (tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    auto tile_coords = [&](int t, int& x0, int& y0, int& img) {
        const int bx = t % tiles_x;
        const int by = (t / tiles_x) % tiles_y;
        img = t / (tiles_x * tiles_y);
        x0 = bx * 128;
        y0 = by * R;
    };
    // A warp-uniform bounded wait: false (and the CTA's stop flag set) when
    // any lane's wait ran out or another warp has stopped the CTA.
    auto warp_wait = [&](uint64_t* bar, unsigned parity) -> bool {
        if (__shfl_sync(0xffffffffu, *fail, 0)) return false;
        const bool w = mbar_wait(bar, parity, a.spin);
        if (__any_sync(0xffffffffu, !w)) {
            if (lane == 0) *fail = 1;
            return false;
        }
        return true;
    };

    if (warp == 0) {
        // TMA producer
        const uint32_t stage_tx = (uint32_t)(G.a_box + G.b_bytes);
        int g = 0, freed = 0;
        bool run = true;
        for (int it = 0; run && it < ntiles_mine; ++it) {
            int x0, y0, img;
            tile_coords((int)blockIdx.x + it * (int)gridDim.x, x0, y0, img);
            for (int c = 0; c < nk; ++c, ++g) {
                const int s = g % NS;
                if (g >= NS) {
                    if (!warp_wait(&empty[s], (unsigned)((g / NS) - 1) & 1u)) {
                        run = false;
                        break;
                    }
                    freed = g - NS + 1;
                }
                if (__shfl_sync(0xffffffffu, *fail, 0)) {
                    run = false;
                    break;
                }
                if (lane == 0 && !a.withhold) {
                    uint8_t* sa = smem + s * G.stage_bytes;
                    mbar_expect_tx(&full[s], stage_tx);
                    tma_load_4d(sa, &xmap, c * 16, x0 - 1, y0 - 1, img, &full[s]);
                    bulk_load(sa + G.a_bytes, a.wt + (size_t)c * (G.b_bytes / 2), (uint32_t)G.b_bytes, &full[s]);
                }
                __syncwarp();
            }
        }
        if (lane == 0) {
            s_loaded = a.withhold ? 0 : g;
            s_freed = freed;
        }
    } else if (warp == 1) {
        // MMA issuer
        const uint32_t idesc = idesc_bf16(128, N);
        // taps stacked along N: one, two or three dy taps of N columns each
        // (R >= 4 and N equal to the row stride kCols, so 3 N <= 192)
        const bool stacked = R >= 4 && N == kCols;
        const uint32_t idesc2 = stacked ? idesc_bf16(128, 2 * N) : idesc;
        const uint32_t idesc3 = stacked ? idesc_bf16(128, 3 * N) : idesc;
        int g = 0, committed = 0;
        bool run = true;
        for (int it = 0; run && it < ntiles_mine; ++it) {
            const int b = it & 1;
            if (it >= 2 && !warp_wait(&acc_empty[b], (unsigned)((it >> 1) - 1) & 1u)) break;
            fence_after();
            const uint32_t acc = tmem + (uint32_t)b * set_cols;
            // output row r's accumulator: rows in reverse order, kCols apart
            auto acc_col = [&](int r) { return acc + (uint32_t)((R - 1 - r) * kCols); };
            for (int c = 0; c < nk; ++c, ++g) {
                const int s = g % NS;
                if (!warp_wait(&full[s], (unsigned)(g / NS) & 1u)) {
                    run = false;
                    break;
                }
                if (lane == 0) {
                    fence_after();
                    // Descriptors of the stage's first A and B matrices; the
                    // others differ only in the start-address field (bits
                    // 0-13, in 16-byte units), and every start stays below
                    // 256 KB, so adding the offset there never carries.
                    // B: tap (dx, dy) at (3 dx + dy) x N x 32 bytes, 8-row
                    // groups 256 B apart, the two K halves 128 B apart.
                    const uint32_t sa = smem_u32(smem + s * G.stage_bytes);
                    const uint64_t ad0 = smem_desc_sw32(sa);
                    const uint64_t bd0 = smem_desc(sa + (uint32_t)G.a_bytes, 128u, 256u);
                    const uint32_t tap_step = (uint32_t)N * 2u;  // N x 32 B / 16
                    if (stacked) {
                        // Slab row ri (input row y0 - 1 + ri) feeds output
                        // row ri - dy through tap dy; the accumulators run
                        // in reverse row order kCols apart, so one MMA with
                        // the taps dlo..dhi stacked along N writes rows
                        // ri - dlo, ri - dlo - 1, ...  On the first stage,
                        // tap (dx 0, dy 0) starts every row's accumulator
                        // (accumulate off) before any stacked MMA adds to it.
                        const bool init = c == 0;
#pragma unroll
                        for (int dx = 0; dx < 3; ++dx) {
                            if (dx == 0 && init) {
#pragma unroll
                                for (int r = 0; r < R; ++r)
                                    mma_bf16(acc_col(r), ad0 + (uint64_t)((r * kSlabRow) >> 4), bd0, idesc, 0u);
                            }
#pragma unroll
                            for (int ri = 0; ri < R + 2; ++ri) {
                                int dlo = ri - R + 1 > 0 ? ri - R + 1 : 0;
                                const int dhi = ri < 2 ? ri : 2;
                                if (dx == 0 && init && dlo == 0) dlo = 1;
                                if (dlo > dhi) continue;
                                const uint64_t ad = ad0 + (uint64_t)((ri * kSlabRow + dx * 32) >> 4);
                                const uint64_t bd = bd0 + (uint64_t)((dx * 3 + dlo) * tap_step);
                                const int nd = dhi - dlo;
                                mma_bf16(acc_col(ri - dlo), ad, bd, nd == 0 ? idesc : nd == 1 ? idesc2 : idesc3, 1u);
                            }
                        }
                    } else {
#pragma unroll
                        for (int t = 0; t < 9; ++t) {
                            const int dy = t / 3, dx = t % 3;
                            const uint64_t bd = bd0 + (uint64_t)((dx * 3 + dy) * tap_step);
                            const uint32_t first = (c > 0 || t > 0) ? 1u : 0u;
#pragma unroll
                            for (int r = 0; r < R; ++r) {
                                const uint64_t ad = ad0 + (uint64_t)(((r + dy) * kSlabRow + dx * 32) >> 4);
                                mma_bf16(acc_col(r), ad, bd, idesc, first);
                            }
                        }
                    }
                    mma_commit(&empty[s]);
                    if (c == nk - 1) mma_commit(&acc_full[b]);
                }
                committed = g + 1;
                __syncwarp();
            }
        }
        if (lane == 0) {
            s_taken = committed;  // every stage taken was also committed
            s_committed = committed;
        }
    } else {
        // epilogue: warps 2..9 -> TMEM lane quarter warp % 4, row half
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        for (int it = 0; it < ntiles_mine; ++it) {
            const int b = it & 1;
            int x0, y0, img;
            tile_coords((int)blockIdx.x + it * (int)gridDim.x, x0, y0, img);
            if (!warp_wait(&acc_full[b], (unsigned)(it >> 1) & 1u)) break;
            fence_after();
            const uint32_t acc = tmem + (uint32_t)b * set_cols;
            const int xo = x0 + q * 32 + lane;
            const uint32_t lane_acc = acc + ((uint32_t)(q * 32) << 16);
            // 32-byte stores where every chunk of the outputs starts on a
            // 32-byte boundary (BF16 chunks of 16 channels)
            const bool v8_y = a.y && (reinterpret_cast<uintptr_t>(a.y) & 31) == 0 && a.y_c % 16 == 0 &&
                              a.y_off % 16 == 0;
            const bool v8_pool = a.pool && (reinterpret_cast<uintptr_t>(a.pool) & 31) == 0;
            auto store_bf16 = [](uint16_t* dst, const uint32_t (&pk)[8], bool v8) {
                if (v8) {
                    st_global_v8(dst, pk);
                } else {
                    uint4* yp = reinterpret_cast<uint4*>(dst);
                    yp[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    yp[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
            };
            // Bias, activation, mask and the stores of one 16-channel chunk
            // (c0..c0 + 15) of output row r at this lane's pixel; the head
            // sums h0 / h1 take the chunk's BF16-rounded values.
            auto finish = [&](int r, int c0, float (&v)[16], float& h0, float& h1) {
                const int yo = y0 + r;
                const long long p = ((long long)img * a.h + yo) * a.w + xo;
                if (a.bias) {
                    const float4* bb = reinterpret_cast<const float4*>(s_bias + c0);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float4 t = bb[j];
                        v[4 * j] += t.x;
                        v[4 * j + 1] += t.y;
                        v[4 * j + 2] += t.z;
                        v[4 * j + 3] += t.w;
                    }
                }
                if (a.act == GI_ACT_RELU) {
#pragma unroll
                    for (int k = 0; k < 16; ++k) v[k] = fmaxf(v[k], 0.0f);
                }
                const long long o = p * a.y_c + a.y_off + c0;
                if (a.mask) {
                    const uint4* mp = reinterpret_cast<const uint4*>(a.mask + o);
                    uint4 m0 = __ldg(mp), m1 = __ldg(mp + 1);
                    const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const uint16_t mv = (uint16_t)(mw[k >> 1] >> ((k & 1) * 16));
                        if (!(bf16_to_f(mv) > 0.0f)) v[k] = 0.0f;
                    }
                }
                if (a.y32) {
                    float4* yp = reinterpret_cast<float4*>(a.y32 + p * N + c0);
#pragma unroll
                    for (int k = 0; k < 4; ++k) yp[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                }
                if (a.hw) {
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const float vb = bf16_to_f(f_to_bf16(v[k]));
                        h0 += s_hw[c0 + k] * vb;
                        h1 += s_hw[N + c0 + k] * vb;
                    }
                }
                if (a.y) {
                    uint32_t pk[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        pk[k] = (uint32_t)f_to_bf16(v[2 * k]) | ((uint32_t)f_to_bf16(v[2 * k + 1]) << 16);
                    if (a.up2) {
                        // nearest 2x upsampling: the pixel's 2 x 2 block of
                        // the (2 h) x (2 w) output
                        const long long W2 = 2LL * a.w;
                        const long long p2 = ((long long)img * 2 * a.h + 2 * yo) * W2 + 2 * xo;
#pragma unroll
                        for (int d = 0; d < 4; ++d)
                            store_bf16(a.y + (p2 + (d >> 1) * W2 + (d & 1)) * a.y_c + a.y_off + c0, pk, v8_y);
                    } else {
                        store_bf16(a.y + o, pk, v8_y);
                    }
                }
            };
            if (a.pool) {
                // Rows in pairs (y0 and R are even): the 2 x 2 maximum of the
                // finished values, the partner pixel from the neighbouring
                // lane; even lanes store the pooled chunk.  Rounding to BF16
                // is monotone, so this equals pooling the stored output.
                const int wo = a.w / 2, ho = a.h / 2;
                for (int r = 2 * half; r < R; r += 4) {
                    const int yo = y0 + r;
                    const bool live = xo < a.w && yo < a.h;  // w, h even: the 2 x 2 window is live as a whole
                    for (int c0 = 0; c0 < N; c0 += 16) {
                        float v0[16], v1[16], hu = 0.0f;
                        uint32_t u0[16], u1[16];
                        tmem_ld16_async(lane_acc + (uint32_t)((R - 1 - r) * kCols + c0), u0);
                        tmem_ld16_async(lane_acc + (uint32_t)((R - 2 - r) * kCols + c0), u1);
                        tmem_wait_ld();
#pragma unroll
                        for (int k = 0; k < 16; ++k) {
                            v0[k] = __uint_as_float(u0[k]);
                            v1[k] = __uint_as_float(u1[k]);
                        }
                        if (live) {
                            finish(r, c0, v0, hu, hu);
                            finish(r + 1, c0, v1, hu, hu);
                        }
                        uint32_t pk[8];
#pragma unroll
                        for (int k = 0; k < 16; k += 2) {
                            float m0 = fmaxf(v0[k], v1[k]), m1 = fmaxf(v0[k + 1], v1[k + 1]);
                            m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 1));
                            m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 1));
                            pk[k >> 1] = (uint32_t)f_to_bf16(m0) | ((uint32_t)f_to_bf16(m1) << 16);
                        }
                        if (live && !(lane & 1)) {
                            const long long pp = ((long long)img * ho + yo / 2) * wo + xo / 2;
                            store_bf16(a.pool + pp * N + c0, pk, v8_pool);
                        }
                    }
                }
            } else {
                for (int r = half; r < R; r += 2) {
                    const int yo = y0 + r;
                    const bool live = xo < a.w && yo < a.h;
                    float h0 = a.hw ? __ldg(a.hb) : 0.0f, h1 = a.hw ? __ldg(a.hb + 1) : 0.0f;
                    // two 16-column chunks in flight per wait
                    for (int c0 = 0; c0 < N; c0 += 32) {
                        const uint32_t col = lane_acc + (uint32_t)((R - 1 - r) * kCols + c0);
                        const bool two = c0 + 16 < N;
                        uint32_t u0[16], u1[16];
                        tmem_ld16_async(col, u0);
                        if (two) tmem_ld16_async(col + 16, u1);
                        tmem_wait_ld();
                        float v[16];
#pragma unroll
                        for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(u0[k]);
                        if (live) finish(r, c0, v, h0, h1);
                        if (two) {
#pragma unroll
                            for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(u1[k]);
                            if (live) finish(r, c0 + 16, v, h0, h1);
                        }
                    }
                    if (a.hout && live) {
                        const long long p = ((long long)img * a.h + yo) * a.w + xo;
                        *reinterpret_cast<float2*>(a.hout + p * 2) = make_float2(h0, h1);
                    }
                }
            }
            fence_before();
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[b])) : "memory");
        }
    }
    // Every role has left its loop (each of its waits is bounded).  After a
    // stop, drain what is still in flight before the tensor memory and the
    // shared memory go away: the TMA loads the MMA warp never took (each in
    // its own stage, waited phase by phase), and the committed MMAs whose
    // `empty` commits nobody saw land (in commit order, so every parity
    // wait names the barrier's next phase).  These waits are bounded too.
    __syncthreads();
    if (*fail && lane == 0) {
        if (warp == 0) {
            for (int g = s_taken; g < s_loaded; ++g) mbar_wait(&full[g % NS], (unsigned)(g / NS) & 1u, a.spin);
        } else if (warp == 1) {
            for (int g = s_freed; g < s_committed; ++g)
                mbar_wait(&empty[g % NS], (unsigned)(g / NS) & 1u, a.spin);
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, tcols);
    if (*fail && tid == 0 && a.err) atomicOr(a.err, 1u);
}

// ---- weight gradient ---------------------------------------------------------
// D[r, co] = sum_p A[r, p] * B[co, p] with r = (K-block, channel) of the
// forward K and p the pixels of this CTA's split.  Both operands are
// staged transposed (pixels along K): a thread loads 8 pixels x 8 channels
// (8 x 16 B) and writes the 8 x 8 block back as one core matrix.
struct WgradArgs {
    const uint16_t* x;
    const uint16_t* dy;
    int n, h, w, cin, cout, ksize, nkb, m_tiles;
    long long P, px_per_split;
    float* scratch;
    uint32_t* err;
    unsigned spin;
    int withhold;
};

__device__ __forceinline__ void transpose8(const uint4 (&in)[8], uint4 (&out)[8]) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(in);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t sel = (j & 1) ? 0x7632u : 0x5410u;
        uint32_t o[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) o[k] = __byte_perm(w[(2 * k) * 4 + (j >> 1)], w[(2 * k + 1) * 4 + (j >> 1)], sel);
        out[j] = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

__global__ void __launch_bounds__(kThreads) k_conv_wgrad(WgradArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bars[kNS];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = a.cout;
    const int stage_bytes = kStageA + (N / 8) * kSBO;
    const uint32_t ncols = tmem_cols(N);
    const int mt = blockIdx.x;
    const long long p_begin = (long long)blockIdx.y * a.px_per_split;
    const long long p_end = min(a.P, p_begin + a.px_per_split);
    if (warp == 0) tmem_alloc(&tmem_slot, ncols);
    if (tid == 0) {
        for (int s = 0; s < kNS; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const int cg = a.cin / 8;
    const long long span = p_end > p_begin ? p_end - p_begin : 0;
    const int nk = (int)((span + 8 * kBKB - 1) / (8 * kBKB));
    bool ok = true;

    auto load_stage = [&](int chunk, int s) {
        uint8_t* sa = smem + s * stage_bytes;
        uint8_t* sb = sa + kStageA;
        const long long pc = p_begin + (long long)chunk * 8 * kBKB;
        const int na = 16 * kBKB, nb = (N / 8) * kBKB;
        for (int task = tid; task < na + nb; task += kThreads) {
            uint4 in[8], out[8];
            const bool is_a = task < na;
            const int t = is_a ? task : task - na;
            const int rg = t / kBKB, q = t % kBKB;
            const long long p0 = pc + q * 8;
            if (is_a) {
                const int kb = mt * 16 + rg;
                int tap = 0, g = 0, dy = 0, dx = 0;
                const bool kb_ok = kb < a.nkb;
                if (kb_ok) {
                    tap = kb / cg;
                    g = kb - tap * cg;
                    if (a.ksize == 3) {
                        dy = tap / 3 - 1;
                        dx = tap % 3 - 1;
                    }
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    in[i] = make_uint4(0, 0, 0, 0);
                    const long long p = p0 + i;
                    if (kb_ok && p < p_end) {
                        const int xx = (int)(p % a.w);
                        const long long tt = p / a.w;
                        const int yy = (int)(tt % a.h);
                        const long long img = tt / a.h;
                        const int x2 = xx + dx, y2 = yy + dy;
                        if (x2 >= 0 && x2 < a.w && y2 >= 0 && y2 < a.h)
                            in[i] = __ldg(reinterpret_cast<const uint4*>(a.x + ((img * a.h + y2) * a.w + x2) * a.cin + g * 8));
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    in[i] = make_uint4(0, 0, 0, 0);
                    const long long p = p0 + i;
                    if (p < p_end) in[i] = __ldg(reinterpret_cast<const uint4*>(a.dy + p * a.cout + rg * 8));
                }
            }
            transpose8(in, out);
            uint8_t* dst = (is_a ? sa : sb) + q * kCore + rg * kSBO;
#pragma unroll
            for (int j = 0; j < 8; ++j) *reinterpret_cast<uint4*>(dst + j * 16) = out[j];
        }
    };

    const uint32_t idesc = idesc_bf16(128, N);
    for (int s = 0; s < kNS - 1; ++s)
        if (s < nk) load_stage(s, s);
    // As in k_conv_fwd: a wait that runs out stops the CTA at the next
    // iteration; `issued` is the last chunk whose MMAs were committed.
    int issued = -1;
    for (int i = 0; i < nk; ++i) {
        const int s = i % kNS;
        fence_proxy_async();
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        if (tid == 0 && !a.withhold) {
            fence_after();
            const uint8_t* sa = smem + s * stage_bytes;
            const uint8_t* sb = sa + kStageA;
#pragma unroll
            for (int kk = 0; kk < kBKB / 2; ++kk) {
                const uint64_t ad = smem_desc(smem_u32(sa + kk * 2 * kCore), kCore, kSBO);
                const uint64_t bd = smem_desc(smem_u32(sb + kk * 2 * kCore), kCore, kSBO);
                mma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&bars[s]);
        }
        if (!a.withhold) issued = i;
        const int j = i + kNS - 1;
        if (j < nk) {
            const int sj = j % kNS;
            if (i >= 1) ok = mbar_wait(&bars[sj], (unsigned)((i - 1) / kNS) & 1u, a.spin);
            if (ok) load_stage(j, sj);
        }
    }
    if (ok && nk > 0) {
        const int last = nk - 1;
        ok = mbar_wait(&bars[last % kNS], (unsigned)(last / kNS) & 1u, a.spin);
    } else if (!ok && issued >= 0) {
        mbar_wait(&bars[issued % kNS], (unsigned)(issued / kNS) & 1u, a.spin);  // let committed MMAs land
    }
    const bool all_ok = __syncthreads_and(ok);
    fence_after();
    const long long row = ((long long)blockIdx.y * a.m_tiles + mt) * 128 + warp * 32 + lane;
    for (int c0 = 0; all_ok && c0 < N; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (nk == 0) {
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = 0.0f;
        }
        float4* o = reinterpret_cast<float4*>(a.scratch + row * N + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
    ok = all_ok;
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
    if (!ok && tid == 0 && a.err) atomicOr(a.err, 1u);
}

// dw[co][r] += sum over splits of scratch[split][r][co], r < 8 * nkb, in a
// fixed order: block (r, 32-channel group) of kReducePhases warps; warp t
// sums the splits t, t + kReducePhases, ... in order, then thread 0 of each
// lane adds the warps' sums in warp order.
constexpr int kReducePhases = 8;
__global__ void __launch_bounds__(32 * kReducePhases) k_wgrad_reduce(const float* __restrict__ scratch, int splits,
                                                                      int m_tiles, int cout, int nkb, int nkb_pad,
                                                                      float* __restrict__ dw) {
    __shared__ float part[kReducePhases][32];
    const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
    const long long r = blockIdx.x;
    const int co = blockIdx.y * 32 + lane;
    float s = 0.0f;
    if (co < cout) {
        const long long stride = (long long)m_tiles * 128 * cout;
        const float* src = scratch + r * cout + co;
#pragma unroll 4
        for (int k = t; k < splits; k += kReducePhases) s += __ldg(src + (long long)k * stride);
    }
    part[t][lane] = s;
    __syncthreads();
    if (t == 0 && co < cout) {
        float v = 0.0f;
#pragma unroll
        for (int q = 0; q < kReducePhases; ++q) v += part[q][lane];
        dw[(long long)co * nkb_pad * 8 + r] += v;
    }
    (void)nkb;
}

// db[co] += sum_p dy[p][co] in a fixed order, so that training runs are
// reproducible: thread row r of block b sums pixels b * rows + r, stepping by
// gridDim.x * rows; the block's rows are added in row order into
// partial[b][co], and k_bias_reduce adds the blocks in a fixed order.
__global__ void k_bias_grad(const uint16_t* __restrict__ dy, long long P, int cout, float* __restrict__ partial) {
    __shared__ float acc[256];
    const int c = threadIdx.x % cout;
    const int rows = blockDim.x / cout;
    const int r0 = threadIdx.x / cout;
    float s = 0.0f;
    if (r0 < rows)
        for (long long p = blockIdx.x * (long long)rows + r0; p < P; p += (long long)gridDim.x * rows)
            s += bf16_to_f(dy[p * cout + c]);
    if (r0 < rows) acc[r0 * cout + c] = s;
    __syncthreads();
    if (threadIdx.x < cout) {
        float t = 0.0f;
        for (int r = 0; r < rows; ++r) t += acc[r * cout + threadIdx.x];
        partial[(long long)blockIdx.x * cout + threadIdx.x] = t;
    }
}

// db[co] += the blocks' partial sums in a fixed order: warp t of the
// 32-channel group sums blocks t, t + 32, ... in order, then the warps'
// sums are added in warp order.
__global__ void __launch_bounds__(1024) k_bias_reduce(const float* __restrict__ partial, int blocks, int cout,
                                                      float* __restrict__ db) {
    __shared__ float part[32][33];
    const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
    const int co = blockIdx.x * 32 + lane;
    float s = 0.0f;
    if (co < cout)
        for (int b = t; b < blocks; b += 32) s += __ldg(partial + (long long)b * cout + co);
    part[t][lane] = s;
    __syncthreads();
    if (t == 0 && co < cout) {
        float v = 0.0f;
        for (int q = 0; q < 32; ++q) v += part[q][lane];
        db[co] += v;
    }
}

__global__ void k_pack_weights(const float* __restrict__ w, int cout, int cin_real, int cin, int ks, int flip,
                               int nkb_pad, uint16_t* __restrict__ out) {
    // out rows: the packed conv's output channels (cout, or cin when flipped)
    const int rows = flip ? cin : cout;
    const int kin = flip ? cout : cin;  // packed conv's input channels
    const long long total = (long long)rows * nkb_pad * 8;
    const int cgk = kin / 8;
    const int taps = ks * ks;
    // the slab kernel reads stage-ordered weights [kin/16][tap'][rows/8][2][8][8]
    // with the taps dx-major (tap' = 3 dx + dy), so that the three dy taps
    // of one dx are one contiguous B operand of 3 x rows rows
    const bool slab = slab_layout(kin, ks);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(i % 8);
        const long long t = i / 8;
        const int kb = (int)(t % nkb_pad);
        const int r = (int)(t / nkb_pad);
        float v = 0.0f;
        long long dst = i;
        if (kb < taps * cgk) {
            const int tap = kb / cgk, g = kb % cgk;
            const int k = g * 8 + j;  // packed conv's input channel
            if (!flip) {
                if (k < cin_real) v = w[(((long long)r * cin_real + k) * ks + tap / ks) * ks + tap % ks];
            } else {
                // dX[ci] = sum_co W[co][ci][taps-1-tap] dY[co]: row r = ci, k = co
                const int src_tap = taps - 1 - tap;
                if (r < cin_real) v = w[(((long long)k * cin_real + r) * ks + src_tap / ks) * ks + src_tap % ks];
            }
            if (slab) {
                const int tap_dx = (tap % 3) * 3 + tap / 3;
                dst = (((((long long)(g >> 1) * 9 + tap_dx) * (rows / 8) + (r >> 3)) * 2 + (g & 1)) * 8 + (r & 7)) * 8 + j;
            }
        } else if (slab) {
            continue;
        }
        out[dst] = f_to_bf16(v);
    }
}

__global__ void k_unpack_grad(const float* __restrict__ dwp, int cout, int cin_real, int cin, int ks, int nkb_pad,
                              float* __restrict__ out) {
    const long long total = (long long)cout * cin_real * ks * ks;
    const int cg = cin / 8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int kx = (int)(i % ks);
        const int ky = (int)((i / ks) % ks);
        const int ci = (int)((i / (ks * ks)) % cin_real);
        const int co = (int)(i / ((long long)ks * ks * cin_real));
        const int tap = ky * ks + kx;
        const int kb = tap * cg + ci / 8;
        out[i] = dwp[((long long)co * nkb_pad + kb) * 8 + ci % 8];
    }
}

__global__ void k_maxpool2(const uint16_t* __restrict__ x, int n, int h, int w, int c, uint16_t* __restrict__ y) {
    const int ho = h / 2, wo = w / 2;
    const long long total = (long long)n * ho * wo * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const long long pix = i / c;
        const int xo = (int)(pix % wo);
        const int yo = (int)((pix / wo) % ho);
        const long long img = pix / ((long long)wo * ho);
        const long long b = ((img * h + 2 * yo) * w + 2 * xo) * c + ch;
        float m = bf16_to_f(x[b]);
        m = fmaxf(m, bf16_to_f(x[b + c]));
        m = fmaxf(m, bf16_to_f(x[b + (long long)w * c]));
        m = fmaxf(m, bf16_to_f(x[b + (long long)w * c + c]));
        y[i] = f_to_bf16(m);
    }
}

// 8-channel variants of the pooling / upsampling / slice helpers (one
// 16-byte vector per thread), used when channel counts, strides and offsets
// are multiples of 8 and the tensors 16-byte aligned.  Each keeps its
// scalar counterpart's per-element arithmetic and order, so the results
// are the same bits.
__device__ __forceinline__ void unpack8(const uint4& v, float (&f)[8]) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) f[k] = bf16_to_f((uint16_t)(w[k >> 1] >> ((k & 1) * 16)));
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k] = (uint32_t)f_to_bf16(f[2 * k]) | ((uint32_t)f_to_bf16(f[2 * k + 1]) << 16);
    return make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ __forceinline__ uint16_t lane16(const uint4& v, int k) {
    const uint32_t ws[4] = {v.x, v.y, v.z, v.w};
    return (uint16_t)(ws[k >> 1] >> ((k & 1) * 16));
}

__global__ void k_maxpool2_v8(const uint16_t* __restrict__ x, int n, int h, int w, int c, uint16_t* __restrict__ y) {
    const int ho = h / 2, wo = w / 2, g8 = c / 8;
    const long long total = (long long)n * ho * wo * g8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % g8);
        const long long pix = i / g8;
        const int xo = (int)(pix % wo);
        const int yo = (int)((pix / wo) % ho);
        const long long img = pix / ((long long)wo * ho);
        const long long b = ((img * h + 2 * yo) * w + 2 * xo) * c + g * 8;
        float a0[8], a1[8], a2[8], a3[8], m[8];
        unpack8(__ldg(reinterpret_cast<const uint4*>(x + b)), a0);
        unpack8(__ldg(reinterpret_cast<const uint4*>(x + b + c)), a1);
        unpack8(__ldg(reinterpret_cast<const uint4*>(x + b + (long long)w * c)), a2);
        unpack8(__ldg(reinterpret_cast<const uint4*>(x + b + (long long)w * c + c)), a3);
#pragma unroll
        for (int k = 0; k < 8; ++k) m[k] = fmaxf(fmaxf(fmaxf(a0[k], a1[k]), a2[k]), a3[k]);
        *reinterpret_cast<uint4*>(y + pix * c + g * 8) = pack8(m);
    }
}

__global__ void k_maxpool2_bwd_v8(const uint16_t* __restrict__ x, const uint16_t* __restrict__ y,
                                  const uint16_t* __restrict__ dy, int n, int h, int w, int c,
                                  uint16_t* __restrict__ dx) {
    const int ho = h / 2, wo = w / 2, g8 = c / 8;
    const long long total = (long long)n * ho * wo * g8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % g8);
        const long long pix = i / g8;
        const int xo = (int)(pix % wo);
        const int yo = (int)((pix / wo) % ho);
        const long long img = pix / ((long long)wo * ho);
        const long long b = ((img * h + 2 * yo) * w + 2 * xo) * c + g * 8;
        const long long off[4] = {0, c, (long long)w * c, (long long)w * c + c};
        const uint4 ym = __ldg(reinterpret_cast<const uint4*>(y + pix * c + g * 8));
        const uint4 gr = __ldg(reinterpret_cast<const uint4*>(dy + pix * c + g * 8));
        uint4 xv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) xv[q] = __ldg(reinterpret_cast<const uint4*>(x + b + off[q]));
        uint32_t out[4][4] = {};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint16_t yk = lane16(ym, k), gk = lane16(gr, k);
            bool taken = false;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const bool hit = !taken && lane16(xv[q], k) == yk;
                if (hit) out[q][k >> 1] |= (uint32_t)gk << ((k & 1) * 16);
                taken |= hit;
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            *reinterpret_cast<uint4*>(dx + b + off[q]) = make_uint4(out[q][0], out[q][1], out[q][2], out[q][3]);
    }
}

__global__ void k_upsample2_bwd_v8(const uint16_t* __restrict__ dy, int n, int h, int w, int c, int ds, int doff,
                                   uint16_t* __restrict__ dx) {
    const int W = 2 * w, g8 = c / 8;
    const long long total = (long long)n * h * w * g8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % g8);
        const long long pix = i / g8;
        const int xx = (int)(pix % w);
        const int yy = (int)((pix / w) % h);
        const long long img = pix / ((long long)w * h);
        const long long b = ((img * 2 * h + 2 * yy) * W + 2 * xx);
        float a[8], bb[8], cc[8], d[8], sum[8];
        unpack8(__ldg(reinterpret_cast<const uint4*>(dy + b * ds + doff + g * 8)), a);
        unpack8(__ldg(reinterpret_cast<const uint4*>(dy + (b + 1) * ds + doff + g * 8)), bb);
        unpack8(__ldg(reinterpret_cast<const uint4*>(dy + (b + W) * ds + doff + g * 8)), cc);
        unpack8(__ldg(reinterpret_cast<const uint4*>(dy + (b + W + 1) * ds + doff + g * 8)), d);
#pragma unroll
        for (int k = 0; k < 8; ++k) sum[k] = a[k] + bb[k] + cc[k] + d[k];
        *reinterpret_cast<uint4*>(dx + pix * c + g * 8) = pack8(sum);
    }
}

__global__ void k_slice_add_v8(const uint16_t* __restrict__ x, long long pixels, int c, uint16_t* __restrict__ y,
                               int stride, int off) {
    const int g8 = c / 8;
    const long long total = pixels * g8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % g8);
        const long long p = i / g8;
        uint4* d = reinterpret_cast<uint4*>(y + p * stride + off + g * 8);
        float a[8], b[8], r[8];
        unpack8(*d, a);
        unpack8(__ldg(reinterpret_cast<const uint4*>(x + p * c + g * 8)), b);
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = a[k] + b[k];
        *d = pack8(r);
    }
}

__global__ void k_maxpool2_bwd(const uint16_t* __restrict__ x, const uint16_t* __restrict__ y,
                               const uint16_t* __restrict__ dy, int n, int h, int w, int c, uint16_t* __restrict__ dx) {
    const int ho = h / 2, wo = w / 2;
    const long long total = (long long)n * ho * wo * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const long long pix = i / c;
        const int xo = (int)(pix % wo);
        const int yo = (int)((pix / wo) % ho);
        const long long img = pix / ((long long)wo * ho);
        const long long b = ((img * h + 2 * yo) * w + 2 * xo) * c + ch;
        const long long off[4] = {0, c, (long long)w * c, (long long)w * c + c};
        const uint16_t ym = y[i], g = dy[i];
        bool taken = false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool hit = !taken && x[b + off[k]] == ym;
            dx[b + off[k]] = hit ? g : (uint16_t)0;
            taken |= hit;
        }
    }
}

__global__ void k_upsample2(const uint16_t* __restrict__ x, int n, int h, int w, int c, uint16_t* __restrict__ y,
                            int ys, int yoff) {
    const int H = 2 * h, W = 2 * w;
    const long long total = (long long)n * H * W * (c / 8);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % (c / 8));
        const long long pix = i / (c / 8);
        const int X = (int)(pix % W);
        const int Y = (int)((pix / W) % H);
        const long long img = pix / ((long long)W * H);
        const uint4 v = *reinterpret_cast<const uint4*>(x + ((img * h + Y / 2) * w + X / 2) * c + g * 8);
        *reinterpret_cast<uint4*>(y + pix * ys + yoff + g * 8) = v;
    }
}

__global__ void k_upsample2_bwd(const uint16_t* __restrict__ dy, int n, int h, int w, int c, int ds, int doff,
                                uint16_t* __restrict__ dx) {
    const int W = 2 * w;
    const long long total = (long long)n * h * w * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const long long pix = i / c;
        const int xx = (int)(pix % w);
        const int yy = (int)((pix / w) % h);
        const long long img = pix / ((long long)w * h);
        const long long b = ((img * 2 * h + 2 * yy) * W + 2 * xx);
        float s = bf16_to_f(dy[b * ds + doff + ch]) + bf16_to_f(dy[(b + 1) * ds + doff + ch]) +
                  bf16_to_f(dy[(b + W) * ds + doff + ch]) + bf16_to_f(dy[(b + W + 1) * ds + doff + ch]);
        dx[i] = f_to_bf16(s);
    }
}

__global__ void k_slice(const uint16_t* __restrict__ x, long long pixels, int stride, int off, int c,
                        uint16_t* __restrict__ y) {
    const long long total = pixels * (c / 8);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i % (c / 8));
        const long long p = i / (c / 8);
        *reinterpret_cast<uint4*>(y + p * c + g * 8) = *reinterpret_cast<const uint4*>(x + p * stride + off + g * 8);
    }
}

__global__ void k_slice_add(const uint16_t* __restrict__ x, long long pixels, int c, uint16_t* __restrict__ y,
                            int stride, int off) {
    const long long total = pixels * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        const long long p = i / c;
        uint16_t* d = y + p * stride + off + ch;
        *d = f_to_bf16(bf16_to_f(*d) + bf16_to_f(x[i]));
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2, float gs) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i] * gs;
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Loss sums in fixed point: |v - t| and |e - |v - t|| scaled by 2^32 and
// rounded per pixel, the pixel count as an integer.  Integer additions are
// exact, so the totals do not depend on the order in which blocks finish
// (the reported loss of a run is reproducible bit for bit).
__device__ __forceinline__ unsigned long long to_fixed32(float v) {
    return __float2ull_rn(fminf(v, 1.0e6f) * 4294967296.0f);
}

__global__ void k_surrogate_loss(const float* __restrict__ head, const float* __restrict__ target,
                                 const uint4* __restrict__ feat, long long P, float inv, float ew,
                                 uint16_t* __restrict__ dhead, unsigned long long* __restrict__ sums) {
    unsigned long long s0 = 0, s1 = 0, s2 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
        const float f3 = __uint_as_float(feat[2 * i].y & 0xFFFF0000u);
        float g0 = 0.0f, g1 = 0.0f;
        if (f3 == 1.0f) {
            const float v = head[i * 16], e = head[i * 16 + 1];
            const float d = v - target[i];
            const float ad = fabsf(d);
            g0 = (d > 0.0f ? 1.0f : d < 0.0f ? -1.0f : 0.0f) * inv;
            const float de = e - ad;
            g1 = (de > 0.0f ? ew : de < 0.0f ? -ew : 0.0f) * inv;
            s0 += to_fixed32(ad);
            s1 += 1;
            s2 += to_fixed32(fabsf(de));
        }
        uint4* o = reinterpret_cast<uint4*>(dhead + i * 16);
        o[0] = make_uint4((uint32_t)f_to_bf16(g0) | ((uint32_t)f_to_bf16(g1) << 16), 0u, 0u, 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sums, s0);
        atomicAdd(sums + 1, s1);
        atomicAdd(sums + 2, s2);
    }
}

// ---- weight gradient from TMA-staged, MN-major operands --------------------
// dW[co][tap][ci] = sum over pixels p of dy[p][co] * x[p + tap][ci], with
// K = pixels.  Both operands come straight from the NHWC tensors: a TMA box
// of AW channels x pixels of one image row lands in shared memory as an
// MN-major swizzled operand (channels contiguous, one 2 * AW-byte row per
// pixel), which the MMA reads with the transpose bits set, so nothing is
// transposed.  A unit is one (dy, AW-channel chunk): its box covers the
// chunk's kpx + 2 pixels of input row y + dy - 1 from x0 - 1, and the
// MMA's M = 128 rows are 128 / AW atoms of that one box at successive
// one-pixel offsets (the atoms' stride is one row), so atom dx is tap
// (dy, dx) and the box serves all three dx taps; atoms past dx = 2 fall in
// TMEM lanes that are not read.  N = cout from dy boxes at the same
// pixels.  A CTA owns a group of units (one TMEM accumulator each) and a
// range of pixel chunks (split K); its partial sums go to scratch rows
// tap * cin + ci, added in a fixed order by k_wgrad_reduce.
constexpr int kWgThreads = 128;  // warp 0 TMA, warp 1 MMA; all four warps drain TMEM
constexpr int kWgMaxStages = 6;
constexpr int kWgMaxUnits = 16;

struct WgradTmaArgs {
    int n, h, w, cin, cout;
    int aw, bw;                   // channels per box of x (16 or 32) / of dy (16, 32 or 64)
    int units, units_per_cta;     // (dy, channel chunk) units in all; per CTA
    int m_tiles, chunks_x;        // scratch rows / 128; pixel chunks per image row
    long long chunks, per_split;  // pixel chunks in all; per CTA
    int kpx;                      // pixels (K) per stage: 64 or 128
    int ns, unit_bytes, a_bytes, b_bytes;
    float* scratch;
    uint32_t* err;
    unsigned spin;
    int withhold;
};

// Layout-type code of the tcgen05 shared-memory descriptor for a swizzle
// span of 2 * channels bytes (32, 64 or 128).
__host__ __device__ constexpr uint32_t swizzle_code(int channels) {
    return channels == 64 ? 2u : channels == 32 ? 4u : 6u;
}

// Descriptor of an MN-major swizzled operand: `lbo` bytes between atoms of
// `channels` MN elements, `sbo` bytes between groups of 8 K rows.
__device__ __forceinline__ uint64_t smem_desc_mn(uint32_t addr, uint32_t lbo, uint32_t sbo, int channels) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)swizzle_code(channels) << 61;
    return d;
}

__global__ void __launch_bounds__(kWgThreads) k_conv_wgrad_tma(WgradTmaArgs a, const __grid_constant__ CUtensorMap xmap,
                                                              const __grid_constant__ CUtensorMap dmap) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[kWgMaxStages], empty[kWgMaxStages], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail, s_loaded, s_taken, s_committed, s_freed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = a.cout, NS = a.ns;
    const int u0 = blockIdx.x * a.units_per_cta;
    const int nu = a.units - u0 < a.units_per_cta ? a.units - u0 : a.units_per_cta;
    const long long c_begin = (long long)blockIdx.y * a.per_split;
    const long long c_end = c_begin + a.per_split < a.chunks ? c_begin + a.per_split : a.chunks;
    const int nk = c_end > c_begin ? (int)(c_end - c_begin) : 0;
    uint32_t ncols = 32;  // a power of two covering the units' accumulators (at most 512)
    while (ncols < (uint32_t)(a.units_per_cta * N)) ncols *= 2;
    const int stage_bytes = a.a_bytes + a.b_bytes;
    const int chunks_c = a.cin / a.aw;
    const int box_a = (a.kpx + 2) * a.aw * 2, box_b = a.kpx * a.bw * 2;
    const int nb = N / a.bw;
    if (warp == 0) tmem_alloc(&tmem_slot, ncols);
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        s_fail = 0;
        s_loaded = s_taken = s_committed = s_freed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    volatile int* fail = &s_fail;
    auto warp_wait = [&](uint64_t* bar, unsigned parity) -> bool {
        if (__shfl_sync(0xffffffffu, *fail, 0)) return false;
        const bool w = mbar_wait(bar, parity, a.spin);
        if (__any_sync(0xffffffffu, !w)) {
            if (lane == 0) *fail = 1;
            return false;
        }
        return true;
    };

    if (warp == 0) {
        // TMA producer: per stage one x box per unit, cout / BW dy boxes
        const uint32_t tx = (uint32_t)(nu * box_a + nb * box_b);
        int g = 0, freed = 0;
        for (; g < nk; ++g) {
            const int s = g % NS;
            if (g >= NS) {
                if (!warp_wait(&empty[s], (unsigned)((g / NS) - 1) & 1u)) break;
                freed = g - NS + 1;
            }
            if (__shfl_sync(0xffffffffu, *fail, 0)) break;
            if (lane == 0 && !a.withhold) {
                const long long c = c_begin + g;
                const int x0 = (int)(c % a.chunks_x) * a.kpx;
                const long long row = c / a.chunks_x;
                const int y = (int)(row % a.h), img = (int)(row / a.h);
                uint8_t* sa = smem + s * stage_bytes;
                mbar_expect_tx(&full[s], tx);
                for (int j = 0; j < nu; ++j) {
                    const int u = u0 + j, dy = u / chunks_c, cc = u - dy * chunks_c;
                    tma_load_4d(sa + j * a.unit_bytes, &xmap, cc * a.aw, x0 - 1, y + dy - 1, img, &full[s]);
                }
                for (int j = 0; j < nb; ++j) tma_load_4d(sa + a.a_bytes + j * box_b, &dmap, j * a.bw, x0, y, img, &full[s]);
            }
            __syncwarp();
        }
        if (lane == 0) {
            s_loaded = a.withhold ? 0 : g;
            s_freed = freed;
        }
    } else if (warp == 1) {
        // MMA issuer: both operands MN-major (transpose bits 15 and 16);
        // A's atoms one pixel row (2 * AW bytes) apart
        const uint32_t idesc = idesc_bf16(128, N) | (1u << 15) | (1u << 16);
        const uint32_t row_a = 2u * (uint32_t)a.aw, sbo_a = 8u * row_a, sbo_b = 16u * (uint32_t)a.bw;
        int committed = 0;
        for (int g = 0; g < nk; ++g) {
            const int s = g % NS;
            if (!warp_wait(&full[s], (unsigned)(g / NS) & 1u)) break;
            if (lane == 0) {
                fence_after();
                const uint32_t sa = smem_u32(smem + s * stage_bytes), sb = sa + (uint32_t)a.a_bytes;
                for (int k = 0; k < a.kpx / 16; ++k) {
                    const uint64_t bd = smem_desc_mn(sb + (uint32_t)k * 2u * sbo_b, (uint32_t)box_b, sbo_b, a.bw);
                    for (int j = 0; j < nu; ++j) {
                        const uint64_t ad = smem_desc_mn(sa + (uint32_t)(j * a.unit_bytes) + (uint32_t)k * 16u * row_a,
                                                         row_a, sbo_a, a.aw);
                        mma_bf16(tmem + (uint32_t)(j * N), ad, bd, idesc, (g > 0 || k > 0) ? 1u : 0u);
                    }
                }
                mma_commit(&empty[s]);
                if (g == nk - 1) mma_commit(&done);
            }
            committed = g + 1;
            __syncwarp();
        }
        if (lane == 0) {
            s_taken = committed;
            s_committed = committed;
        }
    }
    __syncthreads();
    // every MMA landed (the last commit), or a wait ran out: then drain the
    // loads nobody took and the commits nobody saw (bounded waits) first
    bool ok = !*fail;
    if (ok && nk > 0 && !mbar_wait(&done, 0u, a.spin)) ok = false;
    const bool all_ok = __syncthreads_and(ok);
    if (!all_ok && lane == 0) {
        if (warp == 0) {
            for (int g = s_taken; g < s_loaded; ++g) mbar_wait(&full[g % NS], (unsigned)(g / NS) & 1u, a.spin);
        } else if (warp == 1) {
            for (int g = s_freed; g < s_committed; ++g) mbar_wait(&empty[g % NS], (unsigned)(g / NS) & 1u, a.spin);
        }
    }
    fence_after();
    // lane m of unit (dy, cc): tap (dy, m / AW), channel cc * AW + m % AW
    const int m = warp * 32 + lane;
    const int dx = m / a.aw;
    const long long split_row = (long long)blockIdx.y * a.m_tiles * 128;
    for (int j = 0; all_ok && j < nu; ++j) {
        const int u = u0 + j, dy = u / chunks_c, cc = u - dy * chunks_c;
        const long long r = (long long)(dy * 3 + dx) * a.cin + cc * a.aw + m % a.aw;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * N + c0), v);
            if (dx > 2) continue;
            if (nk == 0) {
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = 0.0f;
            }
            float4* o = reinterpret_cast<float4*>(a.scratch + (split_row + r) * N + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
    if (!all_ok && tid == 0 && a.err) atomicOr(a.err, 1u);
}

unsigned grid1d(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
}

int nkb_of(int cin, int ks) { return ks * ks * cin / 8; }
int nkb_pad_of(int cin, int ks) { return (nkb_of(cin, ks) + kBKB - 1) / kBKB * kBKB; }

}  // namespace tc
}  // namespace gi

using gi::fail;
using gi::fail_cuda;
namespace tc = gi::tc;

static inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

namespace {
// Polls per mbarrier wait and the bounded-wait test switch, read at every
// launch (gi_tc_set_wait_limit, gi_tc_set_test_withhold).
std::atomic<unsigned> g_wait_limit{tc::kSpinLimit};
std::atomic<int> g_withhold{0};
}  // namespace

extern "C" gi_status gi_tc_set_wait_limit(uint32_t polls) {
    if (polls == 0) return gi::fail(GI_ERR_INVALID_ARG, "gi_tc_set_wait_limit: polls must be > 0");
    g_wait_limit.store(polls);
    return GI_OK;
}

extern "C" uint32_t gi_tc_wait_limit(void) { return g_wait_limit.load(); }

extern "C" gi_status gi_tc_set_test_withhold(int enable) {
    g_withhold.store(enable ? 1 : 0);
    return GI_OK;
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;

gi_status tensor_map_fn() {
    if (g_encode_tiled) return GI_OK;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return fail(GI_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    g_encode_tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return GI_OK;
}

// 4-D map (c, w, h, n) of an NHWC BF16 tensor with boxes of 16 channels x
// 130 pixels x `rows` rows x 1 image (the halo slab of one stage), written
// to shared memory in the 32-byte swizzled layout.
gi_status slab_map(CUtensorMap* m, const uint16_t* x, int n, int h, int w, int c, int rows) {
    gi_status st = tensor_map_fn();
    if (st != GI_OK) return st;
    const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
    const cuuint32_t box[4] = {16, (cuuint32_t)tc::kSlabPx, (cuuint32_t)rows, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = g_encode_tiled(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<uint16_t*>(x), dims, strides,
                                box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? GI_OK : fail(GI_ERR_CUDA, "cuTensorMapEncodeTiled rejected the activation map");
}

// The TMA weight-gradient kernel serves 3x3 convolutions with cin % 16 == 0
// (every 3x3 layer of the U-Net); 1x1 and other shapes keep the gather kernel.
bool wgrad_uses_tma(int cin, int ks) { return ks == 3 && cin % 16 == 0; }

int box_channels(int c) { return c % 64 == 0 ? 64 : c % 32 == 0 ? 32 : 16; }

tc::WgradTmaArgs wgrad_tma_plan(int n, int h, int w, int cin, int cout) {
    tc::WgradTmaArgs a = {};
    a.n = n;
    a.h = h;
    a.w = w;
    a.cin = cin;
    a.cout = cout;
    a.aw = cin % 32 == 0 ? 32 : 16;  // 128 / AW atoms per MMA, at least the three dx taps
    a.bw = box_channels(cout);
    a.units = 3 * (cin / a.aw);
    a.m_tiles = (9 * cin + 127) / 128;
    // The loads are latency-bound (a TMA round trip takes several thousand
    // cycles), so a stage should carry as many bytes as the ring allows:
    // 128 pixels per stage where every unit of a CTA still fits four
    // stages, else 64 pixels and at least three.  A unit's box region holds
    // kpx + 2 loaded rows plus the rows the atoms past dx = 2 read,
    // 1024-byte aligned for the swizzle; units per CTA are also bounded by
    // TMEM (one cout-wide accumulator each, 512 columns).
    const int want = std::min(std::min(a.units, tc::kWgMaxUnits), 512 / cout);
    for (int kpx : {128, 64}) {
        const int min_stages = kpx == 128 ? 4 : 3;
        a.kpx = kpx;
        a.unit_bytes = ((kpx + 128 / a.aw) * a.aw * 2 + 1023) / 1024 * 1024;
        a.b_bytes = cout * kpx * 2;
        int per = want;
        while (per > 1 && min_stages * (per * a.unit_bytes + a.b_bytes) > 200 * 1024) --per;
        a.units_per_cta = per;
        if (per == want) break;
    }
    a.a_bytes = a.units_per_cta * a.unit_bytes;
    a.ns = std::min(tc::kWgMaxStages, (200 * 1024) / (a.a_bytes + a.b_bytes));
    a.chunks_x = (w + a.kpx - 1) / a.kpx;
    a.chunks = (long long)n * h * a.chunks_x;
    // one wave: a CTA per SM over all unit groups, at least 4 chunks each
    const int groups = (a.units + a.units_per_cta - 1) / a.units_per_cta;
    long long splits = std::max<long long>(1, 152 / groups);
    splits = std::min<long long>(splits, std::max<long long>(1, a.chunks / 4));
    a.per_split = (a.chunks + splits - 1) / splits;
    return a;
}

int wgrad_tma_groups(const tc::WgradTmaArgs& a) { return (a.units + a.units_per_cta - 1) / a.units_per_cta; }

long long wgrad_tma_splits(const tc::WgradTmaArgs& a) { return (a.chunks + a.per_split - 1) / a.per_split; }

// 4-D map (c, w, h, n) of an NHWC BF16 tensor with boxes of `box_c`
// channels x `box_px` pixels of one row, swizzled over 2 * box_c bytes:
// the MN-major operands of the weight-gradient kernel.
gi_status wgrad_map(CUtensorMap* m, const uint16_t* t, int n, int h, int w, int c, int box_c, int box_px) {
    gi_status st = tensor_map_fn();
    if (st != GI_OK) return st;
    const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
    const cuuint32_t box[4] = {(cuuint32_t)box_c, (cuuint32_t)box_px, 1, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUtensorMapSwizzle sw = box_c == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                 : box_c == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
    CUresult r = g_encode_tiled(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<uint16_t*>(t), dims, strides, box,
                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? GI_OK : fail(GI_ERR_CUDA, "cuTensorMapEncodeTiled rejected a weight-gradient map");
}

// Opt a kernel into more than 48 KB of dynamic shared memory, once per
// device (the attribute is per device, and calls may come from several
// threads).
template <typename F>
void smem_opt_in(F* fn, int bytes, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_acq_rel);
}

gi_status launch_slab(const tc::ConvArgs& a, cudaStream_t cs) {
    const tc::SlabGeom G = tc::persist_geom(a.cout, a.cin / 16);
    CUtensorMap m;
    gi_status st = slab_map(&m, a.x, a.n, a.h, a.w, a.cin, G.R + 2);
    if (st != GI_OK) return st;
    static std::atomic<unsigned long long> attr[4];
    auto* kern = G.R == 8 ? tc::k_conv3_slab<8> : G.R == 4 ? tc::k_conv3_slab<4>
               : G.R == 2 ? tc::k_conv3_slab<2> : tc::k_conv3_slab<1>;
    smem_opt_in(kern, 220 * 1024, attr[G.R == 8 ? 3 : G.R == 4 ? 2 : G.R == 2 ? 1 : 0]);
    const int tx = (a.w + 127) / 128, ty = (a.h + G.R - 1) / G.R;
    const long long tiles = (long long)tx * ty * a.n;
    if (tiles > 0x7FFFFFFFLL) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_bf16: too many tiles");
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<long long>(tiles, sms);
    // programmatic dependent launch: the prologue overlaps the previous
    // kernel's tail (the kernel waits for it before any global access)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(tc::kPersistThreads);
    cfg.dynamicSmemBytes = (size_t)(G.NS * G.stage_bytes + 1024);
    cfg.stream = cs;
    cudaLaunchAttribute attr_pdl[1];
    attr_pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr_pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr_pdl;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a, m, tx, ty, (int)tiles);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_conv2d_bf16 launch");
}
}  // namespace

extern "C" gi_status gi_conv2d_bf16(const gi_bf16* x, int n, int h, int w, int cin, const gi_bf16* wt,
                                    const float* bias, int cout, int ksize, int act, const gi_bf16* mask,
                                    gi_bf16* y, int y_stride, int y_off, float* y32, uint32_t* err,
                                    void* stream) {
    if (!x || !wt || (!y && !y32)) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_bf16: NULL argument");
    if (n < 1 || h < 1 || w < 1 || cin < 8 || cin % 8 || cout < 16 || cout > 256 || cout % 16 ||
        (ksize != 1 && ksize != 3) || (act != GI_ACT_NONE && act != GI_ACT_RELU))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_bf16: bad shape (cin % 8, cout % 16 in [16, 256], ksize 1|3)");
    if (y && (y_stride % 8 || y_off % 8 || y_off + cout > y_stride))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_bf16: y_stride / y_off must be multiples of 8 and fit cout");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(wt) | reinterpret_cast<uintptr_t>(y) |
         reinterpret_cast<uintptr_t>(mask) | reinterpret_cast<uintptr_t>(y32)) % 16)
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_bf16: tensors must be 16-byte aligned");
    tc::ConvArgs a = {};
    a.x = x;
    a.n = n;
    a.h = h;
    a.w = w;
    a.cin = cin;
    a.wt = wt;
    a.cout = cout;
    a.nkb = tc::nkb_of(cin, ksize);
    a.nkb_pad = tc::nkb_pad_of(cin, ksize);
    a.ksize = ksize;
    a.bias = bias;
    a.act = act;
    a.mask = mask;
    a.y = y;
    a.y_c = y ? y_stride : cout;
    a.y_off = y ? y_off : 0;
    a.y32 = y32;
    a.err = err;
    a.spin = g_wait_limit.load();
    a.withhold = g_withhold.load();
    a.P = (long long)n * h * w;
    a.hw = nullptr;
    a.hb = nullptr;
    a.hout = nullptr;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (tc::slab_layout(cin, ksize)) return launch_slab(a, cs);
    const int smem = tc::kNS * (tc::kStageA + (cout / 8) * tc::kSBO);
    static std::atomic<unsigned long long> attr{0};
    smem_opt_in(tc::k_conv_fwd, 4 * (8192 + 16384), attr);
    const long long tiles = (a.P + 127) / 128;
    if (tiles > 0x7FFFFFFFLL) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_bf16: too many pixels");
    tc::k_conv_fwd<<<(unsigned)tiles, tc::kThreads, smem, cs>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_conv2d_bf16 launch");
}

namespace {
struct WgradPlan {
    int m_tiles, splits;
    long long px_per_split;
};
WgradPlan wgrad_plan(long long P, int cin, int ks) {
    WgradPlan pl;
    pl.m_tiles = (tc::nkb_of(cin, ks) * 8 + 127) / 128;
    const long long target = 2LL * 152;
    long long splits = std::max<long long>(1, (target + pl.m_tiles - 1) / pl.m_tiles);
    splits = std::min<long long>(splits, std::max<long long>(1, (P + 1023) / 1024));
    long long per = (P + splits - 1) / splits;
    per = (per + 31) / 32 * 32;
    pl.px_per_split = std::max<long long>(per, 32);
    pl.splits = (int)((P + pl.px_per_split - 1) / pl.px_per_split);
    if (pl.splits < 1) pl.splits = 1;
    return pl;
}
}  // namespace

extern "C" size_t gi_conv2d_wgrad_scratch_floats(int n, int h, int w, int cin, int cout, int ksize) {
    if (n < 1 || h < 1 || w < 1 || cin < 8 || cout < 16) return 0;
    if (wgrad_uses_tma(cin, ksize)) {
        const tc::WgradTmaArgs a = wgrad_tma_plan(n, h, w, cin, cout);
        return (size_t)wgrad_tma_splits(a) * a.m_tiles * 128 * cout;
    }
    WgradPlan pl = wgrad_plan((long long)n * h * w, cin, ksize);
    return (size_t)pl.splits * pl.m_tiles * 128 * cout;
}

extern "C" gi_status gi_conv2d_wgrad_bf16(const gi_bf16* x, const gi_bf16* dy, int n, int h, int w, int cin,
                                          int cout, int ksize, float* dw, float* db, float* scratch,
                                          uint32_t* err, void* stream) {
    if (!x || !dy || !dw || !scratch) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_wgrad_bf16: NULL argument");
    if (n < 1 || h < 1 || w < 1 || cin < 8 || cin % 8 || cout < 16 || cout > 256 || cout % 16 ||
        (ksize != 1 && ksize != 3))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_wgrad_bf16: bad shape");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(dy) | reinterpret_cast<uintptr_t>(scratch)) % 16)
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_wgrad_bf16: tensors must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long P = (long long)n * h * w;
    WgradPlan pl = wgrad_plan(P, cin, ksize);
    if (wgrad_uses_tma(cin, ksize)) {
        tc::WgradTmaArgs t = wgrad_tma_plan(n, h, w, cin, cout);
        const long long splits = wgrad_tma_splits(t);
        if (splits > 65535) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_wgrad_bf16: too many pixel splits");
        t.scratch = scratch;
        t.err = err;
        t.spin = g_wait_limit.load();
        t.withhold = g_withhold.load();
        CUtensorMap xm, dm;
        gi_status gs = wgrad_map(&xm, x, n, h, w, cin, t.aw, t.kpx + 2);
        if (gs == GI_OK) gs = wgrad_map(&dm, dy, n, h, w, cout, t.bw, t.kpx);
        if (gs != GI_OK) return gs;
        static std::atomic<unsigned long long> attr_tma{0};
        smem_opt_in(tc::k_conv_wgrad_tma, 220 * 1024, attr_tma);
        const int smem = t.ns * (t.a_bytes + t.b_bytes) + 1024;
        tc::k_conv_wgrad_tma<<<dim3(wgrad_tma_groups(t), (unsigned)splits), tc::kWgThreads, smem, st>>>(t, xm, dm);
        pl.m_tiles = t.m_tiles;  // the reduction below reads this kernel's partial sums
        pl.splits = (int)splits;
    } else {
        tc::WgradArgs a;
        a.x = x;
        a.dy = dy;
        a.n = n;
        a.h = h;
        a.w = w;
        a.cin = cin;
        a.cout = cout;
        a.ksize = ksize;
        a.nkb = tc::nkb_of(cin, ksize);
        a.m_tiles = pl.m_tiles;
        a.P = P;
        a.px_per_split = pl.px_per_split;
        a.scratch = scratch;
        a.err = err;
        a.spin = g_wait_limit.load();
        a.withhold = g_withhold.load();
        const int smem = tc::kNS * (tc::kStageA + (cout / 8) * tc::kSBO);
        static std::atomic<unsigned long long> attr{0};
        smem_opt_in(tc::k_conv_wgrad, 4 * (8192 + 16384), attr);
        tc::k_conv_wgrad<<<dim3(pl.m_tiles, pl.splits), tc::kThreads, smem, st>>>(a);
    }
    const int nkb = tc::nkb_of(cin, ksize);
    tc::k_wgrad_reduce<<<dim3((unsigned)(8 * nkb), (unsigned)((cout + 31) / 32)), 32 * tc::kReducePhases, 0, st>>>(
        scratch, pl.splits, pl.m_tiles, cout, nkb, tc::nkb_pad_of(cin, ksize), dw);
    if (db) {
        // the partial sums reuse the scratch k_wgrad_reduce has finished
        // reading (at least 128 x cout floats)
        const long long cap = (long long)pl.splits * pl.m_tiles * 128;
        const int blocks = (int)std::max<long long>(1, std::min<long long>(std::min<long long>(1216, (P + 63) / 64), cap));
        tc::k_bias_grad<<<blocks, 256, 0, st>>>(dy, P, cout, scratch);
        tc::k_bias_reduce<<<(cout + 31) / 32, 1024, 0, st>>>(scratch, blocks, cout, db);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_conv2d_wgrad_bf16 launch");
}

extern "C" gi_status gi_pack_conv_weights(const float* w, int cout, int cin_real, int cin, int ksize, int flip,
                                          gi_bf16* out, void* stream) {
    if (!w || !out || cout < 1 || cin_real < 1 || cin_real > cin || cin % 8 || (ksize != 1 && ksize != 3))
        return fail(GI_ERR_INVALID_ARG, "gi_pack_conv_weights: bad arguments");
    if (flip && cout % 8) return fail(GI_ERR_INVALID_ARG, "gi_pack_conv_weights: flip needs cout % 8 == 0");
    const int kin = flip ? cout : cin;
    const int rows = flip ? cin : cout;
    const int nkb_pad = tc::nkb_pad_of(kin, ksize);
    const long long total = (long long)rows * nkb_pad * 8;
    tc::k_pack_weights<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        w, cout, cin_real, cin, ksize, flip, nkb_pad, out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_pack_conv_weights launch");
}

extern "C" gi_status gi_unpack_conv_grad(const float* dw_packed, int cout, int cin_real, int cin, int ksize,
                                         float* out, void* stream) {
    if (!dw_packed || !out || cout < 1 || cin_real < 1 || cin % 8 || cin_real > cin || (ksize != 1 && ksize != 3))
        return fail(GI_ERR_INVALID_ARG, "gi_unpack_conv_grad: bad arguments");
    const long long total = (long long)cout * cin_real * ksize * ksize;
    tc::k_unpack_grad<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        dw_packed, cout, cin_real, cin, ksize, tc::nkb_pad_of(cin, ksize), out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_unpack_conv_grad launch");
}

extern "C" gi_status gi_maxpool2_bf16(const gi_bf16* x, int n, int h, int w, int c, gi_bf16* y, void* stream) {
    if (!x || !y || n < 1 || h < 2 || w < 2 || h % 2 || w % 2 || c < 1)
        return fail(GI_ERR_INVALID_ARG, "gi_maxpool2_bf16: bad arguments");
    const long long total = (long long)n * (h / 2) * (w / 2) * c;
    if (c % 8 == 0 && aligned16(x) && aligned16(y))
        tc::k_maxpool2_v8<<<tc::grid1d(total / 8, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, h, w, c, y);
    else
        tc::k_maxpool2<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, h, w, c, y);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_maxpool2_bf16 launch");
}

extern "C" gi_status gi_maxpool2_bwd_bf16(const gi_bf16* x, const gi_bf16* y, const gi_bf16* dy, int n, int h,
                                          int w, int c, gi_bf16* dx, void* stream) {
    if (!x || !y || !dy || !dx || n < 1 || h < 2 || w < 2 || h % 2 || w % 2 || c < 1)
        return fail(GI_ERR_INVALID_ARG, "gi_maxpool2_bwd_bf16: bad arguments");
    const long long total = (long long)n * (h / 2) * (w / 2) * c;
    if (c % 8 == 0 && aligned16(x) && aligned16(y) && aligned16(dy) && aligned16(dx))
        tc::k_maxpool2_bwd_v8<<<tc::grid1d(total / 8, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            x, y, dy, n, h, w, c, dx);
    else
        tc::k_maxpool2_bwd<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, y, dy, n, h, w,
                                                                                                c, dx);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_maxpool2_bwd_bf16 launch");
}

extern "C" gi_status gi_upsample2_bf16(const gi_bf16* x, int n, int h, int w, int c, gi_bf16* y, int y_stride,
                                       int y_off, void* stream) {
    if (!x || !y || n < 1 || h < 1 || w < 1 || c < 8 || c % 8 || y_stride % 8 || y_off < 0 || y_off % 8 ||
        y_off + c > y_stride)
        return fail(GI_ERR_INVALID_ARG, "gi_upsample2_bf16: bad arguments");
    const long long total = (long long)n * 4 * h * w * (c / 8);
    tc::k_upsample2<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, h, w, c, y,
                                                                                         y_stride, y_off);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_upsample2_bf16 launch");
}

extern "C" gi_status gi_upsample2_bwd_bf16(const gi_bf16* dy, int n, int h, int w, int c, int dy_stride,
                                           int dy_off, gi_bf16* dx, void* stream) {
    if (!dy || !dx || n < 1 || h < 1 || w < 1 || c < 1 || dy_off < 0 || dy_off + c > dy_stride)
        return fail(GI_ERR_INVALID_ARG, "gi_upsample2_bwd_bf16: bad arguments");
    const long long total = (long long)n * h * w * c;
    if (c % 8 == 0 && dy_stride % 8 == 0 && dy_off % 8 == 0 && aligned16(dy) && aligned16(dx))
        tc::k_upsample2_bwd_v8<<<tc::grid1d(total / 8, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            dy, n, h, w, c, dy_stride, dy_off, dx);
    else
        tc::k_upsample2_bwd<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            dy, n, h, w, c, dy_stride, dy_off, dx);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_upsample2_bwd_bf16 launch");
}

extern "C" gi_status gi_channel_slice_bf16(const gi_bf16* x, size_t pixels, int stride, int off, int c, gi_bf16* y,
                                           void* stream) {
    if (!x || !y || c < 8 || c % 8 || stride % 8 || off < 0 || off % 8 || off + c > stride)
        return fail(GI_ERR_INVALID_ARG, "gi_channel_slice_bf16: bad arguments");
    const long long total = (long long)pixels * (c / 8);
    tc::k_slice<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, (long long)pixels, stride,
                                                                                     off, c, y);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_channel_slice_bf16 launch");
}

extern "C" gi_status gi_channel_slice_add_bf16(const gi_bf16* x, size_t pixels, int c, gi_bf16* y, int stride,
                                               int off, void* stream) {
    if (!x || !y || c < 1 || off < 0 || off + c > stride)
        return fail(GI_ERR_INVALID_ARG, "gi_channel_slice_add_bf16: bad arguments");
    const long long total = (long long)pixels * c;
    if (c % 8 == 0 && stride % 8 == 0 && off % 8 == 0 && aligned16(x) && aligned16(y))
        tc::k_slice_add_v8<<<tc::grid1d(total / 8, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            x, (long long)pixels, c, y, stride, off);
    else
        tc::k_slice_add<<<tc::grid1d(total, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            x, (long long)pixels, c, y, stride, off);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_channel_slice_add_bf16 launch");
}

extern "C" gi_status gi_adam_f32(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1,
                                 float beta2, float eps, int step, float grad_scale, void* stream) {
    if (!p || !g || !m || !v || step < 1) return fail(GI_ERR_INVALID_ARG, "gi_adam_f32: bad arguments");
    const float c1 = 1.0f - powf(beta1, (float)step);
    const float c2 = 1.0f - powf(beta2, (float)step);
    tc::k_adam<<<tc::grid1d((long long)n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        p, g, m, v, (long long)n, lr, beta1, beta2, eps, c1, c2, grad_scale);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_adam_f32 launch");
}

extern "C" gi_status gi_surrogate_loss(const float* d_head, const float* d_target, const void* d_feat, size_t pixels,
                                       float err_weight, gi_bf16* d_dhead, uint64_t* d_sums, void* stream) {
    if (!d_head || !d_target || !d_feat || !d_dhead || !d_sums || pixels == 0)
        return fail(GI_ERR_INVALID_ARG, "gi_surrogate_loss: bad arguments");
    tc::k_surrogate_loss<<<tc::grid1d((long long)pixels, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        d_head, d_target, static_cast<const uint4*>(d_feat), (long long)pixels, 1.0f / (float)pixels, err_weight,
        d_dhead, reinterpret_cast<unsigned long long*>(d_sums));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_surrogate_loss launch");
}

extern "C" gi_status gi_conv2d_fused_bf16(const gi_bf16* x, int n, int h, int w, int cin, const gi_bf16* wt,
                                          const float* bias, int cout, int act, gi_bf16* y, int y_stride, int y_off,
                                          gi_bf16* pool, int upsample, uint32_t* err, void* stream) {
    if (!x || !wt || (!y && !pool)) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_fused_bf16: NULL argument");
    if (n < 1 || h < 1 || w < 1 || cin < 16 || cin % 16 || cout < 16 || cout > 256 || cout % 16 ||
        (act != GI_ACT_NONE && act != GI_ACT_RELU))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_fused_bf16: bad shape (cin % 16, cout % 16 in [16, 256])");
    if (y && (y_stride % 8 || y_off % 8 || y_off < 0 || y_off + cout > y_stride))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_fused_bf16: y_stride / y_off must be multiples of 8 and fit cout");
    if (pool && (h % 2 || w % 2 || cout > 128))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_fused_bf16: pooling needs even h, w and cout <= 128");
    if (upsample && !y) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_fused_bf16: upsample needs y");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(wt) | reinterpret_cast<uintptr_t>(y) |
         reinterpret_cast<uintptr_t>(pool)) % 16)
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_fused_bf16: tensors must be 16-byte aligned");
    tc::ConvArgs a = {};
    a.x = x;
    a.n = n;
    a.h = h;
    a.w = w;
    a.cin = cin;
    a.wt = wt;
    a.cout = cout;
    a.nkb = tc::nkb_of(cin, 3);
    a.nkb_pad = tc::nkb_pad_of(cin, 3);
    a.ksize = 3;
    a.bias = bias;
    a.act = act;
    a.y = y;
    a.y_c = y ? y_stride : cout;
    a.y_off = y ? y_off : 0;
    a.err = err;
    a.spin = g_wait_limit.load();
    a.withhold = g_withhold.load();
    a.P = (long long)n * h * w;
    a.pool = pool;
    a.up2 = upsample ? 1 : 0;
    gi_status st = launch_slab(a, static_cast<cudaStream_t>(stream));
    if (st != GI_OK) return st;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_conv2d_fused_bf16 launch");
}

extern "C" gi_status gi_conv2d_head_bf16(const gi_bf16* x, int n, int h, int w, int cin, const gi_bf16* wt,
                                         const float* bias, int cout, int act, const float* head_w,
                                         const float* head_b, float* head_out, uint32_t* err, void* stream) {
    if (!x || !wt || !head_w || !head_b || !head_out) return fail(GI_ERR_INVALID_ARG, "gi_conv2d_head_bf16: NULL argument");
    if (n < 1 || h < 1 || w < 1 || cin < 16 || cin % 16 || cout < 16 || cout > 256 || cout % 16 ||
        (act != GI_ACT_NONE && act != GI_ACT_RELU))
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_head_bf16: bad shape (cin % 16, cout % 16 in [16, 256])");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(wt) | reinterpret_cast<uintptr_t>(head_out)) % 16)
        return fail(GI_ERR_INVALID_ARG, "gi_conv2d_head_bf16: tensors must be 16-byte aligned");
    tc::ConvArgs a = {};
    a.x = x;
    a.n = n;
    a.h = h;
    a.w = w;
    a.cin = cin;
    a.wt = wt;
    a.cout = cout;
    a.nkb = tc::nkb_of(cin, 3);
    a.nkb_pad = tc::nkb_pad_of(cin, 3);
    a.ksize = 3;
    a.bias = bias;
    a.act = act;
    a.y_c = cout;
    a.err = err;
    a.spin = g_wait_limit.load();
    a.withhold = g_withhold.load();
    a.P = (long long)n * h * w;
    a.hw = head_w;
    a.hb = head_b;
    a.hout = head_out;
    gi_status st = launch_slab(a, static_cast<cudaStream_t>(stream));
    if (st != GI_OK) return st;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_conv2d_head_bf16 launch");
}
