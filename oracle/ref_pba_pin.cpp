// ref_pba_pin.cpp -- runs the reference's own PBA kernels on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  The reference's only CUDA code is the parallel
// banding algorithm (Cao et al. 2010) in ShadowMapping/include/EDT/
// pba2DKernel.h, launched by ShadowMapping/src/EDT/pba2DHost.cu.  That host
// file binds texture references, which CUDA removed in 12.0, so it cannot be
// built here; this file instead compiles the unmodified kernel header with
// g++ against a small emulation of the CUDA built-ins it uses, and replays
// the host file's launch sequence.  oracle/build_oracle.py builds it into
// oracle/_ref/ only where the reference tree is present; the tests and
// tests/golden/make_edt_golden.py use it to pin the oracle restatement and
// the committed golden fixtures.
//
// Emulation rules (the CUDA semantics the kernels rely on):
//   * threads of a block run one after another, except in the two kernels
//     that call __syncthreads (kernelTranspose, kernelColor), whose threads
//     run as cooperative fibers that all stop at each barrier;
//   * blocks run one after another, so `__shared__` becomes `static`;
//   * tex1Dfetch on linear memory returns zero outside the bound range;
//   * tex2D is point sampled with unnormalised coordinates and clamp
//     addressing (texture-reference defaults): texel floor(x), clamped;
//   * __mul24 keeps the low 32 bits of the product of the sign-extended low
//     24 bits of each operand;
//   * FP32 operations round once each (built with -ffp-contract=off).
// The reference's kernels assume square images (TOID uses one size for both
// dimensions), so only width == height is accepted.
#include <ucontext.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

using std::abs;
using std::max;

// ---- CUDA vocabulary used by pba2DKernel.h ---------------------------------
struct short2 {
    short x, y;
};
struct float4 {
    float x, y, z, w;
};
static inline short2 make_short2(short x, short y) {
    short2 r;
    r.x = x;
    r.y = y;
    return r;
}
struct uint3 {
    unsigned x, y, z;
};
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
static uint3 threadIdx, blockIdx;
static dim3 blockDim, gridDim;

static inline int __mul24(int a, int b) {
    auto s24 = [](int v) -> int64_t {
        int64_t u = (int64_t)((uint32_t)v & 0xFFFFFFu);
        return (u & 0x800000) ? u - 0x1000000 : u;
    };
    return (int)(uint32_t)(uint64_t)(s24(a) * s24(b));
}

enum { cudaTextureType1D = 1, cudaTextureType2D = 2 };
enum { cudaReadModeElementType = 0 };
template <class T, int Dim = cudaTextureType1D, int Mode = cudaReadModeElementType>
struct texture {
    const T* ptr = nullptr;
    long n = 0;
    int w = 0, h = 0;
};
template <class T>
static inline T tex1Dfetch(const texture<T>& t, int i) {
    if (i < 0 || i >= t.n) {
        T z;
        std::memset(&z, 0, sizeof z);
        return z;
    }
    return t.ptr[i];
}
static inline float4 tex2D(const texture<float4, cudaTextureType2D, cudaReadModeElementType>& t, float x, float y) {
    long ix = (long)std::floor(x), iy = (long)std::floor(y);
    ix = std::min<long>(std::max<long>(ix, 0), t.w - 1);
    iy = std::min<long>(std::max<long>(iy, 0), t.h - 1);
    return t.ptr[iy * t.w + ix];
}

// Cooperative fibers for the kernels with barriers.
struct Fiber {
    ucontext_t ctx;
    uint3 tid;
    bool done;
};
static ucontext_t g_sched;
static Fiber* g_cur = nullptr;
static bool g_coop = false;
static std::function<void()>* g_body = nullptr;
static std::vector<Fiber> g_fibers;
static std::vector<std::vector<char>> g_stacks;

static void __syncthreads() {
    if (!g_coop) std::abort();  // a kernel launched without fibers reached a barrier
    swapcontext(&g_cur->ctx, &g_sched);
}

static void fiber_entry() {
    (*g_body)();
    g_cur->done = true;
}

static void launch(dim3 grid, dim3 block, bool coop, std::function<void()> body) {
    gridDim = grid;
    blockDim = block;
    const unsigned nthr = block.x * block.y * block.z;
    g_body = &body;
    g_coop = coop;
    if (coop && g_fibers.size() < nthr) {
        g_fibers.resize(nthr);
        g_stacks.resize(nthr);
        for (auto& s : g_stacks) s.resize(1 << 16);
    }
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx = uint3{bx, by, bz};
                if (!coop) {
                    for (unsigned tz = 0; tz < block.z; ++tz)
                        for (unsigned ty = 0; ty < block.y; ++ty)
                            for (unsigned tx = 0; tx < block.x; ++tx) {
                                threadIdx = uint3{tx, ty, tz};
                                body();
                            }
                    continue;
                }
                unsigned k = 0;
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx, ++k) {
                            Fiber& f = g_fibers[k];
                            f.tid = uint3{tx, ty, tz};
                            f.done = false;
                            getcontext(&f.ctx);
                            f.ctx.uc_stack.ss_sp = g_stacks[k].data();
                            f.ctx.uc_stack.ss_size = g_stacks[k].size();
                            f.ctx.uc_link = &g_sched;
                            makecontext(&f.ctx, fiber_entry, 0);
                        }
                for (;;) {
                    unsigned finished = 0;
                    for (unsigned i = 0; i < nthr; ++i) {
                        Fiber& f = g_fibers[i];
                        if (f.done) {
                            ++finished;
                            continue;
                        }
                        threadIdx = f.tid;
                        g_cur = &f;
                        swapcontext(&g_sched, &f.ctx);
                        if (f.done) ++finished;
                    }
                    if (finished == nthr) break;
                    if (finished != 0) std::abort();  // threads of one block disagree on the barriers
                }
            }
    g_coop = false;
}

// ---- the reference's globals (pba2DHost.cu:50-66) and kernels --------------
#define __global__
#define __device__
#define __host__
#define __shared__ static
#define BLOCKX 16
#define BLOCKY 16
#define BLOCKSIZE 64
#define TILE_DIM 16
#define BLOCK_ROWS 8
typedef void* cudaGraphicsResource_t;

#include "pba2D.h"

static texture<short2> pbaTexColor;
static texture<short2> pbaTexLinks;
static texture<float4, cudaTextureType2D, cudaReadModeElementType> pbaImage;
static texture<float4, cudaTextureType2D, cudaReadModeElementType> pbaGlobalPosition;

#include "pba2DKernel.h"

// ---- the host sequence of pba2DHost.cu (pba2DCompute and its phases) -------
namespace {

struct Buffers {
    int size;
    std::vector<short2> tex[2], transposed;
};

void bind_tex(texture<short2>& t, const std::vector<short2>& v) {
    t.ptr = v.data();
    t.n = (long)v.size();
}

void transpose(std::vector<short2>& out, std::vector<short2>& in, int w, int h) {  // pba2DTranspose
    dim3 block(TILE_DIM, BLOCK_ROWS), grid(w / TILE_DIM, h / TILE_DIM);
    launch(grid, block, true, [&] { kernelTranspose(out.data(), in.data(), w, h); });
}

void phase1(Buffers& b, int m1) {  // pba2DPhase1
    const int s = b.size;
    dim3 block(BLOCKSIZE), grid(s / BLOCKSIZE, m1);
    bind_tex(pbaTexColor, b.tex[0]);
    launch(grid, block, false, [&] { kernelFloodDown(b.tex[1].data(), s, s / m1); });
    bind_tex(pbaTexColor, b.tex[1]);
    launch(grid, block, false, [&] { kernelFloodUp(b.tex[1].data(), s, s / m1); });
    launch(grid, block, false, [&] { kernelPropagateInterband(b.tex[0].data(), s, s / m1); });
    bind_tex(pbaTexLinks, b.tex[0]);
    launch(grid, block, false, [&] { kernelUpdateVertical(b.tex[1].data(), s, m1, s / m1); });
}

void phase2(Buffers& b, int m2) {  // pba2DPhase2
    const int s = b.size;
    dim3 block(BLOCKSIZE), grid(s / BLOCKSIZE, m2);
    bind_tex(pbaTexColor, b.transposed);
    launch(grid, block, false, [&] { kernelProximatePoints(b.tex[0].data(), s, s / m2); });
    bind_tex(pbaTexLinks, b.tex[0]);
    launch(grid, block, false, [&] { kernelCreateForwardPointers(b.tex[0].data(), s, s / m2); });
    for (int noBand = m2; noBand > 1; noBand /= 2) {
        dim3 g(s / BLOCKSIZE, noBand / 2);
        launch(g, block, false, [&] { kernelMergeBands(b.tex[0].data(), s, s / noBand); });
    }
    dim3 g2(s / BLOCKSIZE, s);
    launch(g2, block, false, [&] { kernelDoubleToSingleList(b.tex[0].data(), s); });
}

void phase3(Buffers& b, int m3) {  // pba2DPhase3
    const int s = b.size;
    dim3 block(BLOCKSIZE / m3, m3), grid(s / (BLOCKSIZE / m3));
    bind_tex(pbaTexColor, b.tex[0]);
    launch(grid, block, true, [&] { kernelColor(b.transposed.data(), s, s); });
}

void compute(Buffers& b, int m1, int m2, int m3) {  // pba2DCompute
    phase1(b, m1);
    transpose(b.transposed, b.tex[1], b.size, b.size);
    phase2(b, m2);
    phase3(b, m3);
    transpose(b.tex[1], b.transposed, b.size, b.size);
}

bool shape_ok(int W, int H, int m1, int m2, int m3) {
    return W == H && W >= BLOCKSIZE && W % BLOCKSIZE == 0 && m1 > 0 && W % m1 == 0 && m2 > 0 &&
           W % m2 == 0 && m3 > 0 && BLOCKSIZE % m3 == 0 && W % m3 == 0 && (W * H) % 512 == 0;
}

}  // namespace

// pba2DInitializeInput(short*) + pba2DCompute: sites as (x, y) / (MARKER,
// MARKER) short pairs; out receives textures[1] (nearest site per pixel).
extern "C" int ref_pba_voronoi(const short* sites, int W, int H, int m1, int m2, int m3, short* out) {
    if (!shape_ok(W, H, m1, m2, m3)) return 1;
    Buffers b;
    b.size = W;
    const size_t n = (size_t)W * H;
    b.tex[0].assign((const short2*)sites, (const short2*)sites + n);
    b.tex[1].assign(n, make_short2(0, 0));
    b.transposed.assign(n, make_short2(0, 0));
    compute(b, m1, m2, m3);
    std::memcpy(out, b.tex[1].data(), n * sizeof(short2));
    return 0;
}

// filterHardShadowsUsingEDT's CUDA part (ShadowMapping/src/main.cpp:
// 416-422): initializeInput over the hard-shadow image, pba2DCompute(m1, m2,
// m3), pbaNormalizeDistanceTransform into out4 (channels 0 and 1 written).
// sites / nearest receive textures[0] after initializeInput and textures[1]
// after the transform (either may be NULL).
extern "C" int ref_edt_soft_shadows(const float* image, const float* position, int W, int H, int m1, int m2, int m3,
                                    float penumbra, float intensity, short* sites, short* nearest, float* out4) {
    if (!shape_ok(W, H, m1, m2, m3)) return 1;
    Buffers b;
    b.size = W;
    const size_t n = (size_t)W * H;
    b.tex[0].assign(n, make_short2(0, 0));
    b.tex[1].assign(n, make_short2(0, 0));
    b.transposed.assign(n, make_short2(0, 0));
    pbaImage.ptr = (const float4*)image;
    pbaImage.w = W;
    pbaImage.h = H;
    pbaGlobalPosition.ptr = (const float4*)position;
    pbaGlobalPosition.w = W;
    pbaGlobalPosition.h = H;
    dim3 block(512), grid((int)ceilf((W * H) / 512));
    launch(grid, block, false, [&] { initializeInput(b.tex[0].data(), H, W); });
    if (sites) std::memcpy(sites, b.tex[0].data(), n * sizeof(short2));
    compute(b, m1, m2, m3);
    if (nearest) std::memcpy(nearest, b.tex[1].data(), n * sizeof(short2));
    launch(grid, block, false,
           [&] { pbaNormalizeDistanceTransform(b.tex[1].data(), out4, penumbra, W, intensity); });
    return 0;
}
