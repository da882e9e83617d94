/*
 * gi_surrogate.h -- C ABI of the learned soft-shadow surrogate.
 *
 * The reference has no learned component: its soft shadows come from the
 * PCSS fragment shader (SoftShadowMapping/Shaders/SoftShadow/
 * PlausibleSoftShadow.frag:556-633, selected at SoftShadowMapping/src/
 * main.cpp:1010-1017).  This interface adds a BF16 U-Net that predicts the
 * PCSS visibility of a frame from four cheap per-pixel features, plus an
 * error head; pixels whose predicted error exceeds a threshold are
 * recomputed with the exact PCSS pass.
 *
 * The building blocks are exported so that training (forward, backward,
 * Adam) runs through the same kernels as inference:
 *   - gi_conv2d_bf16: implicit-GEMM convolution (3x3 or 1x1, stride 1,
 *     zero padding) on NHWC BF16 tensors with FP32 accumulation on the
 *     tcgen05 tensor cores (accumulators in tensor memory), with a fused
 *     bias / ReLU / ReLU-derivative-mask epilogue writing into a channel
 *     slice of the output tensor.  A 1x1 convolution of a 1 x P image is a
 *     plain GEMM D[P x N] = A[P x K] . B[N x K]^T.
 *   - gi_conv2d_wgrad_bf16: the weight gradient of the same convolution.
 *   - pooling, upsampling, feature, loss and optimiser kernels.
 *
 * Conventions: tensors are NHWC, channel counts multiples of 8 (16 bytes),
 * row 0 at the bottom as in gi_shadow.h.  Weights are packed as
 * [cout][kblocks][8] BF16 where K-block kb = tap * (cin / 8) + channel
 * group, taps in row-major (dy, dx) order from (-1, -1); 3x3 kernels with
 * cin % 16 == 0 use the same size in the order the persistent slab kernel
 * loads them: per 16 input channels, the nine taps column-major (dx, then
 * dy), each as [cout / 8][2][8][8].  gi_pack_conv_weights builds the right
 * layout from [cout][cin][kh][kw] FP32.  Every call is
 * stream-ordered; `err` (device uint32, may be NULL) collects kernel error
 * bits (1 = a wait on an mbarrier ran out of its iteration limit).
 */
#ifndef GI_SURROGATE_H
#define GI_SURROGATE_H

#include <stdint.h>

#include "gi_shadow.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef uint16_t gi_bf16;

enum {
    GI_ACT_NONE = 0,
    GI_ACT_RELU = 1
};

/* y[n, y, x, y_off + co] = act(bias[co] + sum_{tap, ci} w[co, tap, ci] *
 * x[n, y + dy, x + dx, ci]) (* (mask[n, y, x, co] > 0) when mask is not
 * NULL).  ksize is 3 or 1; cin, cout multiples of 8 with 16 <= cout <= 256
 * and cout % 16 == 0; y_stride (channels per pixel of y) and y_off
 * multiples of 8.  y32 (FP32, cout channels per pixel, may be NULL) also
 * receives the result before the BF16 rounding. */
gi_status gi_conv2d_bf16(const gi_bf16* x, int n, int h, int w, int cin,
                         const gi_bf16* wt, const float* bias, int cout, int ksize,
                         int act, const gi_bf16* mask, gi_bf16* y, int y_stride,
                         int y_off, float* y32, uint32_t* err, void* stream);

/* 3x3 convolution (cin % 16 == 0) as gi_conv2d_bf16 (no mask, no FP32
 * output) with two optional fusions in its epilogue, both bit-identical to
 * running the separate kernels on the stored output:
 *   - pool (may be NULL): also writes the 2x2 max-pooled result,
 *     pool[n][h / 2][w / 2][cout] (BF16; h and w even, cout <= 128), what
 *     gi_maxpool2_bf16 of the output gives;
 *   - upsample != 0: y is [n][2 h][2 w][y_stride] and receives the output
 *     upsampled 2x (nearest) at channel y_off, what gi_upsample2_bf16 of
 *     the output writes.
 * y may be NULL when pool is not (only the pooled result is stored).  The
 * U-Net's encoder layers feed its pooling this way, and its decoder layers
 * their concatenation buffers, without the intermediate tensors. */
gi_status gi_conv2d_fused_bf16(const gi_bf16* x, int n, int h, int w, int cin,
                               const gi_bf16* wt, const float* bias, int cout, int act,
                               gi_bf16* y, int y_stride, int y_off, gi_bf16* pool,
                               int upsample, uint32_t* err, void* stream);

/* 3x3 convolution (cin % 16 == 0) whose epilogue also applies a 1x1 head
 * with two outputs to the activated, BF16-rounded result and writes only
 * that: head_out[p][j] = head_b[j] + sum_c head_w[j][c] * y[p][c], j < 2
 * (FP32, 2 per pixel); the convolution's own output is not stored. */
gi_status gi_conv2d_head_bf16(const gi_bf16* x, int n, int h, int w, int cin,
                              const gi_bf16* wt, const float* bias, int cout, int act,
                              const float* head_w, const float* head_b, float* head_out,
                              uint32_t* err, void* stream);

/* dW[co, tap, ci] += sum over pixels of dy[p, co] * x[p + tap, ci] and
 * db[co] += sum dy[p, co] (db may be NULL); dw is FP32 in the packed
 * [cout][kblocks][8] layout.  scratch: FP32 workspace of at least
 * gi_conv2d_wgrad_scratch_floats(...) floats. */
size_t gi_conv2d_wgrad_scratch_floats(int n, int h, int w, int cin, int cout, int ksize);
gi_status gi_conv2d_wgrad_bf16(const gi_bf16* x, const gi_bf16* dy, int n, int h, int w,
                               int cin, int cout, int ksize, float* dw, float* db,
                               float* scratch, uint32_t* err, void* stream);

/* Packs FP32 [cout][cin_real][k][k] weights into the BF16 layout above
 * (input channels beyond cin_real are zero).  With flip != 0 it packs the
 * transposed, spatially flipped kernel that the data gradient uses
 * (the packed result has cin and cout exchanged). */
gi_status gi_pack_conv_weights(const float* w, int cout, int cin_real, int cin, int ksize,
                               int flip, gi_bf16* out, void* stream);
/* Packs the FP32 packed-layout gradient buffer back to [cout][cin][k][k]. */
gi_status gi_unpack_conv_grad(const float* dw_packed, int cout, int cin_real, int cin,
                              int ksize, float* out, void* stream);

/* 2x2 max pooling (h, w even) and its backward (routes dy to the argmax). */
gi_status gi_maxpool2_bf16(const gi_bf16* x, int n, int h, int w, int c, gi_bf16* y,
                           void* stream);
gi_status gi_maxpool2_bwd_bf16(const gi_bf16* x, const gi_bf16* y, const gi_bf16* dy, int n,
                               int h, int w, int c, gi_bf16* dx, void* stream);
/* Nearest 2x upsampling of x [n, h, w, c] into channels [y_off, y_off + c)
 * of y [n, 2h, 2w, y_stride], and its backward (sum of the 2x2 block). */
gi_status gi_upsample2_bf16(const gi_bf16* x, int n, int h, int w, int c, gi_bf16* y,
                            int y_stride, int y_off, void* stream);
gi_status gi_upsample2_bwd_bf16(const gi_bf16* dy, int n, int h, int w, int c, int dy_stride,
                                int dy_off, gi_bf16* dx, void* stream);
/* Copies channels [off, off + c) of x [.., stride] into y [.., c] (and back
 * with gi_channel_slice_add: y_slice += x). */
gi_status gi_channel_slice_bf16(const gi_bf16* x, size_t pixels, int stride, int off, int c,
                                gi_bf16* y, void* stream);
gi_status gi_channel_slice_add_bf16(const gi_bf16* x, size_t pixels, int c, gi_bf16* y,
                                    int stride, int off, void* stream);

/* Surrogate frame, step 1 (replaces the light map + G-buffer part of
 * gi_render_frame for GI_TECH_PCSS_POISSON): renders the light map into
 * d_depth and the camera visibility keys into the context, then writes
 * the network input d_feat (BF16 [height][width][16]; channels 0-3 used:
 * hard visibility with the pre-test, clamped (z - map depth) * 64,
 * penumbra estimate in map texels / 8 from four blocker taps, and 1 /
 * 0.5 / 0 for pre-test passed / failed / background). */
gi_status gi_surrogate_features(gi_context* ctx, const gi_scene* scene, const gi_map_params* map,
                                const float light_mvp[16], const float camera_mvp[16],
                                const gi_vis_params* vis, int width, int height, float* d_depth,
                                void* d_feat, void* stream);
/* Surrogate frame, step 3 (after the U-Net wrote d_head, FP32
 * [height][width][head_stride]: channel 0 the visibility, 1 the predicted
 * absolute error): background 0, failed pre-test the intensity, else the clamped
 * prediction, or the exact PCSS value where the predicted error exceeds
 * err_threshold (counted into *d_fallback when not NULL).  Uses the keys
 * that gi_surrogate_features left in ctx. */
gi_status gi_surrogate_finish(gi_context* ctx, const gi_scene* scene, int map_width, int map_height,
                              const float* d_depth, const float camera_mvp[16], const gi_vis_params* vis,
                              int width, int height, const float* d_head, int head_stride,
                              const void* d_feat, float err_threshold, float* d_vis,
                              uint32_t* d_fallback, void* stream);
/* Training loss of the surrogate over `pixels` pixels: L1 of the
 * visibility (channel 0 of head) against target on pixels whose feature 3
 * is 1, plus L1 of the error head (channel 1) against the current
 * |visibility - target|.  Writes dhead (BF16 [pixels][16], gradient of
 * the mean loss, other channels 0) and adds {sum |v - t|, pixel count,
 * sum error-head loss} to sums[0..2] in fixed point: sums[0] and sums[2]
 * in units of 2^-32 (each pixel's term rounded once, terms above 1e6
 * clamped), sums[1] an integer count.  The additions are exact integer
 * ones, so the totals do not depend on the order of the GPU's blocks. */
gi_status gi_surrogate_loss(const float* d_head, const float* d_target, const void* d_feat, size_t pixels,
                            float err_weight, gi_bf16* d_dhead, uint64_t* d_sums, void* stream);

/* Adam step on FP32 master weights p with gradient g (both n floats), then
 * the BF16 copy is refreshed by the caller with gi_pack_conv_weights. */
gi_status gi_adam_f32(float* p, const float* g, float* m, float* v, size_t n, float lr,
                      float beta1, float beta2, float eps, int step, float grad_scale,
                      void* stream);

/* Bounded waits.  Every mbarrier wait of the tcgen05 convolution kernels
 * polls at most `polls` times (default 1,048,576, read at each launch).
 * When a wait runs out, the kernel stops issuing loads and MMAs, skips its
 * tensor-memory reads, waits (bounded) for what it had already issued,
 * frees its tensor memory, sets bit 0 of `err` and returns; the outputs of
 * that call are undefined, the context stays usable. */
gi_status gi_tc_set_wait_limit(uint32_t polls);
uint32_t gi_tc_wait_limit(void);
/* Test switch for the bounded-wait path (process-wide, off by default):
 * while enabled, each convolution kernel withholds its first asynchronous
 * stage (the TMA loads of the slab kernel, the MMAs of the others), so the
 * wait on it runs out with nothing in flight.  Never enable it in
 * production. */
gi_status gi_tc_set_test_withhold(int enable);

#ifdef __cplusplus
}
#endif
#endif /* GI_SURROGATE_H */
