// Host entry points of the raster and visibility kernels (internal).
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

namespace gi {

gi_status launch_fill_u32(gi_context* ctx, unsigned* p, size_t n, unsigned v, cudaStream_t st);

gi_status raster_depth_map(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W,
                           int H, int bias_mode, float cbias, float factor, float units,
                           float* d_depth, int small_px, cudaStream_t st);

gi_status raster_gbuffer(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W, int H,
                         float* d_pos, float* d_nrm, int small_px, cudaStream_t st);

// The 6T volume triangles of the stencil pass, 9 floats each, into d_out.
gi_status raster_volume_geometry(gi_context* ctx, const gi_scene* scene, const float L[3],
                                 float infinity, float* d_out, cudaStream_t st);
gi_status raster_shadow_volumes(gi_context* ctx, const gi_scene* scene, const float L[3],
                                float infinity, const float mvp[16], int W, int H, int depth_func,
                                unsigned char* d_stencil, float* d_depth_out, int small_px,
                                cudaStream_t st, bool silhouette = false, int* drawn = nullptr);

// G-buffer visibility keys only (into ctx->d_vkeys), no resolve.
gi_status raster_gbuffer_keys(gi_context* ctx, const gi_scene* scene, const float mvp[16], int W,
                              int H, cudaStream_t st);

// Resolve + visibility in one kernel from ctx->d_vkeys; d_pos / d_nrm may
// be NULL (no G-buffer output).
gi_status launch_frame_visibility(gi_context* ctx, const gi_vis_params* p, const float* d_depth,
                                  int map_w, int map_h, const gi_scene* scene, const float camera_mvp[16],
                                  float* d_vis, int W, int H, float* d_pos, float* d_nrm,
                                  cudaStream_t st);

gi_status launch_visibility(gi_context* ctx, const gi_vis_params* p, const float* d_depth,
                            int map_w, int map_h, const float* d_pos, const float* d_nrm,
                            float* d_vis, int W, int H, cudaStream_t st);

// Learned surrogate: per-pixel features (BF16 x 8) from ctx->d_vkeys and the
// light map, and the final visibility from the network head with exact
// PCSS fallback.
gi_status launch_surrogate_features(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int map_w,
                                    int map_h, const gi_scene* scene, const float camera_mvp[16], int W, int H,
                                    void* d_feat, cudaStream_t st);
gi_status launch_surrogate_finish(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int map_w,
                                  int map_h, const gi_scene* scene, const float camera_mvp[16], int W, int H,
                                  const float* d_head, int head_stride, const void* d_feat, float thr,
                                  float* d_vis, unsigned* d_fallback, cudaStream_t st);

// Area-light ground truth: adds the weighted hard tests of `nw` sample maps
// (one wave, maps[k] of map_s^2 texels, biased translation columns
// trans[k], weights weight[k]) to every pixel's running sum; `first` starts
// the sums at 0, and `last` finishes them into d_vis (sum / count).
struct AreaWave {
    float trans[16][4];
    float weight[16];
    float common[12];  // columns 0..2 of the last sample's biased light MVP
    int pcf_n = 0;     // > 0: pcf_n x pcf_n taps per map at pcf_off[] texels
    float pcf_off[8];
    float pcf_incr_w, pcf_incr_h;
};
gi_status launch_area_accumulate(gi_context* ctx, const gi_scene* scene, const float camera_mvp[16], int W, int H,
                                 const float* maps, int map_s, int nw, const AreaWave& wave, float intensity,
                                 bool first, bool last, float count, float* d_vis, cudaStream_t st);

// Adaptive sampling: one quad-tree node's reprojection (per-pixel count of
// its four corner lights that see the pixel, into d_sums) and evaluation
// over a (W / div) x (H / div) grid of the counts (sets *d_passed when a
// count of 1-3 has eight equal neighbours).
struct QuadCorners {
    const float* maps[4];
    float mvp[4][16];  // biased light MVPs, column-major
};
gi_status launch_qt_evaluate(gi_context* ctx, const float* d_pos, int W, int H, int div, const QuadCorners& q,
                             int map_s, unsigned char* d_sums, unsigned* d_passed, cudaStream_t st);

// Deferred Phong shading of the G-buffer with the visibility as shadow
// term (d_color float4 per pixel or NULL for white); d_out float4.
gi_status launch_phong(gi_context* ctx, const gi_vis_params* p, const float* d_pos, const float* d_nrm,
                       const float* d_vis, const float* d_color, float* d_out, int W, int H, cudaStream_t st);

// The SMSR shaders' EDTSM outputs (NonConservativeSMSR.frag:367-397): the
// hard-shadow image (shadow, depth, preEvaluatedShadow, 1) and the clip
// position MVP * vertex, float4 each; background (0, 0, 0, 1).
gi_status launch_edt_inputs(gi_context* ctx, const gi_vis_params* p, const float camera_mvp[16], const float* d_pos,
                            const float* d_nrm, const float* d_vis, float* d_image, float* d_position, int W, int H,
                            cudaStream_t st);

// PBA exact distance transform with PBA's bands (m1, m2, m3).  Sites come
// from d_sites (short2 per pixel, x != MARKER at a site) or, when d_sites is
// NULL, from initializeInput's test on d_image; d_nearest (short2, may be
// NULL) receives each pixel's site, d_out4 (may be NULL) the normalised EDT
// shadow in channels 0-1 (needs d_image and d_position).
gi_status pba_check_shape(int W, int H, int m1, int m2, int m3, const char* who);
gi_status launch_pba(gi_context* ctx, const int16_t* d_sites, const float* d_image, const float* d_position,
                     int W, int H, int m1, int m2, int m3, float penumbra, float intensity, int16_t* d_nearest,
                     float* d_out4, cudaStream_t st);

// MeanFilter.frag's two passes over an EDT image (x into context scratch,
// then y into d_out), float4 images of W x H.
gi_status launch_edt_mean_filter(gi_context* ctx, const float camera_mv[16], const float* d_image,
                                 const float* d_pos, int W, int H, int order, float* d_out, cudaStream_t st);

// Filtered moment maps (GI_TECH_VSM .. GI_TECH_MSM): the moment map of the
// S x S light map, its 2 x 2 box levels down to the W x W window, the
// separable 7-tap blur; *filtered = the blurred map (float4, W x W).
bool is_moment_technique(int t);
gi_status moment_check_shape(int map_w, int map_h, int W, int H, const char* who);
void moment_quantization(float mq[16], float mqi[16], float* tq0);
gi_status launch_moments(gi_context* ctx, int tech, const float* d_depth, int S, int W, cudaStream_t st,
                         const float** filtered);

// Moment soft shadows (GI_TECH_SAVSM .. GI_TECH_MSSM): the maps the lookups
// read, built from the S x T light map.
// One light-frame of a batch for the persistent visibility pass (device
// table entry): the visibility parameters with the light's matrices, the
// light map, the frame's G-buffer and the output image, and the light-
// frame's first tile in the batch's tile numbering.
struct BatchLightFrame {
    gi_vis_params p;
    const float* map;
    const float4* pos;
    const float4* nrm;
    float* out;
    int map_w, map_h;
    float sx, sy;
    int W, H;
    int tiles_x, tiles_y;
    unsigned tile_begin;
    unsigned pad_;
};
bool batch_visibility_supported(int technique);
gi_status launch_batch_visibility(int technique, const BatchLightFrame* d_lf, int n_lf, unsigned total_tiles,
                                  unsigned* d_queue, int tile_w, int tile_h, int grid, cudaStream_t st);

struct SoftMaps {
    const float4* mom = nullptr;     // moment map or its summed-area table, S x T
    const float2* hsm_lo = nullptr;  // VSSM: min-max level floor(lod); level 0 is
                                     // read from the light map (nullptr here)
    const float2* hsm_hi = nullptr;  // level floor(lod) + 1
    int lo_w = 0, lo_h = 0, hi_w = 0, hi_h = 0;
    float hsm_frac = 0.0f;           // lod - floor(lod)
};
bool is_soft_moment_technique(int t);
gi_status soft_moment_check_shape(int tech, int map_w, int map_h, const char* who);
// The moment map (or its SAT when p->summed_area_table) into dst, or into
// ctx scratch when dst is NULL; *out points at the result.
gi_status launch_soft_moment_map(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T,
                                 cudaStream_t st, float4* dst, const float4** out);
// Min-max level `level` (>= 1) into ctx scratch; *out points at it.
gi_status launch_hsm(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T, int level,
                     cudaStream_t st, const float2** out);
// Everything the lookups of p->technique read.
gi_status soft_moment_prepare(gi_context* ctx, const gi_vis_params* p, const float* d_depth, int S, int T,
                              cudaStream_t st, SoftMaps* out);

// Progressive best-candidate Poisson-disk sequence in the unit disk
// (poisson_table.inc); the n-tap table is its first n points.
extern const float kPoissonDisk[64][2];

}  // namespace gi
