/*
 * gi_oracle.h -- CPU oracle for the shadow-visibility path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain scalar C++,
 * the reference's GLSL passes and the OpenGL fixed-function rules they rely
 * on (rasterisation, depth test, polygon offset, clipping, NEAREST texture
 * fetch with CLAMP_TO_BORDER, stencil INCR_WRAP/DECR_WRAP).  It is the
 * checker of the CUDA path: only the tests, the smoke check and the CPU
 * baseline leg of the benchmark may load it.  The product never calls it.
 *
 * Parity status: the reference's passes run only through OpenGL, which is
 * not available here, so these functions are pinned by hand-derived
 * known-answer tests; the matrix helpers of the product are pinned against
 * the reference's vendored glm.  The GL rules are the ones written in the
 * OpenGL 4.x specification; where the spec leaves a choice (sub-pixel
 * precision, fill convention, polygon-offset r), the choice is stated in
 * gi_oracle.cpp.
 *
 * All images are row-major with row 0 at the bottom; matrices column-major.
 */
#ifndef GI_ORACLE_H
#define GI_ORACLE_H

#include <stdint.h>

#include "../include/gi_shadow.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Light-view depth map: clear to 1, rasterise, LESS, bias, clamp. */
void or_shadow_map(const float* points, int nv, const int* indices, int nt,
                   const float mvp[16], int width, int height, int bias_mode,
                   float constant_bias, float offset_factor, float offset_units,
                   float* out_depth, int threads);

/* G-buffer: (object position, 1) and (normal, frontFacing); background
 * (0,0,0,1) in both. */
void or_gbuffer(const float* points, const float* normals, int nv,
                const int* indices, int nt, const float mvp[16], int width,
                int height, float* out_pos, float* out_nrm, int threads);

/* Per-pixel visibility (r channel).  poisson_xy holds the PCSS Poisson
 * tables: poisson_blocker_taps (x, y) pairs for the blocker search followed
 * by poisson_filter_taps pairs for the filter (NULL for other techniques). */
void or_visibility(const gi_vis_params* p, const float* depth, int map_w,
                   int map_h, const float* pos, const float* nrm, float* out,
                   int width, int height, const float* poisson_xy,
                   int threads);

/* Moment soft shadows (SoftShadowMapping): the moment map of p->technique
 * (SAVSM..MSSM) or, with p->summed_area_table, its summed-area table
 * (float4 [S * T]); and level `level` of the hierarchical min-max map
 * (float2 [(S >> level) * (T >> level)]). */
void or_soft_moment_map(const gi_vis_params* p, const float* depth, int S, int T, float* out);
void or_hierarchical_shadow_map(const gi_vis_params* p, const float* depth, int S, int T, int level,
                                float* out);

/* Shadow-volume stencil counts (uint8, wrapping). out_depth may be NULL. */
/* The 6T volume triangles (9 floats each) of ShadowVolume::build. */
void or_shadow_volume_geometry(const float* points, const float* normals, const int* indices, int nt,
                               const float L[3], float infinity, float* out);
void or_shadow_volume_counts(const float* points, const float* normals,
                             int nv, const int* indices, int nt,
                             const float light_pos[3], float infinity,
                             const float mvp[16], int width, int height,
                             int depth_func, uint8_t* out_stencil,
                             float* out_depth, int threads);

/* Deferred Phong shading (PhongShading.frag); out is float4 per pixel. */
void or_phong_shade(const gi_vis_params* p, const float* pos, const float* nrm, const float* vis,
                    const float* color, int W, int H, float* out);

/* Area-light ground truth (renderMonteCarlo + AccurateSoftShadow.frag):
 * mvps / biased are n x 16 light matrices of the sample lights. */
void or_area_light_visibility(const float* points, const float* normals, int nv,
                              const int* indices, int nt, const float* mvps,
                              const float* biased, int n, int S, int bias_mode, float cbias,
                              float factor, float units, const float camera_mvp[16], float I,
                              int W, int H, float* out, int threads);

/* Adaptive (quad-tree) area-light ground truth (SoftShadowMapping
 * adaptiveSampling).  view_mvp(eye, at, mvp, biased, user) gives the light
 * matrices of a sample; returns the number of sample maps n and writes the
 * visibility (out), each map's eye and at (eyes_out, 6 n floats) and level
 * (levels_out, n floats) in the order the final pass sums them. */
typedef void (*or_view_mvp_fn)(const float* eye, const float* at, float* mvp, float* biased, void* user);
int or_area_light_adaptive(const float* points, const float* normals, int nv, const int* indices, int nt,
                           const float light_eye[3], const float light_at[3], float size, int max_level,
                           int lower_accuracy, or_view_mvp_fn view_mvp, void* user, int S, int bias_mode,
                           float cbias, float factor,
                           float units, const float camera_mvp[16], float I, int W, int H, float* out,
                           float* eyes_out, float* levels_out, int threads);

/* PBA exact distance transform (ShadowMapping/src/EDT/pba2DHost.cu:228-242
 * with the kernels of include/EDT/pba2DKernel.h): sites / out are (x, y)
 * int16 pairs per pixel, a site holding anything but x == -32768; out gets
 * the nearest site of each pixel, equidistant sites resolved as the
 * reference's bands (m1, m2, m3) resolve them. */
void or_pba_voronoi(const int16_t* sites, int W, int H, int m1, int m2, int m3, int16_t* out, int threads);

/* EDTSM (ShadowMapping/src/main.cpp:416-422): site detection over the
 * hard-shadow image (float4 shadow, depth, preEvaluatedShadow, 1), PBA, and
 * the normalisation with the position image (float4); out4 channels 0-1.
 * or_edt_sites / or_edt_normalize are its first and last steps. */
void or_edt_sites(const float* image, int W, int H, int16_t* sites);
void or_edt_normalize(const int16_t* nearest, const float* image, const float* position, int W, int H,
                      float penumbra, float intensity, float* out4);
void or_edt_soft_shadows(const float* image, const float* position, int W, int H, int m1, int m2, int m3,
                         float penumbra, float intensity, int16_t* sites, int16_t* nearest, float* out4,
                         int threads);

/* MeanFilter.frag's x and y passes over an EDT image (float4), out float4. */
void or_edt_mean_filter(const gi_vis_params* p, const float* image, const float* pos, int W, int H, int order,
                        float* out);

/* The SMSR shaders' EDTSM outputs from the G-buffer and visibility. */
void or_edt_inputs(const gi_vis_params* p, const float camera_mvp[16], const float* pos, const float* nrm,
                   const float* vis, int W, int H, float* image, float* position);

/* Hit counts of the return sites of the RBSSM smoothONDS restatement,
 * indexed by source line modulo 4096 (test coverage only). */
void or_rbssm_hits(unsigned long long* out4096, int reset);

#ifdef __cplusplus
}
#endif
#endif
