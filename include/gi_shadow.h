/*
 * gi_shadow.h -- C ABI of the GB300 shadow-visibility engine.
 *
 * This is the drop-in boundary for the shadow passes of
 * MarcioCerqueira/GlobalIllumination.  The reference has no library API:
 * its passes are free functions called from the GLUT display callback and
 * its outputs are OpenGL textures.  Each entry point below names the
 * reference function (file:line) whose work it replaces.  Paths are relative
 * to the reference project root.
 *
 * Conventions
 *   - Every call returns gi_status; gi_last_error_string() gives the text of
 *     the last failure on the calling thread.
 *   - Device buffers (d_*) are owned by the caller and must be allocated on
 *     the device that the gi_context was created for.  Images are row-major
 *     with row 0 at the BOTTOM (OpenGL window/texture convention): pixel
 *     (x, y) of a W x H image lives at index y * W + x.
 *   - Matrices are 4x4 FP32, column-major (m[col * 4 + row]), as glm and
 *     glUniformMatrix4fv(..., GL_FALSE, ...) use them.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     Every pass is stream-ordered and asynchronous; results are valid once
 *     the stream has been synchronised.
 *   - A gi_context owns the scratch memory of the passes (triangle work
 *     queues, visibility keys, an error word).  Use one context per host
 *     thread / stream.
 */
#ifndef GI_SHADOW_H
#define GI_SHADOW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status                                                              */
/* ------------------------------------------------------------------ */
typedef enum gi_status {
    GI_OK = 0,
    GI_ERR_INVALID_ARG = 1,  /* bad pointer, size or enum value            */
    GI_ERR_IO = 2,           /* a file could not be opened (the reference   */
                             /* calls exit(1): Mesh.cpp:336-340,            */
                             /* OBJLoader.cpp:1315-1319)                    */
    GI_ERR_PARSE = 3,        /* malformed OBJ / config content              */
    GI_ERR_CUDA = 4,         /* a CUDA runtime call failed                  */
    GI_ERR_CAPACITY = 5,     /* a device work queue overflowed              */
    GI_ERR_OOM = 6,          /* host or device allocation failed            */
    GI_ERR_DEVICE = 7,       /* a kernel reported an error in its status    */
    GI_ERR_UNSUPPORTED = 8
} gi_status;

/* Text of the last error raised on this thread ("" if none). */
const char* gi_last_error_string(void);
/* Allocation-failure injection, for testing the error paths (process-wide,
 * off by default).  No counterpart in the reference, which exits on a
 * failed load (Mesh.cpp:336-340).  With countdown n >= 0 the library lets
 * n more allocations succeed (host: mesh and scene arrays; device: scene
 * uploads and context scratch) and fails the next one, which the entry
 * point that made it returns as GI_ERR_OOM, leaving its scene or context
 * as it was; the injection then switches itself off.  -1 switches it off. */
gi_status gi_debug_fail_allocation(int countdown);
/* Library version string. */
const char* gi_version(void);

/* ------------------------------------------------------------------ */
/* Context (scratch memory owner)                                      */
/* ------------------------------------------------------------------ */
typedef struct gi_context gi_context;

/* Creates a context bound to CUDA device `device`.  Scratch buffers grow on
 * demand with cudaMalloc and are released by gi_context_destroy. */
gi_status gi_context_create(int device, gi_context** out);
void gi_context_destroy(gi_context* ctx);
/* Number of kernel launches issued through this context since creation. */
uint64_t gi_context_launch_count(const gi_context* ctx);
/* Phase timing for benchmarks: while enabled, gi_render_frame records CUDA
 * events on its stream around its three phases (light map — the camera
 * visibility keys run concurrently on a second stream —, the wait for the
 * keys after the map, resolve + visibility); gi_context_phase_ms waits for
 * the last call's events and returns the three durations in milliseconds. */
gi_status gi_context_set_profiling(gi_context* ctx, int enable);
/* Rasteriser tier thresholds (bounding-box pixels): triangles up to
 * tiny_px are drawn by one thread, up to coop_px by one warp, larger ones
 * by tiles (defaults 96 / 1024; 1 <= tiny_px < coop_px <= 1024).  Results
 * do not depend on them. */
gi_status gi_context_set_tuning(gi_context* ctx, int tiny_px, int coop_px);
gi_status gi_context_phase_ms(gi_context* ctx, float ms[3]);
/* Exact tap skipping of PCSS (GI_TECH_PCSS_POISSON) and PCF: a pixel whose
 * taps can only reach texels on one side of its depth gets the taps' result
 * without running them.  Boxes of up to 3 x 3 texels are always tested from
 * the map itself; with enable != 0 the visibility pass also builds the
 * light map's min-max pyramid (gi_light_map_minmax) to test larger boxes
 * (one more launch per pass).  Off by default.  Results do not depend on
 * it. */
gi_status gi_context_set_tap_pyramid(gi_context* ctx, int enable);
/* Frame graph of gi_render_frame (no counterpart in the reference, whose
 * frame is a sequence of GL draws): with enable != 0 the context keeps the
 * launch sequence of the last gi_render_frame call as a CUDA graph.  A call
 * whose arguments, scene device copy and context settings all equal the
 * previous call's replays it with one graph launch (the first repeat
 * captures it; a new argument set runs the launches directly once).  Any
 * device buffer (re)allocation by the library, or freeing of a scene's
 * device copy, invalidates it.  The graph reads device memory when it
 * runs, so new scene contents uploaded into the same buffers are used.
 * Results do not depend on it; timing events (gi_context_set_profiling)
 * bypass it, and so does a call on a stream the caller is capturing (the
 * launches themselves go into the caller's graph).  Off by default. */
gi_status gi_context_set_frame_graph(gi_context* ctx, int enable);

/* ------------------------------------------------------------------ */
/* Scene (host geometry + optional device copy)                        */
/* ------------------------------------------------------------------ */
typedef struct gi_scene gi_scene;

typedef struct gi_scene_info {
    int num_vertices;
    int num_triangles;
    float camera_eye[3];     /* config key "ve"                            */
    float camera_at[3];      /* config key "va" (any 2nd char but 'e')     */
    float light_eye[3];      /* config key "le"                            */
    float light_at[3];       /* config key "la"                            */
    float depth_threshold;   /* config key "d" (RBSM, A10-A12)             */
    float hsm_alpha;         /* config key "ha" (soft app only)            */
    float hsm_beta;          /* config key "hb"                            */
    int num_objects;         /* number of "+" commits                      */
} gi_scene_info;

/* Parses a Configs/<name>.txt scene file with the grammar of
 * SceneLoader::load (ShadowMapping/src/IO/SceneLoader.cpp:11-94, soft keys
 * ha/hb SoftShadowMapping/src/IO/SceneLoader.cpp:93-97).  Relative OBJ
 * paths are resolved against `base_dir` (NULL = the current directory),
 * which plays the role of the reference's working directory. */
gi_status gi_scene_load_config(const char* cfg_path, const char* base_dir,
                               gi_scene** out);

/* Creates an empty scene. */
gi_status gi_scene_create(gi_scene** out);
void gi_scene_destroy(gi_scene* scene);

/* Reads one Wavefront OBJ (glmReadOBJ, ShadowMapping/src/IO/OBJLoader.cpp:
 * 1309-1387 + Mesh::loadOBJFile, ShadowMapping/src/Mesh.cpp:251-313) into
 * the scene's pending object and computes its normals
 * (Mesh::computeNormals, Mesh.cpp:195-234). */
gi_status gi_scene_object_load_obj(gi_scene* scene, const char* obj_path);
/* Sets the pending object from host arrays (points float[3V], indices
 * int[3T], 0-based) and computes its normals like Mesh::computeNormals. */
gi_status gi_scene_object_from_arrays(gi_scene* scene, const float* points,
                                      int num_vertices, const int* indices,
                                      int num_triangles);
/* Config keys s / t / r on the pending object (Mesh::scale, translate,
 * rotate, Mesh.cpp:378-429; rotate angles are in degrees, p' = Rx Ry Rz p,
 * normals are rotated, scale/translate leave normals untouched). */
gi_status gi_scene_object_scale(gi_scene* scene, float x, float y, float z);
gi_status gi_scene_object_translate(gi_scene* scene, float x, float y, float z);
gi_status gi_scene_object_rotate(gi_scene* scene, float x, float y, float z);
/* Config key "+": appends the pending object (Mesh::addObject,
 * Mesh.cpp:47-193). */
gi_status gi_scene_object_commit(gi_scene* scene);
/* Sets camera / light eye and at, and the RBSM depth threshold. */
gi_status gi_scene_set_views(gi_scene* scene, const float camera_eye[3],
                             const float camera_at[3], const float light_eye[3],
                             const float light_at[3], float depth_threshold);

gi_status gi_scene_get_info(const gi_scene* scene, gi_scene_info* out);
/* Copies the committed geometry out (any pointer may be NULL). */
gi_status gi_scene_get_arrays(const gi_scene* scene, float* points,
                              float* normals, int* indices);

/* Procedural generators for the synthetic benchmark scenes.  Each one
 * replaces the pending object (call gi_scene_object_commit afterwards). */
/* Axis-aligned quad at height y spanning [-h, h] in x and z, face normal +y. */
gi_status gi_gen_ground(gi_scene* scene, float half_size, float y);
/* UV sphere with `slices` x `stacks` segments and single pole vertices. */
gi_status gi_gen_uv_sphere(gi_scene* scene, int slices, int stacks,
                           float radius, const float centre[3]);
/* Icosphere: icosahedron subdivided `level` times (20 * 4^level tris). */
gi_status gi_gen_icosphere(gi_scene* scene, int level, float radius,
                           const float centre[3]);
/* UV-grid sphere (slices x stacks) whose radius is displaced by seeded
 * FP32 Perlin noise of amplitude `amplitude`. */
gi_status gi_gen_displaced_sphere(gi_scene* scene, int slices, int stacks,
                                  float radius, float amplitude,
                                  const float centre[3], uint64_t seed);
/* Batch of `count` icospheres with PCG32(seed) centres uniform in
 * [lo, hi] per axis and radii uniform in [rmin, rmax], each committed. */
gi_status gi_gen_icosphere_field(gi_scene* scene, int count, int level,
                                 const float lo[3], const float hi[3],
                                 float rmin, float rmax, uint64_t seed);

/* Uploads (or re-uploads) the committed geometry to device memory owned by
 * the scene, on `stream` (the reference re-uploads its VBOs every draw:
 * MyGLGeometryViewer::loadVBOs, MyGLGeometryViewer.cpp:383-405). */
gi_status gi_scene_upload(gi_scene* scene, gi_context* ctx, void* stream);
/* Replaces the scene's device geometry with caller-owned host arrays
 * (points/normals float[3V], indices int[3T]) on `stream`; pinned host
 * memory makes the copies asynchronous.  This is the per-draw VBO upload of
 * MyGLGeometryViewer::loadVBOs (MyGLGeometryViewer.cpp:383-405) without the
 * host mesh; the host copy inside the scene is left unchanged.  Index
 * values are trusted: they must lie in [0, V). */
gi_status gi_scene_upload_from(gi_scene* scene, gi_context* ctx,
                               const float* h_points, const float* h_normals,
                               int num_vertices, const int* h_indices,
                               int num_triangles, void* stream);
/* Device pointers of the uploaded geometry (NULL before upload). */
gi_status gi_scene_device_arrays(const gi_scene* scene, const float** d_points,
                                 const float** d_normals, const int** d_indices);

/* ------------------------------------------------------------------ */
/* Matrices (MyGLGeometryViewer::configureAmbient / configureShadow /   */
/* configurePhong, ShadowMapping/src/Viewers/MyGLGeometryViewer.cpp)    */
/* ------------------------------------------------------------------ */
typedef struct gi_view {
    float eye[3];
    float at[3];
    float up[3];      /* the reference uses (0, 0, 1) for light and camera */
    float fovy_deg;   /* reference: 45                                     */
    float znear;      /* reference: 1                                      */
    float zfar;       /* reference: 1000                                   */
    int width;        /* viewport                                          */
    int height;
} gi_view;

typedef struct gi_frame_matrices {
    float light_mvp[16];        /* P V M of the light (main.cpp:255-266)        */
    float light_mvp_biased[16]; /* bias * light_mvp (MyGLGeometryViewer.cpp:139-145) */
    float camera_mvp[16];       /* P V M of the camera                          */
    float camera_mv[16];        /* V M of the camera                            */
    float normal_matrix[9];     /* inverseTranspose(mat3(camera MV)), col-major */
    float light_position[3];    /* lightEye rotated 180 deg about +y
                                   (ShadowMapping/src/main.cpp:283,309)          */
} gi_frame_matrices;

/* glm::perspective(fovy, w/h, n, f) * glm::lookAt(eye, at, up). */
gi_status gi_view_matrices(const gi_view* view, float proj[16], float view_m[16]);
/* Everything the light-view pass and the per-pixel passes need. */
gi_status gi_frame_setup(const gi_view* light, const gi_view* camera,
                         gi_frame_matrices* out);

/* ------------------------------------------------------------------ */
/* A4: light-view depth map                                            */
/* ------------------------------------------------------------------ */
typedef enum gi_bias_mode {
    GI_BIAS_NONE = 0,
    GI_BIAS_CONSTANT = 1,        /* depth += constant_bias                  */
    GI_BIAS_POLYGON_OFFSET = 2   /* glPolygonOffset(factor, units), float   */
                                 /* depth buffer (main.cpp:246-247)         */
} gi_bias_mode;

typedef struct gi_map_params {
    int width;                   /* reference: 2048 (SM), 1024 (Soft)       */
    int height;
    int bias_mode;               /* gi_bias_mode                            */
    float constant_bias;
    float offset_factor;         /* reference: 4                            */
    float offset_units;          /* reference: 20                           */
} gi_map_params;

/* renderShadowMap + displaySceneFromLightPOV (ShadowMapping/src/main.cpp:
 * 221-274, 350-361; soft copy SoftShadowMapping/src/main.cpp:274-318):
 * clears d_depth (float[width*height]) to 1 and rasterises every triangle
 * of the uploaded scene through `light_mvp` with depth test LESS and no
 * culling.  Window depth = 0.5 z_ndc + 0.5; the bias is applied per
 * fragment and the result clamped to [0, 1]. */
gi_status gi_shadow_map(gi_context* ctx, const gi_scene* scene,
                        const gi_map_params* params, const float light_mvp[16],
                        float* d_depth, void* stream);

/* ------------------------------------------------------------------ */
/* A5: G-buffer                                                        */
/* ------------------------------------------------------------------ */
/* renderGBuffer (ShadowMapping/src/main.cpp:363-372, GBuffer.vert:12-23,
 * GBuffer.frag:32-38): d_pos / d_nrm are float4[width*height].  Covered
 * pixels get (object-space position, 1) and (interpolated vertex normal,
 * gl_FrontFacing); background pixels get (0, 0, 0, 1).  Depth test LESS,
 * first-drawn triangle wins depth ties. */
gi_status gi_gbuffer(gi_context* ctx, const gi_scene* scene,
                     const float camera_mvp[16], int width, int height,
                     float* d_pos, float* d_nrm, void* stream);

/* Allocation-free G-buffer.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory (a real-time frame loop where
 * cudaMalloc's implicit device synchronisation would stall the frame, or an
 * application whose device memory is all owned by its own pool).  Same
 * result as gi_gbuffer, with the geometry passed as caller-owned device
 * arrays and no gi_context: the pass's scratch (per-pixel keys, large-
 * triangle records, counters) lives in one static device array of
 * 9,568,512 bytes that each GPU holds from the library's first use on it
 * (the module load) until the process exits.  Limit: width * height <= 1,048,576 (1024 x 1024); larger
 * images return GI_ERR_CAPACITY.  Runs on the calling thread's current
 * device and CUDA context.  The array's device address is per context and
 * is looked up on every call.  The first call in a context loads the
 * library's module and every kernel of the pass (CUDA loads modules lazily
 * by default), which can itself allocate and synchronise: make that first
 * call a warm-up outside the frame loop and before any stream capture (any
 * triangle count, zero included, loads all of them).  Every call
 * reuses the same array: calls that overlap on the GPU (other streams,
 * other threads) race and must be serialised by the caller.  Allocates
 * nothing (no cudaMalloc / cudaFree). */
gi_status gi_gbuffer_noalloc(const float* d_points, const float* d_normals,
                             int num_vertices, const int* d_indices,
                             int num_triangles, const float camera_mvp[16],
                             int width, int height, float* d_pos, float* d_nrm,
                             void* stream);

/* ------------------------------------------------------------------ */
/* A6-A12, A15: per-pixel visibility                                   */
/* ------------------------------------------------------------------ */
typedef enum gi_technique {
    GI_TECH_HARD = 0,           /* Shadow.frag:253-256 ("naive")            */
    GI_TECH_PCF = 1,            /* Shadow.frag:86-116, bilinearPCF flag     */
    GI_TECH_PCF_TRICUBIC = 2,   /* Shadow.frag:54-116, tricubicPCF flag     */
    GI_TECH_PCSS_GRID = 3,      /* PlausibleSoftShadow.frag:166-194,365-398,556-563 */
    GI_TECH_PCSS_POISSON = 4,   /* PCSS with Poisson-disk taps (no ref counterpart) */
    GI_TECH_SMSR_CONSERVATIVE = 5,    /* RBSM/ConservativeSMSR.frag:128-144   */
    GI_TECH_SMSR_NONCONSERVATIVE = 6, /* RBSM/NonConservativeSMSR.frag:288-304 */
    GI_TECH_RPCF_CONSERVATIVE = 7,    /* ConservativeSMSR.frag:146-198 (RPCF v.1, conservative) */
    GI_TECH_RPCF_SMSR = 8,            /* NonConservativeSMSR.frag:306-350 (RPCF v.1) */
    GI_TECH_RSMSS = 9,                /* FilteredRBSM.frag (RSMSS / RPCF v.2) */
    GI_TECH_HARD_SOFTAPP = 10,        /* SoftShadow HardShadow.frag:35-58     */
    GI_TECH_RBSSM = 11,               /* SoftShadow/RBSSM.frag:1202-1376      */
    /* Filtered moment maps (ShadowMapping/src/main.cpp:220-240, 374-396;
     * Shaders/ShadowMap/{Moments,Exponential,ExponentialMoments}.frag;
     * Shaders/Filter/{Gaussian,LogGaussian}Filter.frag; lookups
     * Shadow.frag:118-220).  The light map becomes a moment map, is blurred
     * by the 7-tap Gaussian (log-space for ESM) into a window-size target
     * and read back bilinearly.  Needs a square window (width == height)
     * and a map side equal to the window side times 2^k (k = 0..4), as the
     * reference's 1024^2 window over its 2048^2 map. */
    GI_TECH_VSM = 12,                 /* Shadow.frag:118-141 (Chebyshev)      */
    GI_TECH_ESM = 13,                 /* Shadow.frag:144-157                  */
    GI_TECH_EVSM = 14,                /* Shadow.frag:160-176                  */
    GI_TECH_MSM = 15,                 /* Shadow.frag:178-220 (Hamburger 4MSM) */
    /* Moment soft shadows of SoftShadowMapping (PlausibleSoftShadow.frag;
     * light pass Shaders/Moments/Moments.frag or Shaders/Exponential.frag;
     * src/main.cpp:274-290, 938-973).  The light map becomes an unblurred
     * moment map at the map's size; with summed_area_table set the lookups
     * read its summed-area table (Shaders/Moments/SAT{Horizontal,Vertical}
     * Pass.frag), else they loop over bilinear taps of the moment map.
     * VSSM first classifies each pixel with the hierarchical min-max map
     * (Shaders/Moments/{PrepareMinMax,MinMax}.frag, main.cpp:696-751) and
     * needs a square power-of-two map of side >= 8. */
    GI_TECH_SAVSM = 16,               /* PlausibleSoftShadow.frag:565-572     */
    GI_TECH_VSSM = 17,                /* PlausibleSoftShadow.frag:574-585     */
    GI_TECH_ESSM = 18,                /* PlausibleSoftShadow.frag:587-594     */
    GI_TECH_MSSM = 19,                /* PlausibleSoftShadow.frag:596-603     */
    GI_TECH_COUNT = 20
} gi_technique;

typedef enum gi_pretest_mode {
    GI_PRETEST_REFERENCE = 0,  /* as the reference: world-space light rotated
                                  180 deg vs eye-space vertex (Shadow.frag:222-238) */
    GI_PRETEST_OFF = 1
} gi_pretest_mode;

/* Mirrors ShadowParams (ShadowMapping/include/Viewers/ShadowParams.h:6-37,
 * SoftShadowMapping/include/Viewers/ShadowParams.h:6-69) plus the uniforms
 * the passes receive. */
typedef struct gi_vis_params {
    int technique;              /* gi_technique                             */
    int pretest;                /* gi_pretest_mode                          */
    float shadow_intensity;     /* reference: 0.25                          */
    int kernel_order;           /* PCF k (reference Gaussian order 7)       */
    int penumbra_size;          /* PCF offset in texels (reference 1)       */
    int max_search;             /* RBSM (reference 16)                      */
    float depth_threshold;      /* RBSM, config key "d"                     */
    int blocker_search_size;    /* PCSS grid B (reference 7)                */
    int kernel_size;            /* PCSS grid K (reference 15)               */
    float light_radius;         /* PCSS lightSourceRadius (float here)      */
    float znear;                /* PCSS zNear uniform (reference 1)         */
    float pcss_min_blocker_depth; /* PlausibleSoftShadow.frag:368 (0.99)    */
    int poisson_blocker_taps;   /* PCSS_POISSON: 16                         */
    int poisson_filter_taps;    /* PCSS_POISSON: 32                         */
    int summed_area_table;      /* SAVSM..MSSM: ShadowParams.SAT (key 's')  */
    float hsm_alpha;            /* VSSM: HSMAlpha, config key "ha"          */
    float hsm_beta;             /* VSSM: HSMBeta, config key "hb"           */
    float light_mvp_biased[16];
    float camera_mv[16];
    float normal_matrix[9];
    float light_position[3];
} gi_vis_params;

/* Fills *p with the reference defaults for `technique`. */
gi_status gi_vis_params_default(int technique, gi_vis_params* p);

/* computeHardShadows / renderSoftShadows (ShadowMapping/src/main.cpp:
 * 400-414, SoftShadowMapping/src/main.cpp:1010-1017): writes the r channel
 * of the visibility target, d_vis float[width*height] (background 0). */
gi_status gi_visibility(gi_context* ctx, const gi_vis_params* params,
                        const float* d_depth, int map_width, int map_height,
                        const float* d_pos, const float* d_nrm,
                        float* d_vis, int width, int height, void* stream);

/* One shadowed frame: display() of the reference up to the visibility
 * target (ShadowMapping/src/main.cpp:459-472 renderShadowMap, renderGBuffer,
 * computeHardShadows; SoftShadowMapping/src/main.cpp:925-1017
 * renderSoftShadows).  Renders the light map into d_depth, then the camera
 * visibility keys, then resolves the G-buffer and shades in one kernel, so
 * the G-buffer is never stored unless d_pos / d_nrm are given (float4
 * [width*height] each, may be NULL).  Results equal gi_shadow_map +
 * gi_gbuffer + gi_visibility. */
gi_status gi_render_frame(gi_context* ctx, const gi_scene* scene,
                          const gi_map_params* map, const float light_mvp[16],
                          const float camera_mvp[16], const gi_vis_params* vis,
                          int width, int height, float* d_depth, float* d_vis,
                          float* d_pos, float* d_nrm, void* stream);

/* Poisson-disk sample table used by GI_TECH_PCSS_POISSON (n <= 64 points in
 * the unit disk, interleaved x,y).  Shared with the CPU oracle. */
gi_status gi_poisson_table(int n, float* xy_out);

/* ---- moment soft shadows: the light-side maps ---------------------------
 * The maps GI_TECH_SAVSM..MSSM sample, as the reference builds them from
 * the light pass (SoftShadowMapping/src/main.cpp:274-290 with
 * Shaders/Moments/Moments.frag or Shaders/Exponential.frag, and the SAT
 * loop at :943-971).  d_out (float4 [map_width * map_height]) receives the
 * moment map of vis->technique, or its summed-area table when
 * vis->summed_area_table is set: log2(map_width) iterations of a horizontal
 * pass t(x, y) = m(x, y) + m(x - 2^i, y) followed by a vertical pass
 * m(x, y) = t(x, y) + t(x, y - 2^i), reads outside the map being 0. */
gi_status gi_soft_moment_map(gi_context* ctx, const gi_vis_params* vis, const float* d_depth, int map_width,
                             int map_height, float* d_out, void* stream);

/* renderHSM (SoftShadowMapping/src/main.cpp:696-751): level `level` of the
 * hierarchical min-max shadow map, float2 (min, max) per texel of the
 * (map_width >> level) x (map_height >> level) level.  Level 0 is
 * (depth == 0 ? 1 : depth) + vis->hsm_alpha, depth + vis->hsm_beta
 * (PrepareMinMax.frag); level k takes min / max over the four bilinear
 * reads of level k - 1 at the texel's diagonal neighbours (MinMax.frag).
 * Needs a square power-of-two map, 1 <= level < log2(map_width) (level 0:
 * 0 <= level). */
gi_status gi_hierarchical_shadow_map(gi_context* ctx, const gi_vis_params* vis, const float* d_depth,
                                     int map_width, int map_height, int level, float* d_out, void* stream);

/* ---- EDT-filtered hard shadows (ShadowMapping's EDTSM mode) -------------
 *
 * filterHardShadowsUsingEDT (ShadowMapping/src/main.cpp:416-447) runs the
 * reference's only CUDA code: an exact Euclidean distance transform by the
 * parallel banding algorithm (PBA; src/EDT/pba2DHost.cu, include/EDT/
 * pba2DKernel.h) over sites found in the hard-shadow image, then a
 * normalisation that turns each pixel's distance to its nearest site into a
 * penumbra value.  The reference reaches its images through CUDA-GL interop;
 * here they are plain device buffers.  Results equal the reference's kernels
 * bit for bit for the same bands, equidistant sites included. */

/* MARKER of pba2D.h:60: the x (and y) of a pixel that is not a site. */
#define GI_PBA_MARKER (-32768)

/* pba2DInitializeInput(short*) + pba2DCompute(m1, m2, m3)
 * (pba2DHost.cu:97-101, 208-221; pba2DVoronoiDiagram(16, 16, 16) in the
 * reference): d_sites holds int16 (x, y) per pixel, a site being any pixel
 * whose x is not GI_PBA_MARKER; d_nearest receives the (x, y) of every
 * pixel's nearest site (all (-1, 0) when there is none, as the reference's
 * kernels produce).  width: a multiple of 8 up to 8192; height 2..8192;
 * phase1_band divides height into bands of >= 2 rows; phase2_band is a power
 * of two dividing width into bands of >= 2; phase3_band divides width. */
gi_status gi_pba_voronoi(gi_context* ctx, const int16_t* d_sites, int width, int height, int phase1_band,
                         int phase2_band, int phase3_band, int16_t* d_nearest, void* stream);

/* The CUDA half of filterHardShadowsUsingEDT (main.cpp:419-422):
 * initializeInput over d_image (float4 per pixel: shadow, depth,
 * preEvaluatedShadow, 1 -- the HARD_SHADOW_COLOR texture), the PBA, and
 * pbaNormalizeEDT(out, penumbra_size, shadow_intensity) with d_position
 * (float4 per pixel, the POSITION_MAP_COLOR texture).  Channels 0 (the
 * filtered shadow) and 1 (depth) of d_out (float4 per pixel) are written,
 * channels 2-3 are left as they are.  The reference passes
 * shadowParams.penumbraSize / 5.0 as penumbra_size.  d_nearest (int16 pairs,
 * may be NULL) receives the nearest sites. */
gi_status gi_edt_soft_shadows(gi_context* ctx, const float* d_image, const float* d_position, int width,
                              int height, int phase1_band, int phase2_band, int phase3_band, float penumbra_size,
                              float shadow_intensity, float* d_out, int16_t* d_nearest, void* stream);

/* Rows (summed over calls since the last reset) whose site list was not a
 * strict lower envelope -- the FP32 bisector tests of the reference kept an
 * entry that is nowhere strictly nearest -- and were therefore colored by
 * replaying the reference's chain of group states; every other row is
 * colored by a binary search that gives the same sites.  Synchronises the
 * context's device. */
gi_status gi_pba_chain_rows(gi_context* ctx, uint32_t* rows, int reset);

/* The screen-space mean filter that ends filterHardShadowsUsingEDT
 * (main.cpp:424-447, Shaders/Filter/MeanFilter.frag): an x pass and a y pass
 * over d_image (the EDT output: filtered shadow in channel 0, depth in
 * channel 1), each averaging a depth-aware window whose half-width is
 * dscreen * order * 50 / (2 deye) for the pixel's eye depth (vis->camera_mv
 * and the G-buffer d_pos); d_out (float4, may not alias d_image) receives
 * (mean, depth, 0, 0), background (0, 0, 0, 1).  order is the Gaussian
 * filter order (7 in the reference).  The first pass reads GL_NEAREST, the
 * second bilinearly at level 0. */
gi_status gi_edt_mean_filter(gi_context* ctx, const gi_vis_params* vis, const float* d_image,
                             const float* d_pos, int width, int height, int order, float* d_out,
                             void* stream);

/* The images gi_edt_soft_shadows reads, as the SMSR shaders write them in
 * EDTSM mode (NonConservativeSMSR.frag:367-397, ConservativeSMSR.frag:
 * 215-245) from the G-buffer (d_pos, d_nrm float4) and the visibility of
 * GI_TECH_SMSR_CONSERVATIVE / GI_TECH_SMSR_NONCONSERVATIVE (d_vis):
 * d_image = (shadow, depth, preEvaluatedShadow, 1) and d_position = MVP *
 * vertex with MVP = camera_mvp; background (0, 0, 0, 1) in both. */
gi_status gi_edt_inputs(gi_context* ctx, const gi_vis_params* vis, const float camera_mvp[16],
                        const float* d_pos, const float* d_nrm, const float* d_vis, int width, int height,
                        float* d_image, float* d_position, void* stream);

/* shadeScene / PhongShading.frag (ShadowMapping/src/main.cpp:449-457,
 * Shaders/GBuffer/PhongShading.frag:11-46): deferred Phong shading of the
 * G-buffer (float4 position / normal per pixel) with d_vis as the shadow
 * term: shadow * color * (diffuse 0.5 max(N.L, 0) + (shadow - intensity)
 * 0.25 max(R.E, 0)^3 + ambient 0.4), eye-space light from vis
 * (camera_mv, normal_matrix, light_position, shadow_intensity).  d_color
 * is float4 per pixel (NULL = white); d_out float4 per pixel; background
 * pixels get the clear colour (0.63, 0.82, 0.96, 1). */
gi_status gi_phong_shade(gi_context* ctx, const gi_vis_params* vis, const float* d_pos,
                         const float* d_nrm, const float* d_vis, const float* d_color,
                         int width, int height, float* d_out, void* stream);

/* ------------------------------------------------------------------ */
/* Area-light ground truth (Monte-Carlo over point-light samples)       */
/* ------------------------------------------------------------------ */
/* UniformSampledLightSource::computeUniformSampling
 * (SoftShadowMapping/src/Scene/LightSource/UniformSampledLightSource.cpp:
 * 27-38): the n_side x n_side point lights of an area light of side
 * `size` (the reference: 17 x 17 = 289, size 16).  Sample i shifts eye and
 * at by ((i % n_side - c) / c * size / 2, ((int)(i / n_side) - c) / c *
 * size / 2, 0), c = (n_side - 1) / 2 — in world x and y, as the reference
 * does.  out receives n_side^2 views (the light's other fields copied). */
gi_status gi_area_light_samples(const gi_view* light, float size, int n_side, gi_view* out);

/* renderMonteCarlo (SoftShadowMapping/src/main.cpp:756-811) with
 * AccurateSoftShadow.frag:52-133 (uniform sampling): one light map per
 * sample view (map parameters as gi_shadow_map; square maps), then per
 * camera pixel the average over samples of the hard test (1 or
 * shadow_intensity), using columns 0-2 of the last sample's biased light
 * MVP and each sample's own translation column, as the shader's uniforms
 * do.  No pre-test (it is commented out in the shader); background 0.
 * d_vis is float[width*height].  Maps are rendered in waves into context
 * scratch (at most 1 GiB). */
gi_status gi_area_light_visibility(gi_context* ctx, const gi_scene* scene,
                                   const gi_view* samples, int num_samples,
                                   const gi_map_params* map, const float camera_mvp[16],
                                   float shadow_intensity, int width, int height,
                                   float* d_vis, void* stream);

/* Adaptive area-light ground truth (SoftShadowMapping's adaptiveSampling,
 * main.cpp:440-690 and 820-870, QuadTreeLightSource.cpp, Shaders/QuadTree/
 * Reprojection.frag and Evaluation.frag, the adaptive branch of
 * AccurateSoftShadow.frag:52-133).  A quad tree over the light (side
 * `size`, corner samples on a 17 x 17 grid) is refined depth first up to
 * `max_level` (the reference's 4): a node renders the light maps of its
 * four corners (a grid position is rendered once, by the first node that
 * reaches it), counts per camera pixel how many corners see it, and
 * subdivides if a pixel with a count of 1-3 has eight equal neighbours.
 * The leaves' corners are then rendered if missing and each map takes the
 * level of the last leaf using it; the visibility is the 1 / (2^level + 1)^2
 * weighted average of the maps' hard tests (1 or shadow_intensity), the
 * level carried in the w of each biased translation as the reference's
 * uniforms carry it.  No pre-test; background 0.  d_vis is
 * float[width*height]; samples_out (at most 289 views), levels_out (289
 * floats) and num_samples may be NULL.  Square maps up to 4096^2.
 * lower_accuracy != 0 is the reference's adaptiveSamplingLowerAccuracy
 * (main.cpp:551-555, AccurateSoftShadow.frag:98-116): the evaluation reads
 * the counts on a (width / 4) x (height / 4) grid (each coarse pixel at its
 * centre texel) and the final pass averages 4 x 4 taps per map at offsets
 * -1, -1/3, 1/3, 1 texels (the shader's float loop). */
gi_status gi_area_light_adaptive(gi_context* ctx, const gi_scene* scene, const gi_view* light, float size,
                                 int max_level, int lower_accuracy, const gi_map_params* map,
                                 const float camera_mvp[16],
                                 float shadow_intensity, int width, int height, float* d_vis,
                                 gi_view* samples_out, float* levels_out, int* num_samples, void* stream);

/* Min-max pyramid of a light map.  No counterpart in the reference: with
 * gi_context_set_tap_pyramid the PCSS and PCF passes build it after the
 * light map and skip a pixel's blocker taps when no texel they can reach is
 * below the receiver, and its filter taps when all of those texels lie on
 * one side of it, which gives the same float result as running the taps.
 * This entry point builds it alone: d_levels receives levels 1..6 one after the
 * other, level L as float2(min, max) of every 2^L x 2^L texel block over
 * (width >> L) x (height >> L) cells, row-major (width * height / 3 float2
 * in all, rounded down per level).  width and height must be multiples of
 * 64 and d_map 16-byte aligned (the visibility pass runs every tap for
 * maps that are not). */
gi_status gi_light_map_minmax(gi_context* ctx, const float* d_map, int width, int height,
                              float* d_levels, void* stream);

/* ------------------------------------------------------------------ */
/* A13/A14: shadow volumes with stencil counts                         */
/* ------------------------------------------------------------------ */
typedef enum gi_depth_func {
    GI_DEPTH_LESS = 0,    /* first frame                                    */
    GI_DEPTH_LEQUAL = 1   /* every later frame (ShadowVolumes/src/main.cpp:174) */
} gi_depth_func;

/* One frame of ShadowVolumes display() (ShadowVolumes/src/main.cpp:120-206)
 * up to the stencil buffer: depth prepass of the scene through
 * `camera_mvp`, then the extruded volume of every triangle
 * (ShadowVolume::update, ShadowVolume.cpp:116-194, far vertices
 * (v - L) * infinity) with depth writes off, front faces INCR_WRAP, back
 * faces DECR_WRAP on depth pass.  d_stencil is uint8[width*height]; a pixel
 * is lit iff its count is 0.  d_depth (float[width*height], may be NULL)
 * receives the prepass depth. */
gi_status gi_shadow_volume_counts(gi_context* ctx, const gi_scene* scene,
                                  const float light_pos[3], float infinity,
                                  const float camera_mvp[16], int width,
                                  int height, int depth_func,
                                  uint8_t* d_stencil, float* d_depth,
                                  void* stream);

/* The same frame with silhouette extraction (opt-in; no counterpart in the
 * reference, which extrudes every triangle).  Each edge shared by two
 * triangles gets two coplanar volume quads over the same four points; when
 * their orientations are opposite (the triangles pick the same winding
 * pattern and run the edge in opposite directions, or the other way round)
 * they cancel, and both are left out: only the silhouette quads -- boundary
 * and non-manifold edges, and shared edges whose quads do not cancel -- are
 * rasterised, found one thread per edge and compacted per warp with a
 * ballot.  The counts equal gi_shadow_volume_counts' except at pixels where
 * a cancelling pair's two triangulations (different diagonals, different
 * near-plane clips) round the fragment depth or coverage differently, which
 * happens along the receivers' contact with the occluders; tests and the
 * benchmark count those pixels against the exact path.  The first call
 * after a scene upload builds the edge adjacency on the host (cached), and
 * every call reads the number of silhouette triangles back (a stream
 * synchronisation).  *volume_triangles (may be NULL) receives the number of
 * volume triangles drawn (6T for the exact path). */
gi_status gi_shadow_volume_counts_silhouette(gi_context* ctx, const gi_scene* scene,
                                             const float light_pos[3], float infinity,
                                             const float camera_mvp[16], int width,
                                             int height, int depth_func,
                                             uint8_t* d_stencil, float* d_depth,
                                             int* volume_triangles, void* stream);

/* ShadowVolume::build / update (ShadowVolumes/src/ShadowVolume.cpp:15-194,
 * infinity 100 at ShadowVolumes/src/main.cpp:469-470) for callers that draw
 * the volumes themselves: the 6T volume triangles exactly as
 * gi_shadow_volume_counts rasterises them, resolved through the reference's
 * index buffer.  d_triangles is float[6T * 9]: entry 6t + k is side triangle
 * k of scene triangle t as three object-space vertices (x, y, z), the near
 * vertices copied, the far ones (v - L) * infinity, wound by the sign of
 * dot((n0 + n1 + n2) / 3, light_pos). */
gi_status gi_shadow_volume_geometry(gi_context* ctx, const gi_scene* scene,
                                    const float light_pos[3], float infinity,
                                    float* d_triangles, void* stream);

/* ------------------------------------------------------------------ */
/* Batched frames under one CUDA graph                                 */
/* ------------------------------------------------------------------ */
/* The reference renders one scene from one light per display() call
 * (ShadowMapping/src/main.cpp:459-472).  A gi_batch holds many frames
 * (scene, camera, one or more lights) and replays them as one captured CUDA
 * graph over several streams; per frame the camera's visibility keys are
 * rasterised once and shared by all of its lights.  Each light's result
 * equals gi_render_frame for that light. */
typedef struct gi_batch gi_batch;

typedef struct gi_batch_tuning {
    int tiny_px;              /* bounding-box pixels drawn by one thread    */
    int coop_px;              /* bounding-box pixels drawn by one warp      */
    int streams;              /* streams the frames are dealt over          */
    int frames;
    uint64_t kernel_launches; /* kernel nodes in one gi_batch_run           */
    float best_ms;            /* autotune: time of the chosen setting       */
    int persistent;           /* 1: built by gi_batch_build_persistent      */
    int tile_w, tile_h;       /* persistent: pixels per work item           */
    uint32_t work_items;      /* persistent: (light-frame, tile) items      */
} gi_batch_tuning;

gi_status gi_batch_create(int device, gi_batch** out);
void gi_batch_destroy(gi_batch* batch);
/* Adds a frame: `lights`, `maps` have num_lights entries; the camera view
 * gives the image size.  d_vis is float[num_lights * width * height]: light
 * l's visibility image at offset l * width * height.  Scenes must stay
 * uploaded and unchanged while the batch exists.  Invalidates the graph. */
gi_status gi_batch_add_frame(gi_batch* batch, const gi_scene* scene,
                             const gi_view* camera, const gi_view* lights,
                             const gi_map_params* maps, int num_lights,
                             const gi_vis_params* vis, float* d_vis);
/* Sizes the scratch by running every frame once (synchronising the device),
 * then captures the batch over `streams` streams (1..64). */
gi_status gi_batch_build(gi_batch* batch, int streams);
/* Launches the captured graph on `stream`. */
gi_status gi_batch_run(gi_batch* batch, void* stream);
/* Persistent mode.  The graph rasterises every frame's G-buffer and every
 * light's map into buffers the batch owns (all of them stay resident),
 * then ONE persistent kernel shades every (light-frame, tile_w x tile_h
 * tile) work item of the batch, taken from a device counter.  The frames
 * must share one technique, and not a moment technique.  Results equal
 * gi_batch_build's (and gi_render_frame's) bit for bit. */
gi_status gi_batch_build_persistent(gi_batch* batch, int streams, int tile_w, int tile_h);
/* gi_batch_autotune for the persistent mode: also picks the tile size. */
gi_status gi_batch_autotune_persistent(gi_batch* batch, void* stream, int repeats, gi_batch_tuning* out);
/* Times tier thresholds and stream counts on this batch (each candidate
 * rebuilt and replayed `repeats` times on `stream`), keeps the fastest
 * and rebuilds with it.  *out (may be NULL) receives the choice. */
gi_status gi_batch_autotune(gi_batch* batch, void* stream, int repeats,
                            gi_batch_tuning* out);
gi_status gi_batch_info(const gi_batch* batch, gi_batch_tuning* out);

#ifdef __cplusplus
}
#endif
#endif /* GI_SHADOW_H */
