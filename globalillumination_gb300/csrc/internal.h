// Internal declarations shared by the host C++ and the CUDA translation
// units of libgishadow.so.  Nothing here is part of the public C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gi_shadow.h"

namespace gi {

// Records `msg` as the calling thread's last error and returns `st`.
gi_status fail(gi_status st, const std::string& msg);
// Allocation-failure injection (gi_debug_fail_allocation): true when the
// allocation about to be made must fail.  Device allocations return
// GI_ERR_OOM; host ones call alloc_point(), which throws std::bad_alloc,
// and the C ABI turns that into GI_ERR_OOM.
bool alloc_fail_due();
void alloc_point();
gi_status fail_cuda(int cuda_err, const char* what);

struct Mesh {
    std::vector<float> points;   // float[3V]  (Mesh::pointCloud)
    std::vector<float> normals;  // float[3V]  (Mesh::normalVector)
    std::vector<int> indices;    // int[3T], 0-based (Mesh::indices)
    int num_vertices() const { return (int)(points.size() / 3); }
    int num_triangles() const { return (int)(indices.size() / 3); }
};

// Mesh::computeNormals (ShadowMapping/src/Mesh.cpp:195-234).
void compute_normals(Mesh& m);
// Mesh::scale / translate / rotate (Mesh.cpp:378-429).
void mesh_scale(Mesh& m, float x, float y, float z);
void mesh_translate(Mesh& m, float x, float y, float z);
void mesh_rotate(Mesh& m, float x, float y, float z);
// Mesh::addObject (Mesh.cpp:47-193).
void mesh_append(Mesh& dst, const Mesh& src);
// glmReadOBJ + Mesh::loadOBJFile.
gi_status read_obj(const char* path, Mesh& out);

}  // namespace gi

struct gi_scene {
    gi::Mesh mesh;             // committed objects
    gi::Mesh pending;          // the reference's `temp` object
    bool has_pending = false;
    float camera_eye[3] = {0, 0, 0};
    float camera_at[3] = {0, 0, 0};
    float light_eye[3] = {0, 0, 0};
    float light_at[3] = {0, 0, 0};
    float depth_threshold = 0.0f;
    float hsm_alpha = 0.0f;
    float hsm_beta = 0.0f;
    int num_objects = 0;
    // device copy (owned)
    int device = -1;
    float* d_points = nullptr;
    float* d_normals = nullptr;
    int* d_indices = nullptr;
    size_t cap_vertices = 0;
    size_t cap_triangles = 0;
    int dev_vertices = 0;
    int dev_triangles = 0;
    bool upload_failed = false;  // the last upload ran out of memory: no usable device copy
    uint64_t upload_serial = 0;  // bumped by every upload
    // silhouette mode of the shadow volumes: per triangle edge, the
    // neighbouring triangle across it (see gi_shadow_volume_counts_silhouette)
    int* d_adj = nullptr;
    size_t cap_adj = 0;
    uint64_t adj_serial = ~0ull;  // upload_serial the adjacency was built for
};

// Device scratch owned by a context.  Buffers only grow.
namespace gi {
// Everything a gi_render_frame launch sequence depends on besides device
// memory contents: the scene's device copy, the call's arguments, the
// context's raster tuning and tap-pyramid switch, and the buffer epoch.
// Compared bytewise (filled after a memset).
struct FrameSig {
    const void* scene;
    const void* points;
    const void* normals;
    const void* indices;
    int triangles;
    gi_map_params mp;
    float light_mvp[16];
    float camera_mvp[16];
    gi_vis_params vp;
    int W, H;
    const void* depth;
    const void* vis;
    const void* pos;
    const void* nrm;
    int tiny_px, coop_px;
    int tap_pyramid;
    uint64_t epoch;
};
}  // namespace gi

struct gi_context {
    int device = 0;
    uint64_t launches = 0;
    // raster work queue (large-triangle tiles) and triangle setup records
    void* d_tri_records = nullptr;
    size_t cap_tri_records = 0;
    void* d_tile_items = nullptr;
    size_t cap_tile_items = 0;
    // visibility keys (64-bit depth|primitive) for the G-buffer
    unsigned long long* d_vkeys = nullptr;
    size_t cap_vkeys = 0;
    // prepass depth / stencil counters for shadow volumes
    float* d_depth_tmp = nullptr;
    size_t cap_depth_tmp = 0;
    int* d_counts = nullptr;
    size_t cap_counts = 0;
    // binned rasteriser: records, big-record list, big-record bases, spill
    // list, bin counters (small | big | offset | cursor), bin lists, ranks,
    // bin work items
    void* bin_buf[8] = {};
    size_t bin_cap[8] = {};
    // tiered rasteriser: records, tiny / warp / large lists, large bases,
    // spill, G-buffer triangle -> record map, per-record resolve data.
    // Set 0 serves light maps, set 1 the G-buffer keys (the resolve reads
    // set 1 after any number of light maps).
    void* tier_buf[2][8] = {};
    size_t tier_cap[2][8] = {};
    // tier thresholds (bounding-box pixels): tiny <= tiny_px < warp <= coop_px
    int tiny_px = 96;
    int coop_px = 1024;
    // status words (128): [4..11] counters of the binned raster (records,
    // big records, spills, error bits, admitted big pairs as u64, work
    // items), [32..55] counters of the tiered light-map pass, [64..87] of
    // the tiered camera-key pass (the two passes may run concurrently),
    // [96] rows of the PBA row pass colored by the exact group chain,
    // [100] error bits of the min-max pyramid (bit 0: a copy wait ran out),
    // [101] volume triangles kept by the silhouette mode
    unsigned int* d_status = nullptr;
    unsigned int* h_status = nullptr;  // pinned mirror
    // area-light ground truth: a wave of sample light maps, per-pixel sums
    float* d_area_maps = nullptr;
    size_t cap_area_maps = 0;
    float* d_area_acc = nullptr;
    size_t cap_area_acc = 0;
    float* d_area_gbuf = nullptr;  // adaptive sampling: positions, normals, counts, flag
    size_t cap_area_gbuf = 0;
    // moment techniques: the S x S moment map plus its first mip level, and
    // the two W x W blur targets (float4)
    void* d_mom = nullptr;
    size_t cap_mom = 0;
    void* d_mom_blur = nullptr;
    size_t cap_mom_blur = 0;
    void* d_hsm = nullptr;  // min-max shadow map levels (float2)
    size_t cap_hsm = 0;
    // PBA distance transform: phase-1 site row per pixel (int16)
    int16_t* d_pba_cols = nullptr;
    size_t cap_pba_cols = 0;
    // the x pass of the EDT mean filter (float4 per pixel)
    void* d_edt_meanx = nullptr;
    size_t cap_edt_meanx = 0;
    // nearest site per pixel (short2) when the caller does not keep it
    void* d_pba_near = nullptr;
    size_t cap_pba_near = 0;
    // min-max pyramid of the light map (float2 levels 1..6), status word 100;
    // built for PCSS / PCF only when tap_pyramid is set
    void* d_pyr = nullptr;
    size_t cap_pyr = 0;
    bool tap_pyramid = false;
    // silhouette mode of the shadow volumes: the volume triangles to draw
    // (count in status word 101)
    void* d_sil_list = nullptr;
    size_t cap_sil_list = 0;
    // second stream for the camera-key pass of gi_render_frame, and the
    // fork / join events (cudaStream_t / cudaEvent_t)
    void* aux_stream = nullptr;
    void* fork_ev = nullptr;
    void* join_ev = nullptr;
    // phase timing (cudaEvent_t handles) for gi_render_frame
    bool profiling = false;
    void* phase_ev[4] = {};
    // frame graph (gi_context_set_frame_graph): the arguments of the last
    // gi_render_frame call, whether they have run once eagerly, the graph
    // captured from them (cudaGraphExec_t), the kernels it holds, and the
    // stream it was captured on (cudaStream_t)
    bool frame_graph = false;
    gi::FrameSig fg_sig = {};
    bool fg_seen = false;
    void* fg_exec = nullptr;
    uint64_t fg_launches = 0;
    void* fg_stream = nullptr;
};

namespace gi {
// Grows a device buffer to at least `bytes` (cudaMalloc). Returns GI_OK or an error.
gi_status ensure_buffer(void** ptr, size_t* cap, size_t bytes);
// Bumped by every device allocation of ensure_buffer and every free of a
// scene's device copy: a captured frame graph whose epoch differs may hold
// stale pointers and is captured again.
uint64_t buffer_epoch();
void bump_buffer_epoch();
}
