// batch.cpp -- batched frames under one captured CUDA graph.
//
// A batch is a list of frames (scene, camera, 1..n lights with their map
// sizes, visibility parameters, output buffers).  gi_batch_build runs every
// frame once to size each stream's scratch, then captures the whole batch
// into one CUDA graph: the frames are dealt round-robin to `streams` CUDA
// streams forked from the launching stream, so independent frames (small
// scenes, small maps) overlap on the GPU; each stream owns a gi_context
// (scratch) and one light-map buffer it reuses light after light.  Per
// frame: the camera's visibility keys once, then for every light its depth
// map and the fused G-buffer-resolve + visibility kernel writing that
// light's visibility image.  gi_batch_run launches the graph;
// gi_batch_autotune times candidate tier thresholds (tiny / warp-sized
// bounding boxes) and stream counts on the real batch and keeps the
// fastest.  The reference renders one scene and one light per frame
// (ShadowMapping/src/main.cpp:459-472); batching is new.
//
// Persistent mode (gi_batch_build_persistent): the graph rasterises, per
// frame, its G-buffer into the batch's own per-frame buffers and, per
// light, its light map into a per-light-frame buffer (every map of the
// batch stays resident: about 27 GB for the 256-scene workload), over the
// same streams; then one persistent launch of k_batch_visibility shades
// every (light-frame, tile) work item of the batch from a global counter.
// Its tile size is tuned with the tier thresholds and stream count
// (gi_batch_autotune_persistent).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "host_math.h"
#include "internal.h"
#include "raster.h"

struct gi_batch_frame {
    const gi_scene* scene = nullptr;
    gi_view camera{};
    std::vector<gi_view> lights;
    std::vector<gi_map_params> maps;
    gi_vis_params vis{};
    float* d_vis = nullptr;
    // host-side matrices, computed once at add time
    std::vector<gi_frame_matrices> fm;
};

struct gi_batch {
    int device = 0;
    int num_streams = 0;
    std::vector<gi_batch_frame> frames;
    std::vector<gi_context*> ctxs;
    std::vector<cudaStream_t> streams;
    std::vector<float*> depth;
    std::vector<size_t> depth_cap;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int tiny_px = 96;
    int coop_px = 1024;
    uint64_t launches_per_run = 0;
    // persistent mode
    bool persistent = false;
    int tile_w = 64, tile_h = 8;
    std::vector<float*> lf_map;        // one light map per light-frame
    std::vector<size_t> lf_map_cap;
    std::vector<float*> fr_gbuf;       // per frame: position then normal, float4 each
    std::vector<size_t> fr_gbuf_cap;
    gi::BatchLightFrame* d_lf = nullptr;
    size_t cap_lf = 0;
    unsigned* d_queue = nullptr;
    unsigned total_tiles = 0;
    int n_lf = 0;
};

using gi::fail;
using gi::fail_cuda;

namespace {

void release_persistent(gi_batch* b) {
    for (auto* p : b->lf_map) cudaFree(p);
    for (auto* p : b->fr_gbuf) cudaFree(p);
    b->lf_map.clear();
    b->lf_map_cap.clear();
    b->fr_gbuf.clear();
    b->fr_gbuf_cap.clear();
    cudaFree(b->d_lf);
    cudaFree(b->d_queue);
    b->d_lf = nullptr;
    b->d_queue = nullptr;
    b->cap_lf = 0;
}

void release_streams(gi_batch* b) {
    for (auto* c : b->ctxs) gi_context_destroy(c);
    for (auto s : b->streams) cudaStreamDestroy(s);
    for (auto* d : b->depth) cudaFree(d);
    for (auto e : b->join) cudaEventDestroy(e);
    b->ctxs.clear();
    b->streams.clear();
    b->depth.clear();
    b->depth_cap.clear();
    b->join.clear();
}

void release_graph(gi_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Grows the pool of (context, stream, light-map buffer) slots to n and
// applies the tier thresholds; slots are kept across rebuilds so that
// autotuning does not reallocate scratch.
gi_status make_streams(gi_batch* b, int n) {
    for (int i = (int)b->ctxs.size(); i < n; ++i) {
        gi_context* c = nullptr;
        gi_status st = gi_context_create(b->device, &c);
        if (st != GI_OK) return st;
        b->ctxs.push_back(c);
        cudaStream_t s;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return fail_cuda(e, "gi_batch: cudaStreamCreate");
        b->streams.push_back(s);
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail_cuda(e, "gi_batch: cudaEventCreate");
        b->join.push_back(ev);
        b->depth.push_back(nullptr);
        b->depth_cap.push_back(0);
    }
    b->num_streams = n;
    for (int i = 0; i < n; ++i) {
        b->ctxs[i]->tiny_px = b->tiny_px;
        b->ctxs[i]->coop_px = b->coop_px;
    }
    return GI_OK;
}

// Enqueues frame f on stream slot k.
gi_status enqueue_frame(gi_batch* b, const gi_batch_frame& f, int k) {
    gi_context* ctx = b->ctxs[k];
    cudaStream_t st = b->streams[k];
    const int W = f.camera.width, H = f.camera.height;
    gi_status s = gi::raster_gbuffer_keys(ctx, f.scene, f.fm[0].camera_mvp, W, H, st);
    if (s != GI_OK) return s;
    for (size_t l = 0; l < f.lights.size(); ++l) {
        const gi_map_params& mp = f.maps[l];
        const gi_frame_matrices& m = f.fm[l];
        s = gi::raster_depth_map(ctx, f.scene, m.light_mvp, mp.width, mp.height, mp.bias_mode,
                                 mp.constant_bias, mp.offset_factor, mp.offset_units, b->depth[k], 0, st);
        if (s != GI_OK) return s;
        gi_vis_params vp = f.vis;
        std::memcpy(vp.light_mvp_biased, m.light_mvp_biased, sizeof vp.light_mvp_biased);
        std::memcpy(vp.camera_mv, m.camera_mv, sizeof vp.camera_mv);
        std::memcpy(vp.normal_matrix, m.normal_matrix, sizeof vp.normal_matrix);
        std::memcpy(vp.light_position, m.light_position, sizeof vp.light_position);
        s = gi::launch_frame_visibility(ctx, &vp, b->depth[k], mp.width, mp.height, f.scene,
                                        m.camera_mvp, f.d_vis + l * (size_t)W * H, W, H, nullptr,
                                        nullptr, st);
        if (s != GI_OK) return s;
    }
    return GI_OK;
}

// Persistent mode, phase A for frame i on stream slot k: its G-buffer and
// every light's map into the batch's buffers (lf: index of its first
// light-frame).
gi_status enqueue_frame_persistent(gi_batch* b, size_t i, int k, int lf) {
    const gi_batch_frame& f = b->frames[i];
    gi_context* ctx = b->ctxs[k];
    cudaStream_t st = b->streams[k];
    const int W = f.camera.width, H = f.camera.height;
    float* pos = b->fr_gbuf[i];
    float* nrm = pos + 4 * (size_t)W * H;
    gi_status s = gi::raster_gbuffer(ctx, f.scene, f.fm[0].camera_mvp, W, H, pos, nrm, ctx->tiny_px, st);
    if (s != GI_OK) return s;
    for (size_t l = 0; l < f.lights.size(); ++l) {
        const gi_map_params& mp = f.maps[l];
        const gi_frame_matrices& m = f.fm[l];
        s = gi::raster_depth_map(ctx, f.scene, m.light_mvp, mp.width, mp.height, mp.bias_mode, mp.constant_bias,
                                 mp.offset_factor, mp.offset_units, b->lf_map[lf + l], 0, st);
        if (s != GI_OK) return s;
    }
    return GI_OK;
}

// Phase B on the origin stream: reset the work counter, one persistent launch.
gi_status enqueue_visibility_persistent(gi_batch* b, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch: queue reset");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int grid = std::max(1, sms) * 8;
    gi_status s = gi::launch_batch_visibility(b->frames[0].vis.technique, b->d_lf, b->n_lf, b->total_tiles,
                                              b->d_queue, b->tile_w, b->tile_h, grid, st);
    if (s == GI_OK) b->ctxs[0]->launches++;
    return s;
}

// Sizes the per-frame G-buffers and per-light-frame maps and uploads the
// light-frame table for the current tile size.
gi_status prepare_persistent(gi_batch* b) {
    const int tech = b->frames[0].vis.technique;
    for (const auto& f : b->frames)
        if (f.vis.technique != tech)
            return fail(GI_ERR_UNSUPPORTED, "gi_batch_build_persistent: the frames must share one technique");
    if (!gi::batch_visibility_supported(tech))
        return fail(GI_ERR_UNSUPPORTED, "gi_batch_build_persistent: technique not supported (moment maps)");
    size_t n_lf = 0;
    for (const auto& f : b->frames) n_lf += f.lights.size();
    b->lf_map.resize(n_lf, nullptr);
    b->lf_map_cap.resize(n_lf, 0);
    b->fr_gbuf.resize(b->frames.size(), nullptr);
    b->fr_gbuf_cap.resize(b->frames.size(), 0);
    std::vector<gi::BatchLightFrame> table;
    table.reserve(n_lf);
    unsigned tiles = 0;
    size_t j = 0;
    for (size_t i = 0; i < b->frames.size(); ++i) {
        const gi_batch_frame& f = b->frames[i];
        const int W = f.camera.width, H = f.camera.height;
        gi_status s = gi::ensure_buffer(reinterpret_cast<void**>(&b->fr_gbuf[i]), &b->fr_gbuf_cap[i],
                                        8 * sizeof(float) * (size_t)W * H);
        if (s != GI_OK) return s;
        for (size_t l = 0; l < f.lights.size(); ++l, ++j) {
            const gi_map_params& mp = f.maps[l];
            const gi_frame_matrices& m = f.fm[l];
            s = gi::ensure_buffer(reinterpret_cast<void**>(&b->lf_map[j]), &b->lf_map_cap[j],
                                  sizeof(float) * (size_t)mp.width * mp.height);
            if (s != GI_OK) return s;
            gi::BatchLightFrame e{};
            e.p = f.vis;
            std::memcpy(e.p.light_mvp_biased, m.light_mvp_biased, sizeof e.p.light_mvp_biased);
            std::memcpy(e.p.camera_mv, m.camera_mv, sizeof e.p.camera_mv);
            std::memcpy(e.p.normal_matrix, m.normal_matrix, sizeof e.p.normal_matrix);
            std::memcpy(e.p.light_position, m.light_position, sizeof e.p.light_position);
            e.map = b->lf_map[j];
            e.pos = reinterpret_cast<const float4*>(b->fr_gbuf[i]);
            e.nrm = reinterpret_cast<const float4*>(b->fr_gbuf[i] + 4 * (size_t)W * H);
            e.out = f.d_vis + l * (size_t)W * H;
            e.map_w = mp.width;
            e.map_h = mp.height;
            // shadowMapStep = (1.0 / w, 1.0 / h) in double, stored as float
            e.sx = (float)(1.0 / (double)mp.width);
            e.sy = (float)(1.0 / (double)mp.height);
            e.W = W;
            e.H = H;
            e.tiles_x = (W + b->tile_w - 1) / b->tile_w;
            e.tiles_y = (H + b->tile_h - 1) / b->tile_h;
            e.tile_begin = tiles;
            const unsigned long long nt = (unsigned long long)e.tiles_x * e.tiles_y;
            if (tiles + nt >= (1ull << 32) - 1) return fail(GI_ERR_CAPACITY, "gi_batch_build_persistent: too many tiles");
            tiles += (unsigned)nt;
            table.push_back(e);
        }
    }
    gi_status s = gi::ensure_buffer(reinterpret_cast<void**>(&b->d_lf), &b->cap_lf,
                                    std::max<size_t>(table.size(), 1) * sizeof(gi::BatchLightFrame));
    if (s != GI_OK) return s;
    if (!b->d_queue) {
        size_t cap = 0;
        s = gi::ensure_buffer(reinterpret_cast<void**>(&b->d_queue), &cap, sizeof(unsigned));
        if (s != GI_OK) return s;
    }
    cudaError_t e = cudaMemcpy(b->d_lf, table.data(), table.size() * sizeof(gi::BatchLightFrame),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch_build_persistent: light-frame table");
    b->n_lf = (int)table.size();
    b->total_tiles = tiles;
    return GI_OK;
}

gi_status size_depth(gi_batch* b) {
    size_t need = 0;
    for (const auto& f : b->frames)
        for (const auto& mp : f.maps) need = std::max(need, (size_t)mp.width * mp.height * sizeof(float));
    for (int k = 0; k < b->num_streams; ++k) {
        gi_status s = gi::ensure_buffer(reinterpret_cast<void**>(&b->depth[k]), &b->depth_cap[k], need);
        if (s != GI_OK) return s;
    }
    return GI_OK;
}

// Runs every frame once outside capture so each context's scratch reaches
// its working size (capture must not allocate).
gi_status enqueue_all(gi_batch* b) {
    int lf = 0;
    for (size_t i = 0; i < b->frames.size(); ++i) {
        const int k = (int)(i % b->num_streams);
        gi_status s = b->persistent ? enqueue_frame_persistent(b, i, k, lf) : enqueue_frame(b, b->frames[i], k);
        if (s != GI_OK) return s;
        lf += (int)b->frames[i].lights.size();
    }
    return GI_OK;
}

gi_status dry_run(gi_batch* b) {
    gi_status s = enqueue_all(b);
    if (s != GI_OK) return s;
    if (b->persistent) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return fail_cuda(e, "gi_batch dry run");
        s = enqueue_visibility_persistent(b, b->streams[0]);
        if (s != GI_OK) return s;
    }
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_batch dry run");
}

gi_status capture(gi_batch* b) {
    release_graph(b);
    cudaStream_t origin = b->streams[0];
    cudaError_t e = cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch: cudaStreamBeginCapture");
    gi_status s = GI_OK;
    e = cudaEventRecord(b->fork, origin);
    for (int k = 1; k < b->num_streams && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->streams[k], b->fork, 0);
    uint64_t before = 0;
    for (auto* c : b->ctxs) before += c->launches;
    if (e == cudaSuccess) s = enqueue_all(b);
    for (int k = 1; k < b->num_streams && e == cudaSuccess; ++k) {
        e = cudaEventRecord(b->join[k], b->streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(origin, b->join[k], 0);
    }
    if (b->persistent && s == GI_OK && e == cudaSuccess) s = enqueue_visibility_persistent(b, origin);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(origin, &g);
    if (s != GI_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail_cuda(e != cudaSuccess ? e : e2, "gi_batch: stream capture");
    }
    uint64_t after = 0;
    for (auto* c : b->ctxs) after += c->launches;
    b->launches_per_run = after - before;
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_batch: cudaGraphInstantiate");
}

gi_status build(gi_batch* b, int streams) {
    gi_status s = make_streams(b, streams);
    if (s == GI_OK) s = b->persistent ? prepare_persistent(b) : size_depth(b);
    if (s == GI_OK) s = dry_run(b);
    if (s == GI_OK) s = capture(b);
    return s;
}

}  // namespace

extern "C" gi_status gi_batch_create(int device, gi_batch** out) {
    if (!out) return fail(GI_ERR_INVALID_ARG, "gi_batch_create: out is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return fail(GI_ERR_INVALID_ARG, "gi_batch_create: no such CUDA device");
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch_create: cudaSetDevice");
    gi_batch* b = new gi_batch();
    b->device = device;
    e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete b;
        return fail_cuda(e, "gi_batch_create: cudaEventCreate");
    }
    *out = b;
    return GI_OK;
}

extern "C" void gi_batch_destroy(gi_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    release_graph(b);
    release_streams(b);
    release_persistent(b);
    if (b->fork) cudaEventDestroy(b->fork);
    delete b;
}

extern "C" gi_status gi_batch_add_frame(gi_batch* b, const gi_scene* scene, const gi_view* camera,
                                        const gi_view* lights, const gi_map_params* maps,
                                        int num_lights, const gi_vis_params* vis, float* d_vis) {
    if (!b || !scene || !camera || !lights || !maps || !vis || !d_vis || num_lights < 1)
        return fail(GI_ERR_INVALID_ARG, "gi_batch_add_frame: bad arguments");
    if (scene->device != b->device || (scene->dev_triangles == 0 && scene->mesh.num_triangles() > 0))
        return fail(GI_ERR_INVALID_ARG, "gi_batch_add_frame: scene not uploaded to the batch's device");
    gi_batch_frame f;
    f.scene = scene;
    f.camera = *camera;
    f.vis = *vis;
    f.d_vis = d_vis;
    for (int l = 0; l < num_lights; ++l) {
        if (maps[l].width < 1 || maps[l].height < 1 || maps[l].width > 16384 || maps[l].height > 16384)
            return fail(GI_ERR_INVALID_ARG, "gi_batch_add_frame: map size must be in [1, 16384]");
        if (gi::is_moment_technique(vis->technique)) {
            gi_status st = gi::moment_check_shape(maps[l].width, maps[l].height, camera->width, camera->height,
                                                  "gi_batch_add_frame");
            if (st != GI_OK) return st;
        }
        gi_status sst = gi::soft_moment_check_shape(vis->technique, maps[l].width, maps[l].height, "gi_batch_add_frame");
        if (sst != GI_OK) return sst;
        f.lights.push_back(lights[l]);
        f.maps.push_back(maps[l]);
        gi_frame_matrices m;
        gi_status st = gi_frame_setup(&lights[l], camera, &m);
        if (st != GI_OK) return st;
        f.fm.push_back(m);
    }
    if (camera->width > 16384 || camera->height > 16384)
        return fail(GI_ERR_INVALID_ARG, "gi_batch_add_frame: camera size must be in [1, 16384]");
    b->frames.push_back(std::move(f));
    release_graph(b);  // the graph no longer matches
    return GI_OK;
}

extern "C" gi_status gi_batch_build(gi_batch* b, int streams) {
    if (!b || streams < 1 || streams > 64) return fail(GI_ERR_INVALID_ARG, "gi_batch_build: streams in [1, 64]");
    if (b->frames.empty()) return fail(GI_ERR_INVALID_ARG, "gi_batch_build: empty batch");
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch_build: cudaSetDevice");
    b->persistent = false;
    return build(b, streams);
}

static gi_status check_tile(int tile_w, int tile_h) {
    if (tile_w < 32 || tile_w > 1024 || tile_w % 32 != 0 || tile_h < 1 || tile_h > 256 || tile_w * tile_h > 65536)
        return fail(GI_ERR_INVALID_ARG, "gi_batch_build_persistent: tile_w a multiple of 32 in [32, 1024], "
                                        "tile_h in [1, 256], at most 65536 pixels");
    return GI_OK;
}

extern "C" gi_status gi_batch_build_persistent(gi_batch* b, int streams, int tile_w, int tile_h) {
    if (!b || streams < 1 || streams > 64)
        return fail(GI_ERR_INVALID_ARG, "gi_batch_build_persistent: streams in [1, 64]");
    if (b->frames.empty()) return fail(GI_ERR_INVALID_ARG, "gi_batch_build_persistent: empty batch");
    gi_status s = check_tile(tile_w, tile_h);
    if (s != GI_OK) return s;
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch_build_persistent: cudaSetDevice");
    b->persistent = true;
    b->tile_w = tile_w;
    b->tile_h = tile_h;
    return build(b, streams);
}

extern "C" gi_status gi_batch_run(gi_batch* b, void* stream) {
    if (!b || !b->exec) return fail(GI_ERR_INVALID_ARG, "gi_batch_run: batch not built");
    cudaError_t e = cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? GI_OK : fail_cuda(e, "gi_batch_run: cudaGraphLaunch");
}

extern "C" gi_status gi_batch_info(const gi_batch* b, gi_batch_tuning* out) {
    if (!b || !out) return fail(GI_ERR_INVALID_ARG, "gi_batch_info: NULL argument");
    out->tiny_px = b->tiny_px;
    out->coop_px = b->coop_px;
    out->streams = b->num_streams;
    out->frames = (int)b->frames.size();
    out->kernel_launches = b->launches_per_run;
    out->best_ms = 0.0f;
    out->persistent = b->persistent ? 1 : 0;
    out->tile_w = b->persistent ? b->tile_w : 0;
    out->tile_h = b->persistent ? b->tile_h : 0;
    out->work_items = b->persistent ? b->total_tiles : 0;
    return GI_OK;
}

// Times candidate settings on the real batch and keeps the fastest: tier
// thresholds (tiny / warp-sized bounding boxes) at 8 streams, then the
// stream count, and in persistent mode the work-item tile size.
static gi_status autotune(gi_batch* b, void* stream, int repeats, bool persistent, gi_batch_tuning* out) {
    if (!b || b->frames.empty()) return fail(GI_ERR_INVALID_ARG, "gi_batch_autotune: empty batch");
    if (repeats < 1) repeats = 1;
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch_autotune: cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    b->persistent = persistent;
    auto time_config = [&](int tiny, int coop, int streams, int tw, int th, float* ms) -> gi_status {
        b->tiny_px = tiny;
        b->coop_px = coop;
        b->tile_w = tw;
        b->tile_h = th;
        gi_status s = build(b, streams);
        if (s != GI_OK) return s;
        cudaGraphLaunch(b->exec, st);  // warm
        float best = 1e30f;
        for (int r = 0; r < repeats; ++r) {
            cudaEventRecord(t0, st);
            cudaGraphLaunch(b->exec, st);
            cudaEventRecord(t1, st);
            cudaError_t err = cudaEventSynchronize(t1);
            if (err != cudaSuccess) return fail_cuda(err, "gi_batch_autotune: run");
            float t = 0.0f;
            cudaEventElapsedTime(&t, t0, t1);
            best = std::min(best, t);
        }
        *ms = best;
        return GI_OK;
    };
    const int tinies[] = {16, 32, 64, 96, 128};
    const int coops[] = {256, 512, 1024};
    const int stream_counts[] = {4, 8, 16, 32};
    const int tiles[][2] = {{32, 4}, {64, 4}, {64, 8}, {128, 8}, {256, 8}, {128, 16}};
    int bt = 96, bc = 1024, bs = 8, btw = 64, bth = 8;
    float best = 1e30f;
    gi_status s = GI_OK;
    for (int t : tinies)
        for (int c : coops) {
            if (c <= t || s != GI_OK) continue;
            float ms = 0;
            s = time_config(t, c, 8, btw, bth, &ms);
            if (s == GI_OK && ms < best) {
                best = ms;
                bt = t;
                bc = c;
            }
        }
    for (int n : stream_counts) {
        if (s != GI_OK) break;
        float ms = 0;
        s = time_config(bt, bc, n, btw, bth, &ms);
        if (s == GI_OK && ms < best) {
            best = ms;
            bs = n;
        }
    }
    if (persistent)
        for (const auto& tl : tiles) {
            if (s != GI_OK) break;
            float ms = 0;
            s = time_config(bt, bc, bs, tl[0], tl[1], &ms);
            if (s == GI_OK && ms < best) {
                best = ms;
                btw = tl[0];
                bth = tl[1];
            }
        }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (s != GI_OK) return s;
    b->tiny_px = bt;
    b->coop_px = bc;
    b->tile_w = btw;
    b->tile_h = bth;
    s = build(b, bs);
    if (s != GI_OK) return s;
    if (out) {
        gi_batch_info(b, out);
        out->best_ms = best;
    }
    return GI_OK;
}

extern "C" gi_status gi_batch_autotune(gi_batch* b, void* stream, int repeats, gi_batch_tuning* out) {
    return autotune(b, stream, repeats, false, out);
}

extern "C" gi_status gi_batch_autotune_persistent(gi_batch* b, void* stream, int repeats, gi_batch_tuning* out) {
    if (b && !b->frames.empty()) {
        const int tech = b->frames[0].vis.technique;
        for (const auto& f : b->frames)
            if (f.vis.technique != tech)
                return fail(GI_ERR_UNSUPPORTED, "gi_batch_autotune_persistent: the frames must share one technique");
        if (!gi::batch_visibility_supported(tech))
            return fail(GI_ERR_UNSUPPORTED, "gi_batch_autotune_persistent: technique not supported (moment maps)");
    }
    return autotune(b, stream, repeats, true, out);
}
