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
};

using gi::fail;
using gi::fail_cuda;

namespace {

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
gi_status dry_run(gi_batch* b) {
    for (size_t i = 0; i < b->frames.size(); ++i) {
        gi_status s = enqueue_frame(b, b->frames[i], (int)(i % b->num_streams));
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
    for (size_t i = 0; i < b->frames.size() && s == GI_OK && e == cudaSuccess; ++i)
        s = enqueue_frame(b, b->frames[i], (int)(i % b->num_streams));
    for (int k = 1; k < b->num_streams && e == cudaSuccess; ++k) {
        e = cudaEventRecord(b->join[k], b->streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(origin, b->join[k], 0);
    }
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
    if (s == GI_OK) s = size_depth(b);
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
    return GI_OK;
}

extern "C" gi_status gi_batch_autotune(gi_batch* b, void* stream, int repeats, gi_batch_tuning* out) {
    if (!b || b->frames.empty()) return fail(GI_ERR_INVALID_ARG, "gi_batch_autotune: empty batch");
    if (repeats < 1) repeats = 1;
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return fail_cuda(e, "gi_batch_autotune: cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    auto time_config = [&](int tiny, int coop, int streams, float* ms) -> gi_status {
        b->tiny_px = tiny;
        b->coop_px = coop;
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
    // tier thresholds first (8 streams), then the stream count
    const int tinies[] = {16, 32, 64, 96, 128};
    const int coops[] = {256, 512, 1024};
    const int stream_counts[] = {4, 8, 16, 32};
    int bt = 96, bc = 1024, bs = 8;
    float best = 1e30f;
    gi_status s = GI_OK;
    for (int t : tinies)
        for (int c : coops) {
            if (c <= t) continue;
            float ms = 0;
            s = time_config(t, c, 8, &ms);
            if (s != GI_OK) break;
            if (ms < best) {
                best = ms;
                bt = t;
                bc = c;
            }
        }
    for (int n : stream_counts) {
        if (s != GI_OK) break;
        float ms = 0;
        s = time_config(bt, bc, n, &ms);
        if (s != GI_OK) break;
        if (ms < best) {
            best = ms;
            bs = n;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (s != GI_OK) return s;
    b->tiny_px = bt;
    b->coop_px = bc;
    s = build(b, bs);
    if (s != GI_OK) return s;
    if (out) {
        gi_batch_info(b, out);
        out->best_ms = best;
    }
    return GI_OK;
}
