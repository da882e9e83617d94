// capi.cpp -- the C ABI of libgishadow.so: error reporting, contexts,
// device copies of scenes, frame matrices and the pass entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <atomic>
#include <cstring>
#include <vector>
#include <string>

#include "host_math.h"
#include "internal.h"
#include "../../include/gi_surrogate.h"
#include "raster.h"

namespace {
thread_local std::string g_last_error;

const int kMaxImage = 16384;  // guard-band fixed point stays in int32 below this

gi_status check_device(gi_context* ctx) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return gi::fail_cuda(e, "cudaGetDevice");
    if (cur != ctx->device) {
        e = cudaSetDevice(ctx->device);
        if (e != cudaSuccess) return gi::fail_cuda(e, "cudaSetDevice");
    }
    return GI_OK;
}
}  // namespace

namespace gi {

gi_status fail(gi_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

gi_status fail_cuda(int err, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString((cudaError_t)err);
    return GI_ERR_CUDA;
}

namespace {
// countdown of allocation points until an injected failure (-1: off)
std::atomic<long long> g_alloc_countdown{-1};
}  // namespace

bool alloc_fail_due() {
    long long c = g_alloc_countdown.load();
    while (c >= 0) {
        if (g_alloc_countdown.compare_exchange_weak(c, c - 1)) return c == 0;
    }
    return false;
}

void alloc_point() {
    if (alloc_fail_due()) throw std::bad_alloc();
}

namespace {
std::atomic<uint64_t> g_buffer_epoch{0};
}
uint64_t buffer_epoch() { return g_buffer_epoch.load(std::memory_order_acquire); }
void bump_buffer_epoch() { g_buffer_epoch.fetch_add(1, std::memory_order_acq_rel); }

gi_status ensure_buffer(void** ptr, size_t* cap, size_t bytes) {
    if (*cap >= bytes && *ptr) return GI_OK;
    bump_buffer_epoch();
    if (alloc_fail_due())
        return fail(GI_ERR_OOM, std::string("cudaMalloc of ") + std::to_string(bytes) +
                                    " bytes failed (injected allocation failure)");
    if (*ptr) {
        cudaFree(*ptr);
        *ptr = nullptr;
        *cap = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GI_ERR_OOM, std::string("cudaMalloc of ") + std::to_string(bytes) +
                                    " bytes failed: " + cudaGetErrorString(e));
    }
    *ptr = p;
    *cap = bytes;
    return GI_OK;
}

}  // namespace gi

using gi::fail;

extern "C" const char* gi_last_error_string(void) { return g_last_error.c_str(); }

extern "C" const char* gi_version(void) { return "gi_shadow 0.1.0 (sm_103a)"; }

extern "C" gi_status gi_context_create(int device, gi_context** out) {
    if (!out) return fail(GI_ERR_INVALID_ARG, "gi_context_create: out is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(GI_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    if (device < 0 || device >= n) return fail(GI_ERR_INVALID_ARG, "gi_context_create: bad device");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return gi::fail_cuda(e, "cudaSetDevice");
    gi_context* c = new gi_context();
    c->device = device;
    e = cudaMalloc(&c->d_status, 128 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, 128 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_status, 128 * sizeof(unsigned));
    cudaStream_t aux = nullptr;
    cudaEvent_t fev = nullptr, jev = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking);
    c->aux_stream = aux;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fev, cudaEventDisableTiming);
    c->fork_ev = fev;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&jev, cudaEventDisableTiming);
    c->join_ev = jev;
    if (e != cudaSuccess) {
        gi_context_destroy(c);
        return gi::fail_cuda(e, "gi_context_create allocation");
    }
    std::memset(c->h_status, 0, 128 * sizeof(unsigned));
    *out = c;
    return GI_OK;
}

extern "C" void gi_context_destroy(gi_context* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    cudaFree(c->d_tri_records);
    cudaFree(c->d_tile_items);
    cudaFree(c->d_vkeys);
    cudaFree(c->d_depth_tmp);
    cudaFree(c->d_counts);
    cudaFree(c->d_area_maps);
    cudaFree(c->d_area_acc);
    cudaFree(c->d_pba_cols);
    cudaFree(c->d_mom);
    cudaFree(c->d_mom_blur);
    cudaFree(c->d_hsm);
    cudaFree(c->d_area_gbuf);
    cudaFree(c->d_pba_near);
    cudaFree(c->d_edt_meanx);
    cudaFree(c->d_pyr);
    cudaFree(c->d_sil_list);
    for (int i = 0; i < 8; ++i) cudaFree(c->bin_buf[i]);
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 8; ++i) cudaFree(c->tier_buf[k][i]);
    for (int i = 0; i < 4; ++i)
        if (c->phase_ev[i]) cudaEventDestroy(static_cast<cudaEvent_t>(c->phase_ev[i]));
    if (c->fg_exec) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(c->fg_exec));
    if (c->fg_stream) cudaStreamDestroy(static_cast<cudaStream_t>(c->fg_stream));
    if (c->aux_stream) cudaStreamDestroy(static_cast<cudaStream_t>(c->aux_stream));
    if (c->fork_ev) cudaEventDestroy(static_cast<cudaEvent_t>(c->fork_ev));
    if (c->join_ev) cudaEventDestroy(static_cast<cudaEvent_t>(c->join_ev));
    cudaFree(c->d_status);
    if (c->h_status) cudaFreeHost(c->h_status);
    delete c;
}

extern "C" uint64_t gi_context_launch_count(const gi_context* c) { return c ? c->launches : 0; }

extern "C" gi_status gi_context_set_tap_pyramid(gi_context* c, int enable) {
    if (!c) return fail(GI_ERR_INVALID_ARG, "gi_context_set_tap_pyramid: NULL context");
    c->tap_pyramid = enable != 0;
    return GI_OK;
}

extern "C" gi_status gi_context_set_frame_graph(gi_context* c, int enable) {
    if (!c) return fail(GI_ERR_INVALID_ARG, "gi_context_set_frame_graph: NULL context");
    c->frame_graph = enable != 0;
    if (!c->frame_graph && c->fg_exec) {
        cudaSetDevice(c->device);
        cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(c->fg_exec));
        c->fg_exec = nullptr;
    }
    c->fg_seen = false;
    return GI_OK;
}

extern "C" gi_status gi_context_set_tuning(gi_context* c, int tiny_px, int coop_px) {
    if (!c) return fail(GI_ERR_INVALID_ARG, "gi_context_set_tuning: NULL context");
    if (tiny_px < 1 || coop_px <= tiny_px || coop_px > 1024)
        return fail(GI_ERR_INVALID_ARG, "gi_context_set_tuning: need 1 <= tiny_px < coop_px <= 1024");
    c->tiny_px = tiny_px;
    c->coop_px = coop_px;
    return GI_OK;
}

extern "C" gi_status gi_context_set_profiling(gi_context* c, int enable) {
    if (!c) return fail(GI_ERR_INVALID_ARG, "gi_context_set_profiling: NULL context");
    if (enable && !c->phase_ev[0]) {
        gi_status st = check_device(c);
        if (st != GI_OK) return st;
        for (int i = 0; i < 4; ++i) {
            cudaEvent_t ev;
            cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return gi::fail_cuda(e, "cudaEventCreate");
            c->phase_ev[i] = ev;
        }
    }
    c->profiling = enable != 0;
    return GI_OK;
}

extern "C" gi_status gi_context_phase_ms(gi_context* c, float ms[3]) {
    if (!c || !ms) return fail(GI_ERR_INVALID_ARG, "gi_context_phase_ms: NULL argument");
    if (!c->phase_ev[0]) return fail(GI_ERR_INVALID_ARG, "gi_context_phase_ms: profiling never enabled");
    cudaError_t e = cudaEventSynchronize(static_cast<cudaEvent_t>(c->phase_ev[3]));
    for (int i = 0; i < 3 && e == cudaSuccess; ++i)
        e = cudaEventElapsedTime(&ms[i], static_cast<cudaEvent_t>(c->phase_ev[i]),
                                 static_cast<cudaEvent_t>(c->phase_ev[i + 1]));
    return e == cudaSuccess ? GI_OK : gi::fail_cuda(e, "gi_context_phase_ms");
}

extern "C" void gi_scene_destroy(gi_scene* s) {
    if (!s) return;
    if (s->device >= 0) {
        cudaSetDevice(s->device);
        gi::bump_buffer_epoch();
        cudaFree(s->d_points);
        cudaFree(s->d_normals);
        cudaFree(s->d_indices);
        cudaFree(s->d_adj);
    }
    delete s;
}

// A failed upload leaves no usable device copy: free what is left and mark
// the scene, so that passes refuse it until it is uploaded again.
static gi_status drop_device_copy(gi_scene* s, gi_status st) {
    gi::bump_buffer_epoch();
    cudaFree(s->d_points);
    cudaFree(s->d_normals);
    cudaFree(s->d_indices);
    s->d_points = s->d_normals = nullptr;
    s->d_indices = nullptr;
    s->cap_vertices = s->cap_triangles = 0;
    s->dev_vertices = s->dev_triangles = 0;
    s->upload_failed = true;
    return st;
}

extern "C" gi_status gi_scene_upload(gi_scene* s, gi_context* ctx, void* stream) {
    if (!s || !ctx) return fail(GI_ERR_INVALID_ARG, "gi_scene_upload: NULL argument");
    gi_status st = check_device(ctx);
    if (st != GI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    const size_t nv = (size_t)s->mesh.num_vertices(), nt = (size_t)s->mesh.num_triangles();
    if (s->device >= 0 && s->device != ctx->device) {
        cudaFree(s->d_points);
        cudaFree(s->d_normals);
        cudaFree(s->d_indices);
        cudaFree(s->d_adj);
        s->d_points = s->d_normals = nullptr;
        s->d_indices = nullptr;
        s->d_adj = nullptr;
        s->cap_vertices = s->cap_triangles = 0;
        s->cap_adj = 0;
        s->adj_serial = ~0ull;
    }
    s->device = ctx->device;
    size_t capv = s->cap_vertices * 3 * sizeof(float), capn = capv;
    size_t capi = s->cap_triangles * 3 * sizeof(int);
    st = gi::ensure_buffer(reinterpret_cast<void**>(&s->d_points), &capv, nv * 3 * sizeof(float));
    if (st == GI_OK)
        st = gi::ensure_buffer(reinterpret_cast<void**>(&s->d_normals), &capn, nv * 3 * sizeof(float));
    if (st == GI_OK)
        st = gi::ensure_buffer(reinterpret_cast<void**>(&s->d_indices), &capi, nt * 3 * sizeof(int));
    if (st != GI_OK) return drop_device_copy(s, st);
    s->cap_vertices = capv / (3 * sizeof(float));
    s->cap_triangles = capi / (3 * sizeof(int));
    cudaError_t e = cudaSuccess;
    if (nv) {
        e = cudaMemcpyAsync(s->d_points, s->mesh.points.data(), nv * 3 * sizeof(float),
                            cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d_normals, s->mesh.normals.data(), nv * 3 * sizeof(float),
                                cudaMemcpyHostToDevice, cs);
    }
    if (e == cudaSuccess && nt)
        e = cudaMemcpyAsync(s->d_indices, s->mesh.indices.data(), nt * 3 * sizeof(int),
                            cudaMemcpyHostToDevice, cs);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_scene_upload copy");
    s->dev_vertices = (int)nv;
    s->dev_triangles = (int)nt;
    s->upload_failed = false;
    s->upload_serial++;
    return GI_OK;
}

extern "C" gi_status gi_scene_upload_from(gi_scene* s, gi_context* ctx, const float* hp,
                                          const float* hn, int nv, const int* hi, int nt,
                                          void* stream) {
    if (!s || !ctx || nv < 0 || nt < 0 || (nv > 0 && (!hp || !hn)) || (nt > 0 && !hi))
        return fail(GI_ERR_INVALID_ARG, "gi_scene_upload_from: bad arguments");
    if ((size_t)nt >= ((size_t)1 << 29)) return fail(GI_ERR_CAPACITY, "more than 2^29 triangles");
    gi_status st = check_device(ctx);
    if (st != GI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (s->device >= 0 && s->device != ctx->device) {
        cudaFree(s->d_points);
        cudaFree(s->d_normals);
        cudaFree(s->d_indices);
        cudaFree(s->d_adj);
        s->d_points = s->d_normals = nullptr;
        s->d_indices = nullptr;
        s->d_adj = nullptr;
        s->cap_vertices = s->cap_triangles = 0;
        s->cap_adj = 0;
        s->adj_serial = ~0ull;
    }
    s->device = ctx->device;
    size_t capv = s->cap_vertices * 3 * sizeof(float), capn = capv;
    size_t capi = s->cap_triangles * 3 * sizeof(int);
    const size_t vb = (size_t)nv * 3 * sizeof(float), ib = (size_t)nt * 3 * sizeof(int);
    if (capv < vb || capi < ib) {
        // growing frees the old buffers: let queued work that reads them finish
        cudaError_t e = cudaStreamSynchronize(cs);
        if (e != cudaSuccess) return gi::fail_cuda(e, "gi_scene_upload_from sync");
    }
    st = gi::ensure_buffer(reinterpret_cast<void**>(&s->d_points), &capv, vb);
    if (st == GI_OK) st = gi::ensure_buffer(reinterpret_cast<void**>(&s->d_normals), &capn, vb);
    if (st == GI_OK) st = gi::ensure_buffer(reinterpret_cast<void**>(&s->d_indices), &capi, ib);
    if (st != GI_OK) return drop_device_copy(s, st);
    s->cap_vertices = capv / (3 * sizeof(float));
    s->cap_triangles = capi / (3 * sizeof(int));
    cudaError_t e = cudaSuccess;
    if (vb) e = cudaMemcpyAsync(s->d_points, hp, vb, cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && vb) e = cudaMemcpyAsync(s->d_normals, hn, vb, cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && ib) e = cudaMemcpyAsync(s->d_indices, hi, ib, cudaMemcpyHostToDevice, cs);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_scene_upload_from copy");
    s->dev_vertices = nv;
    s->dev_triangles = nt;
    s->upload_failed = false;
    s->upload_serial++;
    return GI_OK;
}

extern "C" gi_status gi_scene_device_arrays(const gi_scene* s, const float** p, const float** n,
                                            const int** i) {
    if (!s) return fail(GI_ERR_INVALID_ARG, "gi_scene_device_arrays: NULL scene");
    if (p) *p = s->d_points;
    if (n) *n = s->d_normals;
    if (i) *i = s->d_indices;
    return GI_OK;
}

// ---------------------------------------------------------------------------
// Matrices
// ---------------------------------------------------------------------------
static gi_status check_view(const gi_view* v) {
    if (!v) return fail(GI_ERR_INVALID_ARG, "gi_view is NULL");
    if (v->width <= 0 || v->height <= 0)
        return fail(GI_ERR_INVALID_ARG, "gi_view: width/height must be positive");
    if (!(v->znear > 0.0f) || !(v->zfar > v->znear))
        return fail(GI_ERR_INVALID_ARG, "gi_view: need 0 < znear < zfar");
    if (!(v->fovy_deg > 0.0f && v->fovy_deg < 180.0f))
        return fail(GI_ERR_INVALID_ARG, "gi_view: fovy must be in (0, 180)");
    return GI_OK;
}

// MyGLGeometryViewer::configureAmbient (MyGLGeometryViewer.cpp:14-26):
// perspective(fov, (GLfloat)w / h, zNear, zFar) and lookAt(eye, look, up).
static void view_mats(const gi_view* v, gi::M4& P, gi::M4& V) {
    float aspect = (float)v->width / (float)v->height;
    P = gi::perspective(v->fovy_deg, aspect, v->znear, v->zfar);
    V = gi::look_at(gi::v3(v->eye[0], v->eye[1], v->eye[2]), gi::v3(v->at[0], v->at[1], v->at[2]),
                    gi::v3(v->up[0], v->up[1], v->up[2]));
}

extern "C" gi_status gi_view_matrices(const gi_view* v, float proj[16], float view_m[16]) {
    gi_status st = check_view(v);
    if (st != GI_OK) return st;
    gi::M4 P, V;
    view_mats(v, P, V);
    if (proj) gi::store4(P, proj);
    if (view_m) gi::store4(V, view_m);
    return GI_OK;
}

extern "C" gi_status gi_frame_setup(const gi_view* light, const gi_view* camera,
                                    gi_frame_matrices* out) {
    gi_status st = check_view(light);
    if (st == GI_OK) st = check_view(camera);
    if (st != GI_OK) return st;
    if (!out) return fail(GI_ERR_INVALID_ARG, "gi_frame_setup: out is NULL");
    // The model matrix of every pass: identity * translate(0) * rotate(0, x)
    // * rotate(0, y) * rotate(0, z) (ShadowMapping/src/main.cpp:255-260).
    gi::M4 model = gi::identity4();
    model = gi::translate(model, gi::v3(0.0f, 0.0f, 0.0f));
    model = gi::rotate(model, 0.0f, gi::v3(1, 0, 0));
    model = gi::rotate(model, 0.0f, gi::v3(0, 1, 0));
    model = gi::rotate(model, 0.0f, gi::v3(0, 0, 1));
    gi::M4 LP, LV, CP, CV;
    view_mats(light, LP, LV);
    view_mats(camera, CP, CV);
    // lightMVP = projection * view * model (main.cpp:264).
    gi::M4 light_mvp = gi::mul(gi::mul(LP, LV), model);
    // bias matrix (MyGLGeometryViewer.cpp:139-145), lightMVP = bias * lightMVP.
    gi::M4 bias;
    std::memset(&bias, 0, sizeof(bias));
    bias.m[0][0] = 0.5f;
    bias.m[1][1] = 0.5f;
    bias.m[2][2] = 0.5f;
    bias.m[3][0] = 0.5f;
    bias.m[3][1] = 0.5f;
    bias.m[3][2] = 0.5f;
    bias.m[3][3] = 1.0f;
    gi::M4 biased = gi::mul(bias, light_mvp);
    // configurePhong (MyGLGeometryViewer.cpp:108-134): mvp, mv, and the
    // normal matrix latched on the first camera-view call.
    gi::M4 cam_mvp = gi::mul(gi::mul(CP, CV), model);
    gi::M4 cam_mv = gi::mul(CV, model);
    gi::M3 nm = gi::inverse_transpose3(gi::upper3(cam_mv));
    // lightEye = mat3(rotate(180, (0, 1, 0))) * lightEye (main.cpp:283, 309).
    gi::M3 r180 = gi::upper3(gi::rotate(gi::identity4(), 180.0f, gi::v3(0, 1, 0)));
    gi::V3 lp = gi::mul3(r180, gi::v3(light->eye[0], light->eye[1], light->eye[2]));
    gi::store4(light_mvp, out->light_mvp);
    gi::store4(biased, out->light_mvp_biased);
    gi::store4(cam_mvp, out->camera_mvp);
    gi::store4(cam_mv, out->camera_mv);
    gi::store3(nm, out->normal_matrix);
    out->light_position[0] = lp.x;
    out->light_position[1] = lp.y;
    out->light_position[2] = lp.z;
    return GI_OK;
}

// ---------------------------------------------------------------------------
// Passes
// ---------------------------------------------------------------------------
static gi_status check_pass(gi_context* ctx, const gi_scene* s) {
    if (!ctx) return fail(GI_ERR_INVALID_ARG, "context is NULL");
    if (!s) return fail(GI_ERR_INVALID_ARG, "scene is NULL");
    if (s->upload_failed) return fail(GI_ERR_INVALID_ARG, "the scene's last upload failed: upload it again");
    if (s->dev_triangles > 0 && (s->device != ctx->device || !s->d_points))
        return fail(GI_ERR_INVALID_ARG, "scene is not uploaded to the context's device");
    if (s->dev_triangles == 0 && s->mesh.num_triangles() > 0)
        return fail(GI_ERR_INVALID_ARG, "scene has not been uploaded (gi_scene_upload)");
    return check_device(ctx);
}

static gi_status check_image(int w, int h, const char* who) {
    if (w <= 0 || h <= 0 || w > kMaxImage || h > kMaxImage)
        return fail(GI_ERR_INVALID_ARG, std::string(who) + ": image size must be in [1, 16384]");
    return GI_OK;
}

static int small_px_default() { return 128; }

extern "C" gi_status gi_shadow_map(gi_context* ctx, const gi_scene* s, const gi_map_params* mp,
                                   const float light_mvp[16], float* d_depth, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!mp || !light_mvp || !d_depth) return fail(GI_ERR_INVALID_ARG, "gi_shadow_map: NULL argument");
    st = check_image(mp->width, mp->height, "gi_shadow_map");
    if (st != GI_OK) return st;
    if (mp->bias_mode < GI_BIAS_NONE || mp->bias_mode > GI_BIAS_POLYGON_OFFSET)
        return fail(GI_ERR_INVALID_ARG, "gi_shadow_map: bad bias_mode");
    return gi::raster_depth_map(ctx, s, light_mvp, mp->width, mp->height, mp->bias_mode,
                                mp->constant_bias, mp->offset_factor, mp->offset_units, d_depth,
                                small_px_default(), static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_gbuffer(gi_context* ctx, const gi_scene* s, const float camera_mvp[16],
                                int W, int H, float* d_pos, float* d_nrm, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!camera_mvp || !d_pos || !d_nrm) return fail(GI_ERR_INVALID_ARG, "gi_gbuffer: NULL argument");
    st = check_image(W, H, "gi_gbuffer");
    if (st != GI_OK) return st;
    if ((size_t)s->dev_triangles >= ((size_t)1 << 29))
        return fail(GI_ERR_CAPACITY, "gi_gbuffer: more than 2^29 triangles");
    return gi::raster_gbuffer(ctx, s, camera_mvp, W, H, d_pos, d_nrm, small_px_default(),
                              static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_vis_params_default(int technique, gi_vis_params* p) {
    if (!p) return fail(GI_ERR_INVALID_ARG, "gi_vis_params_default: NULL");
    if (technique < 0 || technique >= GI_TECH_COUNT)
        return fail(GI_ERR_INVALID_ARG, "gi_vis_params_default: unknown technique");
    std::memset(p, 0, sizeof(*p));
    p->technique = technique;
    p->pretest = GI_PRETEST_REFERENCE;
    p->shadow_intensity = 0.25f;          // ShadowMapping/src/main.cpp:877
    p->kernel_order = 7;                  // gaussianFilter->buildGaussianKernel(7), main.cpp:859
    p->penumbra_size = 1;                 // main.cpp:871
    p->max_search = 16;                   // main.cpp:872
    p->depth_threshold = 0.0f;            // Configs key "d"
    p->blocker_search_size = 7;           // SoftShadowMapping/src/main.cpp:1612
    p->kernel_size = 15;                  // SoftShadowMapping/src/main.cpp:1613
    p->light_radius = 8.0f;               // lightSource->getSize()/2 with size 16 (:1614)
    p->znear = 1.0f;                      // MyGLGeometryViewer.cpp:7
    p->pcss_min_blocker_depth = 0.99f;    // PlausibleSoftShadow.frag:368
    p->poisson_blocker_taps = 16;
    p->poisson_filter_taps = 32;
    if (technique == GI_TECH_RBSSM) p->kernel_size = 7;  // SoftShadowMapping/src/main.cpp:1450-1455
    // SAVSM .. MSSM: resetShadowParameters sets kernelSize 7 (main.cpp:1341,
    // 1433-1449); SAT starts off (:1606) and HSMAlpha / HSMBeta come from
    // the config keys "ha" / "hb" (default 0, SceneLoader.cpp:8-9)
    if (technique >= GI_TECH_SAVSM && technique <= GI_TECH_MSSM) p->kernel_size = 7;
    for (int i = 0; i < 4; ++i) {
        p->light_mvp_biased[i * 5] = 1.0f;
        p->camera_mv[i * 5] = 1.0f;
    }
    for (int i = 0; i < 3; ++i) p->normal_matrix[i * 4] = 1.0f;
    return GI_OK;
}

static gi_status check_vis_params(const gi_vis_params* p) {
    if (p->technique < 0 || p->technique >= GI_TECH_COUNT)
        return fail(GI_ERR_INVALID_ARG, "gi_visibility: unknown technique");
    if (p->pretest != GI_PRETEST_REFERENCE && p->pretest != GI_PRETEST_OFF)
        return fail(GI_ERR_INVALID_ARG, "gi_visibility: bad pretest mode");
    const int t = p->technique;
    const bool pcf_loop = t == GI_TECH_PCF || t == GI_TECH_PCF_TRICUBIC || t == GI_TECH_RPCF_SMSR ||
                          t == GI_TECH_RPCF_CONSERVATIVE || t == GI_TECH_RSMSS;
    if (pcf_loop) {
        // The reference's FP32 loops run about (2 * penumbra / step + 1)^2
        // taps; bound them so a kernel cannot spin for long.
        if (p->kernel_order < 1 || p->kernel_order > 64 || p->penumbra_size < 1 ||
            p->penumbra_size > 64)
            return fail(GI_ERR_INVALID_ARG,
                        "gi_visibility: kernel_order and penumbra_size must be in [1, 64]");
    }
    if ((t >= GI_TECH_SMSR_CONSERVATIVE && t <= GI_TECH_RSMSS) || t == GI_TECH_RBSSM) {
        if (p->max_search < 0 || p->max_search > 4096)
            return fail(GI_ERR_INVALID_ARG, "gi_visibility: max_search must be in [0, 4096]");
    }
    const bool soft_moment = gi::is_soft_moment_technique(t);
    if (t == GI_TECH_PCSS_GRID || t == GI_TECH_PCSS_POISSON || t == GI_TECH_RBSSM || soft_moment) {
        if (p->kernel_size < 1 || p->kernel_size > 63)
            return fail(GI_ERR_INVALID_ARG, "gi_visibility: kernel_size must be in [1, 63]");
    }
    if ((t == GI_TECH_PCSS_GRID || t == GI_TECH_RBSSM || soft_moment) &&
        (p->blocker_search_size < 1 || p->blocker_search_size > 63))
        return fail(GI_ERR_INVALID_ARG, "gi_visibility: blocker_search_size must be in [1, 63]");
    if (t == GI_TECH_PCSS_POISSON &&
        (p->poisson_blocker_taps < 1 || p->poisson_blocker_taps > 64 ||
         p->poisson_filter_taps < 1 || p->poisson_filter_taps > 64))
        return fail(GI_ERR_INVALID_ARG, "gi_visibility: Poisson tap counts must be in [1, 64]");
    return GI_OK;
}

extern "C" gi_status gi_visibility(gi_context* ctx, const gi_vis_params* p, const float* d_depth,
                                   int map_w, int map_h, const float* d_pos, const float* d_nrm,
                                   float* d_vis, int W, int H, void* stream) {
    if (!ctx || !p || !d_depth || !d_pos || !d_nrm || !d_vis)
        return fail(GI_ERR_INVALID_ARG, "gi_visibility: NULL argument");
    gi_status st = check_image(map_w, map_h, "gi_visibility (map)");
    if (st == GI_OK) st = check_image(W, H, "gi_visibility");
    if (st == GI_OK) st = check_vis_params(p);
    if (st == GI_OK && gi::is_moment_technique(p->technique))
        st = gi::moment_check_shape(map_w, map_h, W, H, "gi_visibility");
    if (st == GI_OK) st = gi::soft_moment_check_shape(p->technique, map_w, map_h, "gi_visibility");
    if (st == GI_OK) st = check_device(ctx);
    if (st != GI_OK) return st;
    return gi::launch_visibility(ctx, p, d_depth, map_w, map_h, d_pos, d_nrm, d_vis, W, H,
                                 static_cast<cudaStream_t>(stream));
}

// The launch sequence of one frame on stream cs: the camera-key pass on the
// context's second stream, concurrently with the light map, then the fused
// resolve + visibility kernel once both are done.
static gi_status enqueue_frame(gi_context* ctx, const gi_scene* s, const gi_map_params* mp,
                               const float light_mvp[16], const float camera_mvp[16], const gi_vis_params* vp,
                               int W, int H, float* d_depth, float* d_vis, float* d_pos, float* d_nrm,
                               cudaStream_t cs) {
    cudaStream_t aux = static_cast<cudaStream_t>(ctx->aux_stream);
    auto mark = [&](int i) {
        if (ctx->profiling) cudaEventRecord(static_cast<cudaEvent_t>(ctx->phase_ev[i]), cs);
    };
    mark(0);
    cudaError_t e = cudaEventRecord(static_cast<cudaEvent_t>(ctx->fork_ev), cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, static_cast<cudaEvent_t>(ctx->fork_ev), 0);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_render_frame: fork");
    gi_status st = gi::raster_gbuffer_keys(ctx, s, camera_mvp, W, H, aux);
    e = cudaEventRecord(static_cast<cudaEvent_t>(ctx->join_ev), aux);
    if (st == GI_OK)
        st = gi::raster_depth_map(ctx, s, light_mvp, mp->width, mp->height, mp->bias_mode,
                                  mp->constant_bias, mp->offset_factor, mp->offset_units, d_depth,
                                  small_px_default(), cs);
    mark(1);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, static_cast<cudaEvent_t>(ctx->join_ev), 0);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_render_frame: join");
    mark(2);
    if (st == GI_OK)
        st = gi::launch_frame_visibility(ctx, vp, d_depth, mp->width, mp->height, s, camera_mvp, d_vis,
                                         W, H, d_pos, d_nrm, cs);
    mark(3);
    return st;
}

extern "C" gi_status gi_render_frame(gi_context* ctx, const gi_scene* s, const gi_map_params* mp,
                                     const float light_mvp[16], const float camera_mvp[16],
                                     const gi_vis_params* vp, int W, int H, float* d_depth,
                                     float* d_vis, float* d_pos, float* d_nrm, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!mp || !light_mvp || !camera_mvp || !vp || !d_depth || !d_vis || (!d_pos != !d_nrm))
        return fail(GI_ERR_INVALID_ARG, "gi_render_frame: bad arguments");
    st = check_image(mp->width, mp->height, "gi_render_frame (map)");
    if (st == GI_OK) st = check_image(W, H, "gi_render_frame");
    if (st == GI_OK) st = check_vis_params(vp);
    if (st == GI_OK && gi::is_moment_technique(vp->technique))
        st = gi::moment_check_shape(mp->width, mp->height, W, H, "gi_render_frame");
    if (st == GI_OK) st = gi::soft_moment_check_shape(vp->technique, mp->width, mp->height, "gi_render_frame");
    if (st != GI_OK) return st;
    if (mp->bias_mode < GI_BIAS_NONE || mp->bias_mode > GI_BIAS_POLYGON_OFFSET)
        return fail(GI_ERR_INVALID_ARG, "gi_render_frame: bad bias_mode");
    if ((size_t)s->dev_triangles >= ((size_t)1 << 29))
        return fail(GI_ERR_CAPACITY, "gi_render_frame: more than 2^29 triangles");
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // A caller that captures its own stream gets the launches themselves in
    // its graph: the frame graph is neither replayed nor captured inside it.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (ctx->frame_graph && cudaStreamIsCapturing(cs, &capture) != cudaSuccess) {
        cudaGetLastError();
        capture = cudaStreamCaptureStatusNone;
    }
    if (!ctx->frame_graph || ctx->profiling || capture != cudaStreamCaptureStatusNone)
        return enqueue_frame(ctx, s, mp, light_mvp, camera_mvp, vp, W, H, d_depth, d_vis, d_pos, d_nrm, cs);
    // Frame graph: a new argument signature runs eagerly once (allocating
    // what the frame needs); the next call with the same signature captures
    // the launch sequence into a graph on the context's capture stream;
    // later ones replay it with one launch.
    gi::FrameSig sig;
    std::memset(&sig, 0, sizeof(sig));
    sig.scene = s;
    sig.points = s->d_points;
    sig.normals = s->d_normals;
    sig.indices = s->d_indices;
    sig.triangles = s->dev_triangles;
    sig.mp = *mp;
    std::memcpy(sig.light_mvp, light_mvp, sizeof(sig.light_mvp));
    std::memcpy(sig.camera_mvp, camera_mvp, sizeof(sig.camera_mvp));
    sig.vp = *vp;
    sig.W = W;
    sig.H = H;
    sig.depth = d_depth;
    sig.vis = d_vis;
    sig.pos = d_pos;
    sig.nrm = d_nrm;
    sig.tiny_px = ctx->tiny_px;
    sig.coop_px = ctx->coop_px;
    sig.tap_pyramid = ctx->tap_pyramid ? 1 : 0;
    sig.epoch = gi::buffer_epoch();
    const bool same = ctx->fg_seen && std::memcmp(&sig, &ctx->fg_sig, sizeof(sig)) == 0;
    if (same && ctx->fg_exec) {
        cudaError_t e = cudaGraphLaunch(static_cast<cudaGraphExec_t>(ctx->fg_exec), cs);
        if (e != cudaSuccess) return gi::fail_cuda(e, "gi_render_frame: graph launch");
        ctx->launches += ctx->fg_launches;
        return GI_OK;
    }
    if (!same) {
        ctx->fg_seen = false;
        st = enqueue_frame(ctx, s, mp, light_mvp, camera_mvp, vp, W, H, d_depth, d_vis, d_pos, d_nrm, cs);
        if (st != GI_OK) return st;
        ctx->fg_sig = sig;
        ctx->fg_sig.epoch = gi::buffer_epoch();  // what this run allocated belongs to the frame
        ctx->fg_seen = true;
        if (ctx->fg_exec) {  // the graph of an older signature is of no further use
            cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(ctx->fg_exec));
            ctx->fg_exec = nullptr;
        }
        return GI_OK;
    }
    cudaError_t e = cudaSuccess;
    if (!ctx->fg_stream) {
        cudaStream_t fs = nullptr;
        e = cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking);
        if (e != cudaSuccess) return gi::fail_cuda(e, "gi_render_frame: capture stream");
        ctx->fg_stream = fs;
    }
    cudaStream_t fs = static_cast<cudaStream_t>(ctx->fg_stream);
    e = cudaStreamBeginCapture(fs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_render_frame: begin capture");
    const uint64_t launches0 = ctx->launches;
    st = enqueue_frame(ctx, s, mp, light_mvp, camera_mvp, vp, W, H, d_depth, d_vis, d_pos, d_nrm, fs);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(fs, &graph);
    const uint64_t held = ctx->launches - launches0;
    ctx->launches = launches0;
    if (st != GI_OK || e != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        ctx->fg_seen = false;
        return st != GI_OK ? st : gi::fail_cuda(e == cudaSuccess ? cudaErrorUnknown : e, "gi_render_frame: capture");
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        ctx->fg_seen = false;
        return gi::fail_cuda(e, "gi_render_frame: graph instantiate");
    }
    ctx->fg_exec = exec;
    ctx->fg_launches = held;
    e = cudaGraphLaunch(exec, cs);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_render_frame: graph launch");
    ctx->launches += held;
    return GI_OK;
}

// UniformSampledLightSource::computeUniformSampling
// (SoftShadowMapping/src/Scene/LightSource/UniformSampledLightSource.cpp:27-38):
// sample i of an n_side x n_side grid shifts eye and at by
// (((i % n_side) - c) / c * half, ((int)(i / n_side) - c) / c * half, 0) with
// half = size / 2 and c = (n_side - 1) / 2, in the reference's float /
// double operation order.
extern "C" gi_status gi_area_light_samples(const gi_view* light, float size, int n_side, gi_view* out) {
    gi_status st = check_view(light);
    if (st != GI_OK) return st;
    if (!out || n_side < 2 || n_side > 32 || !(size >= 0.0f))
        return fail(GI_ERR_INVALID_ARG, "gi_area_light_samples: need out, 2 <= n_side <= 32, size >= 0");
    const int n = n_side * n_side;
    const float half = (float)((double)size / 2.0);
    const float factor = sqrtf((float)n);
    const float sample_size = (float)((double)(factor - 1.0f) / 2.0);
    for (int i = 0; i < n; ++i) {
        const float dx = ((float)(i % (int)factor) - sample_size) / sample_size * half;
        const float dy = ((float)(int)((float)i / factor) - sample_size) / sample_size * half;
        out[i] = *light;
        out[i].eye[0] = light->eye[0] + dx;
        out[i].eye[1] = light->eye[1] + dy;
        out[i].at[0] = light->at[0] + dx;
        out[i].at[1] = light->at[1] + dy;
    }
    return GI_OK;
}

// renderMonteCarlo (SoftShadowMapping/src/main.cpp:756-811) + the uniform
// branch of AccurateSoftShadow.frag:52-133.  Sample maps are rendered in
// waves into context scratch; each wave adds its hard tests to the
// per-pixel sums in sample order.
extern "C" gi_status gi_area_light_visibility(gi_context* ctx, const gi_scene* s, const gi_view* samples, int n,
                                              const gi_map_params* mp, const float camera_mvp[16],
                                              float shadow_intensity, int W, int H, float* d_vis, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!samples || n < 1 || n > 4096 || !mp || !camera_mvp || !d_vis)
        return fail(GI_ERR_INVALID_ARG, "gi_area_light_visibility: bad arguments");
    if (mp->width != mp->height) return fail(GI_ERR_INVALID_ARG, "gi_area_light_visibility: square maps only");
    st = check_image(mp->width, mp->height, "gi_area_light_visibility (map)");
    if (st == GI_OK) st = check_image(W, H, "gi_area_light_visibility");
    if (st != GI_OK) return st;
    if ((size_t)s->dev_triangles >= ((size_t)1 << 29))
        return fail(GI_ERR_CAPACITY, "gi_area_light_visibility: more than 2^29 triangles");
    // per-sample light MVP (projection * view * model) and biased MVP
    std::vector<float> mvp((size_t)n * 16), biased((size_t)n * 16);
    for (int i = 0; i < n; ++i) {
        st = check_view(&samples[i]);
        if (st != GI_OK) return st;
        gi_frame_matrices fm;
        st = gi_frame_setup(&samples[i], &samples[i], &fm);
        if (st != GI_OK) return st;
        std::memcpy(&mvp[(size_t)i * 16], fm.light_mvp, 64);
        std::memcpy(&biased[(size_t)i * 16], fm.light_mvp_biased, 64);
    }
    const int S = mp->width;
    const size_t map_bytes = (size_t)S * S * sizeof(float);
    const int wave_max = (int)std::max<size_t>(1, std::min<size_t>(16, ((size_t)1 << 30) / map_bytes));
    st = gi::ensure_buffer(reinterpret_cast<void**>(&ctx->d_area_maps), &ctx->cap_area_maps, wave_max * map_bytes);
    if (st == GI_OK)
        st = gi::ensure_buffer(reinterpret_cast<void**>(&ctx->d_area_acc), &ctx->cap_area_acc,
                               (size_t)W * H * sizeof(float));
    if (st != GI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    st = gi::raster_gbuffer_keys(ctx, s, camera_mvp, W, H, cs);
    gi::AreaWave wave;
    // the shader's lightMVP uniform is the last sample's (biased) MVP
    std::memcpy(wave.common, &biased[(size_t)(n - 1) * 16], 12 * sizeof(float));
    for (int w0 = 0; w0 < n && st == GI_OK; w0 += wave_max) {
        const int nw = std::min(wave_max, n - w0);
        for (int k = 0; k < nw && st == GI_OK; ++k) {
            const int i = w0 + k;
            st = gi::raster_depth_map(ctx, s, &mvp[(size_t)i * 16], S, S, mp->bias_mode, mp->constant_bias,
                                      mp->offset_factor, mp->offset_units, ctx->d_area_maps + (size_t)k * S * S,
                                      small_px_default(), cs);
            for (int c = 0; c < 4; ++c) wave.trans[k][c] = biased[(size_t)i * 16 + 12 + c];
            wave.weight[k] = 1.0f;  // the uniform branch's accFactor
        }
        if (st == GI_OK)
            st = gi::launch_area_accumulate(ctx, s, camera_mvp, W, H, ctx->d_area_maps, S, nw, wave,
                                            shadow_intensity, w0 == 0, w0 + nw == n, (float)n, d_vis, cs);
    }
    return st;
}

// ---- adaptive area-light sampling -----------------------------------------
// SoftShadowMapping's adaptiveSampling (main.cpp:440-690, 820-870) over a
// QuadTreeLightSource (QuadTreeLightSource.cpp): the tree is evaluated
// depth first as the reference does, so that every sample map is rendered
// by the node that reaches its grid position first (its eye comes from that
// node's own chain of float additions) and maps are numbered in the
// reference's order, which is the order the final pass sums them in.
namespace {

struct QtNode {
    int level;
    float ref_eye[3], ref_at[3];
    int kids[4];  // indices into QtRun::nodes, -1 without children
};

struct QtMap {
    float eye[3], at[3];
    float mvp[16], biased[16];
    float level;  // accFactor[]: the level of the last leaf that used the map
};

struct QtRun {
    gi_context* ctx;
    const gi_scene* scene;
    gi_view light;
    float size;
    int max_level;
    const gi_map_params* mp;
    int S, W, H;
    int div;  // evaluation viewport divisor (4 in the lower-accuracy mode)
    cudaStream_t cs;
    float* pos;
    unsigned char* sums;
    unsigned* passed;
    int hash[17][17];
    std::vector<QtNode> nodes;
    std::vector<QtMap> maps;
};

// QuadTreeLightSource::computeUniformSamples (corner `index` of a node at
// `level`) and computeReferenceSamples (the reference point of child
// `index`): sample[0] += -step + 2 step (index % 2), sample[1] likewise with
// index / 2, step = size / 2^(level + 1) or size / 2^(level + 2).
void qt_offset(const float ref[3], float size, int div_pow, int index, float out[3]) {
    const int div = (int)powf(2.0f, (float)div_pow);
    const float step = size / (float)div;
    out[0] = ref[0];
    out[1] = ref[1];
    out[2] = ref[2];
    out[0] += -step + (2.0f * step * (float)(index % 2));
    out[1] += -step + (2.0f * step * (float)(index / 2));
}

// computeChildIndices (main.cpp:423-436)
void qt_children(int level, int node, int child[4]) {
    const int div = (int)powf(2.0f, (float)level);
    const int x = node % div, y = node / div;
    const int base = 2 * x + (int)powf(2.0f, (float)(level + 2)) * y;
    child[0] = base;
    child[1] = base + 1;
    child[2] = base + (int)powf(2.0f, (float)(level + 1));
    child[3] = base + (int)powf(2.0f, (float)(level + 1)) + 1;
}

// The map of grid position (x, y) for corner `index` of `node`: reused if
// rendered, else rendered now (displaySceneFromLightPOV into the next layer).
gi_status qt_map(QtRun& r, const QtNode& node, int index, int x, int y, int* out) {
    if (r.hash[x][y] >= 0) {
        *out = r.hash[x][y];
        return GI_OK;
    }
    QtMap m;
    qt_offset(node.ref_eye, r.size, node.level + 1, index, m.eye);
    qt_offset(node.ref_at, r.size, node.level + 1, index, m.at);
    gi_view v = r.light;
    for (int c = 0; c < 3; ++c) {
        v.eye[c] = m.eye[c];
        v.at[c] = m.at[c];
    }
    gi_frame_matrices fm;
    gi_status st = gi_frame_setup(&v, &v, &fm);
    if (st != GI_OK) return st;
    std::memcpy(m.mvp, fm.light_mvp, 64);
    std::memcpy(m.biased, fm.light_mvp_biased, 64);
    m.level = 0.0f;
    const int idx = (int)r.maps.size();
    st = gi::raster_depth_map(r.ctx, r.scene, m.mvp, r.S, r.S, r.mp->bias_mode, r.mp->constant_bias,
                              r.mp->offset_factor, r.mp->offset_units, r.ctx->d_area_maps + (size_t)idx * r.S * r.S,
                              small_px_default(), r.cs);
    if (st != GI_OK) return st;
    r.maps.push_back(m);
    r.hash[x][y] = idx;
    *out = idx;
    return GI_OK;
}

void qt_corner(int level, int node, int index, int* x, int* y) {
    const int cf = (int)(16.0f / powf(2.0f, (float)level)), pf = (int)powf(2.0f, (float)level);
    *x = (index % 2) * cf + (node % pf) * cf;
    *y = (index / 2) * cf + (node / pf) * cf;
}

// evaluateSubAreaLightSource (main.cpp:440-570; div = 1, or 4 in the
// lower-accuracy mode, :551-555): the node's four corner maps, the
// reprojection and the evaluation's occlusion query.
gi_status qt_evaluate_sub(QtRun& r, int n, int node, bool* subdivide) {
    gi::QuadCorners q;
    for (int index = 0; index < 4; ++index) {
        int x, y, idx;
        qt_corner(r.nodes[n].level, node, index, &x, &y);
        gi_status st = qt_map(r, r.nodes[n], index, x, y, &idx);
        if (st != GI_OK) return st;
        q.maps[index] = r.ctx->d_area_maps + (size_t)idx * r.S * r.S;
        std::memcpy(q.mvp[index], r.maps[idx].biased, 64);
    }
    cudaError_t e = cudaMemsetAsync(r.passed, 0, sizeof(unsigned), r.cs);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_area_light_adaptive: flag");
    gi_status st = gi::launch_qt_evaluate(r.ctx, r.pos, r.W, r.H, r.div, q, r.S, r.sums, r.passed, r.cs);
    if (st != GI_OK) return st;
    unsigned h = 0;
    e = cudaMemcpyAsync(&h, r.passed, sizeof h, cudaMemcpyDeviceToHost, r.cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.cs);
    if (e != cudaSuccess) return gi::fail_cuda(e, "gi_area_light_adaptive: query");
    *subdivide = h != 0;
    return GI_OK;
}

// evaluateAreaLightSource (main.cpp:572-629, the refinement path)
gi_status qt_evaluate(QtRun& r, int n, int node) {
    if (r.nodes[n].level == r.max_level) return GI_OK;
    int child[4];
    qt_children(r.nodes[n].level, node, child);
    bool sub = false;
    gi_status st = qt_evaluate_sub(r, n, node, &sub);
    if (st != GI_OK || !sub) return st;
    // QuadTreeLightSource::subdivide
    for (int c = 0; c < 4; ++c) {
        QtNode k;
        k.level = r.nodes[n].level + 1;
        qt_offset(r.nodes[n].ref_eye, r.size, r.nodes[n].level + 2, c, k.ref_eye);
        qt_offset(r.nodes[n].ref_at, r.size, r.nodes[n].level + 2, c, k.ref_at);
        k.kids[0] = k.kids[1] = k.kids[2] = k.kids[3] = -1;
        r.nodes[n].kids[c] = (int)r.nodes.size();
        r.nodes.push_back(k);
    }
    for (int c = 0; c < 4 && st == GI_OK; ++c) st = qt_evaluate(r, r.nodes[n].kids[c], child[c]);
    return st;
}

// renderAreaLightSource / renderSubAreaLightSource (main.cpp:631-690): the
// leaves' corner maps (rendering those the evaluation did not), each map
// taking the level of the last leaf that uses it.
gi_status qt_render(QtRun& r, int n, int node) {
    if (r.nodes[n].kids[0] >= 0) {
        int child[4];
        qt_children(r.nodes[n].level, node, child);
        for (int c = 0; c < 4; ++c) {
            gi_status st = qt_render(r, r.nodes[n].kids[c], child[c]);
            if (st != GI_OK) return st;
        }
        return GI_OK;
    }
    for (int index = 0; index < 4; ++index) {
        int x, y, idx;
        qt_corner(r.nodes[n].level, node, index, &x, &y);
        gi_status st = qt_map(r, r.nodes[n], index, x, y, &idx);
        if (st != GI_OK) return st;
        r.maps[idx].level = (float)r.nodes[n].level;
    }
    return GI_OK;
}

}  // namespace

extern "C" gi_status gi_area_light_adaptive(gi_context* ctx, const gi_scene* s, const gi_view* light, float size,
                                            int max_level, int lower_accuracy, const gi_map_params* mp,
                                            const float camera_mvp[16],
                                            float shadow_intensity, int W, int H, float* d_vis, gi_view* samples_out,
                                            float* levels_out, int* num_samples, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st == GI_OK) st = check_view(light);
    if (st != GI_OK) return st;
    if (!mp || !camera_mvp || !d_vis || max_level < 0 || max_level > 4 || !(size >= 0.0f))
        return fail(GI_ERR_INVALID_ARG, "gi_area_light_adaptive: bad arguments (0 <= max_level <= 4)");
    if (mp->width != mp->height) return fail(GI_ERR_INVALID_ARG, "gi_area_light_adaptive: square maps only");
    st = check_image(mp->width, mp->height, "gi_area_light_adaptive (map)");
    if (st == GI_OK) st = check_image(W, H, "gi_area_light_adaptive");
    if (st != GI_OK) return st;
    if (mp->width > 4096) return fail(GI_ERR_CAPACITY, "gi_area_light_adaptive: maps up to 4096^2 (289 are kept)");
    if ((size_t)s->dev_triangles >= ((size_t)1 << 29))
        return fail(GI_ERR_CAPACITY, "gi_area_light_adaptive: more than 2^29 triangles");
    QtRun r;
    r.ctx = ctx;
    r.scene = s;
    r.light = *light;
    r.size = size;
    r.max_level = max_level;
    r.mp = mp;
    r.S = mp->width;
    r.W = W;
    r.H = H;
    r.div = lower_accuracy ? 4 : 1;
    if (W / r.div < 1 || H / r.div < 1)
        return fail(GI_ERR_INVALID_ARG, "gi_area_light_adaptive: the lower-accuracy mode needs width, height >= 4");
    r.cs = static_cast<cudaStream_t>(stream);
    for (auto& row : r.hash)
        for (int& h : row) h = -1;
    const size_t npx = (size_t)W * H;
    const size_t map_bytes = (size_t)r.S * r.S * sizeof(float);
    // every grid position of the 17 x 17 grid is rendered at most once
    st = gi::ensure_buffer(reinterpret_cast<void**>(&ctx->d_area_maps), &ctx->cap_area_maps, 289 * map_bytes);
    if (st == GI_OK)
        st = gi::ensure_buffer(reinterpret_cast<void**>(&ctx->d_area_acc), &ctx->cap_area_acc, npx * sizeof(float));
    if (st == GI_OK)
        st = gi::ensure_buffer(reinterpret_cast<void**>(&ctx->d_area_gbuf), &ctx->cap_area_gbuf,
                               npx * 8 * sizeof(float) + npx + 64);
    if (st != GI_OK) return st;
    r.pos = ctx->d_area_gbuf;
    r.sums = reinterpret_cast<unsigned char*>(ctx->d_area_gbuf + npx * 8);
    r.passed = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(ctx->d_area_gbuf) +
                                           ((npx * 8 * sizeof(float) + npx + 15) & ~(size_t)15));
    // the G-buffer (positions for the reprojections; its keys serve the final pass)
    st = gi::raster_gbuffer(ctx, s, camera_mvp, W, H, r.pos, r.pos + npx * 4, small_px_default(), r.cs);
    if (st != GI_OK) return st;
    // QuadTreeLightSource::buildFirstLevel: the root at the light
    QtNode root;
    root.level = 0;
    for (int c = 0; c < 3; ++c) {
        root.ref_eye[c] = light->eye[c];
        root.ref_at[c] = light->at[c];
    }
    root.kids[0] = root.kids[1] = root.kids[2] = root.kids[3] = -1;
    r.nodes.push_back(root);
    st = qt_evaluate(r, 0, 0);
    if (st == GI_OK) st = qt_render(r, 0, 0);
    if (st != GI_OK) return st;
    const int n = (int)r.maps.size();
    // AccurateSoftShadow.frag's adaptive branch: configureShadow adds
    // accFactor * 10000 to each biased translation's w (float), the shader
    // recovers the level as int(w / 10000) (at most 4) and w - level * 10000,
    // and weighs the map by 1 / (2^level + 1)^2; the lightMVP uniform is the
    // last rendered map's
    gi::AreaWave wave;
    std::memcpy(wave.common, r.maps[n - 1].biased, 12 * sizeof(float));
    if (lower_accuracy) {
        // for (float w = -offset; w <= offset; w += stepSize), offset 1,
        // stepSize 2 * offset / 3.0, in float (AccurateSoftShadow.frag:98-110)
        const float offset = 1.0f, step = 2.0f * offset / 3.0f;
        int k = 0;
        for (float w = -offset; w <= offset && k < 8; w += step) wave.pcf_off[k++] = w;
        wave.pcf_n = k;
        wave.pcf_incr_w = 1.0f / (float)r.S;
        wave.pcf_incr_h = 1.0f / (float)r.S;
    }
    std::vector<float> tr((size_t)n * 4), wt(n);
    float count = 0.0f;
    for (int i = 0; i < n; ++i) {
        const float* b = r.maps[i].biased;
        const float w_enc = b[15] + r.maps[i].level * 10000.0f;
        int ql = (int)(w_enc / 10000.0f);
        if (ql > 4) ql = 4;
        const float wv = w_enc - (float)(ql * 10000);
        float f = 1.0f;
        for (int e = 1; e <= ql; ++e) f *= 2.0f;
        f = f + 1.0f;
        const float acc = 1.0f / (f * f);
        tr[4 * i] = b[12];
        tr[4 * i + 1] = b[13];
        tr[4 * i + 2] = b[14];
        tr[4 * i + 3] = wv;
        wt[i] = acc;
        count += acc;
    }
    for (int w0 = 0; w0 < n && st == GI_OK; w0 += 16) {
        const int nw = std::min(16, n - w0);
        for (int k = 0; k < nw; ++k) {
            for (int c = 0; c < 4; ++c) wave.trans[k][c] = tr[4 * (w0 + k) + c];
            wave.weight[k] = wt[w0 + k];
        }
        st = gi::launch_area_accumulate(ctx, s, camera_mvp, W, H, ctx->d_area_maps + (size_t)w0 * r.S * r.S, r.S,
                                        nw, wave, shadow_intensity, w0 == 0, w0 + nw == n, count, d_vis, r.cs);
    }
    if (st != GI_OK) return st;
    if (num_samples) *num_samples = n;
    for (int i = 0; i < n; ++i) {
        if (samples_out) {
            samples_out[i] = *light;
            for (int c = 0; c < 3; ++c) {
                samples_out[i].eye[c] = r.maps[i].eye[c];
                samples_out[i].at[c] = r.maps[i].at[c];
            }
        }
        if (levels_out) levels_out[i] = r.maps[i].level;
    }
    return GI_OK;
}

extern "C" gi_status gi_phong_shade(gi_context* ctx, const gi_vis_params* vp, const float* d_pos,
                                    const float* d_nrm, const float* d_vis, const float* d_color, int W, int H,
                                    float* d_out, void* stream) {
    if (!ctx || !vp || !d_pos || !d_nrm || !d_vis || !d_out)
        return fail(GI_ERR_INVALID_ARG, "gi_phong_shade: NULL argument");
    gi_status st = check_device(ctx);
    if (st == GI_OK) st = check_image(W, H, "gi_phong_shade");
    if (st != GI_OK) return st;
    return gi::launch_phong(ctx, vp, d_pos, d_nrm, d_vis, d_color, d_out, W, H, static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_pba_voronoi(gi_context* ctx, const int16_t* d_sites, int W, int H, int m1, int m2, int m3,
                                    int16_t* d_nearest, void* stream) {
    if (!ctx || !d_sites || !d_nearest) return fail(GI_ERR_INVALID_ARG, "gi_pba_voronoi: NULL argument");
    gi_status st = check_device(ctx);
    if (st == GI_OK) st = gi::pba_check_shape(W, H, m1, m2, m3, "gi_pba_voronoi");
    if (st != GI_OK) return st;
    return gi::launch_pba(ctx, d_sites, nullptr, nullptr, W, H, m1, m2, m3, 0.0f, 0.0f, d_nearest, nullptr,
                          static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_edt_soft_shadows(gi_context* ctx, const float* d_image, const float* d_position, int W,
                                         int H, int m1, int m2, int m3, float penumbra, float intensity,
                                         float* d_out, int16_t* d_nearest, void* stream) {
    if (!ctx || !d_image || !d_position || !d_out)
        return fail(GI_ERR_INVALID_ARG, "gi_edt_soft_shadows: NULL argument");
    gi_status st = check_device(ctx);
    if (st == GI_OK) st = gi::pba_check_shape(W, H, m1, m2, m3, "gi_edt_soft_shadows");
    if (st != GI_OK) return st;
    return gi::launch_pba(ctx, nullptr, d_image, d_position, W, H, m1, m2, m3, penumbra, intensity, d_nearest,
                          d_out, static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_pba_chain_rows(gi_context* ctx, uint32_t* rows, int reset) {
    if (!ctx || !rows) return fail(GI_ERR_INVALID_ARG, "gi_pba_chain_rows: NULL argument");
    gi_status st = check_device(ctx);
    if (st != GI_OK) return st;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(rows, ctx->d_status + 96, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(ctx->d_status + 96, 0, sizeof(uint32_t));
    return e == cudaSuccess ? GI_OK : gi::fail_cuda(e, "gi_pba_chain_rows");
}

extern "C" gi_status gi_edt_mean_filter(gi_context* ctx, const gi_vis_params* vp, const float* d_image,
                                        const float* d_pos, int W, int H, int order, float* d_out, void* stream) {
    if (!ctx || !vp || !d_image || !d_pos || !d_out) return fail(GI_ERR_INVALID_ARG, "gi_edt_mean_filter: NULL argument");
    if (order < 1 || order > 33) return fail(GI_ERR_INVALID_ARG, "gi_edt_mean_filter: order must be in [1, 33]");
    gi_status st = check_device(ctx);
    if (st == GI_OK) st = check_image(W, H, "gi_edt_mean_filter");
    if (st != GI_OK) return st;
    return gi::launch_edt_mean_filter(ctx, vp->camera_mv, d_image, d_pos, W, H, order, d_out,
                                      static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_edt_inputs(gi_context* ctx, const gi_vis_params* vp, const float camera_mvp[16],
                                   const float* d_pos, const float* d_nrm, const float* d_vis, int W, int H,
                                   float* d_image, float* d_position, void* stream) {
    if (!ctx || !vp || !camera_mvp || !d_pos || !d_nrm || !d_vis || !d_image || !d_position)
        return fail(GI_ERR_INVALID_ARG, "gi_edt_inputs: NULL argument");
    gi_status st = check_device(ctx);
    if (st == GI_OK) st = check_image(W, H, "gi_edt_inputs");
    if (st != GI_OK) return st;
    return gi::launch_edt_inputs(ctx, vp, camera_mvp, d_pos, d_nrm, d_vis, d_image, d_position, W, H,
                                 static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_surrogate_features(gi_context* ctx, const gi_scene* s, const gi_map_params* mp,
                                           const float light_mvp[16], const float camera_mvp[16],
                                           const gi_vis_params* vp, int W, int H, float* d_depth, void* d_feat,
                                           void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!mp || !light_mvp || !camera_mvp || !vp || !d_depth || !d_feat)
        return fail(GI_ERR_INVALID_ARG, "gi_surrogate_features: bad arguments");
    if (vp->technique != GI_TECH_PCSS_POISSON)
        return fail(GI_ERR_INVALID_ARG, "gi_surrogate_features: the surrogate models GI_TECH_PCSS_POISSON");
    st = check_image(mp->width, mp->height, "gi_surrogate_features (map)");
    if (st == GI_OK) st = check_image(W, H, "gi_surrogate_features");
    if (st == GI_OK) st = check_vis_params(vp);
    if (st != GI_OK) return st;
    if ((size_t)s->dev_triangles >= ((size_t)1 << 29))
        return fail(GI_ERR_CAPACITY, "gi_surrogate_features: more than 2^29 triangles");
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    st = gi::raster_depth_map(ctx, s, light_mvp, mp->width, mp->height, mp->bias_mode, mp->constant_bias,
                              mp->offset_factor, mp->offset_units, d_depth, small_px_default(), cs);
    if (st == GI_OK) st = gi::raster_gbuffer_keys(ctx, s, camera_mvp, W, H, cs);
    if (st == GI_OK)
        st = gi::launch_surrogate_features(ctx, vp, d_depth, mp->width, mp->height, s, camera_mvp, W, H, d_feat, cs);
    return st;
}

extern "C" gi_status gi_surrogate_finish(gi_context* ctx, const gi_scene* s, int map_w, int map_h,
                                         const float* d_depth, const float camera_mvp[16], const gi_vis_params* vp,
                                         int W, int H, const float* d_head, int head_stride, const void* d_feat,
                                         float err_threshold, float* d_vis, uint32_t* d_fallback, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!camera_mvp || !vp || !d_depth || !d_head || !d_feat || !d_vis || head_stride < 2 || head_stride % 2)
        return fail(GI_ERR_INVALID_ARG, "gi_surrogate_finish: bad arguments");
    if (vp->technique != GI_TECH_PCSS_POISSON)
        return fail(GI_ERR_INVALID_ARG, "gi_surrogate_finish: the surrogate models GI_TECH_PCSS_POISSON");
    st = check_image(map_w, map_h, "gi_surrogate_finish (map)");
    if (st == GI_OK) st = check_image(W, H, "gi_surrogate_finish");
    if (st == GI_OK) st = check_vis_params(vp);
    if (st != GI_OK) return st;
    if (ctx->cap_vkeys < (size_t)W * H * sizeof(unsigned long long))
        return fail(GI_ERR_INVALID_ARG, "gi_surrogate_finish: call gi_surrogate_features for this frame first");
    return gi::launch_surrogate_finish(ctx, vp, d_depth, map_w, map_h, s, camera_mvp, W, H, d_head, head_stride,
                                       d_feat, err_threshold, d_vis, d_fallback, static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_soft_moment_map(gi_context* ctx, const gi_vis_params* vis, const float* d_depth, int map_w,
                                        int map_h, float* d_out, void* stream) {
    if (!ctx || !vis || !d_depth || !d_out) return fail(GI_ERR_INVALID_ARG, "gi_soft_moment_map: NULL argument");
    if (!gi::is_soft_moment_technique(vis->technique))
        return fail(GI_ERR_INVALID_ARG, "gi_soft_moment_map: technique must be SAVSM, VSSM, ESSM or MSSM");
    gi_status st = check_image(map_w, map_h, "gi_soft_moment_map");
    if (st == GI_OK) st = check_device(ctx);
    if (st != GI_OK) return st;
    if (reinterpret_cast<uintptr_t>(d_out) % 16 != 0)
        return fail(GI_ERR_INVALID_ARG, "gi_soft_moment_map: d_out must be 16-byte aligned");
    const float4* m = nullptr;
    return gi::launch_soft_moment_map(ctx, vis, d_depth, map_w, map_h, static_cast<cudaStream_t>(stream),
                                      reinterpret_cast<float4*>(d_out), &m);
}

extern "C" gi_status gi_hierarchical_shadow_map(gi_context* ctx, const gi_vis_params* vis, const float* d_depth,
                                                int map_w, int map_h, int level, float* d_out, void* stream) {
    if (!ctx || !vis || !d_depth || !d_out)
        return fail(GI_ERR_INVALID_ARG, "gi_hierarchical_shadow_map: NULL argument");
    gi_status st = check_image(map_w, map_h, "gi_hierarchical_shadow_map");
    if (st != GI_OK) return st;
    int m = 0;
    while ((1 << m) < map_w) ++m;
    if (map_w != map_h || (1 << m) != map_w)
        return fail(GI_ERR_UNSUPPORTED, "gi_hierarchical_shadow_map: needs a square power-of-two map");
    // renderHSM writes levels 1 .. log2(width) - 1 after PrepareMinMax's level 0
    if (level < 0 || (level > 0 && level >= m))
        return fail(GI_ERR_INVALID_ARG, "gi_hierarchical_shadow_map: level must be 0 or in [1, log2(width))");
    st = check_device(ctx);
    if (st != GI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    const float2* lv = nullptr;
    st = gi::launch_hsm(ctx, vis, d_depth, map_w, map_h, level, cs, &lv);
    if (st != GI_OK) return st;
    const size_t n = (size_t)(map_w >> level) * (map_h >> level);
    const cudaError_t e = cudaMemcpyAsync(d_out, lv, n * sizeof(float2), cudaMemcpyDeviceToDevice, cs);
    return e == cudaSuccess ? GI_OK : gi::fail_cuda(e, "gi_hierarchical_shadow_map: copy");
}

extern "C" gi_status gi_poisson_table(int n, float* xy) {
    if (n < 1 || n > 64 || !xy) return fail(GI_ERR_INVALID_ARG, "gi_poisson_table: n in [1, 64]");
    for (int i = 0; i < n; ++i) {
        xy[2 * i] = gi::kPoissonDisk[i][0];
        xy[2 * i + 1] = gi::kPoissonDisk[i][1];
    }
    return GI_OK;
}

extern "C" gi_status gi_shadow_volume_counts(gi_context* ctx, const gi_scene* s,
                                             const float light_pos[3], float infinity,
                                             const float camera_mvp[16], int W, int H,
                                             int depth_func, uint8_t* d_stencil, float* d_depth,
                                             void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!light_pos || !camera_mvp || !d_stencil)
        return fail(GI_ERR_INVALID_ARG, "gi_shadow_volume_counts: NULL argument");
    st = check_image(W, H, "gi_shadow_volume_counts");
    if (st != GI_OK) return st;
    if (depth_func != GI_DEPTH_LESS && depth_func != GI_DEPTH_LEQUAL)
        return fail(GI_ERR_INVALID_ARG, "gi_shadow_volume_counts: bad depth_func");
    return gi::raster_shadow_volumes(ctx, s, light_pos, infinity, camera_mvp, W, H, depth_func,
                                     d_stencil, d_depth, small_px_default(),
                                     static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_shadow_volume_geometry(gi_context* ctx, const gi_scene* s,
                                               const float light_pos[3], float infinity,
                                               float* d_triangles, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!light_pos || (!d_triangles && s->dev_triangles > 0))
        return fail(GI_ERR_INVALID_ARG, "gi_shadow_volume_geometry: NULL argument");
    return gi::raster_volume_geometry(ctx, s, light_pos, infinity, d_triangles,
                                      static_cast<cudaStream_t>(stream));
}

extern "C" gi_status gi_debug_fail_allocation(int countdown) {
    if (countdown < -1) return fail(GI_ERR_INVALID_ARG, "gi_debug_fail_allocation: countdown must be >= -1");
    gi::g_alloc_countdown.store(countdown);
    return GI_OK;
}

extern "C" gi_status gi_shadow_volume_counts_silhouette(gi_context* ctx, const gi_scene* s,
                                                        const float light_pos[3], float infinity,
                                                        const float camera_mvp[16], int W, int H,
                                                        int depth_func, uint8_t* d_stencil, float* d_depth,
                                                        int* volume_triangles, void* stream) {
    gi_status st = check_pass(ctx, s);
    if (st != GI_OK) return st;
    if (!light_pos || !camera_mvp || !d_stencil)
        return fail(GI_ERR_INVALID_ARG, "gi_shadow_volume_counts_silhouette: NULL argument");
    st = check_image(W, H, "gi_shadow_volume_counts_silhouette");
    if (st != GI_OK) return st;
    if (depth_func != GI_DEPTH_LESS && depth_func != GI_DEPTH_LEQUAL)
        return fail(GI_ERR_INVALID_ARG, "gi_shadow_volume_counts_silhouette: bad depth_func");
    return gi::raster_shadow_volumes(ctx, s, light_pos, infinity, camera_mvp, W, H, depth_func, d_stencil,
                                     d_depth, small_px_default(), static_cast<cudaStream_t>(stream), true,
                                     volume_triangles);
}
