// The reference's own fragment shaders compiled as C++ (test infrastructure
// only): each shader file is included unmodified, read where it lies in the
// reference tree (paths given by the build recipe as GI_SHADER_* macros),
// inside its own namespace on top of glsl_shim.h, and an extern "C" driver
// runs its main() once per pixel of a G-buffer the caller passes, as the
// reference's full-screen pass does (f_texcoord at the pixel centre), with
// the uniforms the reference's viewers set.  The oracle's visibility is held
// to these outputs bit for bit (tests/test_shader_pin.py).  Built into
// oracle/_ref/ only where the reference tree is present.
#include <cstddef>

#include "glsl_shim.h"

#define uniform
#define varying
#define main shader_main
#define discard          \
    do {                 \
        gl_discarded = true; \
        return;          \
    } while (0)

#define GI_SHADER_GLOBALS \
    using namespace glsl; \
    vec4 gl_FragColor;    \
    vec4 gl_FragData[2];  \
    bool gl_discarded;

namespace pin_pcss {
GI_SHADER_GLOBALS
#include GI_SHADER_PCSS
}  // namespace pin_pcss

namespace {

glsl::mat4 mat4_of(const float* m) {
    glsl::mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) r.c[c].e[k] = m[c * 4 + k];
    return r;
}

glsl::mat3 mat3_of(const float* m) {
    glsl::mat3 r;
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) r.c[c].e[k] = m[c * 3 + k];
    return r;
}

struct Frame {
    const float* depth;
    int S;
    const float* pos;
    const float* nrm;
    int W, H;
    const float* light_mvp;       // the biased light MVP (lightMVP uniform)
    const float* camera_mv;       // MV
    const float* normal_matrix;   // normalMatrix (column-major 3 x 3)
    const float* light_position;  // lightPosition
    float intensity;
};

// Runs `shade` (which sets the namespace's uniforms and calls its main) for
// every pixel; the red channel of gl_FragColor, 0 where main discards.
template <class Run>
void per_pixel(const Frame& f, float* out, Run run) {
    for (int y = 0; y < f.H; ++y)
        for (int x = 0; x < f.W; ++x) {
            const glsl::vec2 tc(((float)x + 0.5f) / (float)f.W, ((float)y + 0.5f) / (float)f.H);
            out[(size_t)y * f.W + x] = run(tc);
        }
}

}  // namespace

extern "C" {

// SoftShadowMapping/Shaders/SoftShadow/PlausibleSoftShadow.frag with PCSS = 1
// (renderSoftShadows, SoftShadowMapping/src/main.cpp:1010-1017).
void ref_pcss(const float* depth, int S, const float* pos, const float* nrm, int W, int H, const float* light_mvp,
              const float* camera_mv, const float* normal_matrix, const float* light_position, float intensity,
              int blocker_search_size, int kernel_size, int light_source_radius, int z_near, int z_far, float* out) {
    using namespace pin_pcss;
    const Frame f{depth, S, pos, nrm, W, H, light_mvp, camera_mv, normal_matrix, light_position, intensity};
    shadowMap = glsl::sampler2D{depth, S, S, 1};
    vertexMap = glsl::sampler2D{pos, W, H, 4};
    normalMap = glsl::sampler2D{nrm, W, H, 4};
    lightMVP = mat4_of(light_mvp);
    MV = mat4_of(camera_mv);
    normalMatrix = mat3_of(normal_matrix);
    lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);
    shadowIntensity = intensity;
    zNear = z_near;
    zFar = z_far;
    windowWidth = W;
    windowHeight = H;
    shadowMapWidth = S;
    shadowMapHeight = S;
    blockerSearchSize = blocker_search_size;
    kernelSize = kernel_size;
    lightSourceRadius = light_source_radius;
    PCSS = 1;
    SAVSM = VSSM = ESSM = MSSM = SAT = 0;
    per_pixel(f, out, [](const glsl::vec2& tc) {
        f_texcoord = tc;
        gl_discarded = false;
        gl_FragColor = glsl::vec4(0.0f);
        shader_main();
        return gl_discarded ? 0.0f : gl_FragColor.x;
    });
}

}  // extern "C"
