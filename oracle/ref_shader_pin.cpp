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

namespace pin_shadow {
GI_SHADER_GLOBALS
#include GI_SHADER_SHADOW
}  // namespace pin_shadow

namespace pin_ncsmsr {
GI_SHADER_GLOBALS
#include GI_SHADER_NCSMSR
}  // namespace pin_ncsmsr

namespace pin_csmsr {
GI_SHADER_GLOBALS
#include GI_SHADER_CSMSR
}  // namespace pin_csmsr

namespace pin_frbsm {
GI_SHADER_GLOBALS
#include GI_SHADER_FRBSM
}  // namespace pin_frbsm

namespace pin_phong {
GI_SHADER_GLOBALS
#include GI_SHADER_PHONG
}  // namespace pin_phong

namespace pin_rbssm {
GI_SHADER_GLOBALS
// RBSSM.frag returns a float from a vec4 function and stores that vec4 in a
// float, which the reference's GL driver accepts (a splat, then the first
// component); in this namespace its vec4 does the same.
struct lenient_vec4 : glsl::vec4 {
    using glsl::vec4::vec4;
    lenient_vec4(float f) : glsl::vec4(f) {}
    lenient_vec4(const glsl::vec4& v) : glsl::vec4(v) {}
    operator float() const { return x; }
};
#define vec4 lenient_vec4
#include GI_SHADER_RBSSM
#undef vec4
}  // namespace pin_rbssm

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

// PlausibleSoftShadow.frag's SAVSM (mode 0) and ESSM (mode 1), with or
// without the summed-area table: `moments` is the soft app's moment map or
// its SAT (float4, S x S, read bilinearly), `depth` the light map the blocker
// search reads.
void ref_soft_moments(int mode, int sat, const float* depth, const float* moments, int S, const float* pos,
                      const float* nrm, int W, int H, const float* light_mvp, const float* camera_mv,
                      const float* normal_matrix, const float* light_position, float intensity,
                      int blocker_search_size, int kernel_size, int light_source_radius, float* out) {
    using namespace pin_pcss;
    const Frame f{depth, S, pos, nrm, W, H, light_mvp, camera_mv, normal_matrix, light_position, intensity};
    shadowMap = glsl::sampler2D{depth, S, S, 1};
    SATShadowMap = glsl::sampler2D{moments, S, S, 4, true};
    vertexMap = glsl::sampler2D{pos, W, H, 4};
    normalMap = glsl::sampler2D{nrm, W, H, 4};
    lightMVP = mat4_of(light_mvp);
    MV = mat4_of(camera_mv);
    normalMatrix = mat3_of(normal_matrix);
    lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);
    shadowIntensity = intensity;
    zNear = 1;
    zFar = 1000;
    windowWidth = W;
    windowHeight = H;
    shadowMapWidth = S;
    shadowMapHeight = S;
    blockerSearchSize = blocker_search_size;
    kernelSize = kernel_size;
    lightSourceRadius = light_source_radius;
    PCSS = VSSM = MSSM = 0;
    SAVSM = mode == 0;
    ESSM = mode == 1;
    SAT = sat;
    per_pixel(f, out, [](const glsl::vec2& tc) {
        f_texcoord = tc;
        gl_discarded = false;
        gl_FragColor = glsl::vec4(0.0f);
        shader_main();
        return gl_discarded ? 0.0f : gl_FragColor.x;
    });
}

// ShadowMapping/Shaders/Shadow.frag (computeHardShadows, ShadowMapping/src/
// main.cpp:400-414): mode 0 the naive hard test, 1 bilinear PCF, 2 tricubic
// PCF.
void ref_shadow(int mode, const float* depth, int S, const float* pos, const float* nrm, int W, int H,
                const float* light_mvp, const float* camera_mv, const float* normal_matrix,
                const float* light_position, float intensity, int kernel_order, int penumbra_size, float* out) {
    using namespace pin_shadow;
    const Frame f{depth, S, pos, nrm, W, H, light_mvp, camera_mv, normal_matrix, light_position, intensity};
    shadowMap = glsl::sampler2D{depth, S, S, 1};
    vertexMap = glsl::sampler2D{pos, W, H, 4};
    normalMap = glsl::sampler2D{nrm, W, H, 4};
    lightMVP = mat4_of(light_mvp);
    MV = mat4_of(camera_mv);
    normalMatrix = mat3_of(normal_matrix);
    lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);
    shadowIntensity = intensity;
    shadowMapWidth = S;
    shadowMapHeight = S;
    kernelOrder = kernel_order;
    penumbraSize = penumbra_size;
    zNear = 1;
    zFar = 1000;
    naive = mode == 0;
    bilinearPCF = mode == 1;
    tricubicPCF = mode == 2;
    VSM = ESM = EVSM = MSM = 0;
    per_pixel(f, out, [](const glsl::vec2& tc) {
        f_texcoord = tc;
        gl_discarded = false;
        gl_FragColor = glsl::vec4(0.0f);
        shader_main();
        return gl_discarded ? 0.0f : gl_FragColor.x;
    });
}

// Shadow.frag's moment lookups (VSM, ESM, EVSM, MSM: mode 3..6) over the
// blurred window-size moment target `moments` (float4, side M, read
// bilinearly), with MSM's quantisation uniforms.
void ref_shadow_moments(int tech_mode, const float* moments, int M, const float* pos, const float* nrm, int W, int H,
                        const float* light_mvp, const float* camera_mv, const float* normal_matrix,
                        const float* light_position, float intensity, const float* mq_inverse, float tq0,
                        float* out) {
    using namespace pin_shadow;
    const Frame f{moments, M, pos, nrm, W, H, light_mvp, camera_mv, normal_matrix, light_position, intensity};
    shadowMap = glsl::sampler2D{moments, M, M, 4, true};
    vertexMap = glsl::sampler2D{pos, W, H, 4};
    normalMap = glsl::sampler2D{nrm, W, H, 4};
    lightMVP = mat4_of(light_mvp);
    MV = mat4_of(camera_mv);
    normalMatrix = mat3_of(normal_matrix);
    lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);
    mQuantizationInverse = mat4_of(mq_inverse);
    tQuantization = glsl::vec4(tq0, 0.0f, 0.0f, 0.0f);
    shadowIntensity = intensity;
    shadowMapWidth = M;
    shadowMapHeight = M;
    zNear = 1;
    zFar = 1000;
    naive = bilinearPCF = tricubicPCF = 0;
    VSM = tech_mode == 3;
    ESM = tech_mode == 4;
    EVSM = tech_mode == 5;
    MSM = tech_mode == 6;
    per_pixel(f, out, [](const glsl::vec2& tc) {
        f_texcoord = tc;
        gl_discarded = false;
        gl_FragColor = glsl::vec4(0.0f);
        shader_main();
        return gl_discarded ? 0.0f : gl_FragColor.x;
    });
}

// The RBSM shaders (computeHardShadows with the RBSM techniques): shader 0
// NonConservativeSMSR.frag, 1 ConservativeSMSR.frag, 2 FilteredRBSM.frag;
// mode 0 SMSR, 1 RPCF (+ SMSR), 2 EDTSM.  out4 receives gl_FragData[0] and,
// when given, out_pos4 gl_FragData[1]; a discarded pixel keeps the clear
// colour (0, 0, 0, 1).
#define GI_RBSM_RUN(NS)                                                                              \
    do {                                                                                             \
        using namespace NS;                                                                          \
        shadowMap = glsl::sampler2D{depth, S, S, 1};                                                 \
        vertexMap = glsl::sampler2D{pos, W, H, 4};                                                   \
        normalMap = glsl::sampler2D{nrm, W, H, 4};                                                   \
        lightMVP = mat4_of(light_mvp);                                                               \
        MV = mat4_of(camera_mv);                                                                     \
        MVP = mat4_of(camera_mvp);                                                                   \
        normalMatrix = mat3_of(normal_matrix);                                                       \
        lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);         \
        shadowMapStep = glsl::vec2((float)(1.0 / S), (float)(1.0 / S));                              \
        shadowIntensity = intensity;                                                                 \
        depthThreshold = depth_threshold;                                                            \
        shadowMapWidth = S;                                                                          \
        shadowMapHeight = S;                                                                         \
        maxSearch = max_search;                                                                      \
        kernelOrder = kernel_order;                                                                  \
        penumbraSize = penumbra_size;                                                                \
        SMSR = mode == 0;                                                                            \
        RPCFPlusSMSR = mode == 1;                                                                    \
        EDTSM = mode == 2;                                                                           \
        for (int y = 0; y < H; ++y)                                                                  \
            for (int x = 0; x < W; ++x) {                                                            \
                const size_t q = (size_t)y * W + x;                                                  \
                f_texcoord = glsl::vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H); \
                gl_discarded = false;                                                                \
                gl_FragData[0] = glsl::vec4(0.0f, 0.0f, 0.0f, 1.0f);                                 \
                gl_FragData[1] = glsl::vec4(0.0f, 0.0f, 0.0f, 1.0f);                                 \
                shader_main();                                                                       \
                if (gl_discarded) {                                                                  \
                    gl_FragData[0] = glsl::vec4(0.0f, 0.0f, 0.0f, 1.0f);                             \
                    gl_FragData[1] = glsl::vec4(0.0f, 0.0f, 0.0f, 1.0f);                             \
                }                                                                                    \
                for (int k = 0; k < 4; ++k) {                                                        \
                    out4[4 * q + k] = gl_FragData[0].e[k];                                           \
                    if (out_pos4) out_pos4[4 * q + k] = gl_FragData[1].e[k];                         \
                }                                                                                    \
            }                                                                                        \
    } while (0)

void ref_rbsm(int shader, int mode, const float* depth, int S, const float* pos, const float* nrm, int W, int H,
              const float* light_mvp, const float* camera_mv, const float* camera_mvp, const float* normal_matrix,
              const float* light_position, float intensity, float depth_threshold, int max_search, int kernel_order,
              int penumbra_size, float* out4, float* out_pos4) {
    if (shader == 0) GI_RBSM_RUN(pin_ncsmsr);
    else if (shader == 1) GI_RBSM_RUN(pin_csmsr);
    else GI_RBSM_RUN(pin_frbsm);
}

// SoftShadowMapping/Shaders/SoftShadow/RBSSM.frag (renderSoftShadows with
// RBSSM).
void ref_rbssm(const float* depth, int S, const float* pos, const float* nrm, int W, int H, const float* light_mvp,
               const float* camera_mv, const float* normal_matrix, const float* light_position, float intensity,
               float depth_threshold, int max_search, int blocker_search_size, int kernel_size,
               int light_source_radius, int z_near, int z_far, float* out) {
    using namespace pin_rbssm;
    const Frame f{depth, S, pos, nrm, W, H, light_mvp, camera_mv, normal_matrix, light_position, intensity};
    shadowMap = glsl::sampler2D{depth, S, S, 1};
    hierarchicalShadowMap = shadowMap;
    vertexMap = glsl::sampler2D{pos, W, H, 4};
    normalMap = glsl::sampler2D{nrm, W, H, 4};
    lightMVP = mat4_of(light_mvp);
    MV = mat4_of(camera_mv);
    normalMatrix = mat3_of(normal_matrix);
    lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);
    shadowMapStep = glsl::vec2((float)(1.0 / S), (float)(1.0 / S));
    shadowIntensity = intensity;
    depthThreshold = depth_threshold;
    zNear = z_near;
    zFar = z_far;
    shadowMapWidth = S;
    shadowMapHeight = S;
    maxSearch = max_search;
    blockerSearchSize = blocker_search_size;
    kernelSize = kernel_size;
    lightSourceRadius = light_source_radius;
    useTextureForColoring = useMeshColor = 0;
    per_pixel(f, out, [](const glsl::vec2& tc) {
        f_texcoord = tc;
        gl_discarded = false;
        gl_FragColor = glsl::vec4(0.0f);
        shader_main();
        return gl_discarded ? 0.0f : gl_FragColor.x;
    });
}

// ShadowMapping/Shaders/GBuffer/PhongShading.frag (shadeScene): RGBA per
// pixel; a discarded (background) pixel keeps the shading target's clear
// colour (0.63, 0.82, 0.96, 1).
void ref_phong(const float* pos, const float* nrm, const float* vis, const float* color, int W, int H,
               const float* camera_mv, const float* normal_matrix, const float* light_position, float intensity,
               float* out4) {
    using namespace pin_phong;
    hardShadowMap = glsl::sampler2D{vis, W, H, 1};
    colorMap = glsl::sampler2D{color, W, H, 4};
    vertexMap = glsl::sampler2D{pos, W, H, 4};
    normalMap = glsl::sampler2D{nrm, W, H, 4};
    MV = mat4_of(camera_mv);
    normalMatrix = mat3_of(normal_matrix);
    lightPosition = glsl::vec3(light_position[0], light_position[1], light_position[2]);
    shadowIntensity = intensity;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t q = (size_t)y * W + x;
            f_texcoord = glsl::vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
            gl_discarded = false;
            gl_FragColor = glsl::vec4(0.0f);
            shader_main();
            const glsl::vec4 c = gl_discarded ? glsl::vec4(0.63f, 0.82f, 0.96f, 1.0f) : gl_FragColor;
            for (int k = 0; k < 4; ++k) out4[4 * q + k] = c.e[k];
        }
}

}  // extern "C"
