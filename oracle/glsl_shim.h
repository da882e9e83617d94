// GLSL 1.20 fragment-shader subset as C++ (test infrastructure only).
//
// Lets the reference's own fragment shaders compile unmodified as C++ so the
// oracle can be held to them: vec2 / vec3 / vec4 with the swizzles those
// shaders use (read and write), mat3 / mat4 (column-major, m[column][row]),
// sampler2D with texture2D / texture / texture2DLod / textureSize, and the
// built-ins they call.  The choices GLSL leaves open are the ones the library
// fixes everywhere else: every float operation rounds once, in the written
// order (build with -ffp-contract=off and -fsingle-precision-constant, so a
// literal such as 0.5 is a float); matrix rows and dot products summed left
// to right; normalize(v) = v * (1 / sqrt(dot(v, v))); mix(x, y, a) =
// x (1 - a) + y a; max(x, y) = x < y ? y : x; min(x, y) = y < x ? y : x;
// clamp(x, a, b) = min(max(x, a), b); step(e, x) = x < e ? 0 : 1; fract(x) =
// x - floor(x); mod(x, y) = x - y floor(x / y); pow(x, 3) = x x x; texture lookups NEAREST at
// level 0 (texel floor(u * size)) with a zero border, a one-channel (depth)
// texture reading as (d, d, d, 1); the moment maps bilinear at level 0 with
// float32 weights and a zero border.
#pragma once

#include <cmath>

namespace glsl {

struct vec2;
struct vec3;
struct vec4;
template <int N>
struct vec_n;
template <>
struct vec_n<2> {
    using type = vec2;
};
template <>
struct vec_n<3> {
    using type = vec3;
};
template <>
struct vec_n<4> {
    using type = vec4;
};

// A swizzle of a vector of S floats that shares the vector's storage.
template <int S, int... I>
struct swz {
    float d[S];
    using V = typename vec_n<sizeof...(I)>::type;
    inline operator V() const;
    inline swz& operator=(const V& v);
    swz& operator=(const swz& o) { return *this = V(o); }
    inline swz& operator+=(const V& v);
    inline swz& operator-=(const V& v);
    inline swz& operator*=(const V& v);
    inline swz& operator/=(const V& v);
    inline swz& operator+=(float f);
    inline swz& operator-=(float f);
    inline swz& operator*=(float f);
    inline swz& operator/=(float f);
};

struct ivec2 {
    int x, y;
};

struct vec2 {
    union {
        float e[2];
        struct {
            float x, y;
        };
        struct {
            float r, g;
        };
        struct {
            float s, t;
        };
        swz<2, 0, 1> xy;
        swz<2, 0, 1> st;
        swz<2, 0, 0, 1, 1> xxyy;
        swz<2, 0, 1, 0, 1> xyxy;
    };
    vec2() : e{0.0f, 0.0f} {}
    explicit vec2(float a) : e{a, a} {}
    vec2(float a, float b) : e{a, b} {}
    explicit vec2(const ivec2& v) : e{(float)v.x, (float)v.y} {}
    inline vec2(const vec3& v);  // truncation, which the reference's driver accepts implicitly
    inline vec2(const vec4& v);
    vec2(const vec2& o) : e{o.e[0], o.e[1]} {}
    vec2& operator=(const vec2& o) {
        e[0] = o.e[0];
        e[1] = o.e[1];
        return *this;
    }
    float& operator[](int i) { return e[i]; }
    float operator[](int i) const { return e[i]; }
};

struct vec3 {
    union {
        float e[3];
        struct {
            float x, y, z;
        };
        struct {
            float r, g, b;
        };
        struct {
            float s, t, p;
        };
        swz<3, 0, 1> xy;
        swz<3, 0, 1> st;
        swz<3, 0, 1, 2> xyz;
    };
    vec3() : e{0.0f, 0.0f, 0.0f} {}
    explicit vec3(float a) : e{a, a, a} {}
    vec3(float a, float b, float c) : e{a, b, c} {}
    vec3(const vec2& v, float c) : e{v.e[0], v.e[1], c} {}
    inline vec3(const vec4& v);  // truncation, as above
    vec3(const vec3& o) : e{o.e[0], o.e[1], o.e[2]} {}
    vec3& operator=(const vec3& o) {
        e[0] = o.e[0];
        e[1] = o.e[1];
        e[2] = o.e[2];
        return *this;
    }
    float& operator[](int i) { return e[i]; }
    float operator[](int i) const { return e[i]; }
};

struct vec4 {
    union {
        float e[4];
        struct {
            float x, y, z, w;
        };
        struct {
            float r, g, b, a;
        };
        struct {
            float s, t, p, q;
        };
        swz<4, 0, 1> xy;
        swz<4, 0, 1> st;
        swz<4, 2, 3> zw;
        swz<4, 1, 3> yw;
        swz<4, 0, 2> xz;
        swz<4, 0, 3> xw;
        swz<4, 1, 2> yz;
        swz<4, 0, 1, 2> xyz;
        swz<4, 0, 1, 2> rgb;
        swz<4, 0, 0, 1, 1> xxyy;
        swz<4, 0, 1, 0, 1> xyxy;
    };
    vec4() : e{0.0f, 0.0f, 0.0f, 0.0f} {}
    explicit vec4(float v) : e{v, v, v, v} {}
    vec4(float a, float b, float c, float d) : e{a, b, c, d} {}
    vec4(const vec2& u, float c, float d) : e{u.e[0], u.e[1], c, d} {}
    vec4(float a, float b, const vec2& u) : e{a, b, u.e[0], u.e[1]} {}
    vec4(const vec2& u, const vec2& v) : e{u.e[0], u.e[1], v.e[0], v.e[1]} {}
    vec4(const vec3& u, float d) : e{u.e[0], u.e[1], u.e[2], d} {}
    vec4(const vec4& o) : e{o.e[0], o.e[1], o.e[2], o.e[3]} {}
    vec4& operator=(const vec4& o) {
        for (int i = 0; i < 4; ++i) e[i] = o.e[i];
        return *this;
    }
    float& operator[](int i) { return e[i]; }
    float operator[](int i) const { return e[i]; }
};

inline vec2::vec2(const vec3& v) : e{v.e[0], v.e[1]} {}
inline vec2::vec2(const vec4& v) : e{v.e[0], v.e[1]} {}
inline vec3::vec3(const vec4& v) : e{v.e[0], v.e[1], v.e[2]} {}

template <int S, int... I>
swz<S, I...>::operator V() const {
    return V(d[I]...);
}
template <int S, int... I>
swz<S, I...>& swz<S, I...>::operator=(const V& v) {
    const int idx[] = {I...};
    for (int k = 0; k < (int)sizeof...(I); ++k) d[idx[k]] = v.e[k];
    return *this;
}

// ---- arithmetic (component-wise, one rounding per operation) -------------
#define GLSL_VEC_OPS(V, N)                                                                  \
    inline V operator+(const V& a, const V& b) {                                            \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r.e[i] = a.e[i] + b.e[i];                               \
        return r;                                                                           \
    }                                                                                       \
    inline V operator-(const V& a, const V& b) {                                            \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r.e[i] = a.e[i] - b.e[i];                               \
        return r;                                                                           \
    }                                                                                       \
    inline V operator*(const V& a, const V& b) {                                            \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r.e[i] = a.e[i] * b.e[i];                               \
        return r;                                                                           \
    }                                                                                       \
    inline V operator/(const V& a, const V& b) {                                            \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r.e[i] = a.e[i] / b.e[i];                               \
        return r;                                                                           \
    }                                                                                       \
    inline V operator+(const V& a, float f) { return a + V(f); }                            \
    inline V operator-(const V& a, float f) { return a - V(f); }                            \
    inline V operator*(const V& a, float f) { return a * V(f); }                            \
    inline V operator/(const V& a, float f) { return a / V(f); }                            \
    inline V operator+(float f, const V& a) { return V(f) + a; }                            \
    inline V operator-(float f, const V& a) { return V(f) - a; }                            \
    inline V operator*(float f, const V& a) { return V(f) * a; }                            \
    inline V operator/(float f, const V& a) { return V(f) / a; }                            \
    inline V operator-(const V& a) {                                                        \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r.e[i] = -a.e[i];                                       \
        return r;                                                                           \
    }                                                                                       \
    inline V& operator+=(V& a, const V& b) { return a = a + b; }                            \
    inline V& operator-=(V& a, const V& b) { return a = a - b; }                            \
    inline V& operator*=(V& a, const V& b) { return a = a * b; }                            \
    inline V& operator/=(V& a, const V& b) { return a = a / b; }                            \
    inline V& operator+=(V& a, float f) { return a = a + f; }                               \
    inline V& operator-=(V& a, float f) { return a = a - f; }                               \
    inline V& operator*=(V& a, float f) { return a = a * f; }                               \
    inline V& operator/=(V& a, float f) { return a = a / f; }                               \
    inline float dot(const V& a, const V& b) {                                              \
        float s = a.e[0] * b.e[0];                                                          \
        for (int i = 1; i < N; ++i) s = s + a.e[i] * b.e[i];                                \
        return s;                                                                           \
    }                                                                                       \
    inline V normalize(const V& a) { return a * (1.0f / std::sqrt(dot(a, a))); }
GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)
#undef GLSL_VEC_OPS

#define GLSL_SWZ_OP(OP, ARG)                                 \
    template <int S, int... I>                               \
    swz<S, I...>& swz<S, I...>::operator OP##=(ARG v) {      \
        return *this = V(*this) OP v;                        \
    }
GLSL_SWZ_OP(+, const V&)
GLSL_SWZ_OP(-, const V&)
GLSL_SWZ_OP(*, const V&)
GLSL_SWZ_OP(/, const V&)
GLSL_SWZ_OP(+, float)
GLSL_SWZ_OP(-, float)
GLSL_SWZ_OP(*, float)
GLSL_SWZ_OP(/, float)
#undef GLSL_SWZ_OP

// ---- matrices (column-major) ------------------------------------------------
struct mat3 {
    vec3 c[3];
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, const vec3& v) {
    vec3 r;
    for (int i = 0; i < 3; ++i) r.e[i] = (m.c[0].e[i] * v.e[0] + m.c[1].e[i] * v.e[1]) + m.c[2].e[i] * v.e[2];
    return r;
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r.e[i] = ((m.c[0].e[i] * v.e[0] + m.c[1].e[i] * v.e[1]) + m.c[2].e[i] * v.e[2]) + m.c[3].e[i] * v.e[3];
    return r;
}

// ---- built-ins ---------------------------------------------------------------
inline float abs(float x) { return std::fabs(x); }
inline float floor(float x) { return std::floor(x); }
inline float fract(float x) { return x - std::floor(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float exp(float x) { return std::exp(x); }
inline float log2(float x) { return std::log2(x); }
inline float max(float x, float y) { return x < y ? y : x; }
inline float min(float x, float y) { return y < x ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float mod(float x, float y) { return x - y * std::floor(x / y); }
// pow(x, 3) as x * x * x (PhongShading.frag's 0.3 * shininess), else the C library's
inline float pow(float x, float y) { return y == 3.0f ? (x * x) * x : std::pow(x, y); }

#define GLSL_VEC_FUNCS(V, N)                                                               \
    inline V abs(const V& a) {                                                             \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = abs(a.e[i]);                                  \
        return r;                                                                          \
    }                                                                                      \
    inline V floor(const V& a) {                                                           \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = floor(a.e[i]);                                \
        return r;                                                                          \
    }                                                                                      \
    inline V fract(const V& a) {                                                           \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = fract(a.e[i]);                                \
        return r;                                                                          \
    }                                                                                      \
    inline V max(const V& a, const V& b) {                                                 \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = max(a.e[i], b.e[i]);                          \
        return r;                                                                          \
    }                                                                                      \
    inline V min(const V& a, const V& b) {                                                 \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = min(a.e[i], b.e[i]);                          \
        return r;                                                                          \
    }                                                                                      \
    inline V max(const V& a, float b) { return max(a, V(b)); }                             \
    inline V min(const V& a, float b) { return min(a, V(b)); }                             \
    inline V clamp(const V& a, float lo, float hi) { return min(max(a, V(lo)), V(hi)); }   \
    inline V mix(const V& x, const V& y, float t) {                                        \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = mix(x.e[i], y.e[i], t);                       \
        return r;                                                                          \
    }                                                                                      \
    inline V mix(const V& x, const V& y, const V& t) {                                     \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = mix(x.e[i], y.e[i], t.e[i]);                  \
        return r;                                                                          \
    }                                                                                      \
    inline V step(const V& e, const V& x) {                                                \
        V r;                                                                               \
        for (int i = 0; i < N; ++i) r.e[i] = step(e.e[i], x.e[i]);                         \
        return r;                                                                          \
    }                                                                                      \
    inline V step(float e, const V& x) { return step(V(e), x); }
GLSL_VEC_FUNCS(vec2, 2)
GLSL_VEC_FUNCS(vec3, 3)
GLSL_VEC_FUNCS(vec4, 4)
#undef GLSL_VEC_FUNCS

inline vec3 reflect(const vec3& i, const vec3& n) { return i - (2.0f * dot(n, i)) * n; }

// ---- textures ----------------------------------------------------------------
struct sampler2D {
    const float* data = nullptr;
    int w = 0, h = 0, channels = 1;
    bool linear = false;  // bilinear at level 0 (the moment maps), else NEAREST
};

inline vec4 texel(const sampler2D& s, int i, int j) {
    if (i < 0 || i >= s.w || j < 0 || j >= s.h) return vec4(0.0f);
    const float* t = s.data + ((size_t)j * s.w + i) * s.channels;
    if (s.channels == 1) return vec4(t[0], t[0], t[0], 1.0f);
    return vec4(t[0], t[1], t[2], t[3]);
}

inline vec4 texture2D(const sampler2D& s, const vec2& uv) {
    if (s.linear) {  // float32 weights, zero border
        const float u = uv.e[0] * (float)s.w - 0.5f, v = uv.e[1] * (float)s.h - 0.5f;
        if (!(u > -2.0f && u < (float)s.w + 1.0f && v > -2.0f && v < (float)s.h + 1.0f)) return vec4(0.0f);
        const float fu = std::floor(u), fv = std::floor(v);
        const int i0 = (int)fu, j0 = (int)fv;
        const float a = u - fu, b = v - fv;
        const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
        const vec4 t0 = texel(s, i0, j0), t1 = texel(s, i0 + 1, j0), t2 = texel(s, i0, j0 + 1),
                   t3 = texel(s, i0 + 1, j0 + 1);
        vec4 r;
        for (int k = 0; k < 4; ++k) r.e[k] = ((w00 * t0.e[k] + w10 * t1.e[k]) + w01 * t2.e[k]) + w11 * t3.e[k];
        return r;
    }
    const float fi = std::floor(uv.e[0] * (float)s.w), fj = std::floor(uv.e[1] * (float)s.h);
    if (!(fi >= 0.0f && fi < (float)s.w && fj >= 0.0f && fj < (float)s.h)) return vec4(0.0f);
    const float* t = s.data + ((size_t)(int)fj * s.w + (int)fi) * s.channels;
    if (s.channels == 1) return vec4(t[0], t[0], t[0], 1.0f);
    return vec4(t[0], t[1], t[2], t[3]);
}
inline vec4 texture(const sampler2D& s, const vec2& uv) { return texture2D(s, uv); }
inline vec4 texture2DLod(const sampler2D& s, const vec2& uv, float) { return texture2D(s, uv); }
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2{s.w, s.h}; }

}  // namespace glsl
