// Host-side FP32 vector / matrix helpers with the operation order of the
// glm 0.9.3 functions the reference calls (vendored under
// ShadowMapping/include/glm).  The order matters because every matrix the
// passes use is built here, and the results are pinned against glm itself
// by the test suite.  This file must be compiled with -ffp-contract=off so
// that no multiply-add is fused.
#pragma once

#include <cmath>
#include <cstring>

namespace gi {

struct V3 {
    float x, y, z;
};

struct M4 {  // column-major: m[c][r]
    float m[4][4];
};

struct M3 {
    float m[3][3];
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 scale(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }

// glm::dot(vec3): x*x + y*y + z*z, left to right.
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// glm::cross (core/func_geometric.inl).
inline V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}

// glm::normalize(vec3): v * inversesqrt(dot(v, v)), inversesqrt = 1 / sqrt.
inline V3 normalize(V3 a) {
    float sqr = a.x * a.x + a.y * a.y + a.z * a.z;
    float inv = 1.0f / std::sqrt(sqr);
    return scale(a, inv);
}

// glm::radians: degrees * (pi / 180) with pi rounded to the value type.
inline float radians(float deg) {
    const float pi = (float)3.1415926535897932384626433832795;
    return deg * (pi / 180.0f);
}

inline M4 identity4() {
    M4 r;
    std::memset(&r, 0, sizeof(r));
    for (int i = 0; i < 4; ++i) r.m[i][i] = 1.0f;
    return r;
}

// glm mat4 * mat4: column j of the result is
// A[0]*B[j][0] + A[1]*B[j][1] + A[2]*B[j][2] + A[3]*B[j][3], left to right.
inline M4 mul(const M4& a, const M4& b) {
    M4 r;
    for (int j = 0; j < 4; ++j)
        for (int row = 0; row < 4; ++row)
            r.m[j][row] = a.m[0][row] * b.m[j][0] + a.m[1][row] * b.m[j][1] +
                          a.m[2][row] * b.m[j][2] + a.m[3][row] * b.m[j][3];
    return r;
}

// glm mat3 * vec3.
inline V3 mul3(const M3& m, V3 v) {
    return V3{m.m[0][0] * v.x + m.m[1][0] * v.y + m.m[2][0] * v.z,
              m.m[0][1] * v.x + m.m[1][1] * v.y + m.m[2][1] * v.z,
              m.m[0][2] * v.x + m.m[1][2] * v.y + m.m[2][2] * v.z};
}

inline M3 upper3(const M4& a) {
    M3 r;
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row) r.m[c][row] = a.m[c][row];
    return r;
}

// glm::translate(m, v): column 3 becomes m[0]*v.x + m[1]*v.y + m[2]*v.z + m[3].
inline M4 translate(const M4& m, V3 v) {
    M4 r = m;
    for (int row = 0; row < 4; ++row)
        r.m[3][row] = m.m[0][row] * v.x + m.m[1][row] * v.y + m.m[2][row] * v.z +
                      m.m[3][row];
    return r;
}

// glm::rotate(m, angle_degrees, axis) (gtc/matrix_transform.inl).
inline M4 rotate(const M4& m, float angle_deg, V3 v) {
    float a = radians(angle_deg);
    float c = std::cos(a);
    float s = std::sin(a);
    V3 axis = normalize(v);
    // glm multiplies scalar * vec: (T(1) - c) * axis, componentwise.
    V3 temp = V3{(1.0f - c) * axis.x, (1.0f - c) * axis.y, (1.0f - c) * axis.z};
    float R[3][3];
    R[0][0] = c + temp.x * axis.x;
    R[0][1] = 0 + temp.x * axis.y + s * axis.z;
    R[0][2] = 0 + temp.x * axis.z - s * axis.y;
    R[1][0] = 0 + temp.y * axis.x - s * axis.z;
    R[1][1] = c + temp.y * axis.y;
    R[1][2] = 0 + temp.y * axis.z + s * axis.x;
    R[2][0] = 0 + temp.z * axis.x + s * axis.y;
    R[2][1] = 0 + temp.z * axis.y - s * axis.x;
    R[2][2] = c + temp.z * axis.z;
    M4 r;
    for (int j = 0; j < 3; ++j)
        for (int row = 0; row < 4; ++row)
            r.m[j][row] = m.m[0][row] * R[j][0] + m.m[1][row] * R[j][1] +
                          m.m[2][row] * R[j][2];
    for (int row = 0; row < 4; ++row) r.m[3][row] = m.m[3][row];
    return r;
}

inline M4 transpose(const M4& a) {
    M4 r;
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) r.m[c][row] = a.m[row][c];
    return r;
}

// glm::perspective(fovy_degrees, aspect, zNear, zFar).
inline M4 perspective(float fovy, float aspect, float zn, float zf) {
    float range = std::tan(radians(fovy / 2.0f)) * zn;
    float left = -range * aspect;
    float right = range * aspect;
    float bottom = -range;
    float top = range;
    M4 r;
    std::memset(&r, 0, sizeof(r));
    r.m[0][0] = (2.0f * zn) / (right - left);
    r.m[1][1] = (2.0f * zn) / (top - bottom);
    r.m[2][2] = -(zf + zn) / (zf - zn);
    r.m[2][3] = -1.0f;
    r.m[3][2] = -(2.0f * zf * zn) / (zf - zn);
    return r;
}

// glm::lookAt(eye, center, up).
inline M4 look_at(V3 eye, V3 center, V3 up) {
    V3 f = normalize(sub(center, eye));
    V3 u = normalize(up);
    V3 s = normalize(cross(f, u));
    u = cross(s, f);
    M4 r = identity4();
    r.m[0][0] = s.x;
    r.m[1][0] = s.y;
    r.m[2][0] = s.z;
    r.m[0][1] = u.x;
    r.m[1][1] = u.y;
    r.m[2][1] = u.z;
    r.m[0][2] = -f.x;
    r.m[1][2] = -f.y;
    r.m[2][2] = -f.z;
    return translate(r, neg(eye));
}

// glm::inverseTranspose(mat3) (gtc/matrix_inverse.inl).
inline M3 inverse_transpose3(const M3& a) {
    const float(*m)[3] = a.m;
    float det = +m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    M3 r;
    r.m[0][0] = +(m[1][1] * m[2][2] - m[2][1] * m[1][2]);
    r.m[0][1] = -(m[1][0] * m[2][2] - m[2][0] * m[1][2]);
    r.m[0][2] = +(m[1][0] * m[2][1] - m[2][0] * m[1][1]);
    r.m[1][0] = -(m[0][1] * m[2][2] - m[2][1] * m[0][2]);
    r.m[1][1] = +(m[0][0] * m[2][2] - m[2][0] * m[0][2]);
    r.m[1][2] = -(m[0][0] * m[2][1] - m[2][0] * m[0][1]);
    r.m[2][0] = +(m[0][1] * m[1][2] - m[1][1] * m[0][2]);
    r.m[2][1] = -(m[0][0] * m[1][2] - m[1][0] * m[0][2]);
    r.m[2][2] = +(m[0][0] * m[1][1] - m[1][0] * m[0][1]);
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row) r.m[c][row] /= det;
    return r;
}

inline void store4(const M4& a, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) out[c * 4 + row] = a.m[c][row];
}

inline M4 load4(const float* in) {
    M4 r;
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) r.m[c][row] = in[c * 4 + row];
    return r;
}

inline void store3(const M3& a, float* out) {
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 3; ++row) out[c * 3 + row] = a.m[c][row];
}

}  // namespace gi
