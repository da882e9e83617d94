// Scene layer: Configs/*.txt grammar, Wavefront OBJ reader, Mesh operations
// and the procedural generators of the synthetic benchmark scenes.
//
// Reference behaviour restated here (paths relative to the reference root):
//   SceneLoader::load          ShadowMapping/src/IO/SceneLoader.cpp:11-94
//                              (+ ha/hb: SoftShadowMapping/src/IO/SceneLoader.cpp:93-97)
//   glmFirstPass/SecondPass    ShadowMapping/src/IO/OBJLoader.cpp:441-776
//   Mesh::loadOBJFile          ShadowMapping/src/Mesh.cpp:251-313
//   Mesh::computeNormals       ShadowMapping/src/Mesh.cpp:195-234
//   Mesh::scale/translate/rotate  ShadowMapping/src/Mesh.cpp:378-429
//   Mesh::addObject            ShadowMapping/src/Mesh.cpp:47-193
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "host_math.h"
#include "internal.h"

namespace gi {

// ---------------------------------------------------------------------------
// Mesh operations
// ---------------------------------------------------------------------------

void compute_normals(Mesh& m) {
    alloc_point();
    const int nv = m.num_vertices();
    if ((int)m.normals.size() != 3 * nv) m.normals.assign(3 * (size_t)nv, 0.0f);
    std::vector<int> nb_seen(nv, 0);
    const float* p = m.points.data();
    for (size_t i = 0; i + 2 < m.indices.size(); i += 3) {
        int a = m.indices[i + 0], b = m.indices[i + 1], c = m.indices[i + 2];
        V3 pa = v3(p[a * 3 + 0], p[a * 3 + 1], p[a * 3 + 2]);
        V3 pb = v3(p[b * 3 + 0], p[b * 3 + 1], p[b * 3 + 2]);
        V3 pc = v3(p[c * 3 + 0], p[c * 3 + 1], p[c * 3 + 2]);
        V3 n = normalize(cross(sub(pb, pa), sub(pc, pa)));
        int v[3] = {a, b, c};
        for (int j = 0; j < 3; ++j) {
            int cur = v[j];
            nb_seen[cur]++;
            float* nv3 = &m.normals[(size_t)cur * 3];
            if (nb_seen[cur] == 1) {
                nv3[0] = n.x;
                nv3[1] = n.y;
                nv3[2] = n.z;
            } else {
                // The reference averages in double: float * (1.0 - 1.0/k)
                // + float * 1.0 / k, then stores to float.
                double k = (double)nb_seen[cur];
                double keep = 1.0 - 1.0 / k;
                nv3[0] = (float)((double)nv3[0] * keep + ((double)n.x * 1.0) / k);
                nv3[1] = (float)((double)nv3[1] * keep + ((double)n.y * 1.0) / k);
                nv3[2] = (float)((double)nv3[2] * keep + ((double)n.z * 1.0) / k);
            }
        }
    }
}

void mesh_scale(Mesh& m, float x, float y, float z) {
    for (size_t i = 0; i + 2 < m.points.size(); i += 3) {
        m.points[i + 0] *= x;
        m.points[i + 1] *= y;
        m.points[i + 2] *= z;
    }
}

void mesh_translate(Mesh& m, float x, float y, float z) {
    for (size_t i = 0; i + 2 < m.points.size(); i += 3) {
        m.points[i + 0] += x;
        m.points[i + 1] += y;
        m.points[i + 2] += z;
    }
}

void mesh_rotate(Mesh& m, float x, float y, float z) {
    M4 r = rotate(identity4(), x, v3(1, 0, 0));
    r = mul(r, rotate(identity4(), y, v3(0, 1, 0)));
    r = mul(r, rotate(identity4(), z, v3(0, 0, 1)));
    M4 t = transpose(r);
    const size_t n = m.points.size();
    if (m.normals.size() != n) m.normals.assign(n, 0.0f);
    for (size_t i = 0; i + 2 < n; i += 3) {
        float px = m.points[i], py = m.points[i + 1], pz = m.points[i + 2];
        float rx = px * t.m[0][0] + py * t.m[0][1] + pz * t.m[0][2];
        float ry = px * t.m[1][0] + py * t.m[1][1] + pz * t.m[1][2];
        float rz = px * t.m[2][0] + py * t.m[2][1] + pz * t.m[2][2];
        m.points[i] = rx;
        m.points[i + 1] = ry;
        m.points[i + 2] = rz;
        float nx = m.normals[i], ny = m.normals[i + 1], nz = m.normals[i + 2];
        rx = nx * t.m[0][0] + ny * t.m[0][1] + nz * t.m[0][2];
        ry = nx * t.m[1][0] + ny * t.m[1][1] + nz * t.m[1][2];
        rz = nx * t.m[2][0] + ny * t.m[2][1] + nz * t.m[2][2];
        m.normals[i] = rx;
        m.normals[i + 1] = ry;
        m.normals[i + 2] = rz;
    }
}

void mesh_append(Mesh& dst, const Mesh& src) {
    alloc_point();
    // Reserve everything first: if an allocation fails, dst is unchanged.
    dst.points.reserve(dst.points.size() + src.points.size());
    dst.normals.reserve(dst.points.size() + src.points.size());
    dst.indices.reserve(dst.indices.size() + src.indices.size());
    const int offset = dst.num_vertices();
    dst.points.insert(dst.points.end(), src.points.begin(), src.points.end());
    if (src.normals.size() == src.points.size())
        dst.normals.insert(dst.normals.end(), src.normals.begin(), src.normals.end());
    else
        dst.normals.resize(dst.points.size(), 0.0f);
    dst.indices.reserve(dst.indices.size() + src.indices.size());
    for (int idx : src.indices) dst.indices.push_back(idx + offset);
}

// ---------------------------------------------------------------------------
// Wavefront OBJ reader with the token semantics of glm.c's fscanf loop
// ---------------------------------------------------------------------------
namespace {

struct Scanner {
    const char* s;
    size_t n;
    size_t pos = 0;

    bool at_end() const { return pos >= n; }
    void skip_ws() {
        while (pos < n && (s[pos] == ' ' || s[pos] == '\t' || s[pos] == '\n' ||
                           s[pos] == '\r' || s[pos] == '\v' || s[pos] == '\f'))
            ++pos;
    }
    // fscanf("%s"): next whitespace-delimited token; false at EOF.
    bool token(std::string& out) {
        skip_ws();
        if (pos >= n) return false;
        size_t b = pos;
        while (pos < n && !(s[pos] == ' ' || s[pos] == '\t' || s[pos] == '\n' ||
                            s[pos] == '\r' || s[pos] == '\v' || s[pos] == '\f'))
            ++pos;
        out.assign(s + b, pos - b);
        return true;
    }
    // fgets(buf, 128, file) used to "eat up the rest of the line".
    void rest_of_line() {
        while (pos < n && s[pos] != '\n') ++pos;
        if (pos < n) ++pos;
    }
    // %d with leading-whitespace skip; false (nothing consumed) on mismatch.
    bool read_int(int& v) {
        size_t save = pos;
        skip_ws();
        size_t b = pos;
        if (pos < n && (s[pos] == '+' || s[pos] == '-')) ++pos;
        size_t digits = pos;
        while (pos < n && s[pos] >= '0' && s[pos] <= '9') ++pos;
        if (pos == digits) {
            pos = save;
            return false;
        }
        v = (int)std::strtol(std::string(s + b, pos - b).c_str(), nullptr, 10);
        return true;
    }
    bool literal(char c) {
        if (pos < n && s[pos] == c) {
            ++pos;
            return true;
        }
        return false;
    }
    // %f: strtof on the text after leading whitespace.
    bool read_float(float& v) {
        skip_ws();
        if (pos >= n) return false;
        // strtof needs a terminated string; copy the token-sized run.
        size_t b = pos, e = pos;
        while (e < n && !(s[e] == ' ' || s[e] == '\t' || s[e] == '\n' || s[e] == '\r'))
            ++e;
        std::string tok(s + b, e - b);
        char* end = nullptr;
        float f = std::strtof(tok.c_str(), &end);
        if (end == tok.c_str()) return false;
        pos = b + (size_t)(end - tok.c_str());
        v = f;
        return true;
    }
    // The four face formats; returns the number of conversions made, as
    // fscanf does.
    int face_vn(int& v, int& nn) {  // %d//%d
        if (!read_int(v)) return 0;
        if (!literal('/') || !literal('/')) return 1;
        return read_int(nn) ? 2 : 1;
    }
    int face_vtn(int& v, int& t, int& nn) {  // %d/%d/%d
        if (!read_int(v)) return 0;
        if (!literal('/')) return 1;
        if (!read_int(t)) return 1;
        if (!literal('/')) return 2;
        return read_int(nn) ? 3 : 2;
    }
    int face_vt(int& v, int& t) {  // %d/%d
        if (!read_int(v)) return 0;
        if (!literal('/')) return 1;
        return read_int(t) ? 2 : 1;
    }
};

// sscanf on a token for the format probe of glmFirstPass/SecondPass.
int probe_vtn(const std::string& tok) {
    Scanner sc{tok.c_str(), tok.size()};
    int a, b, c;
    return sc.face_vtn(a, b, c);
}
int probe_vt(const std::string& tok) {
    Scanner sc{tok.c_str(), tok.size()};
    int a, b;
    return sc.face_vt(a, b);
}

}  // namespace

gi_status read_obj(const char* path, Mesh& out) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return fail(GI_ERR_IO, std::string("can't open OBJ file \"") + path + "\"");
    try {
        alloc_point();
    } catch (...) {
        std::fclose(f);
        throw;
    }
    std::string data;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.append(buf, got);
    std::fclose(f);

    // glm.c keeps vertices 1-based; index 0 is unused.
    std::vector<float> verts(3, 0.0f), norms(3, 0.0f);
    std::vector<int> tri_v;  // 1-based (or relative-resolved) vertex indices
    int numvertices = 1, numnormals = 1;
    Scanner sc{data.c_str(), data.size()};
    std::string tok;
    while (sc.token(tok)) {
        switch (tok[0]) {
            case '#':
                sc.rest_of_line();
                break;
            case 'v':
                if (tok.size() == 1) {
                    float x = 0, y = 0, z = 0;
                    if (!sc.read_float(x) || !sc.read_float(y) || !sc.read_float(z))
                        return fail(GI_ERR_PARSE, std::string("bad vertex in ") + path);
                    verts.push_back(x);
                    verts.push_back(y);
                    verts.push_back(z);
                    numvertices++;
                } else if (tok[1] == 'n' && tok.size() == 2) {
                    float x = 0, y = 0, z = 0;
                    if (!sc.read_float(x) || !sc.read_float(y) || !sc.read_float(z))
                        return fail(GI_ERR_PARSE, std::string("bad normal in ") + path);
                    norms.push_back(x);
                    norms.push_back(y);
                    norms.push_back(z);
                    numnormals++;
                } else if (tok[1] == 't' && tok.size() == 2) {
                    float u = 0, v = 0;
                    sc.read_float(u);
                    sc.read_float(v);
                } else {
                    // glmFirstPass: "Unknown token" then exit(1).
                    return fail(GI_ERR_PARSE,
                                "unknown token \"" + tok + "\" in " + std::string(path));
                }
                break;
            case 'f': {
                std::string first;
                if (!sc.token(first))
                    return fail(GI_ERR_PARSE, std::string("truncated face in ") + path);
                auto resolve = [&](int v) { return v < 0 ? v + numvertices : v; };
                int v = 0, t = 0, nn = 0;
                int fmt;  // 0: v//n, 1: v/t/n, 2: v/t, 3: v
                if (first.find("//") != std::string::npos) fmt = 0;
                else if (probe_vtn(first) == 3) fmt = 1;
                else if (probe_vt(first) == 2) fmt = 2;
                else fmt = 3;
                Scanner fs{first.c_str(), first.size()};
                int v0 = 0;
                if (fmt == 0) fs.face_vn(v, nn);
                else if (fmt == 1) fs.face_vtn(v, t, nn);
                else if (fmt == 2) fs.face_vt(v, t);
                else fs.read_int(v);
                v0 = resolve(v);
                auto next = [&](int& vv) -> bool {
                    if (fmt == 0) return sc.face_vn(vv, nn) > 0;
                    if (fmt == 1) return sc.face_vtn(vv, t, nn) > 0;
                    if (fmt == 2) return sc.face_vt(vv, t) > 0;
                    return sc.read_int(vv);
                };
                // The reference reads the 2nd and 3rd corner without checking
                // the fscanf result (the previous value is kept on failure).
                next(v);
                int v1 = resolve(v);
                next(v);
                int v2 = resolve(v);
                tri_v.push_back(v0);
                tri_v.push_back(v1);
                tri_v.push_back(v2);
                while (next(v)) {
                    int a = tri_v[tri_v.size() - 3];
                    int c = tri_v[tri_v.size() - 1];
                    tri_v.push_back(a);
                    tri_v.push_back(c);
                    tri_v.push_back(resolve(v));
                }
                break;
            }
            default:
                // mtllib, usemtl, g, s, o and anything else: rest of line.
                sc.rest_of_line();
                break;
        }
    }
    const int nv = numvertices - 1;
    out.points.assign(verts.begin() + 3, verts.end());
    out.normals.assign(3 * (size_t)nv, 0.0f);
    // Mesh::loadOBJFile copies OBJ normal i+1 to vertex i when normals exist.
    for (int i = 0; i < nv && i + 1 < numnormals; ++i)
        for (int k = 0; k < 3; ++k) out.normals[i * 3 + k] = norms[(i + 1) * 3 + k];
    out.indices.resize(tri_v.size());
    for (size_t i = 0; i < tri_v.size(); ++i) {
        int idx = tri_v[i] - 1;
        if (idx < 0 || idx >= nv)
            return fail(GI_ERR_PARSE, std::string("face index out of range in ") + path);
        out.indices[i] = idx;
    }
    return GI_OK;
}

// ---------------------------------------------------------------------------
// Procedural generators
// ---------------------------------------------------------------------------

// PCG32 (O'Neill, pcg-random.org, XSH-RR output).
struct Pcg32 {
    uint64_t state = 0, inc = 0;
    Pcg32(uint64_t seed, uint64_t seq) {
        inc = (seq << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // Uniform in [0, 1) with 24 random bits.
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
    float uniform(float lo, float hi) { return lo + (hi - lo) * uniform(); }
};

void gen_ground(Mesh& m, float h, float y) {
    m.points = {-h, y, -h, h, y, -h, h, y, h, -h, y, h};
    // Counter-clockwise seen from +y, so computeNormals yields +y.
    m.indices = {0, 2, 1, 0, 3, 2};
    m.normals.clear();
    compute_normals(m);
}

void gen_uv_grid_sphere(Mesh& m, int slices, int stacks, float radius, const float c[3],
                        const std::vector<float>* radial /* per vertex or null */) {
    m.points.clear();
    m.indices.clear();
    const float pi = 3.14159265358979323846f;
    // north pole, rings 1..stacks-1, south pole
    m.points.insert(m.points.end(), {0.0f, 1.0f, 0.0f});
    for (int i = 1; i < stacks; ++i) {
        float theta = pi * (float)i / (float)stacks;
        float st = std::sin(theta), ct = std::cos(theta);
        for (int j = 0; j < slices; ++j) {
            float phi = 2.0f * pi * (float)j / (float)slices;
            m.points.insert(m.points.end(), {st * std::cos(phi), ct, st * std::sin(phi)});
        }
    }
    m.points.insert(m.points.end(), {0.0f, -1.0f, 0.0f});
    const int nv = m.num_vertices();
    for (int v = 0; v < nv; ++v) {
        float r = radius;
        if (radial) r = (*radial)[v];
        m.points[v * 3 + 0] = m.points[v * 3 + 0] * r + c[0];
        m.points[v * 3 + 1] = m.points[v * 3 + 1] * r + c[1];
        m.points[v * 3 + 2] = m.points[v * 3 + 2] * r + c[2];
    }
    auto ring = [&](int i, int j) { return 1 + (i - 1) * slices + (j % slices); };
    const int south = nv - 1;
    for (int j = 0; j < slices; ++j) {
        // Outward-facing counter-clockwise triangles.
        m.indices.insert(m.indices.end(), {0, ring(1, j + 1), ring(1, j)});
    }
    for (int i = 1; i < stacks - 1; ++i)
        for (int j = 0; j < slices; ++j) {
            int a = ring(i, j), b = ring(i, j + 1), cc = ring(i + 1, j), d = ring(i + 1, j + 1);
            m.indices.insert(m.indices.end(), {a, b, cc, b, d, cc});
        }
    for (int j = 0; j < slices; ++j)
        m.indices.insert(m.indices.end(), {south, ring(stacks - 1, j), ring(stacks - 1, j + 1)});
    m.normals.clear();
    compute_normals(m);
}

void gen_icosphere(Mesh& m, int level, float radius, const float c[3]) {
    const float t = (1.0f + std::sqrt(5.0f)) / 2.0f;
    std::vector<float> p = {-1, t, 0, 1, t, 0, -1, -t, 0, 1, -t, 0, 0, -1, t, 0, 1, t,
                            0, -1, -t, 0, 1, -t, t, 0, -1, t, 0, 1, -t, 0, -1, -t, 0, 1};
    std::vector<int> f = {0, 11, 5, 0, 5,  1, 0, 1, 7, 0, 7,  10, 0, 10, 11,
                          1, 5,  9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
                          3, 9,  4, 3, 4,  2, 3, 2, 6, 3, 6,  8, 3, 8,  9,
                          4, 9,  5, 2, 4,  11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    auto unit = [&](int i) {
        float x = p[i * 3], y = p[i * 3 + 1], z = p[i * 3 + 2];
        float l = std::sqrt(x * x + y * y + z * z);
        p[i * 3] = x / l;
        p[i * 3 + 1] = y / l;
        p[i * 3 + 2] = z / l;
    };
    for (int i = 0; i < 12; ++i) unit(i);
    for (int lv = 0; lv < level; ++lv) {
        std::vector<int> nf;
        std::vector<std::pair<uint64_t, int>> cache;
        auto mid = [&](int a, int b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | (uint32_t)b) : ((uint64_t)b << 32 | (uint32_t)a);
            for (auto& e : cache)
                if (e.first == key) return e.second;
            int idx = (int)(p.size() / 3);
            p.push_back((p[a * 3] + p[b * 3]) * 0.5f);
            p.push_back((p[a * 3 + 1] + p[b * 3 + 1]) * 0.5f);
            p.push_back((p[a * 3 + 2] + p[b * 3 + 2]) * 0.5f);
            unit(idx);
            cache.push_back({key, idx});
            return idx;
        };
        // Per-face midpoint cache keyed linearly is O(F^2); bucket by vertex.
        std::vector<std::vector<std::pair<int, int>>> adj(p.size() / 3 + 3 * f.size());
        auto mid2 = [&](int a, int b) {
            int lo = a < b ? a : b, hi = a < b ? b : a;
            for (auto& e : adj[lo])
                if (e.first == hi) return e.second;
            int idx = (int)(p.size() / 3);
            p.push_back((p[a * 3] + p[b * 3]) * 0.5f);
            p.push_back((p[a * 3 + 1] + p[b * 3 + 1]) * 0.5f);
            p.push_back((p[a * 3 + 2] + p[b * 3 + 2]) * 0.5f);
            unit(idx);
            adj[lo].push_back({hi, idx});
            return idx;
        };
        (void)mid;
        for (size_t i = 0; i < f.size(); i += 3) {
            int a = f[i], b = f[i + 1], cc = f[i + 2];
            int ab = mid2(a, b), bc = mid2(b, cc), ca = mid2(cc, a);
            nf.insert(nf.end(), {a, ab, ca, b, bc, ab, cc, ca, bc, ab, bc, ca});
        }
        f.swap(nf);
    }
    m.points.resize(p.size());
    for (size_t i = 0; i < p.size(); i += 3) {
        m.points[i] = p[i] * radius + c[0];
        m.points[i + 1] = p[i + 1] * radius + c[1];
        m.points[i + 2] = p[i + 2] * radius + c[2];
    }
    m.indices = f;
    m.normals.clear();
    compute_normals(m);
}

// Improved Perlin noise (K. Perlin, "Improving Noise", SIGGRAPH 2002) in
// FP32 with a permutation shuffled by PCG32(seed).
struct Perlin {
    int perm[512];
    explicit Perlin(uint64_t seed) {
        int p[256];
        for (int i = 0; i < 256; ++i) p[i] = i;
        Pcg32 rng(seed, 0x9E3779B97F4A7C15ULL);
        for (int i = 255; i > 0; --i) {
            int j = (int)(rng.next() % (uint32_t)(i + 1));
            int tmp = p[i];
            p[i] = p[j];
            p[j] = tmp;
        }
        for (int i = 0; i < 512; ++i) perm[i] = p[i & 255];
    }
    static float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
    static float lerp(float t, float a, float b) { return a + t * (b - a); }
    static float grad(int hash, float x, float y, float z) {
        int h = hash & 15;
        float u = h < 8 ? x : y;
        float v = h < 4 ? y : (h == 12 || h == 14 ? x : z);
        return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
    }
    float noise(float x, float y, float z) const {
        float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
        int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
        x -= fx;
        y -= fy;
        z -= fz;
        float u = fade(x), v = fade(y), w = fade(z);
        int A = perm[X] + Y, AA = perm[A] + Z, AB = perm[A + 1] + Z;
        int B = perm[X + 1] + Y, BA = perm[B] + Z, BB = perm[B + 1] + Z;
        return lerp(w,
                    lerp(v, lerp(u, grad(perm[AA], x, y, z), grad(perm[BA], x - 1, y, z)),
                         lerp(u, grad(perm[AB], x, y - 1, z), grad(perm[BB], x - 1, y - 1, z))),
                    lerp(v,
                         lerp(u, grad(perm[AA + 1], x, y, z - 1),
                              grad(perm[BA + 1], x - 1, y, z - 1)),
                         lerp(u, grad(perm[AB + 1], x, y - 1, z - 1),
                              grad(perm[BB + 1], x - 1, y - 1, z - 1))));
    }
};

}  // namespace gi

// ---------------------------------------------------------------------------
// C ABI: scene
// ---------------------------------------------------------------------------
using gi::fail;

// Runs an entry point's body, turning a failed host allocation into
// GI_ERR_OOM (the reference exits instead: Mesh.cpp:336-340).  Bodies
// change the scene only after their last allocation, so a failure leaves
// it as it was.
template <class F>
static gi_status guarded(const char* who, F&& body) {
    try {
        return body();
    } catch (const std::bad_alloc&) {
        return fail(GI_ERR_OOM, std::string(who) + ": out of host memory");
    }
}

extern "C" gi_status gi_scene_create(gi_scene** out) {
    if (!out) return fail(GI_ERR_INVALID_ARG, "gi_scene_create: out is NULL");
    try {
        *out = new gi_scene();
    } catch (...) {
        return fail(GI_ERR_OOM, "gi_scene_create: out of host memory");
    }
    return GI_OK;
}

extern "C" gi_status gi_scene_object_load_obj(gi_scene* s, const char* path) {
    return guarded("gi_scene_object_load_obj", [&]() -> gi_status {
        if (!s || !path) return fail(GI_ERR_INVALID_ARG, "gi_scene_object_load_obj: NULL argument");
        gi::Mesh m;
        gi_status st = gi::read_obj(path, m);
        if (st != GI_OK) return st;
        gi::compute_normals(m);
        s->pending = std::move(m);
        s->has_pending = true;
        return GI_OK;
    });
}

extern "C" gi_status gi_scene_object_from_arrays(gi_scene* s, const float* points, int nv,
                                                 const int* indices, int nt) {
    return guarded("gi_scene_object_from_arrays", [&]() -> gi_status {
        if (!s || (nv > 0 && !points) || (nt > 0 && !indices) || nv < 0 || nt < 0)
            return fail(GI_ERR_INVALID_ARG, "gi_scene_object_from_arrays: bad arguments");
        gi::Mesh m;
        m.points.assign(points, points + 3 * (size_t)nv);
        m.indices.assign(indices, indices + 3 * (size_t)nt);
        for (int idx : m.indices)
            if (idx < 0 || idx >= nv)
                return fail(GI_ERR_INVALID_ARG, "gi_scene_object_from_arrays: index out of range");
        gi::compute_normals(m);
        s->pending = std::move(m);
        s->has_pending = true;
        return GI_OK;
    });
}

static gi_status need_pending(gi_scene* s, const char* who) {
    if (!s) return fail(GI_ERR_INVALID_ARG, std::string(who) + ": scene is NULL");
    if (!s->has_pending)
        return fail(GI_ERR_PARSE, std::string(who) + ": no object loaded (config key 'o' missing)");
    return GI_OK;
}

extern "C" gi_status gi_scene_object_scale(gi_scene* s, float x, float y, float z) {
    gi_status st = need_pending(s, "scale");
    if (st != GI_OK) return st;
    gi::mesh_scale(s->pending, x, y, z);
    return GI_OK;
}

extern "C" gi_status gi_scene_object_translate(gi_scene* s, float x, float y, float z) {
    gi_status st = need_pending(s, "translate");
    if (st != GI_OK) return st;
    gi::mesh_translate(s->pending, x, y, z);
    return GI_OK;
}

extern "C" gi_status gi_scene_object_rotate(gi_scene* s, float x, float y, float z) {
    gi_status st = need_pending(s, "rotate");
    if (st != GI_OK) return st;
    gi::mesh_rotate(s->pending, x, y, z);
    return GI_OK;
}

extern "C" gi_status gi_scene_object_commit(gi_scene* s) {
    return guarded("gi_scene_object_commit", [&]() -> gi_status {
        gi_status st = need_pending(s, "commit");
        if (st != GI_OK) return st;
        gi::mesh_append(s->mesh, s->pending);
        if ((size_t)s->mesh.num_triangles() >= ((size_t)1 << 29))
            return fail(GI_ERR_CAPACITY, "scene exceeds 2^29 triangles");
        s->pending = gi::Mesh();
        s->has_pending = false;
        s->num_objects++;
        return GI_OK;
    });
}

extern "C" gi_status gi_scene_set_views(gi_scene* s, const float ce[3], const float ca[3],
                                        const float le[3], const float la[3], float d) {
    if (!s || !ce || !ca || !le || !la) return fail(GI_ERR_INVALID_ARG, "gi_scene_set_views: NULL");
    for (int k = 0; k < 3; ++k) {
        s->camera_eye[k] = ce[k];
        s->camera_at[k] = ca[k];
        s->light_eye[k] = le[k];
        s->light_at[k] = la[k];
    }
    s->depth_threshold = d;
    return GI_OK;
}

extern "C" gi_status gi_scene_get_info(const gi_scene* s, gi_scene_info* out) {
    if (!s || !out) return fail(GI_ERR_INVALID_ARG, "gi_scene_get_info: NULL");
    out->num_vertices = s->mesh.num_vertices();
    out->num_triangles = s->mesh.num_triangles();
    for (int k = 0; k < 3; ++k) {
        out->camera_eye[k] = s->camera_eye[k];
        out->camera_at[k] = s->camera_at[k];
        out->light_eye[k] = s->light_eye[k];
        out->light_at[k] = s->light_at[k];
    }
    out->depth_threshold = s->depth_threshold;
    out->hsm_alpha = s->hsm_alpha;
    out->hsm_beta = s->hsm_beta;
    out->num_objects = s->num_objects;
    return GI_OK;
}

extern "C" gi_status gi_scene_get_arrays(const gi_scene* s, float* p, float* n, int* idx) {
    if (!s) return fail(GI_ERR_INVALID_ARG, "gi_scene_get_arrays: NULL scene");
    if (p) std::memcpy(p, s->mesh.points.data(), s->mesh.points.size() * sizeof(float));
    if (n) std::memcpy(n, s->mesh.normals.data(), s->mesh.normals.size() * sizeof(float));
    if (idx) std::memcpy(idx, s->mesh.indices.data(), s->mesh.indices.size() * sizeof(int));
    return GI_OK;
}

extern "C" gi_status gi_gen_ground(gi_scene* s, float h, float y) {
    return guarded("gi_gen_ground", [&]() -> gi_status {
        if (!s || !(h > 0)) return fail(GI_ERR_INVALID_ARG, "gi_gen_ground: bad arguments");
        gi::alloc_point();
        gi::Mesh m;
        gi::gen_ground(m, h, y);
        s->pending = std::move(m);
        s->has_pending = true;
        return GI_OK;
    });
}

extern "C" gi_status gi_gen_uv_sphere(gi_scene* s, int slices, int stacks, float r,
                                      const float c[3]) {
    return guarded("gi_gen_uv_sphere", [&]() -> gi_status {
        if (!s || !c || slices < 3 || stacks < 2 || !(r > 0))
            return fail(GI_ERR_INVALID_ARG, "gi_gen_uv_sphere: bad arguments");
        gi::alloc_point();
        gi::Mesh m;
        gi::gen_uv_grid_sphere(m, slices, stacks, r, c, nullptr);
        s->pending = std::move(m);
        s->has_pending = true;
        return GI_OK;
    });
}

extern "C" gi_status gi_gen_icosphere(gi_scene* s, int level, float r, const float c[3]) {
    return guarded("gi_gen_icosphere", [&]() -> gi_status {
        if (!s || !c || level < 0 || level > 8 || !(r > 0))
            return fail(GI_ERR_INVALID_ARG, "gi_gen_icosphere: bad arguments");
        gi::alloc_point();
        gi::Mesh m;
        gi::gen_icosphere(m, level, r, c);
        s->pending = std::move(m);
        s->has_pending = true;
        return GI_OK;
    });
}

extern "C" gi_status gi_gen_displaced_sphere(gi_scene* s, int slices, int stacks, float r,
                                             float amp, const float c[3], uint64_t seed) {
    return guarded("gi_gen_displaced_sphere", [&]() -> gi_status {
        if (!s || !c || slices < 3 || stacks < 2 || !(r > 0))
            return fail(GI_ERR_INVALID_ARG, "gi_gen_displaced_sphere: bad arguments");
        // Radius per vertex: r + amp * noise(2 * unit direction), evaluated on
        // the same unit directions the UV grid uses.
        gi::Mesh unit;
        const float zero[3] = {0, 0, 0};
        gi::gen_uv_grid_sphere(unit, slices, stacks, 1.0f, zero, nullptr);
        gi::Perlin noise(seed);
        std::vector<float> radial(unit.num_vertices());
        for (int v = 0; v < unit.num_vertices(); ++v) {
            float x = unit.points[v * 3], y = unit.points[v * 3 + 1], z = unit.points[v * 3 + 2];
            radial[v] = r + amp * noise.noise(2.0f * x + 17.0f, 2.0f * y + 17.0f, 2.0f * z + 17.0f);
        }
        gi::alloc_point();
        gi::Mesh m;
        gi::gen_uv_grid_sphere(m, slices, stacks, r, c, &radial);
        s->pending = std::move(m);
        s->has_pending = true;
        return GI_OK;
    });
}

extern "C" gi_status gi_gen_icosphere_field(gi_scene* s, int count, int level, const float lo[3],
                                            const float hi[3], float rmin, float rmax,
                                            uint64_t seed) {
    return guarded("gi_gen_icosphere_field", [&]() -> gi_status {
        if (!s || !lo || !hi || count < 0 || level < 0 || level > 8 || !(rmin > 0) || rmax < rmin)
            return fail(GI_ERR_INVALID_ARG, "gi_gen_icosphere_field: bad arguments");
        gi::Pcg32 rng(seed, 54u);
        // The spheres are built into one mesh first and committed together,
        // as `count` objects: a failed allocation leaves the scene unchanged.
        gi::Mesh field, sphere;
        for (int i = 0; i < count; ++i) {
            float c[3];
            for (int k = 0; k < 3; ++k) c[k] = rng.uniform(lo[k], hi[k]);
            float r = rng.uniform(rmin, rmax);
            gi::gen_icosphere(sphere, level, r, c);
            gi::mesh_append(field, sphere);
        }
        if ((size_t)s->mesh.num_triangles() + (size_t)field.num_triangles() >= ((size_t)1 << 29))
            return fail(GI_ERR_CAPACITY, "scene exceeds 2^29 triangles");
        gi::mesh_append(s->mesh, field);
        s->num_objects += count;
        s->pending = gi::Mesh();  // each sphere was the pending object once, then committed
        s->has_pending = false;
        return GI_OK;
    });
}

// ---------------------------------------------------------------------------
// Config loader (SceneLoader::load)
// ---------------------------------------------------------------------------
static std::string join_path(const char* base, const std::string& rel) {
    if (!base || !*base || (!rel.empty() && rel[0] == '/')) return rel;
    std::string b(base);
    if (b.back() != '/') b += '/';
    // The reference's configs use '/' separators already; accept '\\' too.
    std::string r = rel;
    for (char& ch : r)
        if (ch == '\\') ch = '/';
    return b + r;
}

extern "C" gi_status gi_scene_load_config(const char* cfg_path, const char* base_dir,
                                          gi_scene** out) {
    return guarded("gi_scene_load_config", [&]() -> gi_status {
        if (!cfg_path || !out) return fail(GI_ERR_INVALID_ARG, "gi_scene_load_config: NULL");
        std::ifstream file(cfg_path);
        if (!file.is_open())
            return fail(GI_ERR_IO, std::string("can't open config \"") + cfg_path + "\"");
        gi_scene* s = nullptr;
        gi_status st = gi_scene_create(&s);
        if (st != GI_OK) return st;
        // `key` and `value` live across lines as in the reference: a blank line
        // leaves both unchanged and repeats the previous key's action with the
        // previous value.
        std::string line, key, value;
        auto val = [&](std::istringstream& split) {
            split >> value;
            return (float)std::atof(value.c_str());
        };
        while (!file.eof()) {
            std::getline(file, line);
            std::istringstream split(line);
            split >> key;
            if (key.empty()) continue;
            const char k0 = key[0];
            const char k1 = key.size() > 1 ? key[1] : '\0';
            st = GI_OK;
            if (k0 == 'o') {
                split >> value;
                st = gi_scene_object_load_obj(s, join_path(base_dir, value).c_str());
            } else if (k0 == 'm') {
                split >> value;  // texture image: not on the visibility path
            } else if (k0 == 's') {
                float v[3];
                for (int a = 0; a < 3; ++a) v[a] = val(split);
                st = gi_scene_object_scale(s, v[0], v[1], v[2]);
            } else if (k0 == 't') {
                float v[3];
                for (int a = 0; a < 3; ++a) v[a] = val(split);
                st = gi_scene_object_translate(s, v[0], v[1], v[2]);
            } else if (k0 == 'r') {
                float v[3];
                for (int a = 0; a < 3; ++a) v[a] = val(split);
                st = gi_scene_object_rotate(s, v[0], v[1], v[2]);
            } else if (k0 == '+') {
                if (line.find('+') != std::string::npos) {
                    st = gi_scene_object_commit(s);
                } else if (!file.eof()) {
                    // A blank line after '+' makes the reference commit the object
                    // it has just deleted (use after free); refuse it.  The empty
                    // read at end of file that `while (!eof)` produces after a
                    // final "+\n" is skipped instead.
                    st = fail(GI_ERR_PARSE, "blank line after '+' repeats a commit");
                }
            } else if (k0 == 'v') {
                for (int a = 0; a < 3; ++a) {
                    float f = val(split);
                    if (k1 == 'e') s->camera_eye[a] = f;
                    else s->camera_at[a] = f;
                }
            } else if (k0 == 'l') {
                for (int a = 0; a < 3; ++a) {
                    float f = val(split);
                    if (k1 == 'e') s->light_eye[a] = f;
                    else s->light_at[a] = f;
                }
            } else if (k0 == 'c') {
                // colours (c r g b / cf obj): not on the visibility path
            } else if (k0 == 'd') {
                s->depth_threshold = val(split);
            } else if (k0 == 'h') {
                float f = val(split);
                if (k1 == 'a') s->hsm_alpha = f;
                else s->hsm_beta = f;
            }
            if (st != GI_OK) {
                gi_scene_destroy(s);
                return st;
            }
        }
        *out = s;
        return GI_OK;
    });
}
