// ref_glm_pin.cpp -- prints the matrices the reference builds for a frame,
// computed with the reference's own vendored glm 0.9.3 headers
// (ShadowMapping/include/glm).  Test infrastructure: built into
// oracle/_ref/ by oracle/build_oracle.py only where the reference tree is
// present, and used by tests/golden/make_glm_golden.py to pin the
// product's matrix code bit for bit.
//
// The composition follows the reference's frame:
//   configureAmbient   projection = perspective(fov, (GLfloat)w / h, n, f),
//                      view = lookAt(eye, look, up), model = mat4(1)
//                      (ShadowMapping/src/Viewers/MyGLGeometryViewer.cpp:14-26)
//   model *= translate(0); model *= rotate(0, x); ... (main.cpp:255-260)
//   lightMVP = projection * view * model (main.cpp:264)
//   bias * lightMVP (MyGLGeometryViewer.cpp:139-145)
//   normalMatrix = inverseTranspose(mat3(view * model)) (:108-117)
//   lightEye = mat3(rotate(180, (0, 1, 0))) * lightEye (main.cpp:283)
//   Mesh::rotate's matrix: transpose(rotate(x, X) * rotate(y, Y) * rotate(z, Z))
//   Mesh::computeNormals' face normal: normalize(cross(b - a, c - a))
//
// Input (stdin), one record per line:
//   F lex ley lez lax lay laz lfov lw lh cex cey cez cax cay caz cfov cw ch
//   R ax ay az
//   N ax ay az bx by bz cx cy cz
// Output: one JSON object per input line with every float as its IEEE-754
// bit pattern in hex.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>

#include <glm/glm.hpp>
#include <glm/gtc/matrix_inverse.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <glm/gtx/transform.hpp>

static unsigned bits(float f) {
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}

static void put_m4(const char* name, const glm::mat4& m, bool comma = true) {
    std::printf("\"%s\": [", name);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) std::printf("\"%08x\"%s", bits(m[c][r]), (c == 3 && r == 3) ? "" : ", ");
    std::printf("]%s", comma ? ", " : "");
}

static void put_m3(const char* name, const glm::mat3& m, bool comma = true) {
    std::printf("\"%s\": [", name);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) std::printf("\"%08x\"%s", bits(m[c][r]), (c == 2 && r == 2) ? "" : ", ");
    std::printf("]%s", comma ? ", " : "");
}

static void put_v3(const char* name, const glm::vec3& v, bool comma = true) {
    std::printf("\"%s\": [\"%08x\", \"%08x\", \"%08x\"]%s", name, bits(v.x), bits(v.y), bits(v.z),
                comma ? ", " : "");
}

int main() {
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string kind;
        if (!(in >> kind)) continue;
        if (kind == "F") {
            float le[3], la[3], lfov, ce[3], ca[3], cfov;
            int lw, lh, cw, ch;
            in >> le[0] >> le[1] >> le[2] >> la[0] >> la[1] >> la[2] >> lfov >> lw >> lh;
            in >> ce[0] >> ce[1] >> ce[2] >> ca[0] >> ca[1] >> ca[2] >> cfov >> cw >> ch;
            const float zn = 1.0f, zf = 1000.0f;
            glm::vec3 up(0.0f, 0.0f, 1.0f);
            glm::vec3 lightEye(le[0], le[1], le[2]);
            // light view
            glm::mat4 lp = glm::perspective(lfov, (float)lw / lh, zn, zf);
            glm::mat4 lv = glm::lookAt(lightEye, glm::vec3(la[0], la[1], la[2]), up);
            glm::mat4 model(1.0f);
            model *= glm::translate(glm::vec3(0.0f, 0.0f, 0.0f));
            model *= glm::rotate(0.0f, glm::vec3(1, 0, 0));
            model *= glm::rotate(0.0f, glm::vec3(0, 1, 0));
            model *= glm::rotate(0.0f, glm::vec3(0, 0, 1));
            glm::mat4 light_mvp = lp * lv * model;
            glm::mat4 bias;
            bias[0][0] = 0.5; bias[0][1] = 0; bias[0][2] = 0; bias[0][3] = 0.0;
            bias[1][0] = 0; bias[1][1] = 0.5; bias[1][2] = 0; bias[1][3] = 0.0;
            bias[2][0] = 0; bias[2][1] = 0; bias[2][2] = 0.5; bias[2][3] = 0.0;
            bias[3][0] = 0.5; bias[3][1] = 0.5; bias[3][2] = 0.5; bias[3][3] = 1.0;
            glm::mat4 biased = bias * light_mvp;
            // camera view
            glm::mat4 cp = glm::perspective(cfov, (float)cw / ch, zn, zf);
            glm::mat4 cv = glm::lookAt(glm::vec3(ce[0], ce[1], ce[2]), glm::vec3(ca[0], ca[1], ca[2]), up);
            glm::mat4 cam_mvp = cp * cv * model;
            glm::mat4 cam_mv = cv * model;
            glm::mat3 nm = glm::inverseTranspose(glm::mat3(cam_mv));
            glm::vec3 lpos = glm::mat3(glm::rotate((float)180.0, glm::vec3(0, 1, 0))) * lightEye;
            std::printf("{\"kind\": \"F\", ");
            put_m4("light_proj", lp);
            put_m4("light_view", lv);
            put_m4("light_mvp", light_mvp);
            put_m4("light_mvp_biased", biased);
            put_m4("camera_mvp", cam_mvp);
            put_m4("camera_mv", cam_mv);
            put_m3("normal_matrix", nm);
            put_v3("light_position", lpos, false);
            std::printf("}\n");
        } else if (kind == "R") {
            float a[3];
            in >> a[0] >> a[1] >> a[2];
            glm::mat4 r = glm::rotate(a[0], glm::vec3(1, 0, 0));
            r *= glm::rotate(a[1], glm::vec3(0, 1, 0));
            r *= glm::rotate(a[2], glm::vec3(0, 0, 1));
            r = glm::transpose(r);
            std::printf("{\"kind\": \"R\", ");
            put_m4("rotation_t", r, false);
            std::printf("}\n");
        } else if (kind == "N") {
            float p[9];
            for (int i = 0; i < 9; ++i) in >> p[i];
            glm::vec3 a(p[0], p[1], p[2]), b(p[3], p[4], p[5]), c(p[6], p[7], p[8]);
            glm::vec3 n = glm::normalize(glm::cross(b - a, c - a));
            std::printf("{\"kind\": \"N\", ");
            put_v3("normal", n, false);
            std::printf("}\n");
        }
    }
    return 0;
}
