// ref_scene_pin.cpp -- test infrastructure only (never linked into the
// product library, never run on the GPU machine).
//
// Pins the product's scene loading and shadow-volume geometry to the
// reference's own C++: this file is compiled together with the reference's
// unmodified sources, read where they lie in the reference tree,
//
//   <app>/src/IO/SceneLoader.cpp   SceneLoader::load      (:11-94)
//   <app>/src/Mesh.cpp             Mesh::addObject, computeNormals,
//                                  loadOBJFile, scale, translate, rotate
//   <app>/src/IO/OBJLoader.cpp     glmReadOBJ (glm.c by Nate Robins)
//   ShadowVolumes/src/ShadowVolume.cpp   ShadowVolume::build (:15-114)
//                                  (only in the ShadowVolumes build)
//
// into oracle/_ref/libscene_ref_<app>.so by oracle/build_oracle.py, against
// a small generated include shim for what does not exist on Linux (GL/glut.h
// types and no-op GL calls for glm.c's drawing functions, which loading never
// calls; the backslash include paths; an empty OpenCV header).  Image.cpp
// (OpenCV texture loading) is replaced by the three members below: loading a
// scene never reads texture pixels for the geometry.
//
// The functions below only drive the reference's classes and copy their
// arrays out; none of the reference's arithmetic is restated here.

#include "IO/SceneLoader.h"
#ifdef GI_PIN_VOLUMES
#include "ShadowVolume.h"
#endif

#include <cstdlib>
#include <cstring>
#include <unistd.h>

// Image.cpp stands outside the pin (it needs OpenCV); these members keep the
// reference's Mesh texture bookkeeping working with blank images.
Image::Image(int w, int h, int channels) : width(w), height(h) {
    data = (unsigned char*)calloc((size_t)(w > 0 ? w : 1) * (h > 0 ? h : 1) * (channels > 0 ? channels : 1), 1);
}
Image::Image(char*) : width(1), height(1) { data = (unsigned char*)calloc(3, 1); }
Image::~Image() { free(data); }

#define PIN_API extern "C" __attribute__((visibility("default")))

struct PinScene {
    int num_vertices;
    int num_triangles;
    float* points;   // [3V]
    float* normals;  // [3V]
    int* indices;    // [3T]
    float views[13]; // camera eye, camera at, light eye, light at, depth threshold
};

// Runs SceneLoader::load on `cfg_path` with `base_dir` as the working
// directory (the reference opens the OBJ paths relative to it) and copies the
// combined mesh out.  Returns 0 on success, -1 if the directory or the file
// cannot be opened.  The reference's Mesh objects are not destroyed: Mesh's
// destructor reads fields its constructors leave uninitialised.
PIN_API int pin_scene_load(const char* cfg_path, const char* base_dir, PinScene* out) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (base_dir && chdir(base_dir) != 0) return -1;
    {
        FILE* f = fopen(cfg_path, "r");
        if (!f) {
            if (base_dir && chdir(cwd) != 0) return -1;
            return -1;
        }
        fclose(f);
    }
    Mesh* mesh = new Mesh();
    SceneLoader loader(const_cast<char*>(cfg_path), mesh);
    loader.load();
    if (base_dir && chdir(cwd) != 0) return -1;
    const int nv = mesh->getPointCloudSize() / 3;
    const int nt = mesh->getIndicesSize() / 3;
    out->num_vertices = nv;
    out->num_triangles = nt;
    out->points = (float*)malloc(sizeof(float) * 3 * (nv > 0 ? nv : 1));
    out->normals = (float*)malloc(sizeof(float) * 3 * (nv > 0 ? nv : 1));
    out->indices = (int*)malloc(sizeof(int) * 3 * (nt > 0 ? nt : 1));
    memcpy(out->points, mesh->getPointCloud(), sizeof(float) * 3 * nv);
    memcpy(out->normals, mesh->getNormalVector(), sizeof(float) * 3 * nv);
    memcpy(out->indices, mesh->getIndices(), sizeof(int) * 3 * nt);
    const float* v[4] = {loader.getCameraPosition(), loader.getCameraAt(), loader.getLightPosition(),
                         loader.getLightAt()};
    for (int k = 0; k < 4; ++k)
        for (int a = 0; a < 3; ++a) out->views[k * 3 + a] = v[k][a];
#ifdef GI_PIN_VOLUMES
    out->views[12] = 0.0f;  // ShadowVolumes' SceneLoader has no "d" key
#else
    out->views[12] = loader.getDepthThreshold();
#endif
    return 0;
}

PIN_API void pin_scene_free(PinScene* s) {
    free(s->points);
    free(s->normals);
    free(s->indices);
    s->points = s->normals = nullptr;
    s->indices = nullptr;
}

#ifdef GI_PIN_VOLUMES
// ShadowVolume::build for a mesh given as arrays: writes the 6T volume
// vertices (float[18T]) and the 6T volume triangles (int[18T]).
PIN_API int pin_shadow_volume_build(const float* points, const float* normals, int num_vertices,
                                    const int* indices, int num_triangles, const float light[3],
                                    int infinity, float* out_points, int* out_indices) {
    if (num_vertices <= 0 || num_triangles <= 0) return -1;
    Mesh* scene = new Mesh(num_vertices, num_triangles);
    memcpy(scene->getPointCloud(), points, sizeof(float) * 3 * num_vertices);
    memcpy(scene->getNormalVector(), normals, sizeof(float) * 3 * num_vertices);
    memcpy(scene->getIndices(), indices, sizeof(int) * 3 * num_triangles);
    ShadowVolume* vol = new ShadowVolume(infinity);
    vol->build(scene, glm::vec3(light[0], light[1], light[2]));
    Mesh* q = vol->getData();
    memcpy(out_points, q->getPointCloud(), sizeof(float) * 18 * (size_t)num_triangles);
    memcpy(out_indices, q->getIndices(), sizeof(int) * 18 * (size_t)num_triangles);
    return 0;  // the meshes are left allocated, as above
}
#endif
