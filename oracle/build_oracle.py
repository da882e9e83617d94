"""Build recipe for the CPU oracle (test infrastructure only).

  oracle/libgioracle.so   the scalar C++ restatement of the reference's
                          passes (gi_oracle.cpp), OpenMP over triangles /
                          rows, -O2 -ffp-contract=off, no -ffast-math.
  oracle/_ref/glm_pin     ref_glm_pin.cpp compiled against the reference's
                          vendored glm 0.9.3 headers; built only where the
                          reference tree is present (never on the GPU machine).
  oracle/_ref/libpba_ref.so
                          ref_pba_pin.cpp: the reference's own PBA kernels
                          (ShadowMapping/include/EDT/pba2DKernel.h, unmodified)
                          compiled for the CPU against a CUDA-emulation shim;
                          built only where the reference tree is present.

  oracle/_ref/libscene_ref_shadowmapping.so, libscene_ref_shadowvolumes.so
                          ref_scene_pin.cpp linked with the reference's own,
                          unmodified SceneLoader.cpp, Mesh.cpp and OBJLoader.cpp
                          of that app (and ShadowVolume.cpp for ShadowVolumes),
                          read where they lie, against a generated include
                          shim under oracle/_ref/shim/; built only where the
                          reference tree is present.

  oracle/_ref/libshader_ref.so
                          ref_shader_pin.cpp: the reference's own fragment
                          shaders (PlausibleSoftShadow.frag, ...) included
                          unmodified as C++ on top of glsl_shim.h; built only
                          where the reference tree is present.

Only the tests, the smoke check, the fixture generators and the CPU-baseline
leg of bench.py use these files; the product library never links or loads
them.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ORACLE_LIB = os.path.join(HERE, "libgioracle.so")
REF_DIR = os.path.join(HERE, "_ref")
GLM_PIN = os.path.join(REF_DIR, "glm_pin")
# The reference tree (read-only); GI_REFERENCE_ROOT overrides the default.
REFERENCE_ROOT = os.environ.get("GI_REFERENCE_ROOT", "/root/reference")
GLM_INCLUDE = os.path.join(REFERENCE_ROOT, "ShadowMapping", "include")
PBA_INCLUDE = os.path.join(REFERENCE_ROOT, "ShadowMapping", "include", "EDT")
PBA_REF_LIB = os.path.join(REF_DIR, "libpba_ref.so")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle() -> str:
    src = os.path.join(HERE, "gi_oracle.cpp")
    deps = [src, os.path.join(HERE, "gi_oracle.h"), os.path.join(ROOT, "include", "gi_shadow.h")]
    if _newer(ORACLE_LIB, deps):
        tmp = ORACLE_LIB + ".tmp"
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                        "-ffp-contract=off", "-fno-fast-math", "-Wall", src, "-o", tmp], check=True)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_ref() -> str | None:
    """Builds oracle/_ref/glm_pin when the reference's glm is available."""
    if not os.path.isdir(os.path.join(GLM_INCLUDE, "glm")):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_glm_pin.cpp")
    if _newer(GLM_PIN, [src]):
        subprocess.run(["g++", "-O0", "-std=c++11", "-ffp-contract=off", "-w", "-I", GLM_INCLUDE,
                        src, "-o", GLM_PIN], check=True)
    return GLM_PIN


def build_pba_ref() -> str | None:
    """Builds oracle/_ref/libpba_ref.so when the reference's PBA kernels are available."""
    kernels = os.path.join(PBA_INCLUDE, "pba2DKernel.h")
    if not os.path.exists(kernels):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_pba_pin.cpp")
    if _newer(PBA_REF_LIB, [src, kernels]):
        tmp = PBA_REF_LIB + ".tmp"
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                        "-w", "-I", PBA_INCLUDE, src, "-o", tmp], check=True)
        os.replace(tmp, PBA_REF_LIB)
    return PBA_REF_LIB


SCENE_PIN_APPS = ("ShadowMapping", "ShadowVolumes")
SHIM_DIR = os.path.join(REF_DIR, "shim")

# What the reference's sources include but Linux does not have: GL types and
# no-op GL calls (only glm.c's drawing functions call them; loading never
# does), the Windows-style backslash include paths, and OpenCV (Image.h's
# include; the pin replaces Image.cpp).
_GLUT_SHIM = """#ifndef GI_PIN_GLUT_SHIM
#define GI_PIN_GLUT_SHIM
typedef float GLfloat;
typedef unsigned int GLuint;
typedef int GLint;
typedef int GLsizei;
typedef unsigned int GLenum;
typedef unsigned char GLboolean;
typedef unsigned char GLubyte;
typedef void GLvoid;
#define GL_FALSE 0
#define GL_TRUE 1
#define GL_TRIANGLES 0x0004
#define GL_FRONT_AND_BACK 0x0408
#define GL_AMBIENT 0x1200
#define GL_DIFFUSE 0x1201
#define GL_SPECULAR 0x1202
#define GL_SHININESS 0x1601
#define GL_COMPILE 0x1300
#define GL_COLOR_MATERIAL 0x0B57
static inline void glBegin(GLenum) {}
static inline void glEnd(void) {}
static inline void glEnable(GLenum) {}
static inline void glDisable(GLenum) {}
static inline void glNormal3fv(const GLfloat*) {}
static inline void glVertex3fv(const GLfloat*) {}
static inline void glTexCoord2fv(const GLfloat*) {}
static inline void glColor3fv(const GLfloat*) {}
static inline void glMaterialfv(GLenum, GLenum, const GLfloat*) {}
static inline void glMaterialf(GLenum, GLenum, GLfloat) {}
static inline GLuint glGenLists(GLsizei) { return 1; }
static inline void glNewList(GLuint, GLenum) {}
static inline void glEndList(void) {}
#endif
"""


def _write_shim() -> None:
    os.makedirs(os.path.join(SHIM_DIR, "GL"), exist_ok=True)
    files = {
        os.path.join(SHIM_DIR, "GL", "glut.h"): _GLUT_SHIM,
        os.path.join(SHIM_DIR, "IO\\SceneLoader.h"): '#include "IO/SceneLoader.h"\n',
        os.path.join(SHIM_DIR, "opencv2\\opencv.hpp"): "/* OpenCV is not needed to load geometry; its header brought in the C\n"
                                                             " * library declarations the reference's files use. */\n"
                                                             "#include <cstring>\n#include <cstdlib>\n#include <cstdio>\n",
    }
    for path, text in files.items():
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)


def scene_ref_lib(app: str) -> str:
    return os.path.join(REF_DIR, f"libscene_ref_{app.lower()}.so")


def build_scene_ref() -> list[str]:
    """Builds the scene / shadow-volume pins when the reference's C++ is available."""
    built = []
    for app in SCENE_PIN_APPS:
        base = os.path.join(REFERENCE_ROOT, app)
        srcs = [os.path.join(base, "src", "IO", "SceneLoader.cpp"), os.path.join(base, "src", "Mesh.cpp"),
                os.path.join(base, "src", "IO", "OBJLoader.cpp")]
        defs = []
        if app == "ShadowVolumes":
            srcs.append(os.path.join(base, "src", "ShadowVolume.cpp"))
            defs.append("-DGI_PIN_VOLUMES")
        if not all(os.path.exists(f) for f in srcs):
            continue
        os.makedirs(REF_DIR, exist_ok=True)
        _write_shim()
        pin = os.path.join(HERE, "ref_scene_pin.cpp")
        lib = scene_ref_lib(app)
        if _newer(lib, [pin, *srcs, os.path.abspath(__file__)]):
            tmp = lib + ".tmp"
            subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                            "-fvisibility=hidden", "-w", *defs, "-I", SHIM_DIR, "-I", os.path.join(base, "include"),
                            pin, *srcs, "-o", tmp], check=True)
            os.replace(tmp, lib)
        built.append(lib)
    return built


SHADER_PIN_LIB = os.path.join(REF_DIR, "libshader_ref.so")
# The reference's fragment shaders compiled by oracle/ref_shader_pin.cpp.
SHADER_PIN_SOURCES = {
    "GI_SHADER_PCSS": os.path.join(REFERENCE_ROOT, "SoftShadowMapping", "Shaders", "SoftShadow",
                                   "PlausibleSoftShadow.frag"),
    "GI_SHADER_SHADOW": os.path.join(REFERENCE_ROOT, "ShadowMapping", "Shaders", "Shadow.frag"),
    "GI_SHADER_NCSMSR": os.path.join(REFERENCE_ROOT, "ShadowMapping", "Shaders", "RBSM", "NonConservativeSMSR.frag"),
    "GI_SHADER_CSMSR": os.path.join(REFERENCE_ROOT, "ShadowMapping", "Shaders", "RBSM", "ConservativeSMSR.frag"),
    "GI_SHADER_FRBSM": os.path.join(REFERENCE_ROOT, "ShadowMapping", "Shaders", "RBSM", "FilteredRBSM.frag"),
    "GI_SHADER_RBSSM": os.path.join(REFERENCE_ROOT, "SoftShadowMapping", "Shaders", "SoftShadow", "RBSSM.frag"),
    "GI_SHADER_PHONG": os.path.join(REFERENCE_ROOT, "ShadowMapping", "Shaders", "GBuffer", "PhongShading.frag"),
}


def build_shader_ref() -> str | None:
    """Builds oracle/_ref/libshader_ref.so when the reference's shaders are present:
    ref_shader_pin.cpp includes each one unmodified on top of glsl_shim.h
    (-fsingle-precision-constant so GLSL's float literals stay float)."""
    shaders = list(SHADER_PIN_SOURCES.values())
    if not all(os.path.exists(f) for f in shaders):
        return None
    pin = os.path.join(HERE, "ref_shader_pin.cpp")
    deps = [pin, os.path.join(HERE, "glsl_shim.h"), *shaders, os.path.abspath(__file__)]
    if _newer(SHADER_PIN_LIB, deps):
        os.makedirs(REF_DIR, exist_ok=True)
        tmp = SHADER_PIN_LIB + ".tmp"
        defs = [f'-D{k}="{v}"' for k, v in SHADER_PIN_SOURCES.items()]
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                        "-fsingle-precision-constant", "-w", "-I", HERE, *defs, pin, "-o", tmp], check=True)
        os.replace(tmp, SHADER_PIN_LIB)
    return SHADER_PIN_LIB


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    print(build_pba_ref())
    print(build_scene_ref())
    print(build_shader_ref())
