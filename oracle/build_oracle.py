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

Only the tests, the smoke check and the CPU-baseline leg of bench.py use
these files; the product library never links or loads them.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ORACLE_LIB = os.path.join(HERE, "libgioracle.so")
REF_DIR = os.path.join(HERE, "_ref")
GLM_PIN = os.path.join(REF_DIR, "glm_pin")
REFERENCE_ROOT = "/root/reference"
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


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    print(build_pba_ref())
