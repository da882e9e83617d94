"""Regenerates tests/golden/edt_pin.npz from the reference's own PBA kernels.

Builds oracle/_ref/libpba_ref.so (oracle/ref_pba_pin.cpp: the reference's
ShadowMapping/include/EDT/pba2DKernel.h compiled for the CPU against a CUDA
emulation, driven in the order of ShadowMapping/src/EDT/pba2DHost.cu) and
records, for every case of tests/edt_cases.py, what the reference's kernels
produce: the nearest-site map of each PBA case, and the sites, nearest
sites and normalised EDT shadow (channels 0-1) of each EDTSM case.  The
oracle and the CUDA path must reproduce every value bit for bit
(tests/test_edt_oracle.py, tests/test_gpu_edt.py).  Needs the reference
tree; the archive is committed.

Run:  python tests/golden/make_edt_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from edt_cases import EDT_CASES, PBA_CASES, hard_shadow_image, pba_case  # noqa: E402
from oracle.build_oracle import build_pba_ref  # noqa: E402

OUT = os.path.join(HERE, "edt_pin.npz")


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def main():
    lib_path = build_pba_ref()
    if lib_path is None:
        raise SystemExit("the reference's PBA kernels are not available here")
    lib = C.CDLL(lib_path)
    rec = {}
    for name, W, H, *_ in PBA_CASES:
        sites, bands = pba_case(name)
        out = np.empty_like(sites)
        if lib.ref_pba_voronoi(_vp(sites), W, H, *bands, _vp(out)) != 0:
            raise SystemExit(f"{name}: shape rejected")
        rec[f"pba/{name}/nearest"] = out
    for name, W, H, seed, pen, inten, bands in EDT_CASES:
        img, pos = hard_shadow_image(W, H, seed)
        out4 = np.zeros((H, W, 4), np.float32)
        sites = np.empty((H, W, 2), np.int16)
        nearest = np.empty((H, W, 2), np.int16)
        rc = lib.ref_edt_soft_shadows(_vp(img), _vp(pos), W, H, *bands, C.c_float(pen / 5.0), C.c_float(inten),
                                      _vp(sites), _vp(nearest), _vp(out4))
        if rc != 0:
            raise SystemExit(f"{name}: shape rejected")
        rec[f"edt/{name}/sites"] = sites
        rec[f"edt/{name}/nearest"] = nearest
        rec[f"edt/{name}/out01"] = np.ascontiguousarray(out4[..., :2])
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
