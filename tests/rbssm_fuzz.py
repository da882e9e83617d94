"""Random binary light maps and light-space G-buffers for the RBSSM tests.

Thin blocker features (one texel wide, isolated texels, corners) drive
every case of the discontinuity-space smoothing; the maps hold blockers at
depth 0.995 over a lit background at 1.0 and the receivers sit at 0.999.
"""
import numpy as np

import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api

I4 = np.eye(4, dtype=np.float32).reshape(-1)
CASES = [(0.5, 1, 0.0), (0.3, 1, 1e-4), (0.7, 1, 0.0), (0.5, 2, 1e-4), (0.2, 1, 0.0), (0.8, 1, 1e-4),
         (0.5, 3, 0.0)]


def case(k, S=64, W=64, H=64, seed=7):
    density, blob, thr = CASES[k]
    rng = np.random.default_rng(seed + k)
    g = rng.random((S // blob + 1, S // blob + 1)) < density
    g = np.kron(g, np.ones((blob, blob)))[:S, :S].astype(bool)
    depth = np.where(g, np.float32(0.995), np.float32(1.0)).astype(np.float32).reshape(-1)
    pos = np.zeros((H, W, 4), np.float32)
    pos[..., 0] = rng.uniform(0.1, 0.9, (H, W))
    pos[..., 1] = rng.uniform(0.1, 0.9, (H, W))
    pos[..., 2] = np.float32(0.999)
    pos[..., 3] = 1.0
    nrm = np.zeros((H, W, 4), np.float32)
    nrm[..., 2] = 1.0
    nrm[..., 3] = 1.0
    p = gi.ShadowParams.defaults(api.GI_TECH_RBSSM)
    p.pretest = api.GI_PRETEST_OFF
    p.pcss_min_blocker_depth = 0.0
    p.light_radius = 8.0
    p.depth_threshold = thr
    fr = gi.Frame(I4, I4, I4, I4, np.eye(3, dtype=np.float32).reshape(-1), np.zeros(3, np.float32))
    return p, fr, depth, pos.reshape(-1), nrm.reshape(-1), S, W, H
