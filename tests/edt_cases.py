"""Seeded inputs for the EDT tests (PBA distance transform and EDTSM).

Used by tests/test_edt_oracle.py, tests/test_gpu_edt.py and
tests/golden/make_edt_golden.py, so the committed golden outputs can be
recomputed from the same inputs anywhere: numpy's PCG64 streams and the
float32 arithmetic below are platform independent.
"""
from __future__ import annotations

import numpy as np

MARKER = -32768

# (name, W, H, kind, parameter, seed, bands)
PBA_CASES = [
    ("random_sparse_64", 64, 64, "random", 0.004, 1, (16, 16, 16)),
    ("random_dense_64", 64, 64, "random", 0.15, 2, (16, 16, 16)),
    ("lattice_64", 64, 64, "lattice", 6, 3, (16, 16, 16)),
    ("lattice_offset_128", 128, 128, "lattice", 10, 4, (16, 16, 16)),
    ("lines_128", 128, 128, "lines", 3, 5, (16, 16, 16)),
    ("clusters_128", 128, 128, "clusters", 5, 6, (16, 16, 16)),
    ("random_128_bands_8_4_8", 128, 128, "random", 0.01, 7, (8, 4, 8)),
    ("random_128_bands_2_64_64", 128, 128, "random", 0.002, 8, (2, 64, 64)),
    ("single_64", 64, 64, "single", 0, 9, (16, 16, 16)),
    ("pair_tie_64", 64, 64, "pair", 0, 10, (16, 16, 16)),
    ("empty_64", 64, 64, "empty", 0, 11, (16, 16, 16)),
    # three sites whose bisectors cross row 0 at one point (35 1/3): the FP32
    # intersections of the reference keep the middle one, so row 0's list is
    # not a strict envelope and is colored by the exact group chain
    ("degenerate_a_64", 64, 64, "points", ((0, 11), (3, 18), (9, 26)), 13, (16, 16, 16)),
    ("degenerate_b_64", 64, 64, "points", ((0, 12), (3, 16), (12, 22)), 14, (16, 16, 16)),
    ("full_64", 64, 64, "full", 0, 12, (16, 16, 16)),
]

# (name, W, H, seed, penumbra_size (the kernels get / 5), intensity, bands)
EDT_CASES = [
    ("edtsm_64", 64, 64, 21, 1.0, 0.25, (16, 16, 16)),
    ("edtsm_128", 128, 128, 22, 1.0, 0.25, (16, 16, 16)),
    ("edtsm_128_wide_penumbra", 128, 128, 23, 20.0, 0.25, (16, 16, 16)),
    ("edtsm_128_intensity_half", 128, 128, 24, 5.0, 0.5, (8, 16, 8)),
]


def site_mask(kind: str, W: int, H: int, param, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    m = np.zeros((H, W), bool)
    if kind == "random":
        m = rng.random((H, W)) < param
    elif kind == "lattice":  # regular lattices: many pixels equidistant from several sites
        st = int(param)
        m[::st, ::st] = True
        m[st // 2::2 * st, st // 2::2 * st] = True
    elif kind == "lines":
        for _ in range(int(param)):
            if rng.random() < 0.5:
                m[rng.integers(H), :] = rng.random(W) < 0.7
            else:
                m[:, rng.integers(W)] = rng.random(H) < 0.7
    elif kind == "clusters":
        yy, xx = np.mgrid[0:H, 0:W]
        for _ in range(int(param)):
            cy, cx, r = rng.integers(H), rng.integers(W), rng.integers(2, 8)
            ring = np.abs(np.hypot(yy - cy, xx - cx) - r) < 0.6
            m |= ring
    elif kind == "single":
        m[rng.integers(H), rng.integers(W)] = True
    elif kind == "pair":  # two sites symmetric about the centre
        cy, cx, d = H // 2, W // 2, 9
        m[cy - d, cx] = m[cy + d, cx] = m[cy, cx - d] = m[cy, cx + d] = True
    elif kind == "points":
        for x, y in param:
            m[y, x] = True
    elif kind == "full":
        m[:] = True
    elif kind != "empty":
        raise ValueError(kind)
    return m


def sites_from_mask(m: np.ndarray) -> np.ndarray:
    s = np.full(m.shape + (2,), MARKER, np.int16)
    ys, xs = np.nonzero(m)
    s[ys, xs, 0] = xs
    s[ys, xs, 1] = ys
    return s


def pba_case(name: str):
    for c in PBA_CASES:
        if c[0] == name:
            _, W, H, kind, param, seed, bands = c
            return sites_from_mask(site_mask(kind, W, H, param, seed)), bands
    raise KeyError(name)


def hard_shadow_image(W: int, H: int, seed: int):
    """A synthetic EDTSM frame: (image, position), float32 [H, W, 4] each.

    image = (shadow, depth, preEvaluatedShadow, 1) with umbra discs at the
    intensity 0.25, lit surface, a few fractional (revectorised) values, a
    depth gradient with one step, back-facing (pre = 0.25) patches and a
    background corner (0, 0, 0, 1); position = a clip-space-like position.
    """
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float32)
    bg = (xx + yy) < (W + H) / 10
    depth = (np.float32(0.97) + np.float32(0.02) * yy / np.float32(H)).astype(np.float32)
    depth = np.where(xx > 0.7 * W, depth - np.float32(0.01), depth).astype(np.float32)
    shadow = np.ones((H, W), np.float32)
    for _ in range(3):
        cy, cx, r = rng.random() * H, rng.random() * W, (0.08 + 0.12 * rng.random()) * min(W, H)
        shadow[(yy - cy) ** 2 + (xx - cx) ** 2 < r * r] = np.float32(0.25)
    frac = rng.random((H, W)) < 0.01
    shadow[frac] = rng.random(int(frac.sum())).astype(np.float32)
    pre = np.ones((H, W), np.float32)
    for _ in range(2):
        y0, x0 = rng.integers(H), rng.integers(W)
        pre[y0:y0 + H // 8, x0:x0 + W // 8] = np.float32(0.25)
    img = np.zeros((H, W, 4), np.float32)
    img[..., 3] = 1.0
    img[..., 0] = np.where(bg, 0, shadow)
    img[..., 1] = np.where(bg, 0, depth)
    img[..., 2] = np.where(bg, 0, pre)
    pos = np.zeros((H, W, 4), np.float32)
    pos[..., 3] = 1.0
    pos[..., 0] = np.where(bg, 0, (xx / np.float32(W) * 2 - 1) * np.float32(3.0))
    pos[..., 1] = np.where(bg, 0, (yy / np.float32(H) * 2 - 1) * np.float32(3.0))
    pos[..., 2] = np.where(bg, 0, depth * np.float32(10.0))
    return img, pos


def brute_force_sqdist(m: np.ndarray) -> np.ndarray:
    """Exact squared distance to the nearest site (small images only)."""
    H, W = m.shape
    ys, xs = np.nonzero(m)
    out = np.empty((H, W), np.int64)
    yy, xx = np.mgrid[0:H, 0:W]
    for r0 in range(0, H, 16):
        d = (yy[r0:r0 + 16, :, None] - ys) ** 2 + (xx[r0:r0 + 16, :, None] - xs) ** 2
        out[r0:r0 + 16] = d.min(-1)
    return out
