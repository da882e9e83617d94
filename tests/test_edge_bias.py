"""The raster kernels' inside test on biased edge values (raster_common.cuh
`tl_bias` / `inside_biased`, the 32-bit paths of raster.cu) is the same
predicate as the top-left rule it replaces:

    E > 0 or (E == 0 and top_left)   <=>   E - (0 if top_left else 1) >= 0

and, for a 64-bit value, `>= 0` is the sign of its high 32-bit word, so three
edges are inside together exactly when the OR of their (biased) values, or
of their high words, is not negative.  Checked here on integers, including
the values next to 0 and to the int32 / int64 limits."""
import numpy as np


def top_left_rule(e, tl):
    return (e > 0) | ((e == 0) & tl)


def biased(e, tl):
    return e - np.where(tl, 0, 1).astype(e.dtype)


def edge_values(rng, n, lo, hi, dtype):
    v = rng.integers(lo, hi, size=n, dtype=np.int64)
    edges = np.array([lo, lo + 1, -2, -1, 0, 1, 2, hi - 2, hi - 1], dtype=np.int64)
    return np.concatenate([v, edges]).astype(dtype)


def test_bias_matches_top_left_rule_int64():
    rng = np.random.default_rng(7)
    # edge values over a box stay well inside int64 (|E| < 2^62)
    e = edge_values(rng, 200_000, -(1 << 62), 1 << 62, np.int64)
    for tl in (False, True):
        t = np.full(e.shape, tl)
        b = biased(e, t)
        assert np.array_equal(top_left_rule(e, t), b >= 0)
        hi = (b >> 32).astype(np.int32)
        assert np.array_equal(b >= 0, hi >= 0)


def test_bias_matches_top_left_rule_int32():
    rng = np.random.default_rng(11)
    # the 32-bit paths run only when every value over the box is below 2^31
    # in magnitude, so the biased value (one less at most) still fits
    e = edge_values(rng, 200_000, -(1 << 31) + 1, 1 << 31, np.int32)
    for tl in (False, True):
        t = np.full(e.shape, tl)
        b = biased(e.astype(np.int64), t)
        assert b.min() >= -(1 << 31)
        assert np.array_equal(top_left_rule(e, t), b.astype(np.int32) >= 0)


def test_three_edges_or_of_values():
    rng = np.random.default_rng(13)
    n = 100_000
    e = rng.integers(-(1 << 40), 1 << 40, size=(3, n), dtype=np.int64)
    e[:, : n // 4] = rng.integers(-2, 3, size=(3, n // 4))  # many zeros and near-zeros
    tl = rng.integers(0, 2, size=(3, n)).astype(bool)
    inside = top_left_rule(e[0], tl[0]) & top_left_rule(e[1], tl[1]) & top_left_rule(e[2], tl[2])
    b = biased(e, tl)
    hi = (b >> 32).astype(np.int32)
    assert np.array_equal(inside, (hi[0] | hi[1] | hi[2]) >= 0)
    small = np.abs(e).max(axis=0) < (1 << 31) - 1
    b32 = b[:, small].astype(np.int32)
    assert np.array_equal(inside[small], (b32[0] | b32[1] | b32[2]) >= 0)
    # adding the bias back gives the value the depth interpolation converts
    assert np.array_equal(b + np.where(tl, 0, 1), e)
