"""Generates poisson_table.inc: a 64-point progressive Poisson-disk sequence.

Mitchell's best-candidate algorithm (D. P. Mitchell, "Spectrally optimal
sampling for distribution ray tracing", SIGGRAPH 1991): point k is the best
of 32 * (k + 1) uniform candidates in the unit disk, "best" meaning the
largest distance to the points already chosen.  Any prefix of the sequence
is itself well spread, so the n-tap table used by the PCSS Poisson
technique is the first n points.  Candidates come from numpy's PCG64 with a
fixed seed; values are stored as float32 and printed with 9 significant
digits so the table round-trips exactly.

Run:  python globalillumination_gb300/csrc/gen_poisson_table.py
"""
import os

import numpy as np


def best_candidate(n=64, seed=0x5EED, k=32):
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = []
    for i in range(n):
        m = k * (i + 1)
        r = np.sqrt(rng.random(m))
        a = 2.0 * np.pi * rng.random(m)
        cand = np.stack([r * np.cos(a), r * np.sin(a)], axis=1)
        if not pts:
            best = cand[np.argmin(np.hypot(cand[:, 0], cand[:, 1]))]
        else:
            p = np.array(pts)
            d = np.min(np.hypot(cand[:, None, 0] - p[None, :, 0], cand[:, None, 1] - p[None, :, 1]), axis=1)
            best = cand[np.argmax(d)]
        pts.append(best)
    return np.array(pts, dtype=np.float32)


def main():
    pts = best_candidate()
    here = os.path.dirname(os.path.abspath(__file__))
    lines = [
        "// Generated by gen_poisson_table.py -- do not edit.",
        "// Initializer of a 64-point progressive Poisson-disk sequence (Mitchell",
        "// best candidate) in the unit disk; the n-tap PCSS table is the first n",
        "// points.  Included by visibility.cu for both the host and the",
        "// __constant__ copy.",
    ]
    for x, y in pts:
        lines.append("{%sf, %sf}," % (repr(float(np.float32(x))), repr(float(np.float32(y)))))
    with open(os.path.join(here, "poisson_table.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")

if __name__ == "__main__":
    main()
