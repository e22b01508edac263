"""Generate tests/golden/reference_mode_r.npz from the reference itself.

Runs the reference's own host path (oracle/_ref, compiled from the reference
sources by oracle/Makefile.ref: s_grid + iterate_2d_jk_blocked with
stencil_<N>_ref_1, real = float or double) on seeded inputs and stores, per
case, the inputs' recipe, a SHA-256 digest of the output interior and, for the
small cases, the output interior itself.  The GPU machine has no reference
sources, so its tests pin the oracle against these fixtures and then compare
the CUDA kernels with the oracle.

Inputs come from the oracle's counter-hash generator (orc_fill_uniform): u in
[-1, 1), v in [-1, 1), s in [0.5, 1.5), halos included, so the halo reads of
the stencil are exercised.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402

# (name, points, dtype, (xs, ys, zs, xh, yh, zh), iterations, seed, keep_array)
CASES = [
    ("p7_small", 7, "f32", (13, 11, 19, 4, 5, 6), 3, 11, True),
    ("p7_odd_min_halo", 7, "f32", (17, 19, 23, 4, 4, 1), 2, 12, True),
    ("p13_small", 13, "f32", (12, 20, 33, 4, 4, 2), 3, 13, True),
    ("p25_small", 25, "f32", (11, 9, 17, 4, 4, 4), 2, 14, True),
    ("p25_refhalo", 25, "f32", (16, 24, 40, 4, 4, 16), 3, 15, True),
    ("p2_small", 2, "f32", (9, 10, 37, 4, 4, 1), 2, 16, True),
    ("p7_f64", 7, "f64", (9, 9, 21, 4, 4, 3), 3, 17, True),
    ("p13_f64", 13, "f64", (10, 11, 12, 4, 4, 2), 2, 18, True),
    ("p25_f64", 25, "f64", (10, 12, 14, 4, 4, 4), 2, 19, True),
    # multi-tile cases: several 128-wide k tiles and 16-row j tiles, ragged
    # edges in both; digest only
    ("p25_tiles", 25, "f32", (20, 37, 300, 4, 4, 4), 2, 20, False),
    ("p13_tiles", 13, "f32", (19, 40, 260, 4, 4, 16), 3, 21, False),
    ("p7_tiles", 7, "f32", (24, 33, 131, 4, 4, 1), 4, 22, False),
    ("p7_nonsquare", 7, "f32", (40, 18, 64, 4, 4, 16), 5, 23, False),
]


def make_inputs(grid, seed, dtype):
    dt = np.float64 if dtype == "f64" else np.float32
    u = O.fill_uniform(grid, seed, 0, -1.0, 1.0, dt)
    v = O.fill_uniform(grid, seed, 1, -1.0, 1.0, dt)
    s = O.fill_uniform(grid, seed, 2, 0.5, 1.5, dt)
    return v, s, u


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if not obuild.build_ref():
        raise SystemExit("the reference sources are not present; cannot regenerate fixtures")
    out = {}
    meta = []
    for name, pts, dtype, grid, iters, seed, keep in CASES:
        v, s, u = make_inputs(grid, seed, dtype)
        O.ref_iterate(v, s, u, grid, pts, iters)
        inner = np.ascontiguousarray(O.interior(v, grid))
        meta.append({"name": name, "points": pts, "dtype": dtype, "grid": list(grid),
                     "iterations": iters, "seed": seed, "sha256": digest(inner),
                     "keep": keep})
        if keep:
            out[name] = inner
        print(name, inner.shape, meta[-1]["sha256"][:16])
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "reference_mode_r.npz"), **out)


if __name__ == "__main__":
    main()
