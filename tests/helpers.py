"""Shared test helpers: seeded inputs and the golden fixtures."""
import json
import os

import numpy as np

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "reference_mode_r.npz")


def golden_cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    arrays = {m["name"]: z[m["name"]] for m in meta if m["keep"]}
    return meta, arrays


def np_dtype(name):
    return np.float64 if name == "f64" else np.float32


def mode_r_inputs(grid, seed, dtype):
    """u, v in [-1, 1), s in [0.5, 1.5): the recipe of tests/golden/make_golden.py."""
    dt = np_dtype(dtype) if isinstance(dtype, str) else dtype
    u = O.fill_uniform(grid, seed, 0, -1.0, 1.0, dt)
    v = O.fill_uniform(grid, seed, 1, -1.0, 1.0, dt)
    s = O.fill_uniform(grid, seed, 2, 0.5, 1.5, dt)
    return v, s, u


def halo_mask(grid):
    xs, ys, zs, xh, yh, zh = grid
    m = np.ones(O.shape(grid), bool)
    m[xh:xh + xs, yh:yh + ys, zh:zh + zs] = False
    return m


def wave_inputs(grid, seed, dtype=np.float32, blobs=False):
    """Wave-form inputs: u, v ~ U[-1e-3, 1e-3) (or seeded Gaussian blobs with
    v = u), s = 0.  The halo is a fixed Dirichlet boundary: u's seeded halo
    values, the same in v, so that it does not change when u and v swap."""
    if blobs:
        u = O.fill_blobs(grid, seed, 8, 20.0, dtype)
        v = u.copy()
    else:
        u = O.fill_uniform(grid, seed, 0, -1e-3, 1e-3, dtype)
        v = O.fill_uniform(grid, seed, 1, -1e-3, 1e-3, dtype)
        m = halo_mask(grid)
        v[m] = u[m]
    s = np.zeros_like(u)
    return v, s, u


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
