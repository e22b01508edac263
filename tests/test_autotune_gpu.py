"""Every configuration the autotuner may pick computes the same bits: the
tiling knobs (tile rows, stages, unit length, fused steps) change the work
decomposition only.  The tensor-core kernel of the 16-bit delta forms sums in
the tensor cores' order: its candidates agree with each other bit for bit and
with the scalar kernel's within the rounding the tensor-core tests bound.
And the tuner runs end to end on the device."""
import numpy as np
import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import autotune
from oracle import oracle as O
from tests.helpers import halo_mask, rel_l2

pytestmark = pytest.mark.gpu


def _zero_halo_inputs(grid, seed):
    u = O.fill_blobs(grid, seed, 4, 5.0)
    v = (u * np.float32(0.999)).astype(np.float32)
    v[halo_mask(grid)] = 0.0
    s = O.fill_uniform(grid, seed, 2, -1.0, 1.0)
    s[halo_mask(grid)] = 0.0
    return v, s, u


@pytest.mark.parametrize("points,storage", [(13, "f32"), (7, "f32"), (25, "f32"), (25, "f16"),
                                            (7, "bf16"), (13, "f16_hilo")])
def test_all_candidates_compute_the_same_bits(points, storage):
    grid = (37, 45, 300, 4, 4, 4)
    g = S.Grid(*grid)
    v, s, u = _zero_halo_inputs(grid, 5 + points)
    results = []
    for cand in autotune.candidates(points, "wave", storage, zero_halo=True):
        try:
            st = S.Stencil(g, points, "wave", storage, dt=5e-4, src=(18, 22, 150), **cand)
        except S.St3dError:
            continue  # a pipeline depth that does not fit this stencil
        with st:
            st.upload(v, s, u)
            st.iterate(9)
            ua, va = g.empty(), g.empty()
            st.download(va, ua)
            st.synchronize()
        results.append((cand, g.interior(ua).copy(), g.interior(va).copy()))
    assert len(results) >= 3
    for group in ([r for r in results if r[0].get("kernel") != "mma"],
                  [r for r in results if r[0].get("kernel") == "mma"]):
        if not group:
            continue
        c0, u0, v0 = group[0]
        for c, uu, vv in group[1:]:
            assert np.array_equal(uu, u0), (c0, c)
            assert np.array_equal(vv, v0), (c0, c)
    mma = [r for r in results if r[0].get("kernel") == "mma"]
    if mma:
        # nine steps: within three units in the last place of the 16-bit words
        ulp = 2.0 ** -7 if storage == "bf16" else 2.0 ** -10
        u0 = results[0][1]
        assert rel_l2(mma[0][1], u0) < 3 * 2 * ulp


def test_tuner_end_to_end(tmp_path):
    g = S.Grid(96, 80, 200, 4, 4, 4)
    path = str(tmp_path / "tune.json")
    best = autotune.tune(g, 13, "wave", "f32", steps=3, cache=path, zero_halo=True)
    assert best["gpts"] > 0 and best["opts"] in [c for c, _ in best["table"]]
    with autotune.tuned_stencil(g, 13, "wave", "f32", cache=path, zero_halo=True, dt=5e-4) as st:
        info = st.info()
        if best["opts"].get("temporal_block", 1) > 1:
            assert info.temporal_block == best["opts"]["temporal_block"]


def test_batch_tuner_end_to_end(tmp_path):
    grids = [S.Grid(70, 90, 130, 4, 4, 4), S.Grid(100, 64, 200, 4, 4, 4), S.Grid(64, 64, 64, 4, 4, 4)]
    pts = [7, 13, 25]
    best = autotune.tune_batch(grids, pts, dts=[1e-3, 5e-4, 5e-4], steps=3,
                               cache=str(tmp_path / "tune.json"))
    assert best["gpts"] > 0 and best["opts"]["schedule"] in ("graph", "persistent", "pipelined")
