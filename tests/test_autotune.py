"""The autotuner's search and cache without a GPU: a model of the timings
replaces the device measurement; every candidate is a configuration the
library's planner accepts."""
import json

import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import api, autotune

DEV = {"sm_count": 152, "cc": (10, 3), "total_bytes": 1 << 38}
GRID = S.Grid(256, 256, 256, 4, 4, 4)


@pytest.mark.parametrize("points,mode,storage", [
    (25, "wave", "f32"), (13, "wave", "f32"), (7, "wave", "f32"), (7, "ref", "f32"),
    (25, "ref", "f64"), (2, "ref", "f32"), (25, "wave", "f16"), (13, "wave", "bf16"),
    (7, "wave", "f16_hilo"), (25, "wave", "f16_hl"), (7, "wave", "f16_hl")])
def test_candidates_are_accepted_by_the_planner(points, mode, storage):
    cands = autotune.candidates(points, mode, storage, zero_halo=True)
    assert cands
    for c in cands:
        o = S.default_opts(points, mode, storage, dt=5e-4, **c)
        info = S.plan(GRID, o)  # raises St3dError when refused
        if c.get("temporal_block", 1) > 1:
            assert info.temporal_block == c["temporal_block"]


def test_temporal_blocking_only_on_request():
    plain = autotune.candidates(13, "wave", "f32")
    fused = autotune.candidates(13, "wave", "f32", zero_halo=True)
    assert not any(c.get("temporal_block", 1) > 1 for c in plain)
    assert any(c.get("temporal_block", 1) == 2 for c in fused)
    assert any(c.get("temporal_block", 1) == 4 for c in fused)  # (T-1)R = 6 <= 8
    deep = autotune.candidates(25, "wave", "f32", zero_halo=True)
    assert {c.get("temporal_block", 1) for c in deep} == {1, 2}  # 25 points: T=4 is (T-1)R = 12


def test_tune_picks_the_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    calls = []

    def model(c):
        calls.append(c)
        if c.get("stages") == 12:
            return None  # refused by the library
        return 10.0 - c.get("stages", 0) * 0.5 - (0.25 if c.get("tile_j") == 8 else 0.0)

    r = autotune.tune(GRID, 13, "wave", "f16", cache=path, measure=model, device=DEV)
    assert r["opts"] == {"kernel": "tma", "tile_j": 20, "stages": 10}
    assert abs(r["ms_per_step"] - 5.0) < 1e-12
    assert r["gpts"] == pytest.approx(256 ** 3 / 5.0e-3 / 1e9)
    n = len(calls)
    assert n == len(autotune.candidates(13, "wave", "f16"))
    # cached: no measurement the second time
    r2 = autotune.tune(GRID, 13, "wave", "f16", cache=path, measure=model, device=DEV)
    assert len(calls) == n and r2["opts"] == r["opts"]
    stored = json.load(open(path))
    assert r["key"] in stored and "|13|wave|f16|256x256x256|" in r["key"]
    # refresh re-measures; another workload gets its own key
    autotune.tune(GRID, 13, "wave", "f16", cache=path, measure=model, device=DEV, refresh=True)
    assert len(calls) == 2 * n
    autotune.tune(GRID, 7, "wave", "f16", cache=path, measure=model, device=DEV)
    assert len(json.load(open(path))) == 2


def test_tune_fails_when_nothing_runs(tmp_path):
    with pytest.raises(S.St3dError) as e:
        autotune.tune(GRID, 25, "wave", "f32", cache=str(tmp_path / "t.json"),
                      measure=lambda c: None, device=DEV)
    assert e.value.status == api.ERR_UNSUPPORTED


def test_cache_survives_a_corrupt_file(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    r = autotune.tune(GRID, 7, "wave", "f32", cache=str(path), measure=lambda c: 1.0, device=DEV)
    assert r["opts"] == autotune.candidates(7, "wave", "f32")[0]
    assert json.load(open(path))[r["key"]]["ms_per_step"] == 1.0


def test_tune_batch_picks_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    grids = [S.Grid(64, 80, 96, 4, 4, 4), S.Grid(120, 64, 200, 4, 4, 4)]
    pts = [7, 25]
    seen = []

    def model(c):
        seen.append(c)
        return {32: 3.0, 64: 2.0, 128: 2.5, 256: 2.6, 512: 2.7}[c["ichunk"]] - \
            (0.1 if c["schedule"] == "graph" else 0.0)

    r = autotune.tune_batch(grids, pts, cache=path, measure=model, device=DEV)
    assert r["opts"] == {"ichunk": 64, "schedule": "graph"}
    assert len(seen) == len(autotune.batch_candidates())
    r2 = autotune.tune_batch(grids, pts, cache=path, measure=model, device=DEV)
    assert r2["opts"] == r["opts"] and len(seen) == len(autotune.batch_candidates())
    # a different batch has its own key
    other = autotune.batch_key(grids[::-1], pts[::-1], DEV)
    assert other != r["key"]
