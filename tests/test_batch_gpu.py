"""GPU tests of the batching form: independent grids of uneven sizes and
stencil orders advancing in one persistent launch per step (device work
queue), optionally replayed from a CUDA graph, or in one launch for all
steps of a call (the pipelined schedule: per-grid step counters), against
the sequential schedule and the oracle.  All schedules run the same
arithmetic, so the fields must agree bit for bit."""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import wave_inputs

pytestmark = pytest.mark.gpu


def _grids(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        xs, ys, zs = (int(x) for x in rng.integers(5, 70, size=3))
        pts = int(rng.choice([7, 13, 25]))
        src = tuple(int(rng.integers(0, d)) for d in (xs, ys, zs))
        out.append(((xs, ys, zs, 4, 4, 4), pts, src))
    return out


def _run(specs, steps_list, schedule, seed, **kw):
    grids = [S.Grid(*g) for g, _, _ in specs]
    pts = [p for _, p, _ in specs]
    dts = [1e-3 if p == 7 else 5e-4 for p in pts]
    srcs = [s for _, _, s in specs]
    inputs = [wave_inputs(g, seed + i) for i, (g, _, _) in enumerate(specs)]
    with S.Batch(grids, pts, dt=dts, srcs=srcs, **kw) as b:
        for i, (v, s, u) in enumerate(inputs):
            b.context(i).upload(v, s, u)
        for n in steps_list:
            b.iterate(n, schedule)
        b.synchronize()
        out = []
        for i, g in enumerate(grids):
            u, v = g.empty(), g.empty()
            b.context(i).download(v, u)
            out.append((g.interior(u).copy(), g.interior(v).copy()))
        info = b.info()
    return out, inputs, info


@pytest.mark.parametrize("schedule", ["persistent", "graph", "pipelined"])
def test_batch_schedules_match_sequential_and_oracle(schedule):
    specs = _grids(7, 9)
    steps_list = [5, 4, 4]  # odd first call: buffer parity and graph reuse
    seq, inputs, _ = _run(specs, steps_list, "sequential", 100)
    got, _, info = _run(specs, steps_list, schedule, 100)
    assert info.grids == len(specs) and info.work_items > 0
    if schedule == "graph":
        assert info.graphs >= 1
    for (ua, va), (ub, vb) in zip(got, seq):
        np.testing.assert_array_equal(ua, ub)
        np.testing.assert_array_equal(va, vb)
    # and the oracle's fused flavour, grid by grid
    total = sum(steps_list)
    for i, ((g, p, src), (v, s, u)) in enumerate(zip(specs, inputs)):
        dt = 1e-3 if p == 7 else 5e-4
        c0, c1, c2 = O.wave_constants(p, 1500.0, dt, 10.0)
        uf, vf = u.copy(), v.copy()
        O.iterate_wave(uf, vf, s, g, p, total, c0, c1, c2, src=src, amps=O.ricker_amps(0, total, dt))
        np.testing.assert_array_equal(got[i][0], O.interior(uf, g))


def test_batch_counts_one_launch_per_step():
    specs = _grids(3, 5)
    _, _, info = _run(specs, [6], "persistent", 1)
    assert info.launches == 6
    _, _, info = _run(specs, [6], "sequential", 1)
    assert info.launches == 6 * 5
    _, _, info = _run(specs, [6, 3], "pipelined", 1)
    assert info.launches == 2  # one launch per call


def test_pipelined_many_steps_few_grids():
    """Two grids of very different sizes over many steps in one launch: the
    small grid runs steps ahead of the large one while each grid's steps stay
    in order (per-grid counters); same bits as the sequential schedule."""
    specs = [((96, 70, 140, 4, 4, 4), 25, (40, 30, 70)), ((9, 7, 20, 4, 4, 4), 7, (4, 3, 10))]
    seq, _, _ = _run(specs, [17], "sequential", 5)
    got, _, _ = _run(specs, [17], "pipelined", 5)
    for (ua, va), (ub, vb) in zip(got, seq):
        np.testing.assert_array_equal(ua, ub)
        np.testing.assert_array_equal(va, vb)


def test_batch_rejects_other_forms():
    g = S.Grid(16, 16, 16, 4, 4, 4)
    opts = (S.api.Opts * 1)(S.default_opts(7, "ref", "f32"))
    h = S.api.C.c_void_p()
    rc = S.lib().st3d_batch_create(1, (S.api.GridDesc * 1)(g.desc()), opts, S.api.C.byref(h))
    assert rc == S.api.ERR_UNSUPPORTED


@pytest.mark.parametrize("ichunk", [1, 3, 32])
def test_pipelined_short_units(ichunk):
    """Units of a few planes: a consumer warp can finish a short unit while
    another warp of its CTA still works on the previous one, so completions
    must be counted per unit; every call ends without a timed-out wait and
    with the sequential schedule's bits."""
    specs = _grids(11, 7)
    seq, _, _ = _run(specs, [6, 5], "sequential", 9, ichunk=ichunk)
    got, _, _ = _run(specs, [6, 5], "pipelined", 9, ichunk=ichunk)
    for (ua, va), (ub, vb) in zip(got, seq):
        np.testing.assert_array_equal(ua, ub)
        np.testing.assert_array_equal(va, vb)
