"""The streamed drop-in call: st3d_iterate_host on pinned host arrays runs
its uploads, steps and downloads in one cooperative launch (chunks of planes
along i, transfer CTAs and stencil CTAs with device-side dependency
counters).  Bar: bit for bit the host arrays the phase-by-phase call leaves
(upload, iterate, download: host path DIRECT), for both update modes, the
7/13/25-point stencils, ragged chunk counts, one and odd step counts,
halos of every width, row lengths that are not a multiple of four points
(the copies' scalar path) and one-plane chunks; and the oracle's fused
flavour.  The call reports host path STREAMED; pageable arrays fall back."""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import mode_r_inputs, wave_inputs

pytestmark = pytest.mark.gpu

STREAMED = 4


def _pinned_copy(a):
    p = S.PinnedArray(a.shape, a.dtype)
    p.array[...] = a
    return p


def _call(grid, points, mode, steps, v, s, u, host_path, **kw):
    g = S.Grid(*grid)
    pv, ps, pu = _pinned_copy(v), _pinned_copy(s), _pinned_copy(u)
    try:
        extra = dict(kw)
        if mode == "wave":
            extra.setdefault("dt", 5e-4)
        with S.Stencil(g, points, mode, "f32", kernel="tma", host_path=host_path, **extra) as st:
            st.iterate_host(pv.array, ps.array, pu.array, steps)
            path = st.info().host_path
            # a second call on the state the first left
            st.iterate_host(pv.array, ps.array, pu.array, steps)
        return pv.array.copy(), pu.array.copy(), path
    finally:
        for p in (pv, ps, pu):
            p.free()


CASES = [
    # grid, points, mode, steps, extra opts
    ((40, 36, 130, 4, 4, 4), 25, "wave", 5, {}),
    ((37, 20, 61, 4, 4, 4), 25, "wave", 1, {}),            # zs % 4 != 0: scalar copies
    ((50, 33, 128, 4, 4, 16), 13, "wave", 7, {"ichunk": 4}),
    ((23, 17, 40, 1, 1, 1), 7, "wave", 6, {"ichunk": 1}),   # one-plane chunks, 1-point halos
    ((64, 48, 96, 4, 5, 8), 25, "ref", 4, {}),
    ((31, 29, 70, 4, 4, 4), 13, "ref", 3, {"ichunk": 5}),
    ((20, 20, 32, 4, 4, 16), 7, "ref", 9, {}),
]


@pytest.mark.parametrize("grid,points,mode,steps,kw", CASES,
                         ids=["%s-%d-%s-%d" % (c[2], c[1], "x".join(map(str, c[0][:3])), c[3])
                              for c in CASES])
def test_streamed_call_equals_phase_by_phase(grid, points, mode, steps, kw):
    if mode == "wave":
        v, s, u = wave_inputs(grid, 31 + points)
        s = O.fill_uniform(grid, 5, 2, -1.0, 1.0, np.float32)
        xs, ys, zs = grid[:3]
        kw = dict(kw, src=(xs // 2, ys // 3, zs - 2))
    else:
        v, s, u = mode_r_inputs(grid, 17 + points, "f32")
    v1, u1, p1 = _call(grid, points, mode, steps, v, s, u, S.api.HOST_AUTO, **kw)
    v2, u2, p2 = _call(grid, points, mode, steps, v, s, u, S.api.HOST_DIRECT, **kw)
    assert p1 == STREAMED and p2 == S.api.HOST_DIRECT
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(u1, u2)
    if mode == "ref":
        vf = v.copy()
        O.iterate_ref(vf, s, u, grid, points, 2 * steps, fma=True)
        np.testing.assert_array_equal(O.interior(v1, grid), O.interior(vf, grid))


def test_streamed_wave_matches_oracle_across_calls():
    grid = (48, 40, 136, 4, 4, 4)
    v, s, u = wave_inputs(grid, 3, blobs=True)
    src = (24, 20, 68)
    vs, us, path = _call(grid, 25, "wave", 6, v, s, u, S.api.HOST_AUTO, src=src)
    assert path == STREAMED
    c0, c1, c2 = O.wave_constants(25, 1500.0, 5e-4, 10.0)
    # each call restarts the source clock at its upload
    uo, vo = u.copy(), v.copy()
    for _ in range(2):
        O.iterate_wave(uo, vo, s, grid, 25, 6, c0, c1, c2, src=src, amps=O.ricker_amps(0, 6, 5e-4),
                       fma=True)
    np.testing.assert_array_equal(O.interior(us, grid), O.interior(uo, grid))
    np.testing.assert_array_equal(O.interior(vs, grid), O.interior(vo, grid))


def test_pageable_arrays_take_the_phase_by_phase_path():
    grid = (20, 24, 64, 4, 4, 4)
    v, s, u = wave_inputs(grid, 9)
    with S.Stencil(S.Grid(*grid), 7, "wave", "f32", kernel="tma", dt=5e-4) as st:
        st.iterate_host(v, s, u, 3)
        assert st.info().host_path != STREAMED


def test_streamed_call_at_256_cubed_twenty_steps():
    """The 7-point configuration's size and run length (256^3, 20 steps):
    streamed and phase-by-phase calls leave the same host arrays."""
    grid = (256, 256, 256, 4, 4, 4)
    v, s, u = wave_inputs(grid, 20251203)
    v1, u1, p1 = _call(grid, 7, "wave", 20, v, s, u, S.api.HOST_AUTO, dt=1e-3)
    v2, u2, p2 = _call(grid, 7, "wave", 20, v, s, u, S.api.HOST_DIRECT, dt=1e-3)
    assert p1 == STREAMED
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(u1, u2)
