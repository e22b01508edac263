"""Parity at the benchmark configurations' full sizes.

  - 7 points, 256^3, 20 steps, 25 points, 528^3, 200 steps, and the
    headline size, 25 points at 1024^3 for 20 steps (stencil_25_ref_1,
    stencil_25.h:75-95), mode R on seeded u, v ~ U[-1, 1), s ~ U[0.5, 1.5):
    the library through the drop-in call equals the oracle's fused flavour
    bit for bit, and the reference order (the oracle's plain flavour, pinned
    to the compiled reference) within 1e-5 relative L2;
  - 13 points, 1040^3, leapfrog wave with 8 seeded Gaussian blobs, 21 steps:
    plain steps equal the oracle's wave restatement bit for bit, and every
    temporal-blocking depth served equals plain steps bit for bit;
  - the 64-grid batch (axes U{64..320}, orders {7, 13, 25}): the graph
    schedule equals the sequential one bit for bit on every grid;
  - 1264^3, the largest grid the reference's command line accepts, in FP32
    (both kernels, known answer) and in the FP16 delta and pair forms.
"""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import mode_r_inputs, rel_l2

pytestmark = pytest.mark.gpu

# temporal-blocking depths the library serves for the 13-point stencil
TB13 = (1, 2, 4)


@pytest.mark.parametrize("points,n,steps", [(7, 256, 20), (25, 528, 200), (25, 1024, 20)])
def test_mode_r_full_size(points, n, steps):
    grid = (n, n, n, 4, 4, 16)
    v, s, u = mode_r_inputs(grid, 20251203 + points, "f32")
    vg = v.copy()
    with S.Stencil(S.Grid(*grid), points, "ref", "f32") as st:
        assert st.info().kernel == S.KERNEL_TMA
        st.iterate_host(vg, s, u, steps)
    vf = v.copy()
    O.iterate_ref(vf, s, u, grid, points, steps, fma=True)
    np.testing.assert_array_equal(O.interior(vg, grid), O.interior(vf, grid))
    del vf
    vp = v.copy()
    O.iterate_ref(vp, s, u, grid, points, steps, fma=False)
    assert rel_l2(O.interior(vg, grid), O.interior(vp, grid)) <= 1e-5


def test_temporal_blocking_full_size():
    g = S.Grid(1040, 1040, 1040, 4, 4, 4)
    grid = g.tuple
    ctx = []
    try:
        for T in TB13:
            st = S.Stencil(g, 13, "wave", "f32", kernel="tma", temporal_block=T, dt=5e-4,
                           src=(520, 520, 520))
            ctx.append(st)
            st.fill(S.FIELD_U, S.FILL_BLOBS, 20251203, 8, 20.0)
            st.fill(S.FIELD_V, S.FILL_BLOBS, 20251203, 8, 20.0)
            st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
            st.iterate(21)
            st.synchronize()
        for other in ctx[1:]:
            for field in (S.FIELD_U, S.FIELD_V):
                d2, b2, dm, bm = other.norms(field, ctx[0], field)
                assert b2 > 0 and d2 == 0.0 and dm == 0.0
        # the plain steps against the oracle's restatement of the wave form
        ug, vg = g.empty(), g.empty()
        ctx[0].download(vg, ug)
    finally:
        for st in ctx:
            st.close()
    u = O.fill_blobs(grid, 20251203, 8, 20.0)
    v = u.copy()
    s = np.zeros_like(u)
    c0, c1, c2 = O.wave_constants(13, 1500.0, 5e-4, 10.0)
    O.iterate_wave(u, v, s, grid, 13, 21, c0, c1, c2, src=(520, 520, 520),
                   amps=O.ricker_amps(0, 21, 5e-4), fma=True)
    np.testing.assert_array_equal(O.interior(ug, grid), O.interior(u, grid))
    np.testing.assert_array_equal(O.interior(vg, grid), O.interior(v, grid))


def test_batch_full_workload_graph_equals_sequential():
    import bench
    specs = bench.batch_specs()
    grids = [S.Grid(xs, ys, zs, 4, 4, 4) for (xs, ys, zs), _, _ in specs]
    pts = [p for _, p, _ in specs]
    dts = [1e-3 if p == 7 else 5e-4 for p in pts]
    srcs = [sp for _, _, sp in specs]
    batches = []
    try:
        for schedule in ("sequential", "graph", "pipelined"):
            b = S.Batch(grids, pts, dt=dts, srcs=srcs)
            batches.append(b)
            for i in range(len(grids)):
                st = b.context(i)
                st.fill(S.FIELD_U, S.FILL_BLOBS, 7 + i, 4, 12.0)
                st.fill(S.FIELD_V, S.FILL_BLOBS, 7 + i, 4, 12.0)
                st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
            b.iterate(5, schedule)
            b.synchronize()
        for other in batches[1:]:
            for i in range(len(grids)):
                a, c = batches[0].context(i), other.context(i)
                for field in (S.FIELD_U, S.FIELD_V):
                    d2, b2, dm, bm = c.norms(field, a, field)
                    assert b2 > 0 and d2 == 0.0, (i, field)
    finally:
        for b in batches:
            b.close()


@pytest.mark.parametrize("points", [7, 25])
def test_largest_grid_the_reference_accepts(points):
    """1264^3, the largest interior the reference's command line accepts
    (main.cpp:125-144): 2.0e9 points, so linear indices run past 2^31.  The
    known-answer run (u = s = 1, v = 0 gives v = n after n steps) holds on
    every point, for the TMA and the direct-load kernels."""
    g = S.Grid(1264, 1264, 1264, 4, 4, 16)
    for kernel in ("tma", "simple"):
        with S.Stencil(g, points, "ref", "f32", kernel=kernel) as st:
            st.fill(S.FIELD_U, S.FILL_CONST, 0, 1.0)
            st.fill(S.FIELD_S, S.FILL_CONST, 0, 1.0)
            st.fill(S.FIELD_V, S.FILL_CONST, 0, 0.0)
            st.iterate(2)
            assert st.check(2.0) == 0
            st.iterate(1)
            assert st.check(3.0) == 0
            assert st.check(2.0) == 1264 ** 3


def test_largest_grid_in_16bit_storage():
    """1264^3 in the FP16 delta form and its hi/lo pair form: word offsets run
    past 2^31 in the 16-bit kernels, encoders and decoders.  Three steps of a
    blob field stay within the forms' rounding of the FP32 run (device
    reductions over every point)."""
    g = S.Grid(1264, 1264, 1264, 4, 4, 4)
    ctx = {}
    try:
        for storage in ("f32", "f16", "f16_hl"):
            st = S.Stencil(g, 25, "wave", storage, dt=5e-4, src=(632, 632, 632))
            ctx[storage] = st
            st.fill(S.FIELD_U, S.FILL_BLOBS, 20251203, 8, 40.0)
            st.fill(S.FIELD_V, S.FILL_BLOBS, 20251203, 8, 40.0)
            st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
            st.iterate(3)
            st.synchronize()
        for storage, bound in (("f16", 2e-3), ("f16_hl", 1e-4)):
            d2, b2, dm, bm = ctx[storage].norms(S.FIELD_U, ctx["f32"], S.FIELD_U)
            assert b2 > 0 and np.isfinite(d2) and (d2 / b2) ** 0.5 < bound, (storage, d2, b2)
    finally:
        for st in ctx.values():
            st.close()
