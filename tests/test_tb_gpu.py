"""GPU parity of temporal blocking: T leapfrog steps fused into one pass.

Bar: bit-identical to the same number of plain steps of the TMA kernel and
to the oracle's fused flavour (the fused pass evaluates every level point
with the single-step operation sequence), for step counts that mix fused
passes with single steps, for every depth served: 7 points T = 2, 4; 13
points T = 2, 4 (tiles with 8 columns of k margin, 112 written); 25 points
T = 2.  Temporal blocking needs a zero halo; a non-zero halo is refused at
upload.
"""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import halo_mask

pytestmark = pytest.mark.gpu

DEPTHS = [(7, 2), (7, 4), (13, 2), (13, 4), (25, 2)]


def _inputs(grid, seed):
    """u, v ~ U[-1e-3, 1e-3), s ~ U[-1, 1) in the interior; zero halo."""
    u = O.fill_uniform(grid, seed, 0, -1e-3, 1e-3, np.float32)
    v = O.fill_uniform(grid, seed, 1, -1e-3, 1e-3, np.float32)
    s = O.fill_uniform(grid, seed, 2, -1.0, 1.0, np.float32)
    m = halo_mask(grid)
    for a in (u, v, s):
        a[m] = 0.0
    return v, s, u


def _run(grid, points, T, steps, v, s, u, src, dt=5e-4, **kw):
    g = S.Grid(*grid)
    with S.Stencil(g, points, "wave", "f32", kernel="tma", temporal_block=T, dt=dt, src=src,
                   **kw) as st:
        assert st.info().temporal_block == T
        st.upload(v, s, u)
        st.iterate(steps)
        ua, va = g.empty(), g.empty()
        st.download(va, ua)
        st.synchronize()
    return g.interior(ua), g.interior(va)


@pytest.mark.parametrize("points,T", DEPTHS)
@pytest.mark.parametrize("grid", [(21, 37, 250, 4, 4, 4), (5, 9, 17, 4, 4, 4),
                                  (40, 30, 123, 4, 4, 8), (17, 48, 121, 4, 4, 4)])
def test_fused_equals_plain_steps(points, T, grid):
    v, s, u = _inputs(grid, 11 + points)
    xs, ys, zs = grid[:3]
    src = (xs // 2, ys // 3, zs - 2)
    steps = 3 * T + 1  # three fused passes and a single step
    uf, vf = _run(grid, points, T, steps, v, s, u, src)
    up, vp = _run(grid, points, 1, steps, v, s, u, src)
    np.testing.assert_array_equal(uf, up)
    np.testing.assert_array_equal(vf, vp)
    c0, c1, c2 = O.wave_constants(points, 1500.0, 5e-4, 10.0)
    amps = O.ricker_amps(0, steps, 5e-4)
    uo, vo = u.copy(), v.copy()
    O.iterate_wave(uo, vo, s, grid, points, steps, c0, c1, c2, src=src, amps=amps, fma=True)
    np.testing.assert_array_equal(uf, O.interior(uo, grid))
    np.testing.assert_array_equal(vf, O.interior(vo, grid))


@pytest.mark.parametrize("points,T", DEPTHS)
def test_fused_small_chunks_many_units(points, T):
    """Short i-chunks: many work units per CTA, rings and queues reused
    across units."""
    grid = (33, 50, 260, 4, 4, 4)
    v, s, u = _inputs(grid, 3)
    uf, vf = _run(grid, points, T, 2 * T, v, s, u, None, ichunk=3)
    up, vp = _run(grid, points, 1, 2 * T, v, s, u, None)
    np.testing.assert_array_equal(uf, up)
    np.testing.assert_array_equal(vf, vp)


def test_fill_on_a_fused_context_keeps_the_halo_zero():
    """Device fills of a context that blocks in time write the interior only;
    its steps then match plain steps from the same (downloaded) start."""
    grid = (24, 40, 200, 4, 4, 4)
    g = S.Grid(*grid)
    src = (12, 20, 100)
    u0, v0, s0 = g.empty(), g.empty(), g.empty()
    u0[:], v0[:], s0[:] = 0.0, 0.0, 0.0
    with S.Stencil(g, 7, "wave", "f32", kernel="tma", temporal_block=4, dt=5e-4, src=src) as st:
        st.fill(S.api.FIELD_U, S.api.FILL_BLOBS, seed=4, a=8, b=20.0)
        st.fill(S.api.FIELD_V, S.api.FILL_BLOBS, seed=4, a=8, b=20.0)
        st.fill(S.api.FIELD_S, S.api.FILL_CONST, a=0.0)
        st.download(v0, u0)
        st.iterate(9)
        ua, va = g.empty(), g.empty()
        st.download(va, ua)
        nf = st.norms()
    assert np.abs(g.interior(u0)).max() > 0
    with S.Stencil(g, 7, "wave", "f32", kernel="tma", temporal_block=1, dt=5e-4, src=src) as st:
        st.upload(v0, s0, u0)
        st.iterate(9)
        ub, vb = g.empty(), g.empty()
        st.download(vb, ub)
        npl = st.norms()
    np.testing.assert_array_equal(g.interior(ua), g.interior(ub))
    np.testing.assert_array_equal(g.interior(va), g.interior(vb))
    assert nf == npl


def test_nonzero_halo_is_refused():
    grid = (10, 12, 40, 4, 4, 4)
    v, s, u = _inputs(grid, 1)
    u[0, 5, 10] = 1.0  # an i-halo plane point the stencil reads
    g = S.Grid(*grid)
    with S.Stencil(g, 7, "wave", "f32", kernel="tma", temporal_block=2, dt=5e-4) as st:
        with pytest.raises(S.St3dError) as e:
            st.upload(v, s, u)
        assert e.value.status == S.api.ERR_UNSUPPORTED


@pytest.mark.parametrize("points,T,rows", [(7, 2, 26), (7, 4, 18), (13, 2, 18), (13, 4, 15),
                                           (25, 2, 15), (7, 1, 0)])
def test_fused_tile_height_is_reported(points, T, rows):
    """st3d_info.tb_tile_j: the level-1 rows of a fused pass's tile (the
    height the plan's tensor maps and the kernel share), 0 without fusion."""
    g = S.Grid(40, 60, 130, 4, 4, 4)
    with S.Stencil(g, points, "wave", "f32", kernel="tma", temporal_block=T, dt=5e-4) as st:
        info = st.info()
        assert info.temporal_block == T
        assert info.tb_tile_j == rows
