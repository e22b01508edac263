"""GPU parity of the precision forms, all arithmetic in FP32:
  - FP16 / BF16: u and the time difference d = u^n - u^{n-1} in 16-bit
    words with a power-of-two scale per i-plane (the delta form);
  - FP16 hi/lo pair: the delta form with u held as two FP16 words;
  - FP16 + a compensating byte: u and v in FP16 words plus a low byte.

The library's scalar 16-bit kernels (kernel "tma") and the oracle's
restatement of the same encoding, scale rule and update must agree bit for
bit (decoded u and v after several steps), for the 7-, 13- and 25-point
stencils; the tensor-core kernel of the delta forms is checked against the
same restatement within rounding in tests/test_mma16_gpu.py.  The 16-bit
forms keep a zero halo (a zero Dirichlet boundary); other halos are refused.
"""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import halo_mask, rel_l2

pytestmark = pytest.mark.gpu


def _inputs(grid, seed, blobs):
    if blobs:
        u = O.fill_blobs(grid, seed, 4, 6.0)
    else:
        u = O.fill_uniform(grid, seed, 0, -1e-3, 1e-3)
        u[halo_mask(grid)] = 0.0
    v = u * np.float32(0.999) if blobs else O.fill_uniform(grid, seed, 1, -1e-3, 1e-3)
    v[halo_mask(grid)] = 0.0
    s = np.zeros_like(u)
    return np.ascontiguousarray(v), s, u


@pytest.mark.parametrize("storage", ["f16", "bf16", "f16_hilo", "f16_hl"])
@pytest.mark.parametrize("points", [7, 13, 25])
@pytest.mark.parametrize("grid,blobs", [((24, 40, 150, 4, 4, 4), True),
                                        ((9, 17, 64, 4, 4, 16), False)])
def test_f16_forms_match_oracle(storage, points, grid, blobs):
    dt = 1e-3 if points == 7 else 5e-4
    steps = 9
    src = (grid[0] // 2, grid[1] // 2, grid[2] // 2)
    v, s, u = _inputs(grid, 3 + points, blobs)
    g = S.Grid(*grid)
    with S.Stencil(g, points, "wave", storage, dt=dt, src=src, kernel="tma") as st:
        assert st.info().kernel == S.KERNEL_TMA
        uu, vv = u.copy(), v.copy()
        st.iterate_host(vv, s, uu, steps)
    ou, ov = _oracle_run(storage, u, v, s, grid, points, steps, dt, src)
    np.testing.assert_array_equal(O.interior(uu, grid), O.interior(ou, grid))
    np.testing.assert_array_equal(O.interior(vv, grid), O.interior(ov, grid))


@pytest.mark.parametrize("points", [7, 25])
@pytest.mark.parametrize("storage,tile_j,stages", [
    ("f16", 16, 12), ("f16", 16, 4), ("f16", 20, 10), ("f16", 20, 6), ("f16", 8, 8),
    ("f16_hl", 16, 8), ("f16_hl", 20, 8), ("f16_hl", 20, 6), ("f16_hl", 8, 4)])
def test_delta_form_tiles_match_oracle(points, storage, tile_j, stages):
    """Every tile height and pipeline depth of the delta kernel gives the
    oracle's bits; ys = 43 leaves a partial tile for 8, 16 and 20 rows."""
    grid = (30, 43, 140, 4, 4, 4)
    dt = 1e-3 if points == 7 else 5e-4
    steps = 7
    src = (15, 21, 70)
    v, s, u = _inputs(grid, 40 + points, True)
    with S.Stencil(S.Grid(*grid), points, "wave", storage, dt=dt, src=src, tile_j=tile_j,
                   stages=stages, kernel="tma") as st:
        assert st.info().tile_j == tile_j
        uu, vv = u.copy(), v.copy()
        st.iterate_host(vv, s, uu, steps)
    ou, ov = _oracle_run(storage, u, v, s, grid, points, steps, dt, src)
    np.testing.assert_array_equal(O.interior(uu, grid), O.interior(ou, grid))
    np.testing.assert_array_equal(O.interior(vv, grid), O.interior(ov, grid))


def _oracle_run(storage, u, v, s, grid, points, steps, dt, src=None, t0=0):
    """(u, v) after `steps` steps of the oracle's restatement of the form."""
    kind, hilo = O.storage_kind(storage)
    c0, c1, c2 = O.wave_constants(points, 1500.0, dt, 10.0)
    amps = O.ricker_amps(t0, steps, dt)
    fs = O.Field16(s, grid, kind, hilo and False)
    if not hilo:
        fu, fd = O.delta_fields(u, v, grid, kind, pair=storage == "f16_hl")
        O.iterate_delta16(fu, fd, fs, grid, points, steps, np.float32(c1), np.float32(c2), src=src,
                          amps=amps)
        return O.delta_decode(fu, fd)
    fu, fv = (O.Field16(x, grid, kind, hilo) for x in (u, v))
    O.iterate_wave16(fu, fv, fs, grid, points, steps, np.float32(c1), np.float32(c2), src=src,
                     amps=amps)
    return fu.decode(), fv.decode()


@pytest.mark.parametrize("storage,bound", [("f16_hilo", 3e-4), ("f16_hl", 6e-4), ("f16", 3e-3),
                                           ("bf16", 2e-2)])
def test_f16_forms_track_fp64(storage, bound):
    """Accuracy of each form against FP64 after 60 steps of a smooth field."""
    grid = (32, 36, 140, 4, 4, 4)
    dt = 5e-4
    v, s, u = _inputs(grid, 11, True)
    g = S.Grid(*grid)
    with S.Stencil(g, 25, "wave", storage, dt=dt) as a, S.Stencil(g, 25, "wave", "f64", dt=dt) as b:
        a.upload(v, s, u)
        b.upload(v.astype(np.float64), s.astype(np.float64), u.astype(np.float64))
        a.iterate(60)
        b.iterate(60)
        a.synchronize()
        b.synchronize()
        err = a.rel_l2(b)
    assert err < bound, err


def test_f16_rejects_nonzero_halo():
    grid = (8, 20, 40, 4, 4, 4)
    u = O.fill_uniform(grid, 1, 0, -1.0, 1.0)
    g = S.Grid(*grid)
    with S.Stencil(g, 7, "wave", "f16") as st:
        with pytest.raises(S.St3dError) as e:
            st.upload(u=u)
        assert e.value.status == S.api.ERR_UNSUPPORTED


def test_f16_norms_and_fill():
    grid = (12, 20, 70, 4, 4, 4)
    g = S.Grid(*grid)
    with S.Stencil(g, 13, "wave", "f16_hilo", dt=5e-4) as st:
        st.fill(S.FIELD_U, S.FILL_BLOBS, 5, 3, 4.0)
        st.fill(S.FIELD_V, S.FILL_CONST, 0, 0.0)
        st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
        u = g.empty()
        st.download(u=u)
        e2, _, em, _ = st.norms(S.FIELD_U)
        ui = g.interior(u).astype(np.float64)
        assert np.isclose(e2, np.sum(ui ** 2), rtol=1e-12) and em == np.max(np.abs(ui))
        assert np.all(u[halo_mask(grid)] == 0.0)


@pytest.mark.parametrize("storage", ["f16", "bf16", "f16_hl"])
def test_delta_form_partial_uploads_and_fills(storage):
    """Setting u or v alone rebuilds the pair from the device state first;
    fills go through the same path; norms of v decode u - d."""
    grid = (10, 18, 70, 4, 4, 4)
    dt = 5e-4
    v, s, u = _inputs(grid, 21, True)
    g = S.Grid(*grid)
    with S.Stencil(g, 13, "wave", storage, dt=dt) as st:
        st.upload(v, s, u)
        st.iterate(3)
        # replace v only: u stays the device's u^3
        u3, v3 = g.empty(), g.empty()
        st.download(v3, u3)
        st.upload(v=v)
        ua, va = g.empty(), g.empty()
        st.download(va, ua)
        # u re-encoded from u3 (its own plane scales), v = dec(U) - dec(D)
        # with D = enc(u3 - v)
        kind, _ = O.storage_kind(storage)
        fu, fd = O.delta_fields(u3, v, grid, kind, pair=storage == "f16_hl")
        eu, ev = O.delta_decode(fu, fd)
        np.testing.assert_array_equal(g.interior(ua), O.interior(eu, grid))
        np.testing.assert_array_equal(g.interior(va), O.interior(ev, grid))
        assert np.max(np.abs(g.interior(ua) - g.interior(u3))) <= 2.0 ** -20 * np.max(np.abs(u3))
        # device norms of v decode the same values
        e2, _, em, _ = st.norms(S.FIELD_V)
        vi = g.interior(va).astype(np.float64)
        assert np.isclose(e2, np.sum(vi ** 2), rtol=1e-12) and em == np.max(np.abs(vi))
        # fills: u blobs, v zero -> d = u
        st.fill(S.FIELD_U, S.FILL_BLOBS, 5, 3, 4.0)
        st.fill(S.FIELD_V, S.FILL_CONST, 0, 0.0)
        ub, vb = g.empty(), g.empty()
        st.download(vb, ub)
        assert np.all(g.interior(vb) == 0.0) or np.max(np.abs(g.interior(vb))) <= \
            2.0 ** -8 * np.max(np.abs(g.interior(ub)))
        assert np.all(ub[halo_mask(grid)] == 0.0)
