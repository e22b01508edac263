"""GPU parity: the CUDA kernels through the C ABI against the oracle and the
reference's golden outputs.

Bars (written in each test):
  - mode R, FP32: relative L2 <= 1e-5 against the reference result (the
    spec bound; only FMA ordering differs), and bit-identical to the
    oracle's fused flavour, which evaluates the same operations in the same
    order.
  - mode R, FP64: relative L2 <= 1e-13 against the reference, bit-identical to
    the fused oracle.
  - mode W: bit-identical to the fused oracle (FP32 and FP64), relative L2
    <= 1e-5 against the oracle's plain flavour.
"""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import golden_cases, mode_r_inputs, np_dtype, rel_l2, wave_inputs

pytestmark = pytest.mark.gpu

META, ARRAYS = golden_cases()
KERNELS = ["simple", "tma"]


def _kernel_ok(kernel, points, dtype):
    return not (kernel == "tma" and (points == 2 or dtype == "f64"))


def _run_mode_r(grid, points, dtype, iters, kernel, v, s, u):
    g = S.Grid(*grid)
    with S.Stencil(g, points, "ref", dtype, kernel=kernel) as st:
        st.iterate_host(v, s, u, iters)
        info = st.info()
    return info


# the TMA kernel serves FP32 7/13/25 points; the simple kernel every case
GOLDEN_RUNS = [pytest.param(m, k, id="%s-%s" % (m["name"], k))
               for m in META for k in KERNELS if _kernel_ok(k, m["points"], m["dtype"])]


@pytest.mark.parametrize("case,kernel", GOLDEN_RUNS)
def test_mode_r_golden(case, kernel):
    pts, dtype, grid, iters = case["points"], case["dtype"], tuple(case["grid"]), case["iterations"]
    v, s, u = mode_r_inputs(grid, case["seed"], dtype)
    v0 = v.copy()
    info = _run_mode_r(grid, pts, dtype, iters, kernel, v, s, u)
    assert info.kernel == (S.KERNEL_TMA if kernel == "tma" else S.KERNEL_SIMPLE)
    got = O.interior(v, grid)
    # the reference result: the fixture, or the oracle pinned to it by digest
    ref = ARRAYS.get(case["name"])
    if ref is None:
        vr, sr, ur = mode_r_inputs(grid, case["seed"], dtype)
        O.iterate_ref(vr, sr, ur, grid, pts, iters)
        ref = O.interior(vr, grid)
    bound = 1e-13 if dtype == "f64" else 1e-5
    assert rel_l2(got, ref) <= bound
    # same operation sequence as the fused oracle: identical bits
    vf, sf, uf = mode_r_inputs(grid, case["seed"], dtype)
    O.iterate_ref(vf, sf, uf, grid, pts, iters, fma=True)
    np.testing.assert_array_equal(got, O.interior(vf, grid))
    # halos of v are never written (the reference writes the interior only)
    mask = np.ones(v.shape, bool)
    xs, ys, zs, xh, yh, zh = grid
    mask[xh:xh + xs, yh:yh + ys, zh:zh + zs] = False
    np.testing.assert_array_equal(v[mask], v0[mask])


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("points", [7, 13, 25])
def test_known_answer(points, kernel):
    """init_arrays + check (iterators.cpp:292-325) through the drop-in call."""
    g = S.Grid(40, 36, 200, 4, 4, 16)
    v, s, u = g.empty(), g.empty(), g.empty()
    S.init_arrays(v, s, u, g.gsize)
    with S.Stencil(g, points, "ref", "f32", kernel=kernel) as st:
        st.iterate_host(v, s, u, 1)
        assert S.check(v, g, 1) == 0
        st.iterate_host(v, s, u, 20)
        assert S.check(v, g, 21) == 0
        assert st.check(21.0, 0.1) == 0


def test_iterate_gb300_drop_in_signature():
    """ITERATE(v, s, u, grid, prefetch_dist, dups, iterations, cacheiter)."""
    g = S.Grid(24, 20, 40, 4, 4, 16)
    v, s, u = mode_r_inputs(g.tuple, 7, "f32")
    vr = v.copy()
    S.iterate_gb300(v, s, u, g, 64, 1, 5, 1, points=13)
    O.iterate_ref(vr, s, u, g.tuple, 13, 5)
    assert rel_l2(g.interior(v), g.interior(vr)) <= 1e-5


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("points", [7, 13, 25])
@pytest.mark.parametrize("grid", [(30, 33, 150, 4, 4, 4), (9, 17, 64, 4, 4, 16),
                                  (5, 40, 300, 4, 4, 8)])
def test_mode_w_fp32(points, kernel, grid):
    dt = 1e-3 if points == 7 else 5e-4
    steps = 12
    src = (grid[0] // 2, grid[1] // 2, grid[2] // 2)
    v, s, u = wave_inputs(grid, 31 + points)
    g = S.Grid(*grid)
    with S.Stencil(g, points, "wave", "f32", kernel=kernel, dt=dt, src=src) as st:
        vv, uu = v.copy(), u.copy()
        st.iterate_host(vv, s, uu, steps)
    c0, c1, c2 = O.wave_constants(points, 1500.0, dt, 10.0)
    amps = O.ricker_amps(0, steps, dt)
    uf, vf = u.copy(), v.copy()
    O.iterate_wave(uf, vf, s, grid, points, steps, c0, c1, c2, src=src, amps=amps, fma=True)
    np.testing.assert_array_equal(O.interior(uu, grid), O.interior(uf, grid))
    np.testing.assert_array_equal(O.interior(vv, grid), O.interior(vf, grid))
    up, vp = u.copy(), v.copy()
    O.iterate_wave(up, vp, s, grid, points, steps, c0, c1, c2, src=src, amps=amps, fma=False)
    assert rel_l2(O.interior(uu, grid), O.interior(up, grid)) <= 1e-5


@pytest.mark.parametrize("points", [7, 13, 25])
def test_mode_w_fp64(points):
    grid = (14, 18, 40, 4, 4, 4)
    dt = 5e-4
    src = (7, 9, 20)
    v, s, u = wave_inputs(grid, 5, np.float64)
    g = S.Grid(*grid)
    with S.Stencil(g, points, "wave", "f64", dt=dt, src=src) as st:
        vv, uu = v.copy(), u.copy()
        st.iterate_host(vv, s, uu, 9)
    c0, c1, c2 = O.wave_constants(points, 1500.0, dt, 10.0)
    amps = O.ricker_amps(0, 9, dt, dtype=np.float64)
    O.iterate_wave(u, v, s, grid, points, 9, c0, c1, c2, src=src, amps=amps, fma=True)
    np.testing.assert_array_equal(O.interior(uu, grid), O.interior(u, grid))


@pytest.mark.parametrize("kernel", KERNELS)
def test_device_resident_steps_match_host_round_trips(kernel):
    """iterate(n) on resident fields == n single-step drop-in calls."""
    grid = (20, 24, 140, 4, 4, 4)
    g = S.Grid(*grid)
    v, s, u = wave_inputs(grid, 8)
    with S.Stencil(g, 25, "wave", "f32", kernel=kernel, dt=5e-4, src=None) as st:
        st.upload(v, s, u)
        st.iterate(6)
        ua, va = g.empty(), g.empty()
        st.download(va, ua)
    ub, vb = u.copy(), v.copy()
    with S.Stencil(g, 25, "wave", "f32", kernel=kernel, dt=5e-4, src=None) as st:
        for _ in range(6):
            st.iterate_host(vb, s, ub, 1)
    np.testing.assert_array_equal(g.interior(ua), g.interior(ub))


@pytest.mark.parametrize("points", [7, 13, 25])
@pytest.mark.parametrize("grid", [(1, 1, 1, 4, 4, 4), (3, 2, 5, 4, 4, 4), (2, 50, 7, 4, 4, 16),
                                  (6, 3, 129, 4, 4, 4)])
def test_ragged_and_tiny_grids(points, grid):
    for kernel in KERNELS:
        v, s, u = mode_r_inputs(grid, 77, "f32")
        vr = v.copy()
        with S.Stencil(S.Grid(*grid), points, "ref", "f32", kernel=kernel) as st:
            st.iterate_host(v, s, u, 2)
        O.iterate_ref(vr, s, u, grid, points, 2, fma=True)
        np.testing.assert_array_equal(v, vr)


def test_errors_are_reported():
    g = S.Grid(8, 8, 8, 4, 4, 4)
    with S.Stencil(g, 7) as st:
        with pytest.raises(S.St3dError) as e:
            st.iterate(1)
        assert e.value.status == S.api.ERR_STATE
    with pytest.raises(S.St3dError) as e:
        S.Stencil(S.Grid(8, 8, 8, 2, 4, 4), 25)
    assert e.value.status == S.api.ERR_INVALID


def test_norms_fp64_reduction():
    grid = (12, 10, 50, 4, 4, 4)
    g = S.Grid(*grid)
    v, s, u = mode_r_inputs(grid, 3, "f32")
    with S.Stencil(g, 7) as a, S.Stencil(g, 7, storage="f64") as b:
        a.upload(v, s, u)
        b.upload(v.astype(np.float64) * 0.5, s.astype(np.float64), u.astype(np.float64) * 2.0)
        d2, b2, dm, bm = a.norms(S.FIELD_U, b, S.FIELD_U)
        ui = g.interior(u).astype(np.float64)
        assert np.isclose(d2, np.sum((ui - 2 * ui) ** 2), rtol=1e-12)
        assert np.isclose(b2, np.sum((2 * ui) ** 2), rtol=1e-12)
        assert dm == np.max(np.abs(ui)) and bm == np.max(np.abs(2 * ui))
        e2, _, em, _ = a.norms(S.FIELD_V)
        vi = g.interior(v).astype(np.float64)
        assert np.isclose(e2, np.sum(vi ** 2), rtol=1e-12) and em == np.max(np.abs(vi))


def test_device_fill_matches_host_generator():
    grid = (10, 12, 33, 4, 4, 4)
    g = S.Grid(*grid)
    with S.Stencil(g, 25) as st:
        st.fill(S.FIELD_U, S.FILL_UNIFORM, 42, -1.0, 1.0)
        st.fill(S.FIELD_V, S.FILL_CONST, 0, 0.25)
        st.fill(S.FIELD_S, S.FILL_BLOBS, 9, 8, 3.0)
        u, v, s = g.empty(), g.empty(), g.empty()
        st.download(v, u)
    np.testing.assert_array_equal(g.interior(u), O.interior(O.fill_uniform(grid, 42, 0, -1.0, 1.0), grid))
    assert np.all(g.interior(v) == 0.25)


def test_vec16_variant_coefficient():
    """Mode R with the 13-point vec_16 K = 6.25 (the reference's variant
    kernel): bit-identical to the oracle's fused flavour with that K."""
    grid = (20, 24, 130, 4, 4, 16)
    v, s, u = mode_r_inputs(grid, 12, "f32")
    o = S.default_opts(13, "ref", "f32")
    o.coef[1] = 6.25
    coefs = O.default_coefs(13, np.float32)
    coefs[1] = 6.25
    for kernel in (S.KERNEL_TMA, S.KERNEL_SIMPLE):
        o.kernel = kernel
        vv = v.copy()
        with S.Stencil(S.Grid(*grid), 13, opts=o) as st:
            st.iterate_host(vv, s, u, 4)
        vf = v.copy()
        O.iterate_ref(vf, s, u, grid, 13, 4, coefs=coefs, fma=True)
        np.testing.assert_array_equal(O.interior(vv, grid), O.interior(vf, grid))


def test_metrics_report_the_timed_region():
    """st3d_metrics_get: steps in the last timer region, throughput, the
    reference's GFlop/s count, energy and max of u, relative L2 to another
    context."""
    grid = (20, 24, 140, 4, 4, 4)
    g = S.Grid(*grid)
    v, s, u = wave_inputs(grid, 8)
    with S.Stencil(g, 13, "wave", "f32", dt=5e-4) as a, S.Stencil(g, 13, "wave", "f32", dt=5e-4) as b:
        for st in (a, b):
            st.upload(v, s, u)
        a.iterate(2)
        a.timer_start()
        a.iterate(5)
        a.timer_stop()
        b.iterate(7)
        m = a.metrics(b)
        assert m["timed_steps"] == 5 and m["steps"] == 7 and m["elapsed_ms"] > 0
        pts = 20 * 24 * 140
        assert abs(m["gpts"] - pts * 5 / (m["elapsed_ms"] * 1e-3) / 1e9) < 1e-9 * m["gpts"] + 1e-12
        assert abs(m["gflops"] - 29 * m["gpts"]) < 1e-9 * m["gflops"]
        e2, _, em, _ = a.norms(S.FIELD_U)
        assert m["energy_u"] == e2 and m["max_abs_u"] == em
        assert m["rel_l2"] == 0.0
        assert a.metrics()["rel_l2"] == -1.0


@pytest.mark.parametrize("dtype", ["f32", "f64"])
@pytest.mark.parametrize("grid,ichunk", [((7, 9, 13, 4, 4, 4), 3), ((5, 30, 67, 4, 4, 16), 64),
                                         ((12, 17, 256, 4, 4, 4), 5), ((3, 4, 1, 4, 4, 4), 0)])
def test_two_point_matches_oracle(dtype, grid, ichunk):
    """stencil_2 (v = 0.5(u + u[k+1]), u's k halo supplying u[zs]) on the
    16-byte-access kernel: ragged rows (zs not a multiple of the vector
    width), odd plane counts per chunk, FP32 and FP64, bit for bit; halos of
    v untouched."""
    v, s, u = mode_r_inputs(grid, 77, dtype)
    v0 = v.copy()
    g = S.Grid(*grid)
    with S.Stencil(g, 2, "ref", dtype, ichunk=ichunk) as st:
        st.iterate_host(v, s, u, 3)
    vf, sf, uf = mode_r_inputs(grid, 77, dtype)
    O.iterate_ref(vf, sf, uf, grid, 2, 3, fma=True)
    np.testing.assert_array_equal(O.interior(v, grid), O.interior(vf, grid))
    mask = np.ones(v.shape, bool)
    xs, ys, zs, xh, yh, zh = grid
    mask[xh:xh + xs, yh:yh + ys, zh:zh + zs] = False
    np.testing.assert_array_equal(v[mask], v0[mask])
