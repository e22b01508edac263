"""The oracle (oracle/st3d_oracle.c) against the reference.

Pins the C restatement to the reference's own host path: against the golden
fixtures generated from the compiled reference (tests/golden/), against the
live reference where it was built on this machine (oracle/_ref), and against
the reference's only built-in test, the constant-field known-answer check of
iterators.cpp:292-325.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from oracle import build as obuild
from oracle import oracle as O
from tests.helpers import golden_cases, halo_mask, mode_r_inputs, np_dtype, wave_inputs, rel_l2

META, ARRAYS = golden_cases()


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", META, ids=[m["name"] for m in META])
def test_oracle_matches_reference_golden(case):
    """Plain flavour of the oracle == the reference, bit for bit."""
    grid = tuple(case["grid"])
    v, s, u = mode_r_inputs(grid, case["seed"], case["dtype"])
    O.iterate_ref(v, s, u, grid, case["points"], case["iterations"])
    inner = np.ascontiguousarray(O.interior(v, grid))
    assert _digest(inner) == case["sha256"]
    if case["keep"]:
        np.testing.assert_array_equal(inner, ARRAYS[case["name"]])


@pytest.mark.parametrize("case", META, ids=[m["name"] for m in META])
def test_fma_flavour_within_tolerance(case):
    """The fused flavour (the device kernels' operation order) stays within
    the 1e-5 relative-L2 parity bound of the reference result."""
    grid = tuple(case["grid"])
    v, s, u = mode_r_inputs(grid, case["seed"], case["dtype"])
    O.iterate_ref(v, s, u, grid, case["points"], case["iterations"], fma=True)
    inner = O.interior(v, grid)
    ref = ARRAYS.get(case["name"])
    if ref is None:
        v2, s2, u2 = mode_r_inputs(grid, case["seed"], case["dtype"])
        O.iterate_ref(v2, s2, u2, grid, case["points"], case["iterations"])
        ref = O.interior(v2, grid)
    tol = 1e-14 if case["dtype"] == "f64" else 1e-6
    assert rel_l2(inner, ref) <= tol


@pytest.mark.parametrize("points", [7, 13, 25])
def test_known_answer(points):
    """init_arrays + check (iterators.cpp:292-325): after n steps v == n."""
    grid = (16, 12, 20, 4, 4, 16)
    v, s, u = O.init_arrays(grid)
    O.iterate_ref(v, s, u, grid, points, 1)
    assert O.check(v, grid, 1) == 0
    O.iterate_ref(v, s, u, grid, points, 6)
    assert O.check(v, grid, 7) == 0
    if points == 7:  # coefficients sum exactly to 1 in float only for 7 points
        assert np.all(O.interior(v, grid) == 7.0)


def test_two_point_fails_known_answer_like_reference():
    """stencil_2 has no v accumulation (stencil_2.h:27), so the reference's own
    check reports every point; the oracle reproduces that."""
    grid = (6, 5, 8, 4, 4, 1)
    v, s, u = O.init_arrays(grid)
    O.iterate_ref(v, s, u, grid, 2, 3)
    assert O.check(v, grid, 3) == 6 * 5 * 8


def test_halos_never_written():
    grid = (7, 6, 9, 4, 4, 4)
    v, s, u = mode_r_inputs(grid, 3, "f32")
    v0 = v.copy()
    O.iterate_ref(v, s, u, grid, 25, 2)
    mask = np.ones(v.shape, bool)
    mask[4:11, 4:10, 4:13] = False
    np.testing.assert_array_equal(v[mask], v0[mask])


def test_default_coefficients_match_reference_constants():
    c = O.default_coefs(25, np.float32)
    assert c[0] == np.float32(1.25) and c[1] == np.float32(6.25)
    assert c[6] == np.float32(np.float32(0.4) * np.float32(1.1))
    d = O.default_coefs(25, np.float64)
    assert d[6] == float(np.float32(0.4)) * float(np.float32(1.1))
    c13 = O.default_coefs(13, np.float32)
    assert c13[1] == np.float32(3.5) and c13[10] == np.float32(np.float32(0.3) * np.float32(0.9))


ref_built = pytest.mark.skipif(not O.ref_available(7), reason="reference not built on this machine")


@ref_built
@pytest.mark.parametrize("points", [2, 7, 13, 25])
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_oracle_matches_live_reference(points, dtype):
    grid = (9, 14, 27, 4, 5, 7)
    v1, s, u = mode_r_inputs(grid, 101 + points, dtype)
    v2 = v1.copy()
    O.iterate_ref(v1, s, u, grid, points, 4)
    O.ref_iterate(v2, s, u, grid, points, 4)
    np.testing.assert_array_equal(v1, v2)


@ref_built
def test_oracle_matches_reference_iterate_3d_square():
    """iterate_3d (the README host recipe) agrees on square grids; it bounds j by
    isize (iterators.cpp:146) so non-square grids are not comparable."""
    grid = (12, 12, 20, 4, 4, 16)
    v1, s, u = mode_r_inputs(grid, 5, "f32")
    v2 = v1.copy()
    O.iterate_ref(v1, s, u, grid, 13, 3)
    O.ref_iterate(v2, s, u, grid, 13, 3, traversal="3d")
    np.testing.assert_array_equal(v1, v2)


@ref_built
@pytest.mark.parametrize("points", [7, 13, 25])
def test_reference_binary_known_answer(points):
    exe = os.path.join(obuild.REF_DIR, "hstencil3d_%d" % points)
    r = subprocess.run([exe, "--xs", "24", "--ys", "24", "--zs", "32", "--iter", "3"],
                       capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="2"),
                       timeout=60)
    assert r.returncode == 0
    assert r.stdout.count("check: 0 errors found") == 2


# ---------------------------------------------------------------- mode W ---
def test_wave_oracle_fp32_tracks_fp64():
    grid = (24, 20, 28, 4, 4, 4)
    c0, c1, c2 = O.wave_constants(13, 1500.0, 5e-4, 10.0)
    v, s, u = wave_inputs(grid, 9)
    vd, sd, ud = v.astype(np.float64), s.astype(np.float64), u.astype(np.float64)
    amps = O.ricker_amps(0, 30, 5e-4)
    src = (12, 10, 14)
    O.iterate_wave(u, v, s, grid, 13, 30, c0, c1, c2, src=src, amps=amps)
    O.iterate_wave(ud, vd, sd, grid, 13, 30, c0, c1, c2, src=src,
                   amps=O.ricker_amps(0, 30, 5e-4, dtype=np.float64))
    assert rel_l2(O.interior(u, grid), O.interior(ud, grid)) < 1e-5


def test_wave_oracle_fma_and_plain_agree():
    grid = (16, 18, 20, 4, 4, 4)
    c0, c1, c2 = O.wave_constants(25, 1500.0, 5e-4, 10.0)
    v, s, u = wave_inputs(grid, 4)
    v2, s2, u2 = v.copy(), s.copy(), u.copy()
    O.iterate_wave(u, v, s, grid, 25, 10, c0, c1, c2, fma=True)
    O.iterate_wave(u2, v2, s2, grid, 25, 10, c0, c1, c2, fma=False)
    assert rel_l2(O.interior(u, grid), O.interior(u2, grid)) < 1e-6


def test_wave_constant_field_is_stationary():
    """c0 = 2 - 2*c1*sum(w) makes u = v = const a fixed point (up to rounding)."""
    grid = (10, 10, 10, 4, 4, 4)
    for pts in (7, 13, 25):
        c0, c1, c2 = O.wave_constants(pts, 1500.0, 1e-3 if pts == 7 else 5e-4, 10.0)
        u = np.full(O.shape(grid), 0.5, np.float64)
        v = u.copy()
        s = np.zeros_like(u)
        O.iterate_wave(u, v, s, grid, pts, 5, c0, c1, c2)
        assert np.max(np.abs(O.interior(u, grid) - 0.5)) < 1e-12


def test_wave_ricker_source():
    t0 = 1.0 / 15.0
    assert O.ricker(t0) == 1.0
    assert abs(O.ricker(0.0)) < 1e-3
    a = O.ricker_amps(0, 200, 1e-3)
    assert np.argmax(a) == 67  # t = 0.067 s, the sample nearest t0


def test_wave_weights_follow_readme_for_seven_points():
    w = O.wave_weights(7)
    assert w[2] == w[6] == w[10] == 1.0
    c0, c1, c2 = O.wave_constants(7, 1500.0, 1e-3, 10.0)
    assert abs(c1 - 0.0225) < 1e-15 and abs(c2 - 1e-6) < 1e-18
    assert abs(c0 - (2 - 6 * 0.0225)) < 1e-15


# ------------------------------------------------------- 16-bit storage ---
def _blob_state(grid, seed):
    u = O.fill_blobs(grid, seed, 4, 6.0)
    v = (u * np.float32(0.999)).astype(np.float32)
    v[halo_mask(grid)] = 0.0
    return u, v


@pytest.mark.parametrize("kind", [0, 1])
def test_delta_form_round_trip(kind):
    """Encoding u and d = u - v and decoding (u, u - d) loses only the 16-bit
    rounding of each word: FP16 keeps 11 significant bits, BF16 8."""
    grid = (10, 12, 40, 4, 4, 4)
    u, v = _blob_state(grid, 2)
    fu, fd = O.delta_fields(u, v, grid, kind)
    uu, vv = O.delta_decode(fu, fd)
    tol = 2.0 ** -11 if kind == 0 else 2.0 ** -8
    ui = O.interior(u, grid)
    assert np.max(np.abs(O.interior(uu, grid) - ui)) <= tol * np.max(np.abs(ui))
    di = ui - O.interior(v, grid)
    dd = O.interior(uu, grid) - O.interior(vv, grid)
    # d is stored at its own scale: its error is relative to |d|, not |u|
    assert np.max(np.abs(dd - di)) <= 2 * tol * np.max(np.abs(di)) + tol * np.max(np.abs(ui)) * 2.0 ** -11


@pytest.mark.parametrize("kind,bound", [(0, 3e-3), (1, 2e-2)])
def test_delta_form_tracks_fp64(kind, bound):
    """The FP16 / BF16 delta form against the FP64 leapfrog after 60 steps of
    a smooth field (25 points): the stated error of the precision form."""
    grid = (32, 36, 140, 4, 4, 4)
    dt = 5e-4
    u, v = _blob_state(grid, 11)
    s = np.zeros_like(u)
    c0, c1, c2 = O.wave_constants(25, 1500.0, dt, 10.0)
    u64, v64 = u.astype(np.float64), v.astype(np.float64)
    O.iterate_wave(u64, v64, s.astype(np.float64), grid, 25, 60, c0, c1, c2, fma=True)
    fu, fd = O.delta_fields(u, v, grid, kind)
    fs = O.Field16(s, grid, kind, False)
    O.iterate_delta16(fu, fd, fs, grid, 25, 60, np.float32(c1), np.float32(c2))
    uu, _ = O.delta_decode(fu, fd)
    assert rel_l2(O.interior(uu, grid), O.interior(u64, grid)) < bound


def test_delta_form_is_more_accurate_than_storing_both_levels():
    """Storing U^{n-1} in FP16 loses the time difference (the velocity) that
    the delta form keeps: after 100 steps the delta form's error is several
    times smaller."""
    grid = (24, 24, 60, 4, 4, 4)
    dt = 5e-4
    u, v = _blob_state(grid, 5)
    s = np.zeros_like(u)
    c0, c1, c2 = O.wave_constants(13, 1500.0, dt, 10.0)
    u64, v64 = u.astype(np.float64), v.astype(np.float64)
    O.iterate_wave(u64, v64, s.astype(np.float64), grid, 13, 100, c0, c1, c2, fma=True)
    fu, fd = O.delta_fields(u, v, grid, 0)
    fs = O.Field16(s, grid, 0, False)
    O.iterate_delta16(fu, fd, fs, grid, 13, 100, np.float32(c1), np.float32(c2))
    e_delta = rel_l2(O.interior(O.delta_decode(fu, fd)[0], grid), O.interior(u64, grid))
    # two levels in FP16 words with the same per-plane scales, FP32 arithmetic
    lu, lv = O.Field16(u, grid, 0, False), O.Field16(v, grid, 0, False)
    O.iterate_wave16(lu, lv, fs, grid, 13, 100, np.float32(c1), np.float32(c2))
    e_levels = rel_l2(O.interior(lu.decode(), grid), O.interior(u64, grid))
    assert e_delta * 4 < e_levels, (e_delta, e_levels)


def test_pair_form_round_trip():
    """The FP16 hi/lo pair keeps about 22 significant bits: decoding the pair
    of a value differs from it by at most 2^-21 of the plane maximum, and the
    hi word alone is the FP16 rounding."""
    grid = (10, 12, 40, 4, 4, 4)
    u, v = _blob_state(grid, 4)
    fp = O.FieldPair(u, grid)
    f16 = O.Field16(u, grid, 0, False)
    np.testing.assert_array_equal(fp.h, f16.h)
    np.testing.assert_array_equal(fp.E, f16.E)
    ui = O.interior(u, grid)
    err = np.abs(O.interior(fp.decode(), grid) - ui)
    assert np.max(err) <= 2.0 ** -21 * np.max(np.abs(ui))
    assert np.max(err) < np.max(np.abs(O.interior(f16.decode(), grid) - ui)) / 100


def test_pair_form_tracks_fp64_closer_than_fp16():
    """u as an FP16 hi/lo pair (d in one FP16 word): against the FP64
    leapfrog after 200 steps (25 points) its error is several times smaller
    than the FP16 delta form's, and within the 1e-3 tolerance."""
    grid = (28, 32, 100, 4, 4, 4)
    dt, steps = 5e-4, 200
    u, v = _blob_state(grid, 13)
    s = np.zeros_like(u)
    c0, c1, c2 = O.wave_constants(25, 1500.0, dt, 10.0)
    u64, v64 = u.astype(np.float64), v.astype(np.float64)
    O.iterate_wave(u64, v64, s.astype(np.float64), grid, 25, steps, c0, c1, c2, fma=True)
    ref = O.interior(u64, grid)
    errs = {}
    for pair in (False, True):
        fu, fd = O.delta_fields(u, v, grid, 0, pair=pair)
        fs = O.Field16(s, grid, 0, False)
        O.iterate_delta16(fu, fd, fs, grid, 25, steps, np.float32(c1), np.float32(c2))
        errs[pair] = rel_l2(O.interior(O.delta_decode(fu, fd)[0], grid), ref)
    assert errs[True] < 1e-3 and errs[True] * 3 < errs[False], errs


def test_delta_form_scales_hold_a_source():
    """With a Ricker source the lagged plane scales still bound every value:
    all words finite, the source plane's d scale follows the amplitude."""
    grid = (12, 14, 30, 4, 4, 4)
    dt = 1e-3
    u = np.zeros(O.shape(grid), np.float32)
    s = np.zeros_like(u)
    c0, c1, c2 = O.wave_constants(7, 1500.0, dt, 10.0)
    src = (6, 7, 15)
    fu, fd = O.delta_fields(u, u, grid, 0)
    fs = O.Field16(s, grid, 0, False)
    amps = O.ricker_amps(0, 120, dt) * np.float32(1e4)
    O.iterate_delta16(fu, fd, fs, grid, 7, 120, np.float32(c1), np.float32(c2), src=src, amps=amps)
    uu, vv = O.delta_decode(fu, fd)
    assert np.all(np.isfinite(uu)) and np.all(np.isfinite(vv))
    assert np.max(np.abs(O.interior(uu, grid))) > 0


def test_vec16_variant_is_ref_with_k_625():
    """The reference's 13-point vec_16 kernel (stencil_13.h:359-430) computes
    the ref kernel's update with K = 6.25 instead of 3.5: the oracle's plain
    flavour with that K reproduces it bit for bit."""
    L = O.ref_vec16_13()
    if L is None:
        pytest.skip("reference vec_16 build not available on this machine")
    coefs = O.default_coefs(13, np.float32)
    coefs[1] = 6.25
    for grid in [(12, 16, 64, 4, 4, 16), (9, 13, 80, 4, 4, 16)]:
        v, s, u = mode_r_inputs(grid, 5, "f32")
        vr = v.copy()
        L.ref_iterate(vr, s, u, *grid, 3)
        vo = v.copy()
        O.iterate_ref(vo, s, u, grid, 13, 3, coefs=coefs)
        np.testing.assert_array_equal(O.interior(vr, grid), O.interior(vo, grid))
