"""GPU checks of the tensor-core kernel of the 16-bit delta forms (kernel
"mma": the j and k neighbour sums as band-matrix products on the tensor
cores with FP32 accumulation).  Its sums round differently from the scalar
kernel's and from the oracle's restatement, so these checks are tolerances,
each stated with its reason:

  - one step from the same encoded state: u^{n+1} = u + dec(enc(d^{n+1}))
    carries at most one unit in the last place of the d word and its own
    rounding, so every decoded u and v = u - d differs from the oracle's by
    at most the units of u and d (2^-10 relative for FP16 words, 2^-7 for
    BF16), and few words differ at all;
  - nine steps: the relative L2 distance to the oracle's run stays below
    three units in the last place (a per-step flip of one unit, growing no
    faster than the steps);
  - accuracy against FP64 after 60 steps: the scalar kernel's bounds.
"""
import numpy as np
import pytest

import stencil3d_gb300 as S
from oracle import oracle as O
from tests.helpers import rel_l2
from tests.test_f16_gpu import _inputs, _oracle_run

pytestmark = pytest.mark.gpu

ULP = {"f16": 2.0 ** -10, "f16_hl": 2.0 ** -10, "bf16": 2.0 ** -7}


def _run(storage, points, grid, steps, dt, src, blobs, seed, **kw):
    v, s, u = _inputs(grid, seed, blobs)
    with S.Stencil(S.Grid(*grid), points, "wave", storage, dt=dt, src=src, kernel="mma", **kw) as st:
        assert st.info().kernel == S.KERNEL_MMA
        uu, vv = u.copy(), v.copy()
        st.iterate_host(vv, s, uu, steps)
    ou, ov = _oracle_run(storage, u, v, s, grid, points, steps, dt, src)
    return (O.interior(uu, grid), O.interior(vv, grid), O.interior(ou, grid), O.interior(ov, grid))


@pytest.mark.parametrize("storage", ["f16", "bf16", "f16_hl"])
@pytest.mark.parametrize("points", [7, 13, 25])
@pytest.mark.parametrize("grid,blobs", [((24, 40, 150, 4, 4, 4), True),
                                        ((9, 17, 64, 4, 4, 16), False),
                                        ((11, 37, 141, 4, 4, 4), True)])
def test_mma_one_step_within_one_unit(storage, points, grid, blobs):
    dt = 1e-3 if points == 7 else 5e-4
    src = (grid[0] // 2, grid[1] // 2, grid[2] // 2)
    ui, vi, oui, ovi = _run(storage, points, grid, 1, dt, src, blobs, 3 + points)
    ulp = ULP[storage]
    floor = 2.0 ** -30 * float(np.max(np.abs(oui)))
    du = np.abs(ui.astype(np.float64) - oui)
    dv = np.abs(vi.astype(np.float64) - ovi)
    d_o = np.abs(oui.astype(np.float64) - ovi)
    assert np.all(du <= ulp * (np.abs(oui) + d_o) + floor), float(np.max(du / (np.abs(oui) + d_o + floor)))
    assert np.all(dv <= ulp * (np.abs(oui) + d_o) + floor)
    assert np.mean(ui != oui) < 0.05 and np.mean(vi != ovi) < 0.05


@pytest.mark.parametrize("storage", ["f16", "bf16", "f16_hl"])
@pytest.mark.parametrize("points", [7, 13, 25])
@pytest.mark.parametrize("stages", [0, -1])
def test_mma_steps_track_oracle(storage, points, stages):
    """ys = 43 and zs = 140 leave partial tiles along j and k."""
    grid = (30, 43, 140, 4, 4, 4)
    dt = 1e-3 if points == 7 else 5e-4
    # stages -1: the kernel's depth named explicitly (8, or 4 for the pair form)
    nv = (4 if storage == "f16_hl" else 8) if stages < 0 else 0
    ui, vi, oui, ovi = _run(storage, points, grid, 9, dt, (15, 21, 70), True, 40 + points,
                            stages=nv)
    bound = 3 * 2 * ULP[storage]
    assert rel_l2(ui, oui) < bound, rel_l2(ui, oui)
    assert rel_l2(vi, ovi) < bound, rel_l2(vi, ovi)


def test_mma_custom_weights():
    """7-point weights that are not exact in one FP16 word (the hi/lo band
    fragments, K = 48) and exact ones (the hi parts alone, K = 24)."""
    grid = (26, 33, 200, 4, 4, 4)
    dt = 1e-3
    for w in (1.0, 0.7):
        coef = [0.0, 0.0] + [w] * 12
        v, s, u = _inputs(grid, 5, True)
        with S.Stencil(S.Grid(*grid), 7, "wave", "f16", dt=dt, kernel="mma", coef=coef) as a, \
                S.Stencil(S.Grid(*grid), 7, "wave", "f16", dt=dt, kernel="tma", coef=coef) as b:
            ua, va, ub, vb = u.copy(), v.copy(), u.copy(), v.copy()
            a.iterate_host(va, s, ua, 9)
            b.iterate_host(vb, s, ub, 9)
        assert rel_l2(O.interior(ua, grid), O.interior(ub, grid)) < 6 * ULP["f16"]


@pytest.mark.parametrize("storage,bound", [("f16_hl", 6e-4), ("f16", 3e-3), ("bf16", 2e-2)])
def test_mma_tracks_fp64(storage, bound):
    """Accuracy against FP64 after 60 steps of a smooth field: the scalar
    kernel's bounds."""
    grid = (32, 36, 140, 4, 4, 4)
    dt = 5e-4
    v, s, u = _inputs(grid, 11, True)
    g = S.Grid(*grid)
    with S.Stencil(g, 25, "wave", storage, dt=dt, kernel="mma") as a, \
            S.Stencil(g, 25, "wave", "f64", dt=dt) as b:
        a.upload(v, s, u)
        b.upload(v.astype(np.float64), s.astype(np.float64), u.astype(np.float64))
        a.iterate(60)
        b.iterate(60)
        a.synchronize()
        b.synchronize()
        err = a.rel_l2(b)
    assert err < bound, err


@pytest.mark.parametrize("storage", ["f16", "f16_hl"])
@pytest.mark.parametrize("zs", [140, 141, 135])
def test_mma_tracks_tma_kernel_on_ragged_rows(storage, zs):
    """zs not a multiple of 8: the last tile's rows end inside a 16-byte
    segment.  Twenty steps stay within rounding of the scalar kernel (a write
    of nonzero words into the zero halo along k grew to 3.3e-3 in this
    configuration) and the k halo downloads as zeros."""
    grid = (16, 36, zs, 4, 4, 4)
    g = S.Grid(*grid)
    v, s, u = _inputs(grid, 11, True)
    with S.Stencil(g, 25, "wave", storage, dt=5e-4, kernel="mma") as a, \
            S.Stencil(g, 25, "wave", storage, dt=5e-4, kernel="tma") as b:
        a.upload(v, s, u)
        b.upload(v, s, u)
        a.iterate(20)
        b.iterate(20)
        ua, ub = g.empty(), g.empty()
        a.download(u=ua)
        b.download(u=ub)
    assert rel_l2(O.interior(ua, grid), O.interior(ub, grid)) < 2e-4
    assert np.all(ua[:, :, :4] == 0.0) and np.all(ua[:, :, 4 + zs:] == 0.0)


@pytest.mark.parametrize("storage", ["f16", "f16_hl", "bf16"])
def test_mma_plane_scales_far_apart(storage):
    """Planes whose scales differ by about 2^40 along i (a blob field and the
    same field times 1e-12): the i-pair weights are the planes' scales as
    exact 16-bit powers of two relative to the largest neighbour, and a plane
    too far below it takes a zero weight.  One step stays within one unit in
    the last place of the oracle's restatement at every point, on both
    sides of the jump."""
    grid = (24, 30, 70, 4, 4, 4)
    v, s, u = _inputs(grid, 9, True)
    scale = np.ones(u.shape, np.float32)
    scale[4 + 12:] = np.float32(1e-12)
    u = (u * scale).astype(np.float32)
    v = (v * scale).astype(np.float32)
    dt, src = 5e-4, None
    with S.Stencil(S.Grid(*grid), 25, "wave", storage, dt=dt, src=src, kernel="mma") as st:
        uu, vv = u.copy(), v.copy()
        st.iterate_host(vv, s, uu, 1)
    ou, ov = _oracle_run(storage, u, v, s, grid, 25, 1, dt, src)
    ui, oui, ovi = O.interior(uu, grid), O.interior(ou, grid), O.interior(ov, grid)
    d_o = np.abs(oui.astype(np.float64) - ovi)
    du = np.abs(ui.astype(np.float64) - oui)
    ulp = ULP[storage]
    # per plane: a floor below the plane's own values (each side of the jump)
    floor = 2.0 ** -30 * np.max(np.abs(oui), axis=(1, 2), keepdims=True)
    assert np.all(du <= ulp * (np.abs(oui) + d_o) + floor)
