"""The precision form's fallback: an FP16 delta-form run moves to the
compensated FP16 + int8 form when its drift against a reference run passes
the tolerance, and continues exactly as a compensated run started from the
moved state (with the source clock carried over)."""
import numpy as np
import pytest

import stencil3d_gb300 as S
from stencil3d_gb300.precision import GuardedWave
from oracle import oracle as O
from tests.helpers import halo_mask

pytestmark = pytest.mark.gpu

GRID = (24, 30, 140, 4, 4, 4)
SRC = (12, 15, 70)


def _inputs():
    u = O.fill_blobs(GRID, 9, 4, 5.0)
    v = (u * np.float32(0.999)).astype(np.float32)
    v[halo_mask(GRID)] = 0.0
    s = np.zeros_like(u)
    return v, s, u


def test_fallback_moves_and_continues_exactly():
    g = S.Grid(*GRID)
    v, s, u = _inputs()
    with S.Stencil(g, 25, "wave", "f64", dt=5e-4, src=SRC) as ref, \
            GuardedWave(g, 25, tol=1e-12, dt=5e-4, src=SRC) as run:
        ref.upload(v.astype(np.float64), s.astype(np.float64), u.astype(np.float64))
        run.upload(v, s, u)
        run.iterate(6)
        ref.iterate(6)
        # the state the move will carry, taken before the check
        um, vm = g.empty(), g.empty()
        run.download(vm, um)
        run.synchronize()
        err = run.check(ref)
        assert err > 1e-12 and run.switched_at == 6 and run.current_storage == "f16_hilo"
        run.iterate(5)
        ua, va = g.empty(), g.empty()
        run.download(va, ua)
        run.synchronize()
    # a compensated run started from the moved state, source clock at 6
    with S.Stencil(g, 25, "wave", "f16_hilo", dt=5e-4, src=SRC) as st:
        st.upload(vm, s, um)
        st.set_step(6)
        st.iterate(5)
        ub, vb = g.empty(), g.empty()
        st.download(vb, ub)
        st.synchronize()
    np.testing.assert_array_equal(g.interior(ua), g.interior(ub))
    np.testing.assert_array_equal(g.interior(va), g.interior(vb))


def test_no_move_within_tolerance():
    g = S.Grid(*GRID)
    v, s, u = _inputs()
    with S.Stencil(g, 13, "wave", "f64", dt=5e-4, src=SRC) as ref, \
            GuardedWave(g, 13, tol=0.5, dt=5e-4, src=SRC) as run:
        ref.upload(v.astype(np.float64), s.astype(np.float64), u.astype(np.float64))
        run.upload(v, s, u)
        for _ in range(3):
            run.iterate(4)
            ref.iterate(4)
            run.check(ref)
        assert run.switched_at is None and len(run.history) == 3
        assert all(e < 0.5 for _, _, e in run.history)


def test_source_clock_is_carried_over():
    """set_step carries the Ricker clock into a new context: from the same
    moved state, a run with the clock at step 70 (near the wavelet's peak,
    t0 = 1/15 s) and one restarted at 0 differ at the source, and the first
    equals a second run with the same clock."""
    g = S.Grid(*GRID)
    v, s, u = _inputs()
    with S.Stencil(g, 7, "wave", "f16_hilo", dt=1e-3, src=SRC) as a:
        a.upload(v, s, u)
        a.iterate(70)
        um, vm = g.empty(), g.empty()
        a.download(vm, um)
        a.synchronize()
    outs = []
    for step in (70, 0, 70):
        with S.Stencil(g, 7, "wave", "f16_hilo", dt=1e-3, src=SRC) as b:
            b.upload(vm, s, um)
            b.set_step(step)
            b.iterate(3)
            ub = g.empty()
            b.download(None, ub)
            b.synchronize()
            outs.append(g.interior(ub).copy())
    np.testing.assert_array_equal(outs[0], outs[2])
    assert not np.array_equal(outs[0], outs[1])
