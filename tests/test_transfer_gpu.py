"""st3d_transfer and device-memory arrays in st3d_upload / st3d_download.

  - a transfer between two FP32 contexts carries the whole time state: both
    continue bit for bit alike, source clock included;
  - a transfer from FP16 delta storage into either compensated storage
    equals the host round trip (download into host arrays, upload, set_step);
  - upload and download take device arrays of the reference layout and move
    the same values as host arrays;
  - mismatched contexts are refused before anything moves.
"""
import ctypes as C

import numpy as np
import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import api
from oracle import oracle as O
from tests.helpers import halo_mask

pytestmark = pytest.mark.gpu

GRID = (20, 28, 150, 4, 4, 4)
SRC = (10, 14, 75)


def _inputs(seed=5):
    u = O.fill_blobs(GRID, seed, 4, 5.0)
    v = (u * np.float32(0.999)).astype(np.float32)
    u[halo_mask(GRID)] = 0.0
    v[halo_mask(GRID)] = 0.0
    s = np.zeros_like(u)
    return v, s, u


def _state(st, g):
    u, v = g.empty(), g.empty()
    st.download(v, u)
    st.synchronize()
    return g.interior(u).copy(), g.interior(v).copy()


@pytest.mark.parametrize("points", [7, 25])
def test_transfer_fp32_continues_alike(points):
    g = S.Grid(*GRID)
    v, s, u = _inputs()
    with S.Stencil(g, points, "wave", "f32", dt=5e-4, src=SRC) as a, \
            S.Stencil(g, points, "wave", "f32", dt=5e-4, src=SRC) as b:
        a.upload(v, s, u)
        a.iterate(9)  # the clock sits at step 9, near no special value
        b.upload(None, s, None)
        b.transfer_from(a)
        for st in (a, b):
            st.iterate(6)
        ua, va = _state(a, g)
        ub, vb = _state(b, g)
    np.testing.assert_array_equal(ua, ub)
    np.testing.assert_array_equal(va, vb)


@pytest.mark.parametrize("fallback", ["f16_hilo", "f16_hl"])
def test_transfer_equals_host_round_trip(fallback):
    g = S.Grid(*GRID)
    v, s, u = _inputs(8)
    with S.Stencil(g, 25, "wave", "f16", dt=5e-4, src=SRC) as a:
        a.upload(v, s, u)
        a.iterate(70)
        hu, hv = g.empty(), g.empty()
        a.download(hv, hu)
        a.synchronize()
        with S.Stencil(g, 25, "wave", fallback, dt=5e-4, src=SRC) as dev, \
                S.Stencil(g, 25, "wave", fallback, dt=5e-4, src=SRC) as host:
            dev.upload(None, s, None)
            dev.transfer_from(a)
            host.upload(hv, s, hu)
            host.set_step(70)
            for st in (dev, host):
                st.iterate(4)
            ud, vd = _state(dev, g)
            uh, vh = _state(host, g)
    np.testing.assert_array_equal(ud, uh)
    np.testing.assert_array_equal(vd, vh)


def test_device_arrays_in_upload_and_download():
    torch = pytest.importorskip("torch")
    g = S.Grid(*GRID)
    v, s, u = _inputs(11)
    dv = torch.from_numpy(v).cuda()
    ds = torch.from_numpy(s).cuda()
    du = torch.from_numpy(u).cuda()
    torch.cuda.synchronize()
    lib = api.lib()
    p = lambda t: C.c_void_p(t.data_ptr())
    with S.Stencil(g, 13, "wave", "f32", dt=5e-4, src=SRC) as a, \
            S.Stencil(g, 13, "wave", "f32", dt=5e-4, src=SRC) as b:
        a.upload(v, s, u)
        assert lib.st3d_upload(b._h, p(dv), p(ds), p(du)) == 0
        for st in (a, b):
            st.iterate(5)
        ua, va = _state(a, g)
        ov = torch.full_like(dv, -7.0)
        ou = torch.full_like(du, -7.0)
        torch.cuda.synchronize()
        assert lib.st3d_download(b._h, p(ov), p(ou)) == 0
        b.synchronize()
        hv, hu = ov.cpu().numpy(), ou.cpu().numpy()
    np.testing.assert_array_equal(g.interior(hu), ua)
    np.testing.assert_array_equal(g.interior(hv), va)
    # the halo planes and rows of the target stay as they were
    assert np.all(hv[halo_mask(GRID) & ~_k_halo(GRID)] == -7.0)


def _k_halo(grid):
    """Points of the k halo inside interior (i, j) rows: the download writes them."""
    xs, ys, zs, xh, yh, zh = grid
    m = np.zeros(O.shape(grid), bool)
    m[xh:xh + xs, yh:yh + ys, :] = True
    m[xh:xh + xs, yh:yh + ys, zh:zh + zs] = False
    return m


def test_transfer_refuses_mismatched_contexts():
    g = S.Grid(*GRID)
    g2 = S.Grid(20, 28, 152, 4, 4, 4)
    v, s, u = _inputs()
    with S.Stencil(g, 13, "wave", "f32", dt=5e-4) as a, \
            S.Stencil(g2, 13, "wave", "f32", dt=5e-4) as b, \
            S.Stencil(g, 13, "wave", "f64", dt=5e-4) as c, \
            S.Stencil(g, 13, "wave", "f32", dt=5e-4) as d:
        with pytest.raises(api.St3dError):
            d.transfer_from(a)  # a holds no fields yet
        a.upload(v, s, u)
        with pytest.raises(api.St3dError):
            b.transfer_from(a)
        with pytest.raises(api.St3dError):
            c.transfer_from(a)
        with pytest.raises(api.St3dError):
            a.transfer_from(a)
