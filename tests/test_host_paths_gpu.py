"""Host transfers: pinned host arrays are read and written by the layout
kernels directly (ST3D_HOST_DIRECT), pageable ones go through the staging
buffer (ST3D_HOST_STAGED).  Both paths move the same points: identical
results and identical host arrays, halos included."""
import numpy as np
import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import api
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _run(g, v, s, u, pinned, path, dtype, points=13, mode="wave"):
    kw = dict(dt=5e-4) if mode == "wave" else {}
    with S.Stencil(g, points, mode, "f64" if dtype == np.float64 else "f32", host_path=path,
                   **kw) as st:
        bufs = []
        if pinned:
            arrs = []
            for a in (v, s, u):
                p = S.PinnedArray(a.shape, dtype)
                p.array[...] = a
                bufs.append(p)
                arrs.append(p.array)
        else:
            arrs = [a.copy() for a in (v, s, u)]
        try:
            st.upload(*arrs)
            up_path = st.info().host_path
            st.iterate(3)
            # the download targets start as sentinels: untouched points keep them
            arrs[0][...] = -7.0
            arrs[2][...] = -7.0
            st.download(arrs[0], arrs[2])
            st.synchronize()
            down_path = st.info().host_path
            out = (arrs[0].copy(), arrs[2].copy())
        finally:
            for p in bufs:
                p.free()
    return out, up_path, down_path


@pytest.mark.parametrize("dtype,mode", [(np.float32, "wave"), (np.float32, "ref"),
                                        (np.float64, "ref")])
def test_direct_and_staged_paths_agree(dtype, mode):
    grid = (20, 30, 150, 4, 4, 8)
    g = S.Grid(*grid)
    u = O.fill_uniform(grid, 3, 0, -1.0, 1.0, dtype)
    v = O.fill_uniform(grid, 3, 1, -1.0, 1.0, dtype)
    s = O.fill_uniform(grid, 3, 2, 0.5, 1.5, dtype)
    a, up_a, down_a = _run(g, v, s, u, True, api.HOST_AUTO, dtype, mode=mode)
    b, up_b, down_b = _run(g, v, s, u, False, api.HOST_AUTO, dtype, mode=mode)
    c, up_c, down_c = _run(g, v, s, u, True, api.HOST_STAGED, dtype, mode=mode)
    assert up_b == down_b == api.HOST_STAGED and up_c == down_c == api.HOST_STAGED
    assert up_a == down_a == api.HOST_DIRECT
    for x, y in ((a, b), (a, c)):
        np.testing.assert_array_equal(x[0], y[0])
        np.testing.assert_array_equal(x[1], y[1])
    # the interior changed, the j/i halos kept the sentinel
    assert np.all(g.interior(a[0]) != -7.0)
    assert a[0][0, 0, 0] == -7.0


def test_direct_path_refuses_pageable_arrays():
    grid = (8, 8, 40, 4, 4, 4)
    g = S.Grid(*grid)
    u = g.empty()
    with S.Stencil(g, 7, "ref", "f32", host_path=api.HOST_DIRECT) as st:
        with pytest.raises(S.St3dError) as e:
            st.upload(u, u, u)
        assert e.value.status == api.ERR_INVALID
