"""Error paths that exist for the GPU only, reached without faulting or
hanging a GPU.

  - A kernel whose bounded device-side wait gives up records a code in the
    context's device status word and returns early; st3d_synchronize turns
    that into ST3D_ERR_TIMEOUT and clears the word.  The word is written from
    the host here (st3d_inject_device_status), as the kernel would write it:
    no device wait is made to run out.  Afterwards the context keeps working
    and computes the same bits as an untouched one.
  - opts.device selects the GPU of a context (one replica per GPU); an
    ordinal beyond the visible devices is refused at st3d_create.
"""
import ctypes as C

import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import api

pytestmark = pytest.mark.gpu


def _wave(kernel="tma", **kw):
    st = S.Stencil(S.Grid(40, 36, 200, 4, 4, 4), 25, "wave", "f32", kernel=kernel, dt=5e-4,
                   src=(20, 18, 100), **kw)
    st.fill(S.FIELD_U, S.FILL_BLOBS, 11, 4, 6.0)
    st.fill(S.FIELD_V, S.FILL_BLOBS, 11, 4, 6.0)
    st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
    return st


@pytest.mark.parametrize("kernel", ["tma", "simple"])
@pytest.mark.parametrize("code", [1, 2])
def test_device_status_maps_to_timeout_and_context_survives(kernel, code):
    with _wave(kernel) as st, _wave(kernel) as ref:
        st.iterate(3)
        st.synchronize()
        st.inject_device_status(code)
        with pytest.raises(S.St3dError) as e:
            st.synchronize()
        assert e.value.status == api.ERR_TIMEOUT
        assert "gave up" in S.last_error()
        # the word was cleared: the next synchronize is clean, and stepping
        # on continues exactly like a context that never saw the error
        st.synchronize()
        st.iterate(4)
        st.synchronize()
        ref.iterate(7)
        ref.synchronize()
        for f in (S.FIELD_U, S.FIELD_V):
            d2, b2, dm, bm = st.norms(f, ref, f)
            assert b2 > 0 and d2 == 0.0 and dm == 0.0


def test_clearing_the_status_word():
    with _wave() as st:
        st.inject_device_status(7)
        st.inject_device_status(0)
        st.synchronize()


def test_device_selection():
    with _wave(device=0) as st:
        info = st.info()
        assert info.device == 0
        st.iterate(2)
        st.synchronize()
    dev = S.device_info()
    o = S.default_opts(25, "wave", "f32")
    o.device = 64  # beyond any node's GPU count
    h = C.c_void_p()
    rc = S.lib().st3d_create(C.byref(S.Grid(16, 16, 16, 4, 4, 4).desc()), C.byref(o), C.byref(h))
    assert rc == api.ERR_INVALID and "out of range" in S.last_error()
    assert dev["sm_count"] > 0


def test_batch_device_must_agree():
    grids = [S.Grid(40, 40, 64, 4, 4, 4), S.Grid(48, 40, 64, 4, 4, 4)]
    opts = (api.Opts * 2)(S.default_opts(7, "wave", "f32"), S.default_opts(13, "wave", "f32"))
    opts[0].device = 0
    opts[1].device = -1
    descs = (api.GridDesc * 2)(*[g.desc() for g in grids])
    h = C.c_void_p()
    rc = S.lib().st3d_batch_create(2, descs, opts, C.byref(h))
    assert rc == api.ERR_INVALID and "one device" in S.last_error()
