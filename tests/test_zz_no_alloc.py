"""st3d_norms_noalloc: the FP64 drift check that allocates nothing.

It exists for callers that cannot allocate device memory where they check
drift, for example a solver running inside another application's time loop
on device buffers that application owns (a cudaMalloc there may synchronise
the device or fail because the memory is reserved).  The caller passes its
fields and a device output; the partial sums live in a fixed 128 KiB array
inside the library (at most 4096 planes along i).

The test plays such a caller: it owns its device buffers (allocated here,
outside the library), calls the entry point through the C ABI twice in a row
on different grids -- the second with fewer planes, so partials left behind by
the first call would show if they were read -- and checks each result
against st3d_norms on contexts holding the same fields: an FP32 field against
an FP64 one and the reverse, on the legacy default stream and on a stream the
test creates and synchronises itself (the use inside a host's time loop).
This file is named to be collected last.
"""
import ctypes as C
import os

import numpy as np
import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import api
from oracle import oracle as O

pytestmark = pytest.mark.gpu

H2D, D2H = 1, 2


def _cudart():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.join(home, "lib64")
    names = sorted((f for f in os.listdir(libdir) if f.startswith("libcudart.so")), key=len)
    rt = C.CDLL(os.path.join(libdir, names[0]))
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaDeviceSynchronize.argtypes = []
    rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
    rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
    rt.cudaStreamDestroy.argtypes = [C.c_void_p]
    return rt


class DeviceBuffer:
    """A caller-owned device buffer (allocated by the test, not the library)."""

    def __init__(self, rt, nbytes):
        self.rt = rt
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), nbytes) == 0
        self.nbytes = nbytes

    def put(self, a):
        assert self.rt.cudaMemcpy(self.ptr, a.ctypes.data, a.nbytes, H2D) == 0

    def get(self, a):
        assert self.rt.cudaMemcpy(a.ctypes.data, self.ptr, a.nbytes, D2H) == 0

    def free(self):
        self.rt.cudaFree(self.ptr)


def _context_norms(grid, a, b):
    g = S.Grid(*grid)
    sa = "f64" if a.dtype == np.float64 else "f32"
    sb = "f64" if b.dtype == np.float64 else "f32"
    with S.Stencil(g, 7, "ref", sa) as ca, S.Stencil(g, 7, "ref", sb) as cb:
        ca.upload(u=a)
        cb.upload(u=b)
        return ca.norms(S.FIELD_U, cb, S.FIELD_U), ca.norms(S.FIELD_U)


def _close(got, want):
    assert got[0] == pytest.approx(want[0], rel=1e-12, abs=1e-300)
    assert got[1] == pytest.approx(want[1], rel=1e-12, abs=1e-300)
    assert got[2] == want[2] and got[3] == want[3]


@pytest.mark.parametrize("ta,tb", [(np.float32, np.float64), (np.float64, np.float32)],
                         ids=["a_f32_b_f64", "a_f64_b_f32"])
@pytest.mark.parametrize("own_stream", [False, True], ids=["default_stream", "own_stream"])
def test_noalloc_norms_match_existing_entry_point_twice(ta, tb, own_stream):
    rt = _cudart()
    lib = S.lib()
    code = {np.float32: S.F32, np.float64: S.F64}
    stream = C.c_void_p()
    if own_stream:
        assert rt.cudaStreamCreate(C.byref(stream)) == 0
    try:
        _two_calls(rt, lib, ta, tb, code, stream)
    finally:
        if own_stream:
            rt.cudaStreamDestroy(stream)


def _two_calls(rt, lib, ta, tb, code, stream):
    def wait():
        if stream.value:
            assert rt.cudaStreamSynchronize(stream) == 0
        else:
            assert rt.cudaDeviceSynchronize() == 0

    for grid, seed in (((40, 24, 70, 4, 4, 4), 1), ((17, 30, 33, 4, 5, 6), 2)):
        a = O.fill_uniform(grid, seed, 0, -1.0, 1.0, ta)
        b = O.fill_uniform(grid, seed, 1, -1.0, 1.0, tb)
        da, db, dout = DeviceBuffer(rt, a.nbytes), DeviceBuffer(rt, b.nbytes), DeviceBuffer(rt, 32)
        try:
            da.put(a)
            db.put(b)
            desc = api.GridDesc(*grid)
            out = np.zeros(4, np.float64)
            rc = lib.st3d_norms_noalloc(C.byref(desc), da.ptr, code[ta], db.ptr, code[tb], dout.ptr,
                                        stream)
            assert rc == 0, S.last_error()
            wait()
            dout.get(out)
            energy = np.zeros(4, np.float64)
            rc = lib.st3d_norms_noalloc(C.byref(desc), da.ptr, code[ta], None, code[tb], dout.ptr,
                                        stream)
            assert rc == 0, S.last_error()
            wait()
            dout.get(energy)
        finally:
            for d in (da, db, dout):
                d.free()
        want, want_energy = _context_norms(grid, a, b)
        _close(out, want)
        _close(energy, want_energy)


def test_noalloc_rejects_grids_beyond_its_scratch():
    desc = api.GridDesc(4097, 8, 8, 4, 4, 4)
    rc = S.lib().st3d_norms_noalloc(C.byref(desc), C.c_void_p(16), S.F32, None, S.F32,
                                    C.c_void_p(16), None)
    assert rc == S.api.ERR_INVALID
    assert "4096" in S.last_error()
