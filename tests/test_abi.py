"""The C ABI without a GPU: exports, struct layout, argument checks, layout
planning and the defaults that mirror the reference's constants."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import stencil3d_gb300 as S
from stencil3d_gb300 import api
from oracle import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "st3d.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(st3d_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", api.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(st3d_\w+)\b", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    lib = S.lib()
    for n in names:
        assert getattr(lib, n) is not None


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirrors of the ABI structs have the C sizes and offsets."""
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "st3d.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(st3d_grid_desc),"
        " sizeof(st3d_opts), sizeof(st3d_info), offsetof(st3d_opts, c0),"
        " offsetof(st3d_opts, src_f), offsetof(st3d_info, bytes_per_point),"
        " sizeof(st3d_metrics), offsetof(st3d_opts, device), offsetof(st3d_info, device));"
        " return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                           check=True).stdout.split()]
    assert vals == [C.sizeof(api.GridDesc), C.sizeof(api.Opts), C.sizeof(api.Info),
                    api.Opts.c0.offset, api.Opts.src_f.offset, api.Info.bytes_per_point.offset,
                    C.sizeof(api.Metrics), api.Opts.device.offset, api.Info.device.offset]


def test_abi_version_and_strings():
    lib = S.lib()
    assert lib.st3d_abi_version() == 2
    assert lib.st3d_status_string(0) == b"ok"
    assert b"out of order" in lib.st3d_status_string(6)


@pytest.mark.parametrize("points", [2, 7, 13, 25])
@pytest.mark.parametrize("storage", ["f32", "f64"])
def test_default_coefficients_equal_oracle(points, storage):
    o = S.default_opts(points, "ref", storage)
    dt = np.float64 if storage == "f64" else np.float32
    ref = O.default_coefs(points, dt)
    got = np.array(list(o.coef), dtype=np.float64)
    if storage == "f32":
        got = got.astype(np.float32)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("points,dt", [(7, 1e-3), (13, 5e-4), (25, 5e-4)])
def test_wave_constants_equal_oracle(points, dt):
    o = S.default_opts(points, "wave", "f32", dt=dt)
    c0, c1, c2 = O.wave_constants(points, 1500.0, dt, 10.0)
    assert (o.c0, o.c1, o.c2) == (c0, c1, c2)
    w = np.array(list(o.coef), dtype=np.float32)
    np.testing.assert_array_equal(w, O.wave_weights(points))


def test_ricker_equals_oracle():
    for t in np.linspace(0.0, 0.3, 31):
        assert S.ricker(t) == O.ricker(t)


def test_plan_layout():
    g = S.Grid(1024, 1024, 1024, 4, 4, 16)
    info = S.plan(g, S.default_opts(25, "wave", "f32"))
    assert info.kernel == S.KERNEL_TMA
    assert info.pk == 32 and info.pj == 4 and info.pi == 4
    assert info.nk == 1088 and (info.nk * 4) % 128 == 0
    assert info.nj == 1032 and info.ni == 1032
    assert info.bytes_per_point == 16.0 and info.flops_per_point == 41
    d = S.plan(g, S.default_opts(25, "ref", "f64"))
    assert d.kernel == S.KERNEL_SIMPLE and d.pk == 16 and d.bytes_per_point == 32.0
    two = S.plan(S.Grid(8, 8, 8, 4, 4, 1), S.default_opts(2))
    assert two.kernel == S.KERNEL_SIMPLE and two.bytes_per_point == 8.0
    odd = S.plan(S.Grid(17, 19, 23, 4, 4, 1), S.default_opts(7))
    assert (odd.nk * 4) % 128 == 0 and odd.nk >= 32 + 23 + 1
    # a context that blocks in time holds a second u/v pair: five fields, and
    # one pass of T steps moves 20 bytes per point
    tb = S.plan(g, S.default_opts(7, "wave", "f32", temporal_block=4))
    assert tb.temporal_block == 4 and tb.device_bytes == 5 * 1032 * 1032 * 1088 * 4
    assert tb.bytes_per_point == 5.0


@pytest.mark.parametrize("grid,opts,status", [
    ((8, 8, 8, 2, 4, 4), dict(points=25), S.api.ERR_INVALID),     # xh < R
    ((8, 8, 8, 4, 4, 3), dict(points=25), S.api.ERR_INVALID),     # zh < R
    ((8, 8, 8, 0, 0, 0), dict(points=7), S.api.ERR_INVALID),      # no halo
    ((8, 8, 8, 0, 0, 1), dict(points=2), S.api.OK),               # 2 points read k+1 only
    ((0, 8, 8, 4, 4, 4), dict(points=7), S.api.ERR_INVALID),      # empty grid
    ((8, 8, 8, 4, 4, 4), dict(points=9), S.api.ERR_INVALID),      # unknown stencil
    ((8, 8, 8, 4, 4, 4), dict(points=2, mode="wave"), S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=7, storage="f64", kernel="tma"), S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=7, mode="wave", src=(8, 0, 0)), S.api.ERR_INVALID),
    ((8, 8, 8, 4, 4, 4), dict(points=7, mode="wave", temporal_block=4), S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=13, mode="wave", temporal_block=2), S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=13, mode="wave", temporal_block=4), S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", temporal_block=2), S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", temporal_block=4), S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=7, mode="ref", temporal_block=2), S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=7, mode="wave", temporal_block=3), S.api.ERR_INVALID),
    ((8, 8, 8, 4, 4, 4), dict(points=7, mode="wave", storage="f16", temporal_block=2),
     S.api.ERR_UNSUPPORTED),
    # the tensor-core kernel: the 16-bit delta forms, 16-row tiles, 6/8/10 stages
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", storage="f16", kernel="mma"), S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=7, mode="wave", storage="bf16", kernel="mma"), S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=13, mode="wave", storage="f16_hl", kernel="mma", stages=4),
     S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=13, mode="wave", storage="f16", kernel="mma", stages=8),
     S.api.OK),
    ((8, 8, 8, 4, 4, 4), dict(points=13, mode="wave", storage="f16_hl", kernel="mma", stages=8),
     S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", storage="f32", kernel="mma"),
     S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", storage="f16_hilo", kernel="mma"),
     S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", storage="f16", kernel="mma", tile_j=20),
     S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", storage="f16", kernel="mma", stages=4),
     S.api.ERR_UNSUPPORTED),
    ((8, 8, 8, 4, 4, 4), dict(points=25, mode="wave", storage="f16_hl", kernel="mma", stages=6),
     S.api.ERR_UNSUPPORTED),
])
def test_plan_rejects_bad_requests(grid, opts, status):
    opts = dict(opts)
    pts = opts.pop("points")
    mode = opts.pop("mode", "ref")
    storage = opts.pop("storage", "f32")
    if pts == 9:
        o = S.default_opts(7)
        o.points = 9
    else:
        o = S.default_opts(pts, mode, storage, **opts)
    info = api.Info()
    rc = S.lib().st3d_plan(C.byref(S.Grid(*grid).desc()), C.byref(o), C.byref(info))
    assert rc == status, S.last_error()


def test_plan_reports_the_tensor_core_kernel():
    g = S.Grid(64, 64, 64, 4, 4, 4)
    for storage in ("f16", "bf16", "f16_hl"):
        info = S.plan(g, S.default_opts(25, "wave", storage, kernel="mma"))
        assert info.kernel == S.KERNEL_MMA and info.tile_j == 16 and info.tile_k == 152
    assert S.plan(g, S.default_opts(25, "wave", "f16", kernel="tma")).kernel == S.KERNEL_TMA
    # AUTO: the tensor-core kernel for the delta forms when no scalar tile or
    # depth is named
    auto = lambda p, st, **kw: S.plan(g, S.default_opts(p, "wave", st, **kw)).kernel
    for p in (7, 13, 25):
        assert auto(p, "f16") == auto(p, "bf16") == auto(p, "f16_hl") == S.KERNEL_MMA
    assert auto(25, "f16", tile_j=20) == auto(25, "f16", stages=8) == S.KERNEL_TMA
    assert auto(25, "f16_hilo") == auto(25, "f32") == S.KERNEL_TMA


@pytest.mark.parametrize("storage,eb", [("f32", 4), ("f64", 8), ("f16", 2), ("bf16", 2),
                                        ("f16_hl", 2), ("f16_hilo", 2)])
@pytest.mark.parametrize("points", [7, 25])
@pytest.mark.parametrize("shape", [(17, 19, 23), (9, 17, 141), (30, 43, 140), (64, 40, 1000)])
def test_layout_keeps_tile_origins_16_byte_aligned(storage, eb, points, shape):
    """A TMA tile copy faults unless its innermost coordinate times the word
    size is a multiple of 16 bytes.  The layout starts the interior one
    128-byte pad into each row and makes rows whole 128-byte lines; the tile
    kernels take columns k0 - kh .. with k0 a multiple of the tile width and
    kh their k margin (4 or 8 floats for FP32, 8 words for 16-bit tiles).
    Every such origin over the grid's tiles, and every store origin k0,
    falls on a 16-byte boundary."""
    info = S.plan(S.Grid(*shape, 4, 4, 4), S.default_opts(points, "wave", storage))
    assert info.pk * eb == 128 and (info.nk * eb) % 128 == 0
    assert info.nk >= info.pk + shape[2] + 8
    if info.tile_k == 0:
        assert info.kernel == S.KERNEL_SIMPLE
        return
    assert (info.tile_k * eb) % 16 == 0
    for kh in ((4, 8) if eb == 4 else (8,)):
        for k0 in range(0, shape[2], info.tile_k):
            assert ((info.pk + k0 - kh) * eb) % 16 == 0
            assert ((info.pk + k0) * eb) % 16 == 0


def test_device_field_defaults_and_planning():
    """opts.device: -1 (the current device) by default; st3d_plan reports
    the requested ordinal and rejects one below -1."""
    o = S.default_opts(25, "wave", "f32")
    assert o.device == -1
    g = S.Grid(16, 16, 16, 4, 4, 4)
    assert S.plan(g, o).device == -1
    o.device = 3
    assert S.plan(g, o).device == 3
    o.device = -2
    info = api.Info()
    assert S.lib().st3d_plan(C.byref(g.desc()), C.byref(o), C.byref(info)) == S.api.ERR_INVALID
    assert "device" in S.last_error()


def _gpu_visible():
    try:
        S.device_info()
        return True
    except S.St3dError:
        return False


@pytest.mark.skipif(_gpu_visible(), reason="a GPU is visible")
def test_no_cpu_fallback_without_gpu():
    """Without a GB300 the library refuses to run instead of computing on the CPU."""
    with pytest.raises(S.St3dError) as e:
        S.Stencil(S.Grid(16, 16, 16, 4, 4, 4), 25)
    assert e.value.status == S.api.ERR_NODEVICE
    v = np.zeros(S.Grid(8, 8, 8, 4, 4, 4).shape, np.float32)
    with pytest.raises(S.St3dError):
        S.iterate_gb300(v, v.copy(), v.copy(), S.Grid(8, 8, 8, 4, 4, 4), points=7)
    # an explicit device ordinal does not bring a CPU path either
    with pytest.raises(S.St3dError) as e:
        S.Stencil(S.Grid(16, 16, 16, 4, 4, 4), 25, device=0)
    assert e.value.status == S.api.ERR_NODEVICE


def test_grid_mirror_matches_reference_strides():
    g = S.Grid(100, 60, 48, 4, 5, 16)
    assert g.jmult == 48 + 32
    assert g.imult == g.jmult * (60 + 10)
    assert g.ijk_ofs == 16 + 5 * g.jmult + 4 * g.imult
    assert g.gsize == (48 + 32) * (60 + 10) * (100 + 8)
    assert g.gvol == 100 * 60 * 48
    a = np.arange(g.gsize, dtype=np.float32).reshape(g.shape)
    assert g.interior(a)[3, 2, 1] == g.idx(3, 2, 1)


def test_host_check_and_init_arrays():
    g = S.Grid(6, 5, 4, 4, 4, 1)
    v, s, u = g.empty(), g.empty(), g.empty()
    S.init_arrays(v, s, u, g.gsize)
    assert np.all(u == 1) and np.all(s == 1) and np.all(v == 0)
    assert S.check(v, g, 0) == 0
    assert S.check(v, g, 1) == 6 * 5 * 4


@pytest.mark.parametrize("desc,what", [
    ((8, 1 << 25, 8, 4, 4, 4), "2^24"),          # ys beyond an axis limit (and INT_MAX as int)
    ((8, 8, (1 << 31) + 5, 4, 4, 4), "2^24"),    # zs that an int cast would make negative
    ((8, 8, 8, 65, 4, 4), "too wide"),           # halo beyond the library's limit
    ((0, 8, 8, 4, 4, 4), ">= 1"),
    ((4097, 8, 8, 4, 4, 4), "4096"),             # the allocation-free array's plane limit
])
def test_noalloc_norms_validate_the_grid_before_any_device_work(desc, what):
    """st3d_norms_noalloc applies every entry point's grid limits before it
    touches a GPU (no device is needed to see the refusal)."""
    g = api.GridDesc(*desc)
    rc = S.lib().st3d_norms_noalloc(C.byref(g), C.c_void_p(256), S.F32, None, S.F32,
                                    C.c_void_p(256), None)
    assert rc == S.api.ERR_INVALID
    assert what in S.last_error()
