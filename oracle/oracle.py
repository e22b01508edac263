"""ctypes front end of the CPU oracle (test infrastructure only).

Wraps ``oracle/_build/libst3d_oracle.so`` (the C restatement in
``st3d_oracle.c``) and, where it was built, the reference's own host path in
``oracle/_ref/libref<N>[d].so`` (see ``ref_harness.cpp``).  Arrays are numpy
arrays in the reference layout of grid.cpp:20-24: shape
``(xs+2xh, ys+2yh, zs+2zh)``, C order, so that element ``[xh+i, yh+j, zh+k]``
is ``IDX(i,j,k)`` of stencils.h:5.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        for T, p in (("f32", _f32p), ("f64", _f64p)):
            getattr(L, "orc_default_coefs_" + T).argtypes = [C.c_int, C.c_int, p]
            f = getattr(L, "orc_iterate_ref_" + T)
            f.argtypes = [p, p, p, _u32p, C.c_int, p, C.c_uint, C.c_int]
            f.restype = C.c_int
            f = getattr(L, "orc_iterate_wave_" + T)
            fl = C.c_float if T == "f32" else C.c_double
            f.argtypes = [p, p, p, _u32p, C.c_int, p, fl, fl, fl, C.c_void_p,
                          C.c_void_p, C.c_uint, C.c_int]
            f.restype = C.c_int
            f = getattr(L, "orc_fill_uniform_" + T)
            f.argtypes = [p, _u32p, C.c_uint64, C.c_uint, C.c_double, C.c_double]
            f = getattr(L, "orc_fill_blobs_" + T)
            f.argtypes = [p, _u32p, C.c_uint64, C.c_int, C.c_double]
        L.orc_wave_constants.argtypes = [_f32p, C.c_double, C.c_double, C.c_double, _f64p]
        L.orc_ricker.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_ricker.restype = C.c_double
        L.orc_unit_at.argtypes = [C.c_uint64, C.c_uint, C.c_longlong, C.c_longlong, C.c_longlong]
        L.orc_unit_at.restype = C.c_double
        L.orc_blob_params.argtypes = [C.c_uint64, C.c_int, _u32p, _f64p]
        L.orc_init_arrays_f32.argtypes = [_f32p, _f32p, _f32p, C.c_size_t]
        L.orc_check_f32.argtypes = [_f32p, _u32p, C.c_uint]
        L.orc_check_f32.restype = C.c_uint
        for name, pa, pb in (("f32_f32", _f32p, _f32p), ("f32_f64", _f32p, _f64p),
                             ("f64_f64", _f64p, _f64p)):
            getattr(L, "orc_diff_" + name).argtypes = [pa, pb, _u32p, _f64p]
        _lib = L
    return _lib


def _dt(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def gvec(grid):
    """grid = (xs, ys, zs, xh, yh, zh) -> uint32 vector for the C calls."""
    return np.asarray(grid, dtype=np.uint32)


def shape(grid):
    xs, ys, zs, xh, yh, zh = grid
    return (xs + 2 * xh, ys + 2 * yh, zs + 2 * zh)


def interior(a, grid):
    xs, ys, zs, xh, yh, zh = grid
    return a[xh:xh + xs, yh:yh + ys, zh:zh + zs]


def default_coefs(points, dtype=np.float32, isotropic=False):
    c = np.zeros(14, dtype=dtype)
    getattr(lib(), "orc_default_coefs_" + _dt(dtype))(points, int(isotropic), c)
    return c


def fill_uniform(grid, seed, field, lo, hi, dtype=np.float32):
    a = np.empty(shape(grid), dtype=dtype)
    getattr(lib(), "orc_fill_uniform_" + _dt(dtype))(a, gvec(grid), seed, field, lo, hi)
    return a


def fill_blobs(grid, seed, nblobs=8, sigma=20.0, dtype=np.float32):
    a = np.empty(shape(grid), dtype=dtype)
    getattr(lib(), "orc_fill_blobs_" + _dt(dtype))(a, gvec(grid), seed, nblobs, sigma)
    return a


def iterate_ref(v, s, u, grid, points, iterations, coefs=None, fma=False):
    """Mode R in place on v (stencil_*_ref_1 update, u and s fixed)."""
    if coefs is None:
        coefs = default_coefs(points, v.dtype)
    rc = getattr(lib(), "orc_iterate_ref_" + _dt(v.dtype))(
        v, s, u, gvec(grid), points, np.ascontiguousarray(coefs, dtype=v.dtype),
        iterations, int(fma))
    assert rc == 0, rc
    return v


def wave_constants(points, vel, dt, dx, coefs=None):
    if coefs is None:
        coefs = wave_weights(points)
    out = np.zeros(3, dtype=np.float64)
    lib().orc_wave_constants(np.ascontiguousarray(coefs, dtype=np.float32), vel, dt, dx, out)
    return out


def wave_weights(points, isotropic=False):
    """Mode W neighbour weights: 1 for 7 points (README.md:11-20), the
    stencil_{13,25}.h cx/cy/cz otherwise."""
    c = default_coefs(points, np.float32, isotropic)
    if points == 7:
        c[2] = c[6] = c[10] = 1.0
    c[0] = c[1] = 0.0
    return c


def ricker(t, f=15.0, t0=None):
    if t0 is None:
        t0 = 1.0 / f
    return lib().orc_ricker(t, f, t0)


def ricker_amps(step0, n, dt, f=15.0, t0=None, dtype=np.float32):
    """Source amplitudes of steps step0 .. step0+n-1: w((step0+m)*dt)."""
    return np.array([ricker((step0 + m) * dt, f, t0) for m in range(n)], dtype=dtype)


def iterate_wave(u, v, s, grid, points, iterations, c0, c1, c2, weights=None,
                 src=None, amps=None, fma=True):
    """Mode W in place: afterwards u = U^{n+it}, v = U^{n+it-1}."""
    if weights is None:
        weights = wave_weights(points)
    T = u.dtype
    srcv = None
    if src is not None:
        srcv = np.asarray(src, dtype=np.int64)
    ampv = None
    if amps is not None:
        ampv = np.ascontiguousarray(amps, dtype=T)
        assert ampv.size >= iterations
    rc = getattr(lib(), "orc_iterate_wave_" + _dt(T))(
        u, v, s, gvec(grid), points, np.ascontiguousarray(weights, dtype=T),
        c0, c1, c2,
        srcv.ctypes.data if srcv is not None else None,
        ampv.ctypes.data if ampv is not None else None,
        iterations, int(fma))
    assert rc == 0, rc
    return u, v


def diff(a, b, grid):
    """(sum (a-b)^2, sum b^2, max|a-b|, max|b|) over the interior."""
    out = np.zeros(4, dtype=np.float64)
    name = _dt(a.dtype) + "_" + _dt(b.dtype)
    getattr(lib(), "orc_diff_" + name)(a, b, gvec(grid), out)
    return out


def rel_l2(a, b, grid):
    d2, b2, _, _ = diff(a, b, grid)
    return float(np.sqrt(d2 / b2)) if b2 > 0 else float(np.sqrt(d2))


def init_arrays(grid):
    n = int(np.prod(shape(grid)))
    v = np.empty(shape(grid), np.float32)
    s = np.empty(shape(grid), np.float32)
    u = np.empty(shape(grid), np.float32)
    lib().orc_init_arrays_f32(v, s, u, n)
    return v, s, u


def check(v, grid, maxiter):
    return int(lib().orc_check_f32(v, gvec(grid), maxiter))


# ---------------------------------------------------------------------------
# The reference itself (oracle/_ref), where it was built on this machine.
# ---------------------------------------------------------------------------
_ref_libs = {}


def ref_available(points=7, dtype=np.float32):
    return ref_lib(points, dtype) is not None


def ref_lib(points, dtype=np.float32):
    key = (points, _dt(dtype))
    if key in _ref_libs:
        return _ref_libs[key]
    name = "libref%d%s.so" % (points, "d" if _dt(dtype) == "f64" else "")
    path = os.path.join(_build.REF_DIR, name)
    L = None
    if os.path.exists(path):
        try:
            L = C.CDLL(path)
        except OSError:
            L = None  # built for another architecture
    if L is not None:
        p = _f64p if _dt(dtype) == "f64" else _f32p
        for fn in ("ref_iterate", "ref_iterate_3d"):
            getattr(L, fn).argtypes = [p, p, p] + [C.c_uint] * 7
            getattr(L, fn).restype = C.c_int
        L.ref_check_count.argtypes = [p] + [C.c_uint] * 7
        L.ref_check_count.restype = C.c_uint
    _ref_libs[key] = L
    return L


def ref_vec16_13():
    """The reference's 13-point vec_16 kernel build (K = 6.25), or None."""
    path = os.path.join(_build.REF_DIR, "libref13vec16.so")
    if not os.path.exists(path):
        return None
    try:
        L = C.CDLL(path)
    except OSError:
        return None
    L.ref_iterate.argtypes = [_f32p, _f32p, _f32p] + [C.c_uint] * 7
    return L


def ref_iterate(v, s, u, grid, points, iterations, traversal="2d_jk_blocked"):
    """The reference's ITERATE (iterate_2d_jk_blocked, or iterate_3d) in place."""
    L = ref_lib(points, v.dtype)
    if L is None:
        raise RuntimeError("reference library for %d points is not built here" % points)
    fn = L.ref_iterate if traversal == "2d_jk_blocked" else L.ref_iterate_3d
    fn(v, s, u, *[int(x) for x in grid], iterations)
    return v


# ---------------------------------------------------------------------------
# 16-bit storage forms (FP16 / BF16 words with per-plane scales, optional
# compensating byte), restated in oracle/st3d_oracle.c
# ---------------------------------------------------------------------------
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def _lib16():
    L = lib()
    if not getattr(L, "_f16_ready", False):
        L.orc16_encode.argtypes = [C.c_int, C.c_int, _f32p, _u32p, _u16p, C.c_void_p, _i32p, _f32p]
        L.orc16_decode.argtypes = [C.c_int, C.c_int, _u16p, C.c_void_p, _i32p, _u32p, _f32p]
        L.orc16_iterate_wave.argtypes = [
            C.c_int, C.c_int, _u16p, C.c_void_p, _i32p, _f32p, _u16p, C.c_void_p, _i32p, _f32p,
            _u16p, _i32p, _f32p, _u32p, C.c_int, _f32p, C.c_float, C.c_float, C.c_float,
            C.c_void_p, C.c_void_p, C.c_uint]
        L.orc16_iterate_wave.restype = C.c_int
        L.orc16_iterate_delta.argtypes = [
            C.c_int, _u16p, _i32p, _f32p, _u16p, _i32p, _f32p, _u16p, _i32p, _f32p, _u32p, C.c_int,
            _f32p, C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p]
        L.orc16_iterate_delta.restype = C.c_int
        L.orc16_encode_pair.argtypes = [_f32p, _u32p, _u16p, _u16p, _i32p, _f32p]
        L.orc16_decode_pair.argtypes = [_u16p, _u16p, _i32p, _u32p, _f32p]
        L.orc16_scale_exponent.argtypes = [C.c_float]
        L.orc16_scale_exponent.restype = C.c_int
        L._f16_ready = True
    return L


class Field16:
    """A field in 16-bit storage: words h, bytes q (compensated form), per-plane
    scale exponents E and maxima M."""

    def __init__(self, x, grid, kind, hilo):
        self.kind, self.hilo, self.grid = kind, hilo, grid
        self.h = np.zeros(shape(grid), np.uint16)
        self.q = np.zeros(shape(grid), np.int8) if hilo else None
        self.E = np.zeros(grid[0], np.int32)
        self.M = np.zeros(grid[0], np.float32)
        _lib16().orc16_encode(kind, int(hilo), np.ascontiguousarray(x, np.float32), gvec(grid),
                              self.h, self.q.ctypes.data if hilo else None, self.E, self.M)

    def decode(self):
        x = np.zeros(shape(self.grid), np.float32)
        _lib16().orc16_decode(self.kind, int(self.hilo), self.h,
                              self.q.ctypes.data if self.hilo else None, self.E,
                              gvec(self.grid), x)
        return x


class FieldPair:
    """A field in the FP16 hi/lo pair storage (the u of the F16_HL form):
    words h and l with x = (h + l) * 2^E, per-plane scale exponents E and
    maxima M."""

    def __init__(self, x, grid):
        self.kind, self.hilo, self.grid = 0, False, grid
        self.h = np.zeros(shape(grid), np.uint16)
        self.l = np.zeros(shape(grid), np.uint16)
        self.E = np.zeros(grid[0], np.int32)
        self.M = np.zeros(grid[0], np.float32)
        _lib16().orc16_encode_pair(np.ascontiguousarray(x, np.float32), gvec(grid), self.h, self.l,
                                   self.E, self.M)

    def decode(self):
        x = np.zeros(shape(self.grid), np.float32)
        _lib16().orc16_decode_pair(self.h, self.l, self.E, gvec(self.grid), x)
        return x


def storage_kind(storage):
    """(kind, hilo) of a 16-bit storage name (the F16_HL form is FP16 words
    without the compensating byte)."""
    return {"f16": (0, False), "bf16": (1, False), "f16_hilo": (0, True), "f16_hl": (0, False)}[storage]


def k4_of(points, c1):
    """4*c1*sum(w) rounded to float, as the library forms it."""
    w = wave_weights(points)
    return float(np.float32(4.0 * c1 * sum(float(x) for x in w[2:14])))


def iterate_wave16(u, v, s, grid, points, iterations, c1, c2, src=None, amps=None, weights=None):
    """Mode W on Field16 states u, v (in place; u newest afterwards) and s."""
    if weights is None:
        weights = wave_weights(points)
    srcv = None if src is None else np.asarray(src, dtype=np.int64)
    ampv = None if amps is None else np.ascontiguousarray(amps, dtype=np.float32)
    rc = _lib16().orc16_iterate_wave(
        u.kind, int(u.hilo), u.h, u.q.ctypes.data if u.hilo else None, u.E, u.M,
        v.h, v.q.ctypes.data if v.hilo else None, v.E, v.M, s.h, s.E, s.M, gvec(grid), points,
        np.ascontiguousarray(weights, np.float32), c1, c2, k4_of(points, c1),
        srcv.ctypes.data if srcv is not None else None,
        ampv.ctypes.data if ampv is not None else None, iterations)
    assert rc == 0, rc
    return u, v


def delta_fields(u, v, grid, kind, pair=False):
    """The FP16 / BF16 storage state of (u, v): Field16 of u (FieldPair with
    `pair`, the F16_HL form) and of the time difference d = u - v (FP32
    subtraction, as the library forms it)."""
    u = np.ascontiguousarray(u, np.float32)
    d = u - np.ascontiguousarray(v, np.float32)
    fu = FieldPair(u, grid) if pair else Field16(u, grid, kind, False)
    return fu, Field16(d, grid, kind, False)


def delta_decode(fu, fd):
    """(u, v) of a delta-form state: u = dec(U), v = u - dec(D) (FP32)."""
    u = fu.decode()
    return u, u - fd.decode()


def iterate_delta16(u, d, s, grid, points, iterations, c1, c2, src=None, amps=None, weights=None):
    """Mode W in the FP16 / BF16 delta form on Field16 states u, d (in place,
    newest level afterwards) and s; u a FieldPair runs the F16_HL form."""
    if weights is None:
        weights = wave_weights(points)
    srcv = None if src is None else np.asarray(src, dtype=np.int64)
    ampv = None if amps is None else np.ascontiguousarray(amps, dtype=np.float32)
    rc = _lib16().orc16_iterate_delta(
        u.kind, u.h, u.E, u.M, d.h, d.E, d.M, s.h, s.E, s.M, gvec(grid), points,
        np.ascontiguousarray(weights, np.float32), c1, c2, k4_of(points, c1),
        srcv.ctypes.data if srcv is not None else None,
        ampv.ctypes.data if ampv is not None else None, iterations,
        u.l.ctypes.data if isinstance(u, FieldPair) else None)
    assert rc == 0, rc
    return u, d
