"""ctypes binding of libst3d (include/st3d.h) and the Python mirror of the
reference's host interface.

The reference's interface for the hot path is C++ (iterators.h:6-36,
grid.h:7-71): ``s_grid`` describes the fields, ``ITERATE(v, s, u, grid,
prefetch_dist, dups, iterations, cacheiter)`` advances them in place, and
``init_arrays`` / ``check`` are the known-answer harness.  This module keeps
those names and argument meanings on numpy arrays in the reference layout and
runs the work through the CUDA library; there is no CPU path for the stencil:
without the built library or a GB300 every call raises ``St3dError``.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libst3d.so")

OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT, ERR_STATE, ERR_NODEVICE = range(8)
MODE_REF, MODE_WAVE = 0, 1
F32, F64, F16, BF16, F16_HILO, F16_HL = 0, 1, 2, 3, 4, 5
KERNEL_AUTO, KERNEL_SIMPLE, KERNEL_TMA, KERNEL_MMA = 0, 1, 2, 3
FIELD_U, FIELD_V, FIELD_S = 0, 1, 2
FILL_CONST, FILL_UNIFORM, FILL_BLOBS = 0, 1, 2
HOST_AUTO, HOST_STAGED, HOST_DIRECT, HOST_STRIDED, HOST_STREAMED = 0, 1, 2, 3, 4

_MODES = {"ref": MODE_REF, "wave": MODE_WAVE}
_STORAGES = {"f32": F32, "f64": F64, "f16": F16, "bf16": BF16, "f16_hilo": F16_HILO, "f16_hl": F16_HL}
_KERNELS = {"auto": KERNEL_AUTO, "simple": KERNEL_SIMPLE, "tma": KERNEL_TMA, "mma": KERNEL_MMA}


class St3dError(RuntimeError):
    def __init__(self, status, detail):
        super().__init__("st3d status %d: %s" % (status, detail))
        self.status = status


class GridDesc(C.Structure):
    _fields_ = [("xs", C.c_uint32), ("ys", C.c_uint32), ("zs", C.c_uint32),
                ("xh", C.c_uint32), ("yh", C.c_uint32), ("zh", C.c_uint32)]


class Opts(C.Structure):
    _fields_ = [("points", C.c_int32), ("mode", C.c_int32), ("storage", C.c_int32),
                ("kernel", C.c_int32), ("coef", C.c_double * 14),
                ("c0", C.c_double), ("c1", C.c_double), ("c2", C.c_double),
                ("src_i", C.c_int32), ("src_j", C.c_int32), ("src_k", C.c_int32),
                ("pad0", C.c_int32),
                ("src_f", C.c_double), ("src_t0", C.c_double), ("dt", C.c_double),
                ("temporal_block", C.c_int32), ("tile_j", C.c_int32), ("tile_k", C.c_int32),
                ("ichunk", C.c_int32), ("stages", C.c_int32), ("host_path", C.c_int32),
                ("device", C.c_int32), ("reserved", C.c_int32 * 5)]


class Info(C.Structure):
    _fields_ = [("interior_points", C.c_uint64), ("device_bytes", C.c_uint64),
                ("step", C.c_uint64), ("launches", C.c_uint64),
                ("nk", C.c_uint32), ("nj", C.c_uint32), ("ni", C.c_uint32),
                ("pk", C.c_uint32), ("pj", C.c_uint32), ("pi", C.c_uint32),
                ("kernel", C.c_int32), ("radius", C.c_int32),
                ("bytes_per_point", C.c_double), ("flops_per_point", C.c_double),
                ("tile_j", C.c_int32), ("tile_k", C.c_int32), ("ichunk", C.c_int32),
                ("temporal_block", C.c_int32), ("host_path", C.c_int32), ("tb_tile_j", C.c_int32),
                ("device", C.c_int32), ("reserved", C.c_int32 * 5)]


class Metrics(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("timed_steps", C.c_uint64), ("elapsed_ms", C.c_double),
                ("gpts", C.c_double), ("gflops", C.c_double), ("mem_gbs", C.c_double),
                ("energy_u", C.c_double), ("max_abs_u", C.c_double), ("rel_l2", C.c_double),
                ("reserved", C.c_double * 4)]


class BatchInfo(C.Structure):
    _fields_ = [("grids", C.c_uint32), ("work_items", C.c_uint32), ("ctas", C.c_uint32),
                ("graphs", C.c_uint32), ("interior_points", C.c_uint64), ("launches", C.c_uint64),
                ("reserved", C.c_int32 * 8)]


BATCH_SEQUENTIAL, BATCH_PERSISTENT, BATCH_GRAPH, BATCH_PIPELINED = 0, 1, 2, 3
_SCHEDULES = {"sequential": BATCH_SEQUENTIAL, "persistent": BATCH_PERSISTENT, "graph": BATCH_GRAPH,
              "pipelined": BATCH_PIPELINED}

_lib = None


def lib():
    """Load libst3d.so (built in-tree by ``stencil3d_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise St3dError(ERR_NODEVICE, "libst3d.so is not built (%s); run "
                            "stencil3d_gb300.build.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, i = C.c_void_p, C.c_int
        sig = {
            "st3d_abi_version": ([], i),
            "st3d_status_string": ([i], C.c_char_p),
            "st3d_last_error": ([], C.c_char_p),
            "st3d_device_info": ([C.POINTER(i), C.POINTER(i), C.POINTER(i), C.POINTER(C.c_size_t)], i),
            "st3d_default_opts": ([i, i, i, C.POINTER(Opts)], i),
            "st3d_set_wave_physics": ([C.POINTER(Opts), C.c_double, C.c_double, C.c_double], i),
            "st3d_plan": ([C.POINTER(GridDesc), C.POINTER(Opts), C.POINTER(Info)], i),
            "st3d_create": ([C.POINTER(GridDesc), C.POINTER(Opts), C.POINTER(vp)], i),
            "st3d_destroy": ([vp], i),
            "st3d_get_info": ([vp, C.POINTER(Info)], i),
            "st3d_get_stream": ([vp, C.POINTER(vp)], i),
            "st3d_upload": ([vp, vp, vp, vp], i),
            "st3d_download": ([vp, vp, vp], i),
            "st3d_iterate": ([vp, C.c_uint32], i),
            "st3d_iterate_host": ([vp, vp, vp, vp, C.c_uint32], i),
            "st3d_synchronize": ([vp], i),
            "st3d_inject_device_status": ([vp, C.c_uint32], i),
            "st3d_fill": ([vp, i, i, C.c_uint64, C.c_double, C.c_double], i),
            "st3d_check": ([vp, C.c_double, C.c_double, C.POINTER(C.c_uint64)], i),
            "st3d_norms": ([vp, i, vp, i, C.POINTER(C.c_double)], i),
            "st3d_timer_start": ([vp], i),
            "st3d_timer_stop": ([vp, C.POINTER(C.c_float)], i),
            "st3d_set_step": ([vp, C.c_uint64], i),
            "st3d_transfer": ([vp, vp], i),
            "st3d_metrics_get": ([vp, vp, C.POINTER(Metrics)], i),
            "st3d_host_alloc": ([C.c_size_t, C.POINTER(vp)], i),
            "st3d_host_free": ([vp], i),
            "st3d_ricker": ([C.c_double, C.c_double, C.c_double], C.c_double),
            "st3d_norms_noalloc": ([C.POINTER(GridDesc), vp, i, vp, i, vp, vp], i),
            "st3d_batch_create": ([C.c_uint32, C.POINTER(GridDesc), C.POINTER(Opts), C.POINTER(vp)], i),
            "st3d_batch_destroy": ([vp], i),
            "st3d_batch_context": ([vp, C.c_uint32, C.POINTER(vp)], i),
            "st3d_batch_get_info": ([vp, C.POINTER(BatchInfo)], i),
            "st3d_batch_iterate": ([vp, C.c_uint32, i], i),
            "st3d_batch_synchronize": ([vp], i),
            "st3d_batch_timer_start": ([vp], i),
            "st3d_batch_timer_stop": ([vp, C.POINTER(C.c_float)], i),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _ck(status):
    if status != OK:
        raise St3dError(status, lib().st3d_last_error().decode())


def last_error():
    return lib().st3d_last_error().decode()


def device_info():
    sm, ma, mi, tot = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
    _ck(lib().st3d_device_info(C.byref(sm), C.byref(ma), C.byref(mi), C.byref(tot)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value), "total_bytes": tot.value}


def ricker(t, f=15.0, t0=None):
    return lib().st3d_ricker(t, f, 1.0 / f if t0 is None else t0)


# ---------------------------------------------------------------------------
# s_grid mirror (grid.h:7-71, grid.cpp:9-48)
# ---------------------------------------------------------------------------
class Grid:
    """Geometry of the reference's s_grid: interior sizes, halos and the
    strides of the reference layout (grid.cpp:20-24).  The block, superblock
    and checkerboard members tile the CPU caches (grid.cpp:56-230) and have no
    GPU meaning; they are accepted and ignored."""

    def __init__(self, xs, ys, zs, xh=4, yh=4, zh=16, xb=1, yb=1, zb=None, sbm=12.0,
                 jshuffle=13, kshuffle=3):
        self.xsize, self.ysize, self.zsize = int(xs), int(ys), int(zs)
        self.xhalo, self.yhalo, self.zhalo = int(xh), int(yh), int(zh)
        self.xb_size, self.yb_size = int(xb), int(yb)
        self.zb_size = int(zb) if zb is not None else self.zsize
        self.sb_mib, self.jshuf, self.kshuf = sbm, jshuffle, kshuffle
        self.jmult = self.zsize + 2 * self.zhalo
        self.imult = self.jmult * (self.ysize + 2 * self.yhalo)
        self.ijk_ofs = self.zhalo + self.yhalo * self.jmult + self.xhalo * self.imult
        self.gsize = (self.zsize + 2 * self.zhalo) * (self.ysize + 2 * self.yhalo) * \
                     (self.xsize + 2 * self.xhalo)
        self.gvol = self.zsize * self.ysize * self.xsize

    def idx(self, i, j, k):
        return self.ijk_ofs + k + self.jmult * j + self.imult * i

    @property
    def shape(self):
        return (self.xsize + 2 * self.xhalo, self.ysize + 2 * self.yhalo,
                self.zsize + 2 * self.zhalo)

    @property
    def tuple(self):
        return (self.xsize, self.ysize, self.zsize, self.xhalo, self.yhalo, self.zhalo)

    def desc(self):
        return GridDesc(*self.tuple)

    def interior(self, a):
        a = a.reshape(self.shape)
        return a[self.xhalo:self.xhalo + self.xsize, self.yhalo:self.yhalo + self.ysize,
                 self.zhalo:self.zhalo + self.zsize]

    def empty(self, dtype=np.float32):
        return np.zeros(self.shape, dtype=dtype)


def default_opts(points, mode="ref", storage="f32", **kw):
    o = Opts()
    _ck(lib().st3d_default_opts(points, _MODES.get(mode, mode), _STORAGES.get(storage, storage),
                                C.byref(o)))
    phys = {k: kw.pop(k) for k in ("vel", "dt", "dx") if k in kw}
    if phys:
        _ck(lib().st3d_set_wave_physics(C.byref(o), phys.get("vel", 1500.0),
                                        phys.get("dt", 1e-3), phys.get("dx", 10.0)))
    for k, v in kw.items():
        if k == "kernel":
            v = _KERNELS.get(v, v)
        if k == "coef":
            for m, x in enumerate(v):
                o.coef[m] = float(x)
            continue
        if k == "src":
            if v is None:
                o.src_i = -1
            else:
                o.src_i, o.src_j, o.src_k = (int(x) for x in v)
            continue
        setattr(o, k, v)
    return o


def plan(grid, opts):
    info = Info()
    _ck(lib().st3d_plan(C.byref(grid.desc()), C.byref(opts), C.byref(info)))
    return info


def _ptr(a, dtype):
    if a is None:
        return None
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous %s array" % np.dtype(dtype).name)
    return a.ctypes.data


class Stencil:
    """One device context: the fields of one grid and one update rule.

    ``Stencil(grid, points, mode="ref"|"wave", storage="f32"|"f64", ...)``
    allocates the device fields; ``upload``/``download`` move reference-layout
    numpy arrays in and out; ``iterate(n)`` advances n steps on the device.
    """

    def __init__(self, grid, points=7, mode="ref", storage="f32", opts=None, _handle=None, **kw):
        self.grid = grid
        self.opts = opts if opts is not None else default_opts(points, mode, storage, **kw)
        self.dtype = np.float64 if self.opts.storage == F64 else np.float32
        self._owned = _handle is None
        if _handle is None:
            h = C.c_void_p()
            _ck(lib().st3d_create(C.byref(grid.desc()), C.byref(self.opts), C.byref(h)))
            self._h = h
        else:
            self._h = _handle

    def close(self):
        if getattr(self, "_h", None):
            if self._owned:
                lib().st3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def info(self):
        info = Info()
        _ck(lib().st3d_get_info(self._h, C.byref(info)))
        return info

    def upload(self, v=None, s=None, u=None):
        _ck(lib().st3d_upload(self._h, _ptr(v, self.dtype), _ptr(s, self.dtype), _ptr(u, self.dtype)))

    def download(self, v=None, u=None):
        _ck(lib().st3d_download(self._h, _ptr(v, self.dtype), _ptr(u, self.dtype)))

    def iterate(self, iterations=1):
        _ck(lib().st3d_iterate(self._h, int(iterations)))

    def set_step(self, step):
        """The mode W source clock (reset to 0 by upload and fill)."""
        _ck(lib().st3d_set_step(self._h, int(step)))

    def transfer_from(self, src):
        """Take u, v and the step clock of `src` (same grid and mode) on the
        device, encoded in this context's storage; s stays as it is."""
        _ck(lib().st3d_transfer(self._h, src._h))

    def iterate_host(self, v, s, u, iterations):
        _ck(lib().st3d_iterate_host(self._h, _ptr(v, self.dtype), _ptr(s, self.dtype),
                                    _ptr(u, self.dtype), int(iterations)))

    def synchronize(self):
        _ck(lib().st3d_synchronize(self._h))

    def inject_device_status(self, code):
        """Diagnostics: set the device status word as a timed-out device wait
        does (st3d_synchronize then reports ST3D_ERR_TIMEOUT once)."""
        _ck(lib().st3d_inject_device_status(self._h, int(code)))

    def fill(self, field, kind, seed=0, a=0.0, b=0.0):
        _ck(lib().st3d_fill(self._h, field, kind, seed, a, b))

    def check(self, expected, tol=0.1):
        n = C.c_uint64()
        _ck(lib().st3d_check(self._h, float(expected), float(tol), C.byref(n)))
        return n.value

    def norms(self, field=FIELD_U, other=None, other_field=FIELD_U):
        out = (C.c_double * 4)()
        _ck(lib().st3d_norms(self._h, field, other._h if other is not None else None,
                             other_field, out))
        return tuple(out)

    def metrics(self, ref=None):
        """st3d_metrics_get: the last timer region's throughput and the
        reference's GFlop/s and memory figures, energy and max of u, and the
        relative L2 of u from `ref`'s u (-1 without)."""
        m = Metrics()
        _ck(lib().st3d_metrics_get(self._h, ref._h if ref is not None else None, C.byref(m)))
        return {f: getattr(m, f) for f, _ in Metrics._fields_ if f != "reserved"}

    def rel_l2(self, other, field=FIELD_U, other_field=FIELD_U):
        d2, b2, dm, bm = self.norms(field, other, other_field)
        return (d2 / b2) ** 0.5 if b2 > 0 else d2 ** 0.5

    def timer_start(self):
        _ck(lib().st3d_timer_start(self._h))

    def timer_stop(self):
        ms = C.c_float()
        _ck(lib().st3d_timer_stop(self._h, C.byref(ms)))
        return ms.value


class Batch:
    """Many independent grids (FP32 wave form, 7/13/25 points) advancing
    together: ``Batch(grids, points, dt=..., srcs=...)``; ``context(i)`` is a
    Stencil view of grid i for upload/download/fill/norms; ``iterate(n,
    schedule)`` with schedule "sequential", "persistent", "graph" or
    "pipelined"."""

    def __init__(self, grids, points, dt=None, srcs=None, **kw):
        n = len(grids)
        self.grids = list(grids)
        descs = (GridDesc * n)(*[g.desc() for g in grids])
        opts = (Opts * n)()
        for i, (g, p) in enumerate(zip(grids, points)):
            extra = dict(kw)
            if dt is not None:
                extra["dt"] = dt[i] if isinstance(dt, (list, tuple)) else dt
            if srcs is not None:
                extra["src"] = srcs[i]
            opts[i] = default_opts(p, "wave", "f32", **extra)
        self.opts = opts
        h = C.c_void_p()
        _ck(lib().st3d_batch_create(n, descs, opts, C.byref(h)))
        self._h = h
        self._views = []
        for i in range(n):
            c = C.c_void_p()
            _ck(lib().st3d_batch_context(self._h, i, C.byref(c)))
            self._views.append(Stencil(grids[i], opts=opts[i], _handle=c))

    def context(self, i):
        return self._views[i]

    def __len__(self):
        return len(self._views)

    def iterate(self, steps, schedule="graph"):
        _ck(lib().st3d_batch_iterate(self._h, int(steps), _SCHEDULES.get(schedule, schedule)))

    def synchronize(self):
        _ck(lib().st3d_batch_synchronize(self._h))

    def info(self):
        info = BatchInfo()
        _ck(lib().st3d_batch_get_info(self._h, C.byref(info)))
        return info

    def timer_start(self):
        _ck(lib().st3d_batch_timer_start(self._h))

    def timer_stop(self):
        ms = C.c_float()
        _ck(lib().st3d_batch_timer_stop(self._h, C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "_h", None):
            for v in self._views:
                v.close()
            lib().st3d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class PinnedArray:
    """A numpy view of pinned host memory from st3d_host_alloc."""

    def __init__(self, shape, dtype=np.float32):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        _ck(lib().st3d_host_alloc(self.nbytes, C.byref(p)))
        self._p = p
        buf = (C.c_byte * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            lib().st3d_host_free(self._p)
            self._p = None


# ---------------------------------------------------------------------------
# The reference's harness functions (iterators.h:6-36) on host arrays
# ---------------------------------------------------------------------------
_ctx_cache = {}


def iterate_gb300(v, s, u, grid, prefetch_dist=64, dups=1, iterations=1, cacheiter=1,
                  points=7, mode="ref"):
    """Drop-in for ITERATE(v, s, u, grid, prefetch_dist, dups, iterations,
    cacheiter) (iterators.h:6-29): advances the reference-layout arrays in
    place on the GPU.  prefetch_dist, dups and cacheiter steer CPU traversal
    and cache emulation in the reference (iterators.cpp:42-89, 262-289) and
    have no effect here; points selects the stencil (STENCIL_SIZE,
    config.h:35-38)."""
    key = (grid.tuple, points, mode, v.dtype.str)
    st = _ctx_cache.get(key)
    if st is None:
        st = Stencil(grid, points, mode, "f64" if v.dtype == np.float64 else "f32")
        _ctx_cache[key] = st
    st.iterate_host(v, s, u, iterations)


def init_arrays(v, s, u, gsize=None):
    """init_arrays (iterators.cpp:292-301): v = 0, u = s = 1 everywhere."""
    v.reshape(-1)[:gsize] = 0.0
    u.reshape(-1)[:gsize] = 1.0
    s.reshape(-1)[:gsize] = 1.0


def check(v, grid, maxiter):
    """check (iterators.cpp:304-325): interior points with |v - maxiter| > 0.1."""
    return int(np.count_nonzero(np.abs(grid.interior(v) - v.dtype.type(maxiter)) > 0.1))
