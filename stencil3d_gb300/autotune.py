"""Autotuner for the stencil kernels: picks the launch configuration of one
(grid, stencil order, mode, storage) by timing candidate configurations on the
device, and keeps the choice in a JSON cache.

For a batch of grids (``tune_batch``) the knobs are the planes per work
unit and the schedule (CUDA graph, plain persistent launches, or one
pipelined launch per call).

The knobs are the ``st3d_opts`` fields that change how the work is tiled,
never what is computed: the kernel (TMA pipeline, plain, or for the 16-bit
delta forms the tensor-core kernel), tile rows (``tile_j``), pipeline stages
(``stages``), planes per work unit (``ichunk``) and, for the FP32 wave form
of the 7- and 13-point stencils on a zero halo, steps fused per pass
(``temporal_block``).  Every candidate produces the same bits as any other
(the per-point operation sequence is fixed), except that the tensor-core
kernel sums in the tensor cores' order (within one unit in the last place of
the 16-bit words per step), so the tuner only ranks speed.  The reference
has no counterpart (its tile sizes are command-line options,
main.cpp:125-144).

    best = tune(Grid(1024, 1024, 1024, 4, 4, 4), 25, "wave", "f16")
    st = Stencil(grid, 25, "wave", "f16", **best["opts"])

``tune`` looks the key up in the cache first; ``measure`` may be replaced (the
tests pass a model of the timings) so the search and the cache run without a
GPU.
"""
import json
import os
import time

from . import api

CACHE_ENV = "ST3D_TUNE_CACHE"
KNOBS = ("kernel", "tile_j", "stages", "ichunk", "temporal_block")


def default_cache_path():
    return os.environ.get(CACHE_ENV) or os.path.join(
        os.path.expanduser("~"), ".cache", "stencil3d_gb300", "tune.json")


def candidates(points, mode, storage, zero_halo=False):
    """The configurations worth timing for one stencil/mode/storage, as
    dicts of ``st3d_opts`` overrides (0 = the library's automatic choice)."""
    out = []
    if storage == "f16_hl":
        for tj, depths in ((16, (4, 6, 8)), (20, (6, 8)), (8, (4, 6, 8))):
            for nv in depths:
                out.append({"kernel": "tma", "tile_j": tj, "stages": nv})
        return out + [{"kernel": "mma", "ichunk": ic} for ic in (0, 64, 256)]
    if storage in ("f16", "bf16"):
        for tj, depths in ((16, (4, 6, 8, 12)), (20, (6, 8, 10)), (8, (4, 6, 8, 12))):
            for nv in depths:
                out.append({"kernel": "tma", "tile_j": tj, "stages": nv})
        return out + [{"kernel": "mma", "ichunk": ic} for ic in (0, 64, 256)]
    if storage == "f16_hilo":
        return [{"kernel": "tma", "tile_j": 16, "stages": nv} for nv in (4, 6, 8, 12)]
    if storage == "f64" or points == 2:
        return [{"kernel": "simple", "ichunk": ic} for ic in (32, 64, 128)]
    # FP32: the TMA pipeline shapes the kernel serves, a few unit lengths,
    # and the plain kernel as a floor
    for tj, nv in ((16, 4), (16, 3), (16, 2), (8, 4), (8, 3)):
        for ic in (0, 64, 256):
            out.append({"kernel": "tma", "tile_j": tj, "stages": nv, "ichunk": ic})
    out.append({"kernel": "simple", "ichunk": 64})
    if zero_halo and mode == "wave":
        # the fused depths the library serves: (T - 1) * R <= 8
        for T in ((2, 4) if points in (7, 13) else (2,)):
            for ic in (0, 64):
                out.append({"kernel": "tma", "temporal_block": T, "ichunk": ic})
    return out


def cache_key(grid, points, mode, storage, device=None):
    d = device if device is not None else api.device_info()
    return "sm%d_cc%d%d|%d|%s|%s|%dx%dx%d|h%d,%d,%d" % (
        d["sm_count"], d["cc"][0], d["cc"][1], points, mode, storage, grid.xsize, grid.ysize,
        grid.zsize, grid.xhalo, grid.yhalo, grid.zhalo)


def load_cache(path):
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(path, data):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def measure_device(grid, points, mode, storage, cand, steps=10, warmup=3, phys=None):
    """Milliseconds per step of one candidate on the device: seeded blob
    fields (zero halo), `warmup` untimed steps, CUDA events around `steps`.
    Returns None when the library refuses the configuration."""
    phys = dict(phys or {})
    try:
        st = api.Stencil(grid, points, mode, storage, **phys, **cand)
    except api.St3dError:
        return None
    try:
        st.fill(api.FIELD_U, api.FILL_BLOBS, 1, 8, 20.0)
        st.fill(api.FIELD_V, api.FILL_BLOBS, 1, 8, 20.0)
        st.fill(api.FIELD_S, api.FILL_CONST, 0, 0.0)
        st.iterate(warmup)
        st.synchronize()
        st.timer_start()
        st.iterate(steps)
        ms = st.timer_stop()
        st.synchronize()
        return ms / steps
    except api.St3dError:
        return None
    finally:
        st.close()


def tune(grid, points, mode="wave", storage="f32", steps=10, cache=None, refresh=False,
         zero_halo=False, measure=None, device=None, phys=None):
    """Best configuration for the workload: {"opts": overrides, "ms_per_step",
    "gpts", "table": [[candidate, ms], ...], "key"}.  The result is cached
    under the workload's key (device, stencil, mode, storage, sizes, halos)."""
    path = cache if cache is not None else default_cache_path()
    key = cache_key(grid, points, mode, storage, device)
    data = load_cache(path)
    if not refresh and key in data:
        return data[key]
    if measure is None:
        def measure(c):
            return measure_device(grid, points, mode, storage, c, steps=steps, phys=phys)
    table = []
    t0 = time.perf_counter()
    for cand in candidates(points, mode, storage, zero_halo):
        ms = measure(cand)
        table.append([cand, ms])
    timed = [(c, ms) for c, ms in table if ms is not None and ms > 0]
    if not timed:
        raise api.St3dError(api.ERR_UNSUPPORTED, "no candidate configuration ran")
    best, ms = min(timed, key=lambda x: x[1])
    pts = grid.xsize * grid.ysize * grid.zsize
    result = {"key": key, "opts": best, "ms_per_step": ms, "gpts": pts / (ms * 1e-3) / 1e9,
              "table": table, "tuning_s": time.perf_counter() - t0}
    data = load_cache(path)  # another process may have added keys meanwhile
    data[key] = result
    save_cache(path, data)
    return result


def batch_key(grids, points, device=None):
    """Cache key of a batch: device, and a digest of the (sizes, halos,
    order) list in order."""
    import hashlib
    d = device if device is not None else api.device_info()
    desc = ";".join("%dx%dx%d|%d,%d,%d|%d" % (g.xsize, g.ysize, g.zsize, g.xhalo, g.yhalo, g.zhalo, p)
                    for g, p in zip(grids, points))
    return "sm%d_cc%d%d|batch|%d|%s" % (d["sm_count"], d["cc"][0], d["cc"][1], len(grids),
                                         hashlib.sha1(desc.encode()).hexdigest()[:16])


def batch_candidates():
    """Batch knobs: planes per work unit (shorter units balance the shared
    queue, longer ones re-read fewer warm-up planes; 512 is a whole column
    of every grid up to 512 planes) and the schedule."""
    return [{"ichunk": ic, "schedule": sch} for ic in (32, 64, 128, 256, 512)
            for sch in ("graph", "persistent", "pipelined")]


def measure_batch_device(grids, points, cand, dts=None, srcs=None, steps=20, warmup=3):
    """Milliseconds per step of a batch under one candidate (seeded blob
    fields, CUDA events around `steps` steps)."""
    try:
        b = api.Batch(grids, points, dt=dts, srcs=srcs, ichunk=cand["ichunk"])
    except api.St3dError:
        return None
    try:
        for i in range(len(grids)):
            st = b.context(i)
            st.fill(api.FIELD_U, api.FILL_BLOBS, 1 + i, 4, 12.0)
            st.fill(api.FIELD_V, api.FILL_BLOBS, 1 + i, 4, 12.0)
            st.fill(api.FIELD_S, api.FILL_CONST, 0, 0.0)
        b.iterate(warmup, cand["schedule"])
        b.synchronize()
        b.timer_start()
        b.iterate(steps, cand["schedule"])
        ms = b.timer_stop()
        b.synchronize()
        return ms / steps
    except api.St3dError:
        return None
    finally:
        b.close()


def tune_batch(grids, points, dts=None, srcs=None, steps=20, cache=None, refresh=False,
               measure=None, device=None):
    """Best batch configuration: {"opts": {"ichunk", "schedule"}, "ms_per_step",
    "gpts", "table", "key"}, cached like `tune`."""
    path = cache if cache is not None else default_cache_path()
    key = batch_key(grids, points, device)
    data = load_cache(path)
    if not refresh and key in data:
        return data[key]
    if measure is None:
        def measure(c):
            return measure_batch_device(grids, points, c, dts=dts, srcs=srcs, steps=steps)
    t0 = time.perf_counter()
    table = [[c, measure(c)] for c in batch_candidates()]
    timed = [(c, ms) for c, ms in table if ms is not None and ms > 0]
    if not timed:
        raise api.St3dError(api.ERR_UNSUPPORTED, "no batch configuration ran")
    best, ms = min(timed, key=lambda x: x[1])
    pts = sum(g.xsize * g.ysize * g.zsize for g in grids)
    result = {"key": key, "opts": best, "ms_per_step": ms, "gpts": pts / (ms * 1e-3) / 1e9,
              "table": table, "tuning_s": time.perf_counter() - t0}
    data = load_cache(path)
    data[key] = result
    save_cache(path, data)
    return result


def tuned_stencil(grid, points, mode="wave", storage="f32", cache=None, zero_halo=False,
                  **kw):
    """A Stencil with the tuned configuration (tuning on first use)."""
    phys = {k: kw[k] for k in ("vel", "dt", "dx") if k in kw}
    best = tune(grid, points, mode, storage, cache=cache, zero_halo=zero_halo, phys=phys)
    opts = dict(best["opts"])
    opts.update({k: v for k, v in kw.items() if k not in KNOBS})
    return api.Stencil(grid, points, mode, storage, **opts)
