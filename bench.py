#!/usr/bin/env python3
"""Benchmark of the stencil3d hot path on GB300.

Workload (default): the 25-point cross stencil (radius 4, the reference's
stencil_25.h coefficients) in its leapfrog wave form, 1024^3 interior with
4-point halos, FP32 fields; Gaussian-blob initial field (8 seeded blobs,
sigma = 20 cells, v = u), 15 Hz Ricker point source at the grid centre,
c = 1500 m/s, dx = 10 m, dt = 0.5 ms.  Synthetic data: the reference ships
no dataset.

One step = one leapfrog time step over the whole grid (one kernel launch).
``value`` is whole-job throughput in Gpoints/s with the fields resident in
HBM; ``e2e`` is the same metric through the drop-in C-ABI call
``st3d_iterate_host`` (ITERATE's replacement) on pinned host arrays, host
to device and device to host copies inside the timed region.  The u, v and
s fields of the default workload take 13.9 GB in the device layout, far more
than the 129 MB L2, so no flush is needed between steps.

Beside the headline the line carries: the 16-bit storage forms (``fp16``:
FP16 and BF16 delta forms, the FP16 hi/lo pair form, FP16 + int8) with their
error against an FP64 run every 100 steps over 1000 steps, and the guarded
FP16 run that moves to a compensated form past half of a 1e-3 tolerance;
the FP64 path; the 64-grid batch (sequential, persistent, graph, tuned);
temporal blocking (1/2/4 fused steps); ``e2e``; ``cpu_baseline``.

``--impl reference`` times the CPU restatement of the path (the oracle; the
reference's own compiled path where it runs on this machine) with every host
core on the same workload, one full time step per step.

Multi-GPU: the path does not shard (a single grid would need a halo
exchange the reference does not have), so ``--gpus N`` under torchrun runs N
independent replicas, one grid per GPU (weak scaling), barrier and max-over-
ranks timing over gloo.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOADS = {
    # name: (points, xs, ys, zs, halo, dt, init)
    "wave25_1024": (25, 1024, 1024, 1024, 4, 5e-4, "blobs"),
    "wave25_512": (25, 512, 512, 512, 4, 5e-4, "blobs"),
    "wave25_528": (25, 528, 528, 528, 4, 5e-4, "uniform"),
    "wave13_1040": (13, 1040, 1040, 1040, 2, 5e-4, "blobs"),
    "wave7_256": (7, 256, 256, 256, 1, 1e-3, "uniform"),
    "wave7_1024": (7, 1024, 1024, 1024, 4, 1e-3, "blobs"),
    "wave7_512": (7, 512, 512, 512, 4, 1e-3, "blobs"),
    "wave13_512": (13, 512, 512, 512, 4, 5e-4, "blobs"),
}
# fused steps per pass served for each stencil order
TB_DEPTHS = {7: (1, 2, 4), 13: (1, 2, 4), 25: (1, 2)}
# timed steps of a temporal-blocking workload that has a stated run length:
# the 13-point 1040^3 configuration runs 2000 steps at every depth
TB_STEPS = {"wave13_1040": 2000}
# the smaller benchmark configurations, each at its stated run length, FP32
# plain steps of the wave form (the 256^3 and 528^3 runs of the reference's
# host driver)
CONFIG_RUNS = (("wave7_256", 20), ("wave25_528", 200))
SEED = 20251203
# st3d_kernel values by name
KERNEL_NAMES = {1: "simple", 2: "tma", 3: "mma"}
# CUDA device of this replica (LOCAL_RANK under torchrun)
DEVICE = -1


def parse():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=sorted(WORKLOADS), default="wave25_1024")
    p.add_argument("--kernel", choices=["auto", "simple", "tma"], default="auto")
    p.add_argument("--accuracy-steps", type=int, default=1000,
                   help="steps of the FP32-vs-FP64 drift run (0: skip)")
    p.add_argument("--e2e-calls", type=int, default=3)
    p.add_argument("--e2e-iters", type=int, default=20,
                   help="time steps per drop-in call (the README host run uses --iter 20)")
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="target CPU time of the cpu_baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--batch-steps", type=int, default=500,
                   help="steps of the batching-form run: 64 seeded grids (0 to skip)")
    p.add_argument("--batch-grids", type=int, default=64,
                   help="grids of the batching-form run (the first n of the seeded list)")
    p.add_argument("--precision-forms", default="f16_hilo,f16_hl,f16,bf16",
                   help="16-bit storage forms timed and judged against FP64 ('' to skip)")
    p.add_argument("--guard-fallback", default="f16_hilo", choices=["f16_hilo", "f16_hl"],
                   help="storage the guarded FP16 run moves to past half the tolerance")
    p.add_argument("--fp64-steps", type=int, default=5,
                   help="timed steps of the FP64 (USE_DOUBLE) run of the workload (0 to skip)")
    p.add_argument("--temporal-workloads", default="wave7_1024,wave13_1040,wave25_1024",
                   help="workloads timed with 1, 2 and 4 fused steps per pass ('' to skip)")
    p.add_argument("--temporal-steps", type=int, default=40,
                   help="timed steps of each temporal-blocking run without a stated run length "
                        "(a multiple of 4; wave13_1040 runs its 2000)")
    p.add_argument("--mode-r-steps", type=int, default=20,
                   help="timed steps of the mode R (reference update) run of the workload (0: skip)")
    p.add_argument("--no-configs", dest="configs", action="store_false",
                   help="skip the smaller benchmark configurations (wave7_256, wave25_528)")
    return p.parse_args()


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.2)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(kernel_tag, workload):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/<kernel>_<workload>.md, line 'traffic_bytes_per_launch:')."""
    path = os.path.join(REPO, "profiles", "%s_%s.md" % (kernel_tag, workload))
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


# --------------------------------------------------------------------------
def make_stencil(S, wl, storage="f32", kernel="auto", temporal_block=1, **kw):
    kw.setdefault("device", DEVICE)
    points, xs, ys, zs, halo, dt, init = WORKLOADS[wl]
    g = S.Grid(xs, ys, zs, halo, halo, halo)
    st = S.Stencil(g, points, "wave", storage, kernel=kernel, dt=dt,
                   src=(xs // 2, ys // 2, zs // 2), temporal_block=temporal_block, **kw)
    init_fields(S, st, init)
    return g, st


def l2_note(info):
    """How the timed steps avoid L2 reuse: the u, v and s fields each step
    streams are far larger than the 129 MB L2."""
    fields = 3 * info.nk * info.nj * info.ni * 4 / 1e9
    return "fields %.1f GB >> 129 MB L2, no flush needed" % fields


def init_fields(S, st, init):
    if init == "blobs":
        st.fill(S.FIELD_U, S.FILL_BLOBS, SEED, 8, 20.0)
        st.fill(S.FIELD_V, S.FILL_BLOBS, SEED, 8, 20.0)
    else:
        st.fill(S.FIELD_U, S.FILL_UNIFORM, SEED, -1e-3, 1e-3)
        st.fill(S.FIELD_V, S.FILL_UNIFORM, SEED + 1, -1e-3, 1e-3)
    st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
    st.synchronize()


def accuracy_run(S, wl, steps, kernel, storages, guard_tol=1e-3, fallback="f16_hilo"):
    """Runs of the same workload in each storage next to an FP64 run; relative
    L2 and max error of u against FP64 every 100 steps (FP64 device
    reductions).  With guard_tol, also the guarded precision form: FP16 delta
    storage that moves to the compensated form when its error against the
    FP64 run passes guard_tol at a check (stencil3d_gb300.precision)."""
    from stencil3d_gb300.precision import GuardedWave
    points, xs, ys, zs, halo, dt, init = WORKLOADS[wl]
    ref_g, ref = make_stencil(S, wl, "f64")
    runs = {st: make_stencil(S, wl, st, kernel if st == "f32" else "auto")[1] for st in storages}
    report = {st: [] for st in storages}
    guard = None
    if guard_tol:
        guard = GuardedWave(ref_g, points, tol=guard_tol, fallback=fallback, dt=dt,
                            src=(xs // 2, ys // 2, zs // 2), device=DEVICE)
        init_fields(S, guard, init)
        guard_s = 0.0
    # The FP64 run advances in chunks of `every`: the guarded run is checked
    # after each chunk until it has moved, then every 100 steps like the rest.
    every = 10
    done = 0
    while done < steps:
        n = min(every, steps - done)
        ref.iterate(n)
        ref.synchronize()
        done += n
        if guard is not None:
            t0 = time.perf_counter()
            guard.iterate(n)
            guard.synchronize()
            if guard.switched_at is None or done % 100 == 0 or done == steps:
                guard.check(ref)  # the move to the fallback, when it happens, is timed too
            guard_s += time.perf_counter() - t0
        if done % 100 and done != steps:
            continue
        m = done - (done - 1) // 100 * 100
        for st in storages:
            runs[st].iterate(m)
        for st in storages:
            runs[st].synchronize()
            d2, b2, dm, bm = runs[st].norms(S.FIELD_U, ref, S.FIELD_U)
            report[st].append({"step": done, "rel_l2": (d2 / b2) ** 0.5 if b2 > 0 else None,
                               "max_abs": dm, "rel_max": dm / bm if bm > 0 else None})
    for r in runs.values():
        r.close()
    ref.close()
    if guard is not None:
        report["guarded"] = {
            "tol": guard_tol, "margin": guard.margin, "storage": guard.storage,
            "fallback": guard.fallback, "switched_at": guard.switched_at,
            "checks": "every %d steps until the move, then every 100" % every,
            "value": xs * ys * zs * steps / guard_s / 1e9, "unit": "Gpts/s",
            "value_note": "host wall clock per 100-step chunk, incl. the error check and the move",
            "accuracy_vs_fp64": [{"step": st, "storage": sto, "rel_l2": e} for st, sto, e in guard.history
                                 if st % 100 == 0 or st == guard.switched_at],
            "l2_err_vs_fp64": guard.history[-1][2] if guard.history else None}
        guard.close()
    return report


def batch_specs(seed=SEED, n=64):
    """The batching workload: n grids, each axis uniform in 64..320 cells,
    stencil order from {7, 13, 25}, a Ricker source at a random interior
    point, FP32 wave form (seeded)."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        xs, ys, zs = (int(x) for x in rng.integers(64, 321, size=3))
        pts = int(rng.choice([7, 13, 25]))
        src = tuple(int(rng.integers(0, d)) for d in (xs, ys, zs))
        specs.append(((xs, ys, zs), pts, src))
    return specs


def batch_run(S, steps, warmup, n=64):
    """Aggregate throughput of the batching form under each schedule."""
    specs = batch_specs(n=n)
    grids = [S.Grid(xs, ys, zs, 4, 4, 4) for (xs, ys, zs), _, _ in specs]
    pts = [p for _, p, _ in specs]
    dts = [1e-3 if p == 7 else 5e-4 for p in pts]
    srcs = [s for _, _, s in specs]
    out = {"grids": len(specs), "steps": steps,
           "workload": "%d grids, axes U{64..320}, orders {7,13,25}, FP32 wave, seeded sources" % n}
    with S.Batch(grids, pts, dt=dts, srcs=srcs, device=DEVICE) as b:
        for i in range(len(grids)):
            st = b.context(i)
            st.fill(S.FIELD_U, S.FILL_BLOBS, SEED + i, 4, 12.0)
            st.fill(S.FIELD_V, S.FILL_BLOBS, SEED + i, 4, 12.0)
            st.fill(S.FIELD_S, S.FILL_CONST, 0, 0.0)
        info = b.info()
        total = info.interior_points
        out["points"] = int(total)
        out["work_items_per_step"] = int(info.work_items)
        for schedule in ("sequential", "persistent", "graph", "pipelined"):
            b.iterate(warmup, schedule)
            b.synchronize()
            l0 = b.info().launches
            b.timer_start()
            b.iterate(steps, schedule)
            ms = b.timer_stop()
            b.synchronize()
            out[schedule] = {"value": total * steps / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
                             "ms_per_step": ms / steps,
                             "launches": int(b.info().launches - l0)}
    out["graph_vs_sequential"] = out["graph"]["value"] / out["sequential"]["value"]
    out["pipelined_vs_sequential"] = out["pipelined"]["value"] / out["sequential"]["value"]
    # the autotuner's pick of unit length and schedule for this batch
    import tempfile
    from stencil3d_gb300 import autotune
    with tempfile.TemporaryDirectory() as tmp:
        best = autotune.tune_batch(grids, pts, dts=dts, srcs=srcs, steps=20,
                                   cache=os.path.join(tmp, "tune.json"))
    out["tuned"] = {"opts": best["opts"], "value": best["gpts"], "unit": "Gpts/s",
                    "table": [[c, None if ms is None else total / (ms * 1e-3) / 1e9]
                              for c, ms in best["table"]]}
    return out


def time_storage(S, wl, storage, steps, warmup, kernel="auto"):
    """Device time of `steps` steps in one storage (fresh fields, W warm-up)."""
    g, st = make_stencil(S, wl, storage, kernel)
    info = st.info()
    st.iterate(warmup)
    st.synchronize()
    st.timer_start()
    st.iterate(steps)
    ms = st.timer_stop()
    st.synchronize()
    st.close()
    return g.gvol * steps / (ms * 1e-3) / 1e9, ms / steps, info


def temporal_run(S, workloads, steps, warmup, peak):
    """Throughput of each workload with 1, 2 and 4 leapfrog steps fused per
    pass over HBM (temporal blocking), and the fused result's agreement with
    plain steps (bitwise: max |difference| of u after the run)."""
    out = {}
    for wl in workloads:
        points = WORKLOADS[wl][0]
        n = TB_STEPS.get(wl, steps)
        n = max(4, n - n % 4)
        res = {"steps": n}
        ref = None
        for T in TB_DEPTHS.get(points, (1,)):
            g, st = make_stencil(S, wl, "f32", "tma", temporal_block=T)
            info = st.info()
            st.iterate(4 * warmup)  # the same start time for every depth
            st.synchronize()
            l0 = st.info().launches
            st.timer_start()
            st.iterate(n)
            ms = st.timer_stop()
            st.synchronize()
            launches = st.info().launches - l0
            pts = g.gvol
            ach = info.bytes_per_point * pts * n / (ms * 1e-3) / 1e9
            entry = {"value": pts * n / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
                     "ms_per_step": ms / n, "launches": int(launches),
                     "bytes_per_point_step": info.bytes_per_point,
                     "tile_rows": int(info.tb_tile_j or info.tile_j),
                     "roofline": {"achieved": ach, "peak": peak, "unit": "GB/s",
                                  "frac": ach / peak}}
            if ref is None:
                ref = st
            else:
                d2, b2, dm, bm = st.norms(S.FIELD_U, ref, S.FIELD_U)
                entry["max_abs_diff_vs_T1"] = dm
                st.close()
            res["T%d" % T] = entry
        ref.close()
        base = res["T1"]["value"]
        for k, e in res.items():
            if isinstance(e, dict):
                e["speedup_vs_T1"] = e["value"] / base
        out[wl] = res
    return out


def mode_r_run(S, wl, steps, warmup, peak):
    """The reference's own update (mode R: stencil_25_ref_1, stencil_25.h:75-95
    for 25 points) on the workload's grid, FP32: seeded u, v ~ U[-1, 1) and
    s ~ U[0.5, 1.5) (the fields of the parity tests), u and s fixed, v
    accumulating; one launch per step, CUDA events on the context's stream."""
    points, xs, ys, zs, halo, dt, init = WORKLOADS[wl]
    g = S.Grid(xs, ys, zs, halo, halo, halo)
    with S.Stencil(g, points, "ref", "f32", device=DEVICE) as st:
        st.fill(S.FIELD_U, S.FILL_UNIFORM, SEED, -1.0, 1.0)
        st.fill(S.FIELD_V, S.FILL_UNIFORM, SEED + 1, -1.0, 1.0)
        st.fill(S.FIELD_S, S.FILL_UNIFORM, SEED + 2, 0.5, 1.5)
        info = st.info()
        st.iterate(warmup)
        st.synchronize()
        l0 = st.info().launches
        st.timer_start()
        st.iterate(steps)
        ms = st.timer_stop()
        st.synchronize()
        launches = st.info().launches - l0
    value = g.gvol * steps / (ms * 1e-3) / 1e9
    ach = info.bytes_per_point * g.gvol / (ms / max(1, launches) * 1e-3) / 1e9
    return {"workload": "%s, mode R (the reference's update), seeded u, v ~ U[-1,1), "
                        "s ~ U[0.5,1.5)" % wl,
            "value": value, "unit": "Gpts/s", "steps": steps, "ms_per_step": ms / steps,
            "launches": int(launches), "kernel": "k_tma<%d,ref>" % points,
            "parity": "bit-exact to the oracle's fused flavour, <= 1e-5 relative L2 from the "
                      "reference order (tests/test_configs_gpu.py, 20 steps at 1024^3)",
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "bytes_per_point": info.bytes_per_point}}


def config_runs(S, warmup, peak):
    """The smaller benchmark configurations at their stated run lengths: the
    plain FP32 wave steps, Gpts/s and the fraction of the HBM roofline."""
    out = {}
    for wl, steps in CONFIG_RUNS:
        g, st = make_stencil(S, wl, "f32", "auto")
        try:
            info = st.info()
            st.iterate(warmup)
            st.synchronize()
            st.timer_start()
            st.iterate(steps)
            ms = st.timer_stop()
            st.synchronize()
        finally:
            st.close()
        ach = info.bytes_per_point * g.gvol * steps / (ms * 1e-3) / 1e9
        out[wl] = {"value": g.gvol * steps / (ms * 1e-3) / 1e9, "unit": "Gpts/s", "steps": steps,
                   "ms_per_step": ms / steps, "fields_gb": round(3 * g.gsize * 4 / 1e9, 3),
                   "roofline": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak}}
    return out


def _r(x, n=4):
    """x rounded to n significant digits (None stays None)."""
    if x is None:
        return None
    return float("%.*g" % (n, x))


def summary_of(result):
    """The figures a reader needs first, in one short object: the FP32
    headline, mode R, each 16-bit form (Gpts/s, speed-up over FP32, roofline
    fraction, relative L2 against FP64 after the accuracy run), the batch,
    temporal blocking per depth and the smaller configurations."""
    out = {"fp32": [_r(result["value"]), _r(result["roofline"]["frac"], 3),
                    _r(result.get("l2_err_fp32_vs_fp64"), 3)],
           "cols": "[Gpts/s, x FP32, HBM frac, rel L2 vs FP64 after the accuracy run]"}
    if result.get("mode_r"):
        out["mode_r"] = [_r(result["mode_r"]["value"]), _r(result["mode_r"]["roofline"]["frac"], 3)]
    for form, e in (result.get("fp16") or {}).items():
        if form == "f16_guarded":
            out[form] = [_r(e.get("value")), None, None, _r(e.get("l2_err_vs_fp64"), 3)]
            continue
        out[form] = [_r(e["value"]), _r(e["speedup_vs_fp32"], 3), _r(e["roofline"]["frac"], 3),
                     _r(e.get("l2_err_vs_fp64"), 3)]
        if e.get("kernel"):
            out.setdefault("fp16_kernel", {})[form] = e["kernel"]
    b = result.get("batch")
    if b:
        out["batch"] = {"seq": _r(b["sequential"]["value"]), "persistent": _r(b["persistent"]["value"]),
                        "graph": _r(b["graph"]["value"]), "graph_vs_seq": _r(b["graph_vs_sequential"], 3)}
        if "pipelined" in b:
            out["batch"]["pipelined"] = _r(b["pipelined"]["value"])
    for wl, r in (result.get("temporal_blocking") or {}).items():
        out["tb_" + wl] = {k: _r(e["value"]) for k, e in r.items() if isinstance(e, dict)}
        out["tb_" + wl]["steps"] = r["steps"]
    for wl, e in (result.get("configs") or {}).items():
        out[wl] = [_r(e["value"]), _r(e["roofline"]["frac"], 3)]
    if result.get("e2e"):
        out["e2e"] = _r(result["e2e"]["value"])
    return out


def e2e_run(S, st, g, calls, iters):
    """Drop-in calls on pinned host arrays: upload v, s, u; `iters` steps;
    download v and u; CUDA events on the context's stream bracket it all."""
    shape = g.shape
    pv, ps, pu = S.PinnedArray(shape), S.PinnedArray(shape), S.PinnedArray(shape)
    try:
        st.download(pv.array, pu.array)  # current device state as the host input
        ps.array[...] = 0.0
        st.iterate_host(pv.array, ps.array, pu.array, iters)  # warm-up call
        times = []
        for _ in range(calls):
            st.timer_start()
            st.iterate_host(pv.array, ps.array, pu.array, iters)
            times.append(st.timer_stop())
        path = st.info().host_path  # of the timed calls
        # the same call split into its phases, for the record
        phases = {}
        st.timer_start()
        st.upload(pv.array, ps.array, pu.array)
        phases["upload_ms"] = st.timer_stop()
        st.timer_start()
        st.iterate(iters)
        phases["iterate_ms"] = st.timer_stop()
        st.timer_start()
        st.download(pv.array, pu.array)
        phases["download_ms"] = st.timer_stop()
        host = (pv.array.copy(), pu.array.copy())
    finally:
        for p in (pv, ps, pu):
            p.free()
    pts = g.gvol
    ms = statistics.median(times)
    # bytes copied per call: each upload moves a whole host array, each
    # download the span of the interior rows of every interior plane
    xs, ys, zs = g.xsize, g.ysize, g.zsize
    h2d = 3 * g.gsize * 4
    d2h = 2 * xs * ys * (zs + 2 * g.zhalo) * 4
    return {"value": pts * iters / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "host_path": {0: "auto", 1: "staged", 2: "direct", 3: "strided",
                          4: "streamed"}[path],
            "step": "one ITERATE-equivalent call (st3d_iterate_host) of %d time steps" % iters,
            "ms_per_call": ms, "phases": phases,
            "h2d_gbs": h2d / (phases["upload_ms"] * 1e-3) / 1e9,
            "d2h_gbs": d2h / (phases["download_ms"] * 1e-3) / 1e9}, host


def cpu_wave_sample(wl, u, v, target_s, threads):
    """Time the CPU restatement (oracle, plain flavour, OpenMP) of the same
    leapfrog update on the same fields: one full time step per sample step."""
    from oracle import oracle as O
    points, xs, ys, zs, halo, dt, init = WORKLOADS[wl]
    grid = (xs, ys, zs, halo, halo, halo)
    c0, c1, c2 = O.wave_constants(points, 1500.0, dt, 10.0)
    s = np.zeros_like(u)
    src = (xs // 2, ys // 2, zs // 2)
    amps = O.ricker_amps(0, 10000, dt)
    t0 = time.perf_counter()
    O.iterate_wave(u, v, s, grid, points, 1, c0, c1, c2, src=src, amps=amps, fma=False)
    one = time.perf_counter() - t0
    n = max(2, min(200, int(target_s / max(one, 1e-6))))
    n += n % 2  # even: no trailing copy of the newest field back into u
    t0 = time.perf_counter()
    O.iterate_wave(u, v, s, grid, points, n, c0, c1, c2, src=src, amps=amps[1:], fma=False)
    el = time.perf_counter() - t0
    out = {"value": xs * ys * zs * n / el / 1e9, "unit": "Gpts/s", "cores": threads,
           "kind": "port",
           "sample": "%d full %s leapfrog steps (%.1f s) of the oracle's C restatement, "
                     "OpenMP %d threads" % (n, wl, el, threads)}
    # the reference's own update (mode R) restated: the plain flavour is bit
    # for bit the reference's compiled stencil_*_ref_1 over its jk-blocked
    # traversal; fields as they are (the timing does not depend on them)
    s[...] = 1.0
    t0 = time.perf_counter()
    O.iterate_ref(v, s, u, grid, points, 1, fma=False)
    one = time.perf_counter() - t0
    nr = max(1, min(50, int(0.5 * target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    O.iterate_ref(v, s, u, grid, points, nr, fma=False)
    el = time.perf_counter() - t0
    out["mode_r"] = {"value": xs * ys * zs * nr / el / 1e9, "unit": "Gpts/s",
                     "sample": "%d mode R steps (%.1f s) of %s, the reference's update restated, "
                               "OpenMP %d threads" % (nr, el, wl, threads)}
    return out


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# --------------------------------------------------------------------------
def run_gb300(args, dist):
    global DEVICE
    import stencil3d_gb300 as S
    DEVICE = dist.local_rank  # one replica per GPU
    points, xs, ys, zs, halo, dt, init = WORKLOADS[args.workload]
    g, st = make_stencil(S, args.workload, "f32", args.kernel)
    info = st.info()
    st.iterate(args.warmup)
    st.synchronize()

    dist.barrier()
    st.synchronize()
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    launches0 = st.info().launches
    st.timer_start()
    st.iterate(args.steps)
    ms = st.timer_stop()
    st.synchronize()
    launches = st.info().launches - launches0
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)

    pts = g.gvol
    value = dist.world * pts * args.steps / (ms_max * 1e-3) / 1e9
    launch_ms = ms / max(1, launches)
    peak, peak_kind = measured_peak()
    achieved = info.bytes_per_point * pts / (launch_ms * 1e-3) / 1e9
    kernel_tag = "tma" if info.kernel == S.KERNEL_TMA else "simple"
    traffic = profile_traffic(kernel_tag, args.workload)

    result = {
        "metric": "Gpts/s + % of HBM roofline, 25-pt 1024^3: FP32 vs FP16-store at stated L2 err",
        "value": value, "unit": "Gpts/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded Gaussian blobs + Ricker source (no dataset in the reference)",
        "config": {"workload": args.workload, "points": points, "grid": [xs, ys, zs],
                   "halo": halo, "form": "leapfrog wave", "dt": dt, "storage": "f32",
                   "kernel": kernel_tag, "tile_j": info.tile_j, "tile_k": info.tile_k,
                   "ichunk": info.ichunk,
                   "l2": l2_note(info),
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "gflops": pts * args.steps * info.flops_per_point / (ms * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "bytes_per_point": info.bytes_per_point,
                     "traffic": traffic,
                     "kernel": "k_tma<%d,wave>" % points if kernel_tag == "tma" else
                               "k_simple<float,%d,wave>" % points},
        "gpu_launches": int(launches),
        "clocks": clk,
        "fp16": None,
    }

    forms = [f for f in args.precision_forms.split(",") if f]
    if forms:
        result["fp16"] = {}
        for form in forms:
            gp, msf, finfo = time_storage(S, args.workload, form, args.steps, args.warmup)
            gp = dist.world * gp * (ms / ms_max)  # same replica scaling as value
            ach = finfo.bytes_per_point * pts / (msf * 1e-3) / 1e9
            result["fp16"][form] = {"value": gp, "unit": "Gpts/s", "ms_per_step": msf,
                                    "speedup_vs_fp32": gp / value,
                                    "bytes_per_point": finfo.bytes_per_point,
                                    "kernel": KERNEL_NAMES.get(finfo.kernel, finfo.kernel),
                                    "roofline": {"achieved": ach, "peak": peak, "unit": "GB/s",
                                                 "frac": ach / peak}}
            if finfo.kernel == S.KERNEL_MMA:
                # the scalar 16-bit kernel on the same workload, for comparison
                gs, mss, _ = time_storage(S, args.workload, form, args.steps, args.warmup, "tma")
                result["fp16"][form]["scalar_kernel"] = {
                    "kernel": "tma", "value": dist.world * gs * (ms / ms_max), "ms_per_step": mss,
                    "frac": finfo.bytes_per_point * pts / (mss * 1e-3) / 1e9 / peak}
    if args.fp64_steps > 0:
        # the reference's USE_DOUBLE build (config.h:96-97) on the device:
        # the plain kernel in FP64, 32 algorithmic bytes per point
        gp, msd, dinfo = time_storage(S, args.workload, "f64", args.fp64_steps, min(args.warmup, 3))
        ach = dinfo.bytes_per_point * pts / (msd * 1e-3) / 1e9
        # FP64 arithmetic per point of the wave update: 3 per neighbour pair
        # ((a+b), -2u, fma) plus 2u, -v and two fma; each one FP64-pipe
        # instruction, against the nominal 1.25 TFLOP/s = 0.625 T FP64 fma/s
        npairs = {7: 3, 13: 6, 25: 12}[points]
        dp_ops = 3 * npairs + 4
        dp_rate = dp_ops * pts / (msd * 1e-3) / 1e12
        result["fp64"] = {"value": dist.world * gp * (ms / ms_max), "unit": "Gpts/s",
                          "ms_per_step": msd, "bytes_per_point": dinfo.bytes_per_point,
                          "gflops": pts * dinfo.flops_per_point / (msd * 1e-3) / 1e9,
                          "roofline": {"bound": "fp64", "achieved": dp_rate, "peak": 0.625,
                                       "unit": "T fp64 instr/s", "frac": dp_rate / 0.625,
                                       "peak_kind": "nominal (1.25 TFLOP/s FP64)",
                                       "fp64_ops_per_point": dp_ops,
                                       "hbm_frac": ach / peak},
                          "kernel": "k_simple<double,%d,wave>" % points}
    if dist.rank == 0 and args.accuracy_steps > 0:
        acc = accuracy_run(S, args.workload, args.accuracy_steps, args.kernel, ["f32"] + forms,
                           guard_tol=1e-3 if "f16" in forms else 0, fallback=args.guard_fallback)
        result["accuracy_vs_fp64"] = acc["f32"]
        if "guarded" in acc:
            result["fp16"]["f16_guarded"] = acc["guarded"]
        result["l2_err_fp32_vs_fp64"] = acc["f32"][-1]["rel_l2"]
        for form in forms:
            result["fp16"][form]["accuracy_vs_fp64"] = acc[form]
            result["fp16"][form]["l2_err_vs_fp64"] = acc[form][-1]["rel_l2"]

    if dist.rank == 0 and args.mode_r_steps > 0:
        result["mode_r"] = mode_r_run(S, args.workload, args.mode_r_steps, args.warmup, peak)

    if dist.rank == 0 and args.configs:
        result["configs"] = config_runs(S, args.warmup, peak)

    if dist.rank == 0 and args.batch_steps > 0:
        result["batch"] = batch_run(S, args.batch_steps, args.warmup, args.batch_grids)

    tws = [w for w in args.temporal_workloads.split(",") if w]
    if dist.rank == 0 and tws:
        result["temporal_blocking"] = temporal_run(S, tws, args.temporal_steps, args.warmup, peak)

    host = None
    if args.e2e_calls > 0:
        e2e, host = e2e_run(S, st, g, args.e2e_calls, args.e2e_iters)
        e2e["value"] = dist.world * e2e["value"] if dist.world > 1 else e2e["value"]
        result["e2e"] = e2e
    st.close()
    if args.e2e_calls > 0 and result["e2e"]["host_path"] in ("direct", "streamed"):
        # the same calls phase by phase (upload, steps, download) on the
        # direct path and through the staging buffer, for comparison
        for name, hp in (("direct", S.api.HOST_DIRECT), ("staged", S.api.HOST_STAGED)):
            if name == result["e2e"]["host_path"]:
                continue
            g2, st2 = make_stencil(S, args.workload, "f32", args.kernel, host_path=hp)
            e2s, _ = e2e_run(S, st2, g2, args.e2e_calls, args.e2e_iters)
            st2.close()
            result["e2e"][name] = {k: e2s[k] for k in ("value", "ms_per_call", "phases", "h2d_gbs",
                                                      "d2h_gbs", "host_path")}

    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline and host is not None:
        v_host, u_host = host
        result["cpu_baseline"] = cpu_wave_sample(args.workload, u_host, v_host,
                                                 args.cpu_seconds, host_threads())
    if dist.rank == 0:
        # last key of the line: the short summary stays inside any tail of
        # the output a reader keeps
        result["summary"] = summary_of(result)
        print(json.dumps(result), flush=True)


def run_reference(args, dist):
    """The reference arm: the CPU implementation of the path on the host
    cores, same workload and metric.  Rank 0 alone runs it."""
    if dist.rank != 0:
        return
    from oracle import build as obuild
    from oracle import oracle as O
    obuild.build_oracle()
    points, xs, ys, zs, halo, dt, init = WORKLOADS[args.workload]
    grid = (xs, ys, zs, halo, halo, halo)
    if init == "blobs":
        u = O.fill_blobs(grid, SEED, 8, 20.0)
        v = u.copy()
    else:
        u = O.fill_uniform(grid, SEED, 0, -1e-3, 1e-3)
        v = O.fill_uniform(grid, SEED + 1, 1, -1e-3, 1e-3)
    s = np.zeros_like(u)
    c0, c1, c2 = O.wave_constants(points, 1500.0, dt, 10.0)
    src = (xs // 2, ys // 2, zs // 2)
    # an even number of timed steps: the oracle moves the newest field back
    # into `u` after an odd count, a copy that is not part of the update
    timed = args.steps + (args.steps % 2)
    amps = O.ricker_amps(0, args.warmup + timed + 1, dt)
    O.iterate_wave(u, v, s, grid, points, args.warmup, c0, c1, c2, src=src, amps=amps)
    t0 = time.perf_counter()
    O.iterate_wave(u, v, s, grid, points, timed, c0, c1, c2, src=src,
                   amps=amps[args.warmup:], fma=False)
    el = time.perf_counter() - t0
    value = xs * ys * zs * timed / el / 1e9
    threads = host_threads()
    # the wave form has no reference code: what runs is always the oracle's
    # C restatement (kind "port"), whose mode R is pinned bit for bit to the
    # reference's compiled path
    kind = "port"
    sample = ("%d full leapfrog steps of %s on the CPU restatement (oracle), OpenMP %d threads"
              % (timed, args.workload, threads))
    print(json.dumps({
        "impl": "reference",
        "metric": "Gpts/s + % of HBM roofline, 25-pt 1024^3: FP32 vs FP16-store at stated L2 err",
        "value": value, "unit": "Gpts/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el * 1e3 / timed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "points": points, "grid": [xs, ys, zs],
                   "halo": halo, "form": "leapfrog wave", "dt": dt},
        "cpu_baseline": {"value": value, "unit": "Gpts/s", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "Gpts/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference has no wave form; its CPU path restated in C (oracle/st3d_oracle.c, "
                "pinned bit-exact to the reference's mode R) runs the same update",
    }), flush=True)


def main():
    args = parse()
    from stencil3d_gb300.replicas import Replicas
    dist = Replicas()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_gb300(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
