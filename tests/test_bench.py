"""bench.py without a GPU: the reference arm's JSON line, the committed ncu
traffic it quotes, and the seeded batch workload."""
import json
import os
import subprocess
import sys
from types import SimpleNamespace

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def test_reference_arm_line():
    """`--impl reference` prints one JSON line with the contract's keys: the
    CPU implementation's throughput, its own cpu_baseline description and an
    e2e block with no host-device bytes."""
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                          "--workload", "wave7_256", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Gpts/s"
    assert line["config"]["workload"] == "wave7_256"
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_traffic_comes_from_the_committed_profile():
    t = bench.profile_traffic("tma", "wave25_1024")
    assert t is not None and 17.18e9 < t < 20e9  # 1.0 .. 1.16 x the 16 B/pt algorithmic bytes
    assert bench.profile_traffic("tma", "no_such_workload") is None


def test_batch_workload_is_seeded_and_prefix_stable():
    a, b = bench.batch_specs(), bench.batch_specs()
    assert a == b and len(a) == 64
    assert bench.batch_specs(n=16) == a[:16]
    for (xs, ys, zs), pts, src in a:
        assert all(64 <= d <= 320 for d in (xs, ys, zs)) and pts in (7, 13, 25)
        assert all(0 <= s < d for s, d in zip(src, (xs, ys, zs)))


def test_l2_note_uses_the_device_layout():
    info = SimpleNamespace(nk=1088, nj=1032, ni=1032)
    assert bench.l2_note(info) == "fields 13.9 GB >> 129 MB L2, no flush needed"


def test_summary_is_short_and_last():
    """The summary object closes the line and stays short enough to survive
    in a kept tail of the output."""
    form = {"value": 300.0, "speedup_vs_fp32": 0.75, "roofline": {"frac": 0.45},
            "l2_err_vs_fp64": 6.6e-3}
    tb = {"steps": 2000, "T1": {"value": 405.0}, "T2": {"value": 470.0}, "T4": {"value": 440.0}}
    result = {"value": 398.3, "roofline": {"frac": 0.939}, "l2_err_fp32_vs_fp64": 3.4e-6,
              "mode_r": {"value": 395.0, "roofline": {"frac": 0.93}},
              "fp16": {"f16": form, "bf16": form, "f16_hl": form, "f16_hilo": form,
                       "f16_guarded": {"value": 197.0, "l2_err_vs_fp64": 8.4e-4}},
              "batch": {"sequential": {"value": 186.0}, "persistent": {"value": 357.0},
                        "graph": {"value": 358.0}, "graph_vs_sequential": 1.92},
              "temporal_blocking": {"wave7_1024": tb, "wave13_1040": tb, "wave25_1024": tb},
              "configs": {"wave7_256": {"value": 300.0, "roofline": {"frac": 0.7}},
                          "wave25_528": {"value": 380.0, "roofline": {"frac": 0.9}}},
              "e2e": {"value": 126.5}}
    sm = bench.summary_of(result)
    text = json.dumps(sm)
    assert len(text) < 1200, len(text)
    assert sm["fp32"][0] == 398.3 and sm["f16"][1] == 0.75 and sm["tb_wave13_1040"]["steps"] == 2000
