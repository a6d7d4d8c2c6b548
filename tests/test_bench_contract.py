"""bench.py's output contract on small cases: one JSON line with the metric,
value, unit, counts, timing, scaling, dtype, data and config keys, plus e2e
(with the bytes copied each step), gpu_launches, roofline, cpu_baseline and
clocks for our arm, and impl/cpu_baseline/e2e for the reference arm."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "e2e")


def _run(args, timeout):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def _check_base(d):
    for k in BASE_KEYS:
        assert k in d, k
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["unit"] == "IP-updates/s" and d["data"] == "synthetic" and d["scaling"] == "weak"
    assert d["warmup"] >= 3
    assert "workload" in d["config"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in d["e2e"], k


def test_reference_arm_line():
    d = _run(["--impl", "reference", "--n", "8", "--steps", "2", "--warmup", "3"], timeout=600)
    assert d["config"]["elements"] == 512 and d["config"]["parallelism"] == "replicas1"
    _check_base(d)
    assert d["impl"] == "reference" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


@pytest.mark.gpu
def test_our_arm_line():
    d = _run(["--n", "16", "--steps", "5", "--warmup", "3", "--no-variants"], timeout=900)
    _check_base(d)
    assert d["n_gpus"] == 1 and d["dtype"] == "f64"
    assert d["e2e"]["h2d_bytes_per_step"] == 24 * d["config"]["nodes"] == d["e2e"]["d2h_bytes_per_step"]
    assert d["gpu_launches"] > 0
    # the FP64 element kernel's binding roof is the FP64 pipe; its HBM figure beside it
    r = d["roofline"]
    assert r["bound"] == "fp64" and r["unit"] == "TFLOP/s" and r["peak"] > 0 and "traffic" in r
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12 and 0 < r["pipe_instruction_frac"] < 1.5
    h = d["roofline_hbm"]
    assert h["bound"] == "hbm" and h["unit"] == "GB/s" and h["peak"] > 0
    assert abs(h["frac"] - h["achieved"] / h["peak"]) < 1e-12 and "traffic" in h
    # both arms describe the workload with the same dict
    ref = _run(["--impl", "reference", "--n", "16", "--steps", "1", "--warmup", "3"], timeout=600)
    assert ref["config"] == d["config"]
    assert d["cpu_baseline"]["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
