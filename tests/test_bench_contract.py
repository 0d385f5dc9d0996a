"""The bench's reference arm on CPU: the line the measurement contract asks
for (one JSON object from rank 0 with the workload, the metric and the
reported CPU baseline; nothing, and exit 0, from the other ranks)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, env_extra=None, timeout=300):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                          env=env, timeout=timeout, cwd=ROOT)


def test_reference_arm_line():
    # the line's format on a 256^2 grid (the default 4096^2 takes ~4 s per step here)
    r = _run(["--impl", "reference", "--steps", "5", "--warmup", "3", "--grid", "256"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["unit"] == "cell-updates/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 5 and d["warmup"] == 3
    assert d["config"]["workload"] == "shear layer 256x256, SSP-RK3, WENO-Z, CFL 0.7, seed 2024"
    assert "5 timed" in d["cpu_baseline"]["sample"] and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert isinstance(cb["sample"], str) and cb["sample"]
    one = cb["single_core"]
    assert one["cores"] == 1 and one["value"] > 0 and one["unit"] == d["unit"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_are_silent():
    r = _run(["--impl", "reference", "--gpus", "2"], env_extra={"RANK": "1", "WORLD_SIZE": "2"}, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_warmup_below_three_is_rejected():
    r = _run(["--warmup", "2"], timeout=120)
    assert r.returncode != 0
    assert "--warmup" in r.stderr


@pytest.mark.gpu
def test_kernel_tour_runs():
    """Every kernel of the path once at a small size (the per-kernel counter
    capture's workload)."""
    r = _run(["--kernel-tour", "256"], timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    tour = d["kernel_tour"]
    for k in ("fp64", "fp32", "fp64_rk1", "wave_fp64", "learned", "batch_fp32", "batch_fp64"):
        assert tour[k]["steps"] == 1, k
    assert 0.0 <= tour["learned"]["flagged"] <= 1.0
    assert tour["noalloc_dt"]["rc"] == 0 and tour["noalloc_dt"]["dt"] > 0.0
