"""The benchmark's command-line contract, on the CPU: the reference arm (the
oracle port of pplacer's placement flow, core.ml:113-409, timed on the host
cores) prints one JSON line with the keys the GPU arm's line has, and the GPU
arm fails loudly where there is no CUDA device instead of falling back to a
CPU path."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args, timeout=300):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_prints_one_contract_line():
    r = _bench("--impl", "reference", "--steps", "2", "--warmup", "1", "--cpu-sample", "16", "--workload",
               "cpu_small")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["metric"] == "query placements/s" and line["unit"] == "placements/s"
    assert line["steps"] == 2 and line["warmup"] == 1 and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"] == "cpu_small"
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_gpu_arm_fails_loudly_without_a_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present")
    except ImportError:
        pass
    r = _bench("--steps", "1", "--warmup", "3", "--workload", "cpu_small", "--cpu-sample", "8")
    assert r.returncode != 0
    assert "no CUDA device" in r.stderr
    assert not any(ln.startswith("{") for ln in r.stdout.splitlines())
