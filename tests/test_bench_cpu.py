"""The benchmark's reference arm (the CPU oracle port, no GPU needed) prints one JSON line with
the contract's keys, on small cases of the named workloads."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("args", [["--workload", "c1", "--scale", "0.05"],
                                  ["--workload", "range", "--scale", "0.02", "--dims", "9", "--structure", "kd"],
                                  ["--workload", "range", "--scale", "0.02", "--dims", "16", "--structure", "ball"]])
def test_reference_arm_line(args):
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1", *args],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
