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


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    """Two ranks on gloo (no GPU): rank 0 alone times the CPU reference and prints the line, the
    other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--workload", "c1", "--scale", "0.02"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(s) for s in out.stdout.splitlines() if s.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0


def _rank_helpers(rank, world, port, results):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup()
    try:
        bench.barrier(w)
        # Each rank reports its own step time; every rank must see the slowest one.
        results[r] = bench.max_over_ranks(w, 10.0 + 5.0 * r)
        bench.barrier(w)
    finally:
        bench.dist_teardown(w)


def test_rank_helpers_take_the_slowest_rank_over_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        results = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_helpers, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(results) == {0: 15.0, 1: 15.0}
