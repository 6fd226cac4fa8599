"""Benchmark of the exact-kNN engine on GB300: exact kNN queries/sec.

Default workload (the configuration the headline metric is quoted on): KdTreeGpu<3>,
depthSkips 0, N = 4,194,304 points from a 64-component Gaussian mixture (sigma 0.01),
Q = 1,048,576 queries from the same mixture, K = 16, max radius +inf; seeded synthetic data.
After it, the same run measures the other configurations (`--configs`, default c1,c3,c4,c5) and
reports each in the line's `configs` block with the same fields.  Other headline workloads
(`--workload`): c1, c3, c4, c5 (uneven batch) and `range`, the reference's range-limited speed
test (N = 500,000 uniform points, Q = 10,000, K = 5, maxDistance2 = 0.01 D; `--dims 6..17`,
`--structure kd|ball|bf`).

One step = one exact query pass over the Q queries on the prebuilt tree (construction is timed
once and reported separately as build_ms).  Timed steps: CUDA events on the query stream, L2
flushed (a 256 MB write) before every step, synchronize + barrier on both sides, max over ranks;
every time is the median over the timed steps, with min, max and mean in `step_ms`.

Reported per workload:
  value      queries/sec of the chosen form (engine-selected plan: autotune, plus the learned
             radius where the workload has a training sample), inputs resident in HBM;
  no_model   the same autotuned form without the radius model, and learned_radius_gain;
  plain      queries/sec of the plain form (the reference benchmarks' template arguments);
  e2e        the chosen form through the C ABI with pinned HOST buffers (knn_query_host: copies
             of the queries in and the results out inside the timed region);
  roofline   the dominant kernel's algorithmic bytes (visit counts from the plain form's device
             counters x node/leaf/query/result sizes) or MMA work per pass / the summed CUDA-event
             spans of its launches, against the measured HBM or tensor peak; DRAM traffic, L2 byte
             rate and active lanes from the committed ncu summary;
  cpu_baseline  the reference algorithm on the host cores (oracle port), all threads.

`--impl reference` times the reference's CPU implementation of the same workload instead.
Multi-GPU (`--gpus N` under torchrun): independent replicas, one per GPU (the path has no
exchange step); value = all ranks' queries / the slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from cudaexactknn_gb300 import workloads as W  # noqa: E402

L2_FLUSH_BYTES = 256 << 20
METRIC = "exact kNN queries/sec on 1 GB300: chosen vs plain GPU form, 100% exact match"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "range"])
    ap.add_argument("--dims", type=int, default=16, help="range workload: D in 6..17")
    ap.add_argument("--structure", default="kd", choices=["kd", "ball", "bf"], help="range workload: index type")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the workload (debug only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--configs", default="c1,c3,c4,c5",
                    help="with the default c2 workload: further configurations measured after it and "
                         "reported in the line's `configs` block (comma list, or `none`)")
    ap.add_argument("--profile-once", choices=["chosen", "plain", "no_model", "build"], default=None,
                    help="set up (train, autotune), then run one query of that form between "
                         "cudaProfilerStart/Stop and exit (for ncu --profile-from-start off); "
                         "`build`: the index construction (after one untimed warm-up build)")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def profile_summary(kernel: str, workload: str) -> dict:
    """Figures of the committed ncu summary of `kernel` on `workload` (profiles/ncu_<kernel>_<workload>.txt):
    lines `name: value` for dram_bytes_per_launch, l2_gbs and lanes_active."""
    path = os.path.join(ROOT, "profiles", f"ncu_{kernel}_{workload}.txt")
    out = {}
    if not os.path.exists(path):
        return out
    for line in open(path):
        for name in ("dram_bytes_per_launch", "l2_gbs", "lanes_active"):
            if line.startswith(name + ":"):
                try:
                    out[name] = float(line.split(":", 1)[1].split()[0])
                except (ValueError, IndexError):
                    pass
    return out


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(mhz)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(mhz)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        # NCCL between GPUs; gloo where there is none (the reference arm and the rank helpers
        # need no device).
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def dist_teardown(world):
    if world > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(args):
    if args.workload == "range":
        return W.range_limited(args.scale, args.dims, args.structure)
    return W.CONFIGS[args.workload](args.scale)


def tree_kind_label(w):
    return {"bf": f"BruteForceGpu<{w.dims}>", "kd": f"KdTreeGpu<{w.dims}>", "ball": f"BallTreeGpu<{w.dims}>"}[w.structure]


def algorithmic_bytes(w, counters, count):
    """Bytes per launch by the per-query figure: nodes x node size + leaf slots x slot size +
    query + result row.  k-d node = 4 B split; ball visit = two child balls; slot = 4(D+1) B."""
    d = w.dims
    slot = 4 * (d + 1)
    if w.structure == "kd":
        node_b = 4
    elif w.structure == "ball":
        node_b = 2 * 4 * (d + 1)
    else:
        node_b = 0
    per_result = 8 * w.k
    if w.structure == "bf":
        return count * (4 * d + per_result) + w.points.shape[0] * 4 * d, 0
    total = counters.nodes_visited * node_b + counters.points_scanned * slot + count * (4 * d + per_result)
    floor = count * (4 * d + per_result) + w.points.shape[0] * slot
    return total, floor


def fp64_error(w, rows, idx, dist):
    """Largest error of the returned FP32 squared distances against the same pairs summed in
    FP64 on the host: absolute, relative, and the bound (D + 4) 2^-23 relative."""
    valid = idx >= 0
    if not valid.any():
        return None
    q = np.repeat(w.queries[rows].astype(np.float64), idx.shape[1], axis=0)[valid.ravel()]
    p = w.points[idx[valid]].astype(np.float64)
    exact = ((q - p) ** 2).sum(axis=1)
    got = dist[valid].astype(np.float64)
    err = np.abs(got - exact)
    rel = err[exact > 0] / exact[exact > 0]
    return {"max_abs": float(err.max()), "max_rel": float(rel.max()) if rel.size else 0.0,
            "bound_rel": (w.dims + 4) * 2.0 ** -23, "pairs": int(valid.sum())}


def cpu_baseline(w, threads, sample=None):
    import oracle
    qs = w.queries if sample is None else w.queries[:sample]
    t0 = time.perf_counter()
    if w.structure == "kd":
        tree = oracle.kd_tree(w.points, w.depth_skips)
    elif w.structure == "ball":
        tree = oracle.ball_tree(w.points, w.depth_skips)
    else:
        tree = None
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    if tree is None:
        oracle.bf_knn(w.points, qs, w.k, w.max_dist2, heap=w.heap, fma=True, threads=threads)
    else:
        tree.knn(qs, w.k, w.max_dist2, heap=w.heap, fma=True, strict=False, threads=threads)
    dt = time.perf_counter() - t0
    return len(qs) / dt, build_s, len(qs)


PLAIN_KW = {"kd": dict(block_size=32, shmem_stack=True),
            "ball": dict(block_size=16, heap=True, shmem_tracking=True, shmem_stack=True),
            "bf": dict(block_size=32)}


def run_reference_c5(args):
    """The reference's CPU trees on every set of the uneven batch (a sample of each set's queries)."""
    import oracle
    threads = os.cpu_count() or 1
    sets = W.c5_sets(args.scale)
    trees = [(oracle.kd_tree(w.points, w.depth_skips) if w.structure == "kd" else
              oracle.ball_tree(w.points, w.depth_skips), w) for w in sets]
    per_set = 256

    def step():
        for tree, w in trees:
            tree.knn(w.queries[:per_set], w.k, w.max_dist2, fma=True, strict=False, threads=threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    nq = sum(min(per_set, len(w.queries)) for w in sets)
    qps = nq * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1000 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "c5_uneven_batch_64_sets", "structure": "KdTree<3|8> / BallTree<32> (CPU)",
                   "queries_per_step": nq},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"first {per_set} queries of each of the {len(sets)} sets per step, oracle "
                                   f"port of src/KdTree.cuh and src/BallTree.cuh, {threads} host threads"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args, world, rank):
    if rank != 0:
        return
    if args.workload == "c5":
        run_reference_c5(args)
        return
    w = workload(args)
    threads = os.cpu_count() or 1
    import oracle
    kind = "port"
    sample = {"c1": None, "c2": 262144, "c3": 4096, "c4": 64, "range": None}[args.workload]
    label = {"kd": "KdTree", "ball": "BallTree", "bf": "BruteForce"}[w.structure]
    if w.structure == "kd":
        tree = oracle.kd_tree(w.points, w.depth_skips)
    elif w.structure == "ball":
        tree = oracle.ball_tree(w.points, w.depth_skips)
    else:
        tree = None
    qs = w.queries if sample is None else w.queries[:sample]

    def step():
        if tree is None:
            oracle.bf_knn(w.points, qs, w.k, w.max_dist2, heap=w.heap, fma=True, threads=threads)
        else:
            tree.knn(qs, w.k, w.max_dist2, heap=w.heap, fma=True, strict=False, threads=threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    qps = len(qs) * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1000 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w.name, "structure": f"{label}<{w.dims}> (CPU)", "k": w.k,
                   "depth_skips": w.depth_skips, "queries_per_step": len(qs)},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": kind,
                         "sample": f"{len(qs)} of {len(w.queries)} queries per step, "
                                   f"oracle port of src/{label}.cuh, {threads} host threads"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def step_stats(ms):
    """Median, spread and mean of per-step times (ms)."""
    a = np.asarray(ms, dtype=np.float64)
    return {"median_ms": float(np.median(a)), "min_ms": float(a.min()), "max_ms": float(a.max()),
            "mean_ms": float(a.mean()), "steps": int(a.size)}


class Device:
    """The GPU of this rank, its torch stream and the L2 flush buffer."""

    def __init__(self, local):
        import torch
        from cudaexactknn_gb300 import _lib
        torch.cuda.set_device(local)
        self.local = local
        self.dev = torch.device("cuda", local)
        self.lib = _lib.load()
        self.stream = torch.cuda.current_stream(self.dev)
        self.flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=self.dev)

    def release(self):
        import torch
        torch.cuda.synchronize(self.dev)
        torch.cuda.empty_cache()


# Rows checked against the oracle's brute force (outside timing) and the CPU-baseline sample
# (queries) per workload: sized so that the oracle finishes in seconds on the host cores.
EXACT_ROWS = {"c1": 4096, "c2": 2048, "c3": 1024, "c4": 256, "range": 2048}
CPU_SAMPLE = {"c1": None, "c2": None, "c3": 16384, "c4": 256, "range": None}


def measure(D, w, key, steps, warmup, plain_steps, world, rank, cpu=True):
    """One workload on a prebuilt index: chosen form (autotune, learned radius where the workload
    has a training sample), the same without the radius model, the plain form, end to end through
    knn_query_host, exactness against the oracle, roofline and CPU baseline.  Returns the result
    dict (times are medians over the timed steps)."""
    import ctypes
    import torch
    from cudaexactknn_gb300 import _lib, knn
    import oracle

    dev, lib, stream, flush = D.dev, D.lib, D.stream, D.flush
    pts = torch.from_numpy(w.points).to(dev)
    qs = torch.from_numpy(w.queries).to(dev)
    count, k = len(w.queries), w.k
    index = knn.build_index(w.structure, pts, w.depth_skips)
    build_ms = index.info().build_ms
    out_i = torch.empty((count, k), dtype=torch.int32, device=dev)
    out_d = torch.empty((count, k), dtype=torch.float32, device=dev)
    query = knn.Query(qs, count, w.max_dist2, out_i, out_d)

    # Plain form: the reference benchmarks' template choices (kd <K,32,false,false,true>,
    # ball <K,16,true,true,true>, brute force <K,32,false,false>; tests/Dim3SpeedTests.cu:38,43,
    # tests/DimXSpeedTests.cu:52), no autotune, no learned radius.
    plain_kw = PLAIN_KW[w.structure]
    train = w.extra.get("train")
    report = None
    if train is not None:
        report = index.train_radius_model(torch.from_numpy(train).to(dev), k)
        chosen_kw = dict(flags=_lib.QF_AUTOTUNE | _lib.QF_LEARNED_RADIUS)
    else:
        chosen_kw = dict(flags=_lib.QF_AUTOTUNE)
    learned = bool(chosen_kw["flags"] & _lib.QF_LEARNED_RADIUS)

    def timed(kw, n_steps, n_warm):
        for _ in range(n_warm):
            index.batch_knn(query, k, sync=False, **kw)
        torch.cuda.synchronize(dev)
        barrier(world)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_steps)]
        kern_ms = []
        launches0 = lib.knn_launch_count()
        timed_kw = dict(kw)
        timed_kw["flags"] = timed_kw.get("flags", 0) | _lib.QF_TIMING
        for s in range(n_steps):
            flush.zero_()
            ev[s][0].record(stream)
            index.batch_knn(query, k, sync=False, **timed_kw)
            ev[s][1].record(stream)
            tot, ker = ctypes.c_float(), ctypes.c_float()
            _lib.check(lib.knn_last_query_timing(index.handle, ctypes.byref(tot), ctypes.byref(ker)))
            kern_ms.append(ker.value)
        torch.cuda.synchronize(dev)
        launches = lib.knn_launch_count() - launches0
        barrier(world)
        step_ms = [max_over_ranks(world, a.elapsed_time(b)) for a, b in ev]
        return step_ms, kern_ms, launches

    # Exactness of every form on a sample, checked against the CPU oracle (outside timing).
    sample = np.sort(np.random.default_rng(0).choice(count, size=min(count, EXACT_ROWS.get(key, 1024)),
                                                     replace=False))
    want = oracle.row_keys(*oracle.bf_knn(w.points, w.queries[sample], k, w.max_dist2, fma=True,
                                          threads=os.cpu_count() or 1))
    forms = [("plain", plain_kw), ("chosen", chosen_kw)]
    if learned:
        forms.append(("no_model", dict(flags=_lib.QF_AUTOTUNE)))
    exact = {}
    for name, kw in forms:
        index.batch_knn(query, k, **kw)
        got = oracle.row_keys(out_i[sample].cpu().numpy(), out_d[sample].cpu().numpy())
        exact[name] = float((got == want).all(axis=1).mean())
    index.batch_knn(query, k, **chosen_kw)
    fp64 = fp64_error(w, sample, out_i[sample].cpu().numpy(), out_d[sample].cpu().numpy())

    counters = index.stats(query, k, **plain_kw)
    alg_bytes, floor_bytes = algorithmic_bytes(w, counters, count)
    chosen_counters = index.stats(query, k, **chosen_kw)

    def plan_of(learned_flag):
        tuned = _lib.QueryOpts()
        tuned_ms = ctypes.c_float()
        _lib.check(lib.knn_tuned_plan(index.handle, k, int(learned_flag), ctypes.byref(tuned), ctypes.byref(tuned_ms)))
        return dict(bf16_filter=bool(tuned.flags & _lib.QF_BF16_FILTER), block_size=tuned.block_size,
                    heap=bool(tuned.heap_tracking), shmem_tracking=bool(tuned.shmem_tracking),
                    shmem_stack=bool(tuned.shmem_stack), leaf_scan=tuned.leaf_scan,
                    traversal={0: "thread", 1: "warp", 2: "group", 3: "box"}.get(tuned.traversal, str(tuned.traversal)),
                    candidates_timed=tuned.reserved)

    tuned_plan = plan_of(learned)
    with ClockSampler(D.local) as clocks:
        chosen_ms, chosen_kern, launches = timed(chosen_kw, steps, warmup)
    plain_ms, plain_kern, _ = timed(plain_kw, plain_steps, 1)
    chosen_st, plain_st = step_stats(chosen_ms), step_stats(plain_ms)
    value = world * count / (chosen_st["median_ms"] / 1e3)
    plain_qps = world * count / (plain_st["median_ms"] / 1e3)

    no_model = None
    if learned:
        nm_kw = dict(flags=_lib.QF_AUTOTUNE)
        nm_ms, nm_kern, _ = timed(nm_kw, steps, warmup)
        nm_counters = index.stats(query, k, **nm_kw)
        nm_st = step_stats(nm_ms)
        nm_value = world * count / (nm_st["median_ms"] / 1e3)
        no_model = {"form": "autotune without the radius model", "value": nm_value, "ms_per_step": nm_st["median_ms"],
                    "step_ms": nm_st, "kernel_ms": float(np.median(nm_kern)), "plan": plan_of(False),
                    "exact_match": exact["no_model"],
                    "visits": {"nodes": int(nm_counters.nodes_visited), "leaves": int(nm_counters.leaves_visited),
                               "points": int(nm_counters.points_scanned)},
                    "learned_radius_gain": value / nm_value}

    # End to end through the C ABI with pinned host buffers.
    h_q = torch.from_numpy(w.queries).pin_memory()
    h_i = torch.empty((count, k), dtype=torch.int32).pin_memory()
    h_d = torch.empty((count, k), dtype=torch.float32).pin_memory()
    for _ in range(warmup):
        index.knn_host(h_q, k, w.max_dist2, h_i, h_d, **chosen_kw)
    torch.cuda.synchronize(dev)
    barrier(world)
    e2e_ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        index.knn_host(h_q, k, w.max_dist2, h_i, h_d, **chosen_kw)
        e2e_ms.append(max_over_ranks(world, (time.perf_counter() - t0) * 1e3))
    e2e_st = step_stats(e2e_ms)
    e2e_exact = float((oracle.row_keys(h_i.numpy()[sample], h_d.numpy()[sample]) == want).all(axis=1).mean())

    kernel_ms = float(np.median(chosen_kern))
    kernel_name = {"kd": "kd_knn_kernel", "ball": "ball_knn_kernel", "bf": "bf_knn_kernel"}[w.structure]
    if tuned_plan["traversal"] == "group":
        kernel_name = "kd_group_kernel"
    elif tuned_plan["traversal"] == "box":
        kernel_name = "kd_box_knn_kernel"
    if tuned_plan["bf16_filter"]:
        # Tensor-core filter: the MMA work it issues, 2 x 128 queries x 256 rows x (16 per K step,
        # ceil(D/16) steps) per point tile scanned (device counter), against the dense 16-bit peak.
        kernel_name = "tc_filter_kernel"
        peak, peak_kind = bf16_peak()
        mma_tiles = int(chosen_counters.leaves_visited)
        flops = 2.0 * 128 * 256 * 16 * math.ceil(w.dims / 16) * mma_tiles
        achieved = flops / (kernel_ms / 1e3) / 1e12
        roof_bound, roof_unit = "tensor", "TFLOP/s"
    else:
        peak, peak_kind = peaks()
        achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
        roof_bound, roof_unit = "hbm", "GB/s"
    prof = profile_summary(kernel_name, key)
    roofline = {"bound": roof_bound, "achieved": achieved, "peak": peak, "unit": roof_unit, "frac": achieved / peak,
                "traffic": prof.get("dram_bytes_per_launch"),
                "peak_source": f"{peak_kind} " + ("bf16_tflops" if roof_bound == "tensor" else "hbm_gbs"),
                "kernel": kernel_name, "kernel_ms": kernel_ms,
                "kernel_span": "sum of the CUDA-event spans of every search kernel of the pass "
                               "(seeded search and retries)",
                "algorithmic_bytes_per_launch": int(alg_bytes), "compulsory_bytes_per_launch": int(floor_bytes),
                "l2_gbs": prof.get("l2_gbs"), "lanes_active": prof.get("lanes_active"),
                "mma_tiles_scanned": int(chosen_counters.leaves_visited) if tuned_plan["bf16_filter"] else None,
                "visits": {"nodes": int(counters.nodes_visited), "leaves": int(counters.leaves_visited),
                           "points": int(counters.points_scanned)}}

    res = {
        "value": value, "unit": "queries/s", "ms_per_step": chosen_st["median_ms"], "step_ms": chosen_st,
        "config": {"workload": w.name, "structure": tree_kind_label(w), "n": int(w.points.shape[0]),
                   "queries": count, "k": k, "depth_skips": w.depth_skips,
                   "max_distance2": "inf" if math.isinf(w.max_dist2) else w.max_dist2,
                   "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas x{world}"},
        "exact_match": {**exact, "e2e": e2e_exact, "sample_queries": int(len(sample))},
        "distance_error_vs_fp64": fp64,
        "plain": {"value": plain_qps, "ms_per_step": plain_st["median_ms"], "step_ms": plain_st, "plan": plain_kw,
                  "kernel_ms": float(np.median(plain_kern))},
        "chosen": {"form": "autotune + learned radius" if learned else "autotune", "plan": tuned_plan,
                   "kernel_ms": kernel_ms, "fallback_queries": int(chosen_counters.fallback_queries),
                   "visits": {"nodes": int(chosen_counters.nodes_visited),
                              "leaves": int(chosen_counters.leaves_visited),
                              "points": int(chosen_counters.points_scanned)},
                   "radius_model": None if report is None else {
                       "train_ms": report.train_ms, "samples": report.samples, "steps": report.steps,
                       "rmse_log_kth": report.rmse, "margin": report.margin, "coverage": report.coverage}},
        "speedup_vs_plain": value / plain_qps,
        "no_model": no_model,
        "build_ms": build_ms,
        "e2e": {"value": world * count / (e2e_st["median_ms"] / 1e3), "unit": "queries/s", "step_ms": e2e_st,
                "h2d_bytes_per_step": int(w.queries.nbytes), "d2h_bytes_per_step": int(count * k * 8)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clocks.summary(),
    }
    index.close()
    del pts, qs, out_i, out_d, query, h_q, h_i, h_d
    D.release()
    if cpu and rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        qps, build_s, nq = cpu_baseline(w, threads, CPU_SAMPLE.get(key))
        res["cpu_baseline"] = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"{nq} of {count} queries, oracle port of the reference's CPU "
                                         f"{w.structure} algorithm, {threads} threads (tree build {build_s:.1f} s, untimed)"}
    return res


def measure_c5(D, scale, steps, warmup, plain_steps, world, rank, cpu=True):
    """Uneven batch: 64 independent sets in one CUDA-graph launch against one plain batchKnn per
    set (each ending in a device synchronisation, as the reference's does), both over every
    query of every set.  The plain form takes ~35 s per step (its 32-dimensional ball trees visit
    most of their nodes), so it is timed over `plain_steps` steps after a warm-up on 64 queries
    per set."""
    import torch
    from cudaexactknn_gb300 import knn
    import oracle

    dev, lib, stream, flush = D.dev, D.lib, D.stream, D.flush
    sets = W.c5_sets(scale)
    built = []
    build_ms = 0.0
    for w in sets:
        ix = knn.build_index(w.structure, torch.from_numpy(w.points).to(dev), w.depth_skips)
        build_ms += ix.info().build_ms
        q = torch.from_numpy(w.queries).to(dev)
        few = min(64, len(w.queries))
        built.append((w, ix, knn.Query(q, len(w.queries), w.max_dist2), knn.Query(q[:few], few, w.max_dist2)))
    total_q = sum(len(w.queries) for w in sets)

    def plain_step():
        for w, ix, q, _ in built:
            ix.batch_knn(q, w.k, **PLAIN_KW[w.structure])

    def plain_warm():
        for w, ix, _, fq in built:
            ix.batch_knn(fq, w.k, **PLAIN_KW[w.structure])

    batch = knn.Batch([(ix, q.points, w.k, w.max_dist2) for w, ix, q, _ in built], autotune=True)
    classes, kernels_per_run = batch.info()

    def timed(fn, n_steps, n_warm):
        for _ in range(n_warm):
            fn()
        torch.cuda.synchronize(dev)
        barrier(world)
        out = []
        for _ in range(n_steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            out.append(max_over_ranks(world, a.elapsed_time(b)))
        barrier(world)
        return out

    launches0 = lib.knn_launch_count()
    with ClockSampler(D.local) as clocks:
        chosen_ms = timed(lambda: batch.run(sync=False), steps, warmup)
    graph_launches = lib.knn_launch_count() - launches0
    plain_warm()
    plain_ms = timed(plain_step, plain_steps, 0)
    chosen_st, plain_st = step_stats(chosen_ms), step_stats(plain_ms)
    value = world * total_q / (chosen_st["median_ms"] / 1e3)
    plain_qps = world * total_q / (plain_st["median_ms"] / 1e3)

    # Exactness: a sample of every set's rows from the batch and from the plain form against the
    # oracle's brute force.
    rows_ok = rows = plain_ok = 0
    res = batch.run()
    rng = np.random.default_rng(0)
    for (w, ix, q, _), (oi, od) in zip(built, res):
        pick = np.sort(rng.choice(q.count, size=min(64, q.count), replace=False))
        want = oracle.row_keys(*oracle.bf_knn(w.points, w.queries[pick], w.k, w.max_dist2, fma=True,
                                              threads=os.cpu_count() or 1))
        got = oracle.row_keys(oi[pick].cpu().numpy(), od[pick].cpu().numpy())
        rows_ok += int((got == want).all(axis=1).sum())
        # The plain form on the picked rows alone (its answer for a query does not depend on the batch).
        pq = knn.Query(torch.from_numpy(np.ascontiguousarray(w.queries[pick])).to(dev), len(pick), w.max_dist2)
        pi, pd = ix.batch_knn(pq, w.k, **PLAIN_KW[w.structure])
        plain_ok += int((oracle.row_keys(pi.cpu().numpy(), pd.cpu().numpy()) == want).all(axis=1).sum())
        rows += len(pick)

    # End to end: pinned host queries in, the graph launch, every result out.
    h_q = [torch.from_numpy(w.queries).pin_memory() for w, _, _, _ in built]
    h_out = [(torch.empty(oi.shape, dtype=torch.int32).pin_memory(), torch.empty(od.shape).pin_memory())
             for oi, od in res]

    def e2e_step():
        for (w, ix, q, _), hq in zip(built, h_q):
            q.points.copy_(hq, non_blocking=True)
        batch.run(sync=False)
        for (oi, od), (hi, hd) in zip(res, h_out):
            hi.copy_(oi, non_blocking=True)
            hd.copy_(od, non_blocking=True)
        torch.cuda.synchronize(dev)

    for _ in range(warmup):
        e2e_step()
    e2e_ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append(max_over_ranks(world, (time.perf_counter() - t0) * 1e3))
    e2e_st = step_stats(e2e_ms)

    # Roofline: bytes the batch must move (every set's points, queries and result rows once)
    # over the batch time -- the compulsory traffic, HBM bound.
    compulsory = sum(w.points.nbytes + w.queries.nbytes + len(w.queries) * w.k * 8 for w in sets)
    peak, peak_kind = peaks()
    achieved = compulsory / (chosen_st["median_ms"] / 1e3) / 1e9
    out = {
        "value": value, "unit": "queries/s", "ms_per_step": chosen_st["median_ms"], "step_ms": chosen_st,
        "config": {"workload": "c5_uneven_batch_64_sets", "sets": len(sets), "queries": total_q,
                   "points": int(sum(len(w.points) for w in sets)), "classes": classes,
                   "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas x{world}"},
        "exact_match": {"chosen": rows_ok / rows, "plain": plain_ok / rows, "sample_queries": rows},
        "plain": {"value": plain_qps, "ms_per_step": plain_st["median_ms"], "step_ms": plain_st,
                  "queries_per_step": total_q,
                  "form": "one batchKnn per set with the reference benchmarks' template choices, every query; "
                          f"{plain_steps} timed steps after a warm-up on 64 queries per set"},
        "chosen": {"form": "one CUDA-graph launch: a persistent kernel per (tree, dims, k) class, or the "
                           "tensor-core filter for classes of dims >= 16 where it times faster; autotuned",
                   "kernels_per_run": kernels_per_run},
        "speedup_vs_plain": value / plain_qps,
        "build_ms": build_ms,
        "e2e": {"value": world * total_q / (e2e_st["median_ms"] / 1e3), "unit": "queries/s", "step_ms": e2e_st,
                "h2d_bytes_per_step": int(sum(w.queries.nbytes for w in sets)),
                "d2h_bytes_per_step": int(sum(len(w.queries) * w.k * 8 for w in sets))},
        "gpu_launches": int(kernels_per_run * steps),
        "graph_launches": int(graph_launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": f"{peak_kind} hbm_gbs", "kernel": "kd/ball_batch_kernel",
                     "algorithmic_bytes_per_launch": int(compulsory)},
        "clocks": clocks.summary(),
    }
    batch.close()
    for _, ix, _, _ in built:
        ix.close()
    del built, res, h_q, h_out
    D.release()
    if cpu and rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        per_set = 256
        trees = [(oracle.kd_tree(w.points, w.depth_skips) if w.structure == "kd" else
                  oracle.ball_tree(w.points, w.depth_skips), w) for w in sets]
        t0 = time.perf_counter()
        for tree, w in trees:
            tree.knn(w.queries[:per_set], w.k, w.max_dist2, fma=True, strict=False, threads=threads)
        dt = time.perf_counter() - t0
        nq = sum(min(per_set, len(w.queries)) for w in sets)
        out["cpu_baseline"] = {"value": nq / dt, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"first {per_set} queries of each of the {len(sets)} sets, oracle port of "
                                         f"src/KdTree.cuh and src/BallTree.cuh, {threads} threads (builds untimed)"}
    return out


HEADER_KEYS = {"metric": METRIC, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded, shapes of the config)"}


def main():
    args = parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    D = Device(local)
    cpu = not args.no_cpu_baseline
    if args.profile_once:
        profile_once(D, args)
        return
    if args.workload == "c5":
        res = measure_c5(D, args.scale, args.steps, args.warmup, 1, world, rank, cpu)
    else:
        res = measure(D, workload(args), args.workload, args.steps, args.warmup,
                      max(5, min(args.steps, 20)), world, rank, cpu)
    line = {"metric": METRIC, "value": res.pop("value"), "unit": res.pop("unit"), "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, **HEADER_KEYS, **res}
    line["n_gpus"] = world
    # The other configurations, each on the same GPU after the headline one, with fewer timed
    # steps (median of at least five).
    names = [] if args.configs == "none" or args.workload != "c2" else args.configs.split(",")
    if names:
        block = {}
        sec_steps, sec_warm = max(5, min(args.steps, 10)), max(3, min(args.warmup, 3))
        for name in names:
            t0 = time.perf_counter()
            if name == "c5":
                sub = measure_c5(D, args.scale, sec_steps, sec_warm, 1, world, rank, cpu)
            else:
                sub = measure(D, W.CONFIGS[name](args.scale), name, sec_steps, sec_warm, 5, world, rank, cpu)
            sub["wall_s"] = time.perf_counter() - t0
            block[name] = sub
        line["configs"] = block
    if rank == 0:
        print(json.dumps(line), flush=True)


def profile_once(D, args):
    """Set up (train, autotune), then run one query of the requested form between
    cudaProfilerStart/Stop (for ncu --profile-from-start off)."""
    import torch
    from cudaexactknn_gb300 import _lib, knn
    w = workload(args)
    pts = torch.from_numpy(w.points).to(D.dev)
    qs = torch.from_numpy(w.queries).to(D.dev)
    if args.profile_once == "build":
        knn.build_index(w.structure, pts, w.depth_skips).close()  # warm-up (module load, pools)
        torch.cuda.synchronize(D.dev)
        torch.cuda.profiler.start()
        index = knn.build_index(w.structure, pts, w.depth_skips)
        torch.cuda.synchronize(D.dev)
        torch.cuda.profiler.stop()
        index.close()
        return
    index = knn.build_index(w.structure, pts, w.depth_skips)
    query = knn.Query(qs, len(w.queries), w.max_dist2)
    if args.profile_once == "plain":
        kw = PLAIN_KW[w.structure]
    elif w.extra.get("train") is not None and args.profile_once == "chosen":
        index.train_radius_model(torch.from_numpy(w.extra["train"]).to(D.dev), w.k)
        kw = dict(flags=_lib.QF_AUTOTUNE | _lib.QF_LEARNED_RADIUS)
    else:
        kw = dict(flags=_lib.QF_AUTOTUNE)
    index.batch_knn(query, w.k, **kw)  # autotunes on the first call
    torch.cuda.synchronize(D.dev)
    torch.cuda.profiler.start()
    index.batch_knn(query, w.k, **kw)
    torch.cuda.synchronize(D.dev)
    torch.cuda.profiler.stop()
    index.close()


if __name__ == "__main__":
    try:
        main()
    finally:
        dist_teardown(int(os.environ.get("WORLD_SIZE", "1")))
