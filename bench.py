"""Benchmark: multi-pass gather / scatter and STREAM on one GB300.

Workload (one "step"): on n = 2^28 int32 payloads in[i] = i and a
Fisher-Yates permutation loc (seed 2), gather and scatter at pass counts
1, 2, 4, 8, 16; then STREAM copy, scale, add, triad on 2^28 float32 arrays
a[i] = i, b[i] = i + 10 with scalar 3.0.  Every array is 1 GiB, larger than
L2, so no L2 flush is needed between steps.

Metric: effective GB/s = algorithmic bytes / time (decimal GB).  Algorithmic
bytes: gather / scatter 12 B per element per call (read index, read
payload, write payload), independent of the pass count; copy / scale 8 B,
add / triad 12 B per element.

Schedule: gather / scatter run the shared-memory-window form by default
(--method tiled; "partition" = L2 windows, "sweep" = the reference's pass-by-
pass schedule); results are identical for every pass count and schedule.
The tiled form does not use the pass count: its windows are fixed by the
shared-memory size, so the five gather (and five scatter) calls of a step run
the same kernels on the same arrays five times; the p1..p16 entries are not
five schedules.  The reference's pass-by-pass schedule is timed per pass
count under `compare.sweep`.

value     device-timed, inputs resident in HBM (CUDA events, max over ranks)
e2e       same metric through the C ABI with host buffers: every step copies
          its inputs from pinned host memory and every output back, the
          copies on two copy streams overlapping the calls
roofline  the dominant call of the step against the measured HBM copy rate
cpu_baseline  the reference's CPU path (OpenMP ports, oracle/) on the host
          cores, on a bounded sample; rank 0 at N=1 only

The same line also carries the other configurations as keys (skipped with
--no-extras): config1_scan (2^24 int32 exclusive scan, warm and L2-flushed),
config4_scan (2^30 int32 / int64 / f32 scans under the three schemes, with the
f32 error against an f64 accumulation), config3_split (2^28 key/value stable
split, 2..1024 buckets, uniform and Zipf keys), config5_batch (4096 uneven
segments batched vs one plain call per segment, and the persistent work-queue
form) and config5_serve (Poisson request stream, p50 / p99 latency).  Each has
its own GB/s, fraction of HBM and, where the reference has a CPU path, its
cpu_baseline.

--impl reference runs the reference's CPU implementation of the same step at
the same size (OpenMP ports of openmp/test_gather_scatter_CPU.cpp and
openmp/test_bandwidth_CPU.cpp; add/triad restated) on all host threads; it
loads only the oracle, never this library.

Multi-GPU: the primitives do not shard (replicas only); under torchrun each
rank runs the full step on its own GPU, value = all ranks' bytes / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "efficient-dpp_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

PASSES = (1, 2, 4, 8, 16)
STREAM_OPS = ("copy", "scale", "add", "triad")
STREAM_BYTES = {"copy": 8, "scale": 8, "add": 12, "triad": 12}
GS_BYTES = 12
METRIC = "effective GB/s (% of HBM roofline) per primitive; batched vs plain elems/s; p99"


def step_calls():
    calls = []
    for p in PASSES:
        calls.append(("gather", p))
        calls.append(("scatter", p))
    for op in STREAM_OPS:
        calls.append((op, 0))
    return calls


def call_bytes(name, n):
    return n * (GS_BYTES if name in ("gather", "scatter") else STREAM_BYTES[name])


def call_launches(name, p, method="tiled"):
    """Kernels of this library one call launches."""
    if name not in ("gather", "scatter"):
        return 1
    if method == "tiled":  # count, scan, partition, refine, (fetch, refine,) apply
        return 7 if name == "gather" else 5
    if method == "sweep" or p == 1:
        return p
    return 5 if name == "gather" else 4  # count, bases, partition, (fetch,) apply


def step_config(n, world):
    """The `config` of the gather/scatter + STREAM step, the same object in
    both arms (this library and --impl reference)."""
    workload = ("multipass gather/scatter (2^28 int32, Fisher-Yates seed 2, passes 1,2,4,8,16) "
                "+ STREAM copy/scale/add/triad (2^28 f32, scalar 3.0)" if n == 1 << 28 else
                f"multipass gather/scatter (n={n} int32, Fisher-Yates seed 2, passes 1,2,4,8,16) "
                f"+ STREAM copy/scale/add/triad (n={n} f32, scalar 3.0)")
    return {"workload": workload, "n": n, "passes": list(PASSES),
            "parallelism": f"replicas{world}",
            "l2": "inputs (1 GiB each at 2^28) larger than L2; no flush"}


def measured_peak_gbs():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# distributed helpers (replicas only)
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        # let the sampler start before the timed region opens (its first
        # sample), so that every sample falls inside the timed region's span
        t0 = time.time()
        while time.time() - t0 < 3.0 and self.proc.poll() is None:
            self.file.flush()
            if os.path.getsize(self.file.name) > 0:
                break
            time.sleep(0.02)
        self.skip = sum(1 for _ in open(self.file.name))
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines()[getattr(self, "skip", 0):]:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v == "Active"})
        loaded = [r for r in rows if r[2] > 200.0] or rows
        return {"sm_mhz": statistics.median(r[0] for r in loaded),
                "sm_max_mhz": max(r[1] for r in rows), "power_w_max": max(r[2] for r in rows),
                "samples": len(rows), "reasons": reasons}


# ---------------------------------------------------------------------------
def cpu_baseline(n_sample: int, reps: int = 5):
    """The reference's CPU path (OpenMP ports in oracle/) on a bounded
    sample; returns the same metric (GB/s) and a description."""
    import numpy as np

    from oracle import oracle as orc
    threads = orc.max_threads()
    loc = orc.gen_permutation(n_sample, 2)
    inp = np.arange(n_sample, dtype=np.int32)
    a = np.arange(n_sample, dtype=np.float32)
    b = a + 10
    out = np.zeros(n_sample, np.int32)
    fout = np.zeros(n_sample, np.float32)
    t = {}
    times = [orc.gather_omp(inp, loc, threads, out)[1] for _ in range(reps)]
    t["gather"] = orc.average_hampel(times)
    times = [orc.scatter_omp(inp, loc, threads, out)[1] for _ in range(reps)]
    t["scatter"] = orc.average_hampel(times)
    for op in STREAM_OPS:
        times = [orc.stream(op, a, b, 3.0, threads, fout)[1] for _ in range(reps)]
        t[op] = orc.average_hampel(times)
    step_ms = sum(t[name] for name, _ in step_calls())  # no passes on the CPU
    step_bytes = sum(call_bytes(name, n_sample) for name, _ in step_calls())
    return {
        "value": step_bytes / (step_ms * 1e-3) / 1e9, "unit": "GB/s", "cores": threads,
        "kind": "port",
        "sample": f"n=2^{n_sample.bit_length() - 1}: OpenMP gather+scatter (single pass, as "
                  f"openmp/test_gather_scatter_CPU.cpp) once per pass count, copy/scale/add/"
                  f"triad; Hampel mean of {reps} reps per call",
        "ms_per_call": {k: round(v, 3) for k, v in t.items()},
    }


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU implementation of the step, at
    the GPU arm's size (2^28 by default) on all host threads.  It loads only
    the oracle (OpenMP ports of the reference's CPU functions and the seeded
    permutation generator), never this library."""
    if rank != 0:
        return 0
    import numpy as np

    from oracle import oracle as orc
    n = args.ref_n or (1 << args.log2n)
    threads = orc.max_threads()
    loc = orc.gen_permutation(n, 2)
    inp = np.arange(n, dtype=np.int32)
    a = np.arange(n, dtype=np.float32)
    b = a + 10
    out = np.zeros(n, np.int32)
    fout = np.zeros(n, np.float32)

    def step():
        for name, _p in step_calls():
            if name == "gather":
                orc.gather_omp(inp, loc, threads, out)
            elif name == "scatter":
                orc.scatter_omp(inp, loc, threads, out)
            else:
                orc.stream(name, a, b, 3.0, threads, fout)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    step_bytes = sum(call_bytes(name, n) for name, _ in step_calls())
    ms = dt / args.steps * 1e3
    value = step_bytes / (ms * 1e-3) / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic",
        "config": step_config(n, world),
        "reference_note": "the reference's CPU path on the same arrays and sizes as the GPU arm",
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                         "kind": "port",
                         "sample": f"the whole step at n=2^{n.bit_length() - 1} (OpenMP ports of "
                                   f"openmp/test_gather_scatter_CPU.cpp:24-41 and "
                                   f"test_bandwidth_CPU.cpp:39-56; add/triad restated"
                                   + ("; the reference's AVX2 sources do not build on this Arm "
                                      "host)" if platform.machine() in ("aarch64", "arm64")
                                      else ")")},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _device(args):
    import torch
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    return dev


def measure_batch(args, dev, world, steps, warmup, autotune=False):
    """Config 5: 4096 uneven segments (scan / 64-bucket split / permutation
    gather, total <= 2^30 int32): the batched launches (tuned schedule,
    captured in a CUDA graph) and the persistent work-queue launch against
    one plain C-ABI call per segment.  Returns the figures as a dict."""
    import numpy as np
    import torch

    import edpp
    from edpp import batch as B
    segs = B.config5_segments(cap=1 << args.batch_log2_total)
    in0, in1 = B.gen_inputs(segs, seed=4)
    n = len(in0)
    elems = int(segs["length"].sum())
    nbytes = B.algorithmic_bytes(segs)
    d0 = torch.from_numpy(in0).to(dev)
    d1 = torch.from_numpy(in1).to(dev)
    o0 = torch.zeros(n, dtype=torch.int32, device=dev)
    o1 = torch.zeros(n, dtype=torch.int32, device=dev)
    q0 = torch.zeros_like(o0)
    q1 = torch.zeros_like(o1)
    stream = torch.cuda.current_stream()

    tuning = B.tuned(segs)
    tune_info = None
    if autotune:
        plan0 = B.Plan(segs)
        ws0 = plan0.workspace(dev)
        tuning, tms = B.autotune(segs, d0, d1, o0, o1, ws0, reps=3)
        B.record_tuning(segs, tuning, tms, {"segments": len(segs), "elements": elems})
        tune_info = {"tuning": tuning.as_dict(), "ms": round(tms, 4)}
        del ws0, plan0
    plan = B.Plan(segs, tuning)
    ws = plan.workspace(dev)
    plan.upload(ws)
    pws = B.plain_workspace(segs, dev)

    def timed(fn, reps):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / reps, world)

    plain_ms = timed(lambda: B.run_plain(segs, d0, d1, q0, q1, pws), steps)
    # batched: capture one launch in a CUDA graph, replay it
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(g):
            plan.launch(d0, d1, o0, o1, ws)
    stream.wait_stream(side)
    with ClockSampler(int(dev.index or 0)) as clk:
        batch_ms = timed(g.replay, steps)
    stream_ms = timed(lambda: plan.launch(d0, d1, o0, o1, ws), steps)
    identical = bool(torch.equal(o0, q0) and torch.equal(o1, q1))
    # the persistent work-queue schedule (one launch) on the same segments,
    # at the best of the knobs the batch autotuner searches (blocks per SM,
    # split deferral, segment order), each timed the same way
    queue_ms, queue_tu, queue_identical = None, None, True
    qws = B.Plan(segs, B.Tuning(4, 1, 0, B.SCHEDULE_QUEUE)).workspace(dev)  # same size for all
    for bps in (2, 3, 4):
        for defer in (0, 1, 2, 4):
            for lf in (0, 1):
                tu = B.Tuning(bps, defer, lf, B.SCHEDULE_QUEUE)
                qplan = B.Plan(segs, tu)
                qplan.upload(qws)
                o0.zero_()
                o1.zero_()
                ms = timed(lambda: qplan.launch(d0, d1, o0, o1, qws), max(2, steps // 2))
                queue_identical = queue_identical and bool(torch.equal(o0, q0) and
                                                           torch.equal(o1, q1))
                if queue_ms is None or ms < queue_ms:
                    queue_ms, queue_tu = ms, tu.as_dict()
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the batch workload")
    peak, peak_kind = measured_peak_gbs()
    gbs = nbytes / (batch_ms * 1e-3) / 1e9
    ops = {B.OP_NAMES[k]: int((segs["op"] == k).sum()) for k in (0, 1, 2)}
    kinds = tuning is None or tuning.schedule == B.SCHEDULE_KINDS
    # kernels per batch: KINDS launches one kernel per tile kind present
    # (a split takes three: histogram, per-segment histogram scans, scatter)
    launches = (int(bool(ops["scan"])) + int(bool(ops["gather"])) + 3 * int(bool(ops["split"]))
                if kinds else 1)
    del d0, d1, o0, o1, q0, q1, ws, pws, qws
    torch.cuda.empty_cache()
    return {
        "workload": "4096 segments, log-uniform 2^10..2^24 rescaled to <= 2^30 int32 (seed 4), "
                    "ops scan / 64-bucket split / gather",
        "segments": len(segs), "elements": elems, "ops": ops, "tasks": plan.num_tasks,
        "tuning": tuning.as_dict() if tuning else "default (kinds)",
        "plain": {"ms": round(plain_ms, 4), "elements/s": round(elems / (plain_ms * 1e-3), 1)},
        "batched_graph": {"ms": round(batch_ms, 4), "elements/s": round(elems / (batch_ms * 1e-3), 1),
                          "GB/s": round(gbs, 1), "frac_of_hbm": round(gbs / peak, 4)},
        "batched_stream_launch_ms": round(stream_ms, 4),
        "persistent_queue": {"ms": round(queue_ms, 4), "tuning": queue_tu,
                             "elements/s": round(elems / (queue_ms * 1e-3), 1),
                             "speedup_vs_plain": round(plain_ms / queue_ms, 3),
                             "identical_to_plain": queue_identical},
        "speedup_vs_plain": round(plain_ms / batch_ms, 3),
        "identical_to_plain": identical,
        "autotune": tune_info,
        "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(gbs / peak, 4), "traffic": None,
                     "kernel": "batch kernels (whole batch)", "peak_source": peak_kind},
        "launches_per_batch": launches,
        "clocks": clk.summary(),
        "cpu_baseline": None,
        "cpu_baseline_note": "the batched form is compared with plain per-segment C-ABI calls "
                             "on the same GPU (plain.ms)",
    }


def run_batch_workload(args, rank, world):
    """--workload batch: config 5 alone, as one JSON line."""
    import edpp
    edpp.lib()
    dev = _device(args)
    r = measure_batch(args, dev, world, args.steps, args.warmup, autotune=args.autotune)
    if rank == 0:
        line = {"metric": METRIC,
                "workload_metric": "batched elements/s (one launch per tile kind, graph-captured) "
                                   "vs plain per-segment launches",
                "value": round(world * r["elements"] / (r["batched_graph"]["ms"] * 1e-3), 1),
                "unit": "elements/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["batched_graph"]["ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic",
                "config": {"workload": r["workload"], "segments": r["segments"],
                           "elements": r["elements"], "ops": r["ops"], "tasks": r["tasks"],
                           "tuning": r["tuning"]},
                "gpu_launches": r["launches_per_batch"] * args.steps}
        line.update({k: v for k, v in r.items() if k not in line and k != "workload"})
        print(json.dumps(line), flush=True)
    return 0


def measure_serve(args, dev, rates, requests):
    """Config 5, serving: Poisson arrivals at swept rates of requests with
    log-uniform sizes 4K..64M elements (op scan / 64-bucket split / gather),
    host buffers in pinned memory, admission cap 40 GB of HBM, continuous
    batching; p50 / p99 latency (submit -> outputs in host memory)."""
    import numpy as np

    import edpp
    from edpp import batch as B
    from edpp import serve as S
    npay = args.serve_payloads
    sizes, ops = [], []
    for i in range(npay):
        u = (edpp.lib().edpp_gen_draw(4 ^ 0x5E, i) >> 11) * (1.0 / 9007199254740992.0)
        sizes.append(int(2.0 ** (12 + 14 * u)))
        ops.append(edpp.lib().edpp_gen_draw(4 ^ 0x5F, i) % 3)
    segs = B.layout(sizes, ops, 64)
    in0, in1 = B.gen_inputs(segs, seed=5)
    total = len(in0)
    p_in0, p_in1 = S.pinned_empty(total), S.pinned_empty(total)
    p_o0, p_o1 = S.pinned_empty(total), S.pinned_empty(total)
    p_in0[:] = in0
    p_in1[:] = in1
    pay = [(int(s["op"]), int(s["offset"]), int(s["length"])) for s in segs]
    rng = np.random.default_rng(6)
    results = []
    srv = S.Server(pool_bytes=int(args.pool_gb * 1e9), slots=args.serve_slots)
    # warm-up: every payload once
    ids = [srv.submit(op, p_in0[o:o + L], p_in1[o:o + L], p_o0[o:o + L], p_o1[o:o + L], 64)
           for op, o, L in pay]
    for rid in ids:
        st, _ = srv.wait(rid)
        assert st == 0
    with ClockSampler(int(dev.index or 0)) as clk:
        for rate in rates:
            n = requests
            gaps = rng.exponential(1.0 / rate, size=n)
            arrivals = np.cumsum(gaps)
            inflight = {}
            lat, queue, elems = [], [], 0
            t0 = time.perf_counter()
            for i in range(n):
                k = i % npay
                if k in inflight:  # payload buffers still in use: wait for them
                    st, tm = srv.wait(inflight.pop(k))
                    assert st == 0
                    lat.append(tm.latency_ms)
                    queue.append(tm.queue_ms)
                now = time.perf_counter() - t0
                if arrivals[i] > now:
                    time.sleep(arrivals[i] - now)
                op, o, L = pay[k]
                inflight[k] = srv.submit(op, p_in0[o:o + L], p_in1[o:o + L], p_o0[o:o + L],
                                         p_o1[o:o + L], 64)
                elems += L
            for rid in inflight.values():
                st, tm = srv.wait(rid)
                assert st == 0
                lat.append(tm.latency_ms)
                queue.append(tm.queue_ms)
            wall = time.perf_counter() - t0
            lat = np.array(lat)
            results.append({"rate_req_s": rate, "requests": n,
                            "achieved_req_s": round(n / wall, 1),
                            "elements/s": round(elems / wall, 1),
                            "p50_ms": round(float(np.percentile(lat, 50)), 3),
                            "p99_ms": round(float(np.percentile(lat, 99)), 3),
                            "mean_ms": round(float(lat.mean()), 3),
                            "queue_p99_ms": round(float(np.percentile(queue, 99)), 3)})
    stats = srv.stats()
    srv.close()
    return {"workload": "Poisson arrivals, sizes log-uniform 2^12..2^26 int32, ops scan / "
                        "64-bucket split / gather, pinned host buffers",
            "payloads": npay, "pool_bytes": int(args.pool_gb * 1e9), "slots": args.serve_slots,
            "rates": results, "server": stats, "clocks": clk.summary()}


def run_serve_workload(args, rank, world):
    """--workload serve: the serving sweep alone, as one JSON line."""
    import edpp
    edpp.lib()
    dev = _device(args)
    if rank != 0:
        return 0
    r = measure_serve(args, dev, [float(x) for x in args.rates.split(",")], args.serve_requests)
    best = max(r["rates"], key=lambda x: x["elements/s"])
    print(json.dumps({
        "metric": METRIC, "workload_metric": "served elements/s with p50/p99 latency",
        "value": best["elements/s"], "unit": "elements/s", "n_gpus": world,
        "steps": len(r["rates"]), "warmup": 1, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": r["workload"], "payloads": r["payloads"],
                   "pool_bytes": r["pool_bytes"], "slots": r["slots"]},
        "rates": r["rates"], "server": r["server"], "clocks": r["clocks"],
        "e2e": {"value": best["elements/s"], "unit": "elements/s",
                "note": "every request copies inputs host->device and outputs back"},
    }), flush=True)
    return 0


def _event_ms(fn, reps, warmup, flush=None):
    """Mean CUDA-event time of fn() over reps calls (after warm-up); with
    `flush`, an L2-sized buffer is rewritten before every call and the flush
    is timed separately and subtracted."""
    import torch
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(reps):
        if flush is not None:
            flush.add_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
    return total / reps


def _hampel_ms(fn, reps):
    from oracle import oracle as orc
    return orc.average_hampel([fn() for _ in range(reps)])


FP32_EPS = 1.0  # relative error of an f32 scan: |gpu - f64| / max(|f64|, FP32_EPS)


def measure_scans(args, dev, reps, warmup, config1=True, config4=True, cpu=True):
    """Configs 1 and 4: int32 exclusive scan of 2^24 values in [0,15]
    (seed 1), warm and with L2 flushed; global scans of 2^30 int32 / int64
    (inclusive and exclusive, values in [0,100], seed 1) and f32 inclusive
    (values in [-1,1], seed 1) under the three schemes, with the f32 result's
    error against an f64 accumulation of the same inputs (the oracle).
    cpu: the OpenMP ports of scan_SSA_omp / scan_RTS_omp on the host cores
    (config 1 at full size, config 4 on a 2^28 sample)."""
    import numpy as np
    import torch

    import edpp
    peak, peak_kind = measured_peak_gbs()
    out = {"peak": peak, "peak_source": peak_kind}
    rows = []
    if config1:
        flush = torch.empty(64 << 20, dtype=torch.int32, device=dev)  # 256 MB > L2
        h24 = edpp.gen_uniform_i32(1 << 24, 1, 0, 15)
        x24 = torch.from_numpy(h24).to(dev)
        y24 = torch.empty_like(x24)
        for algo in ("lookback", "rts", "ssa"):
            ws = edpp.workspace(edpp.scan_workspace_bytes(1 << 24, "int32", algo), dev)
            for l2 in ("warm", "flushed"):
                ms = _event_ms(lambda: edpp.scan(x24, algo=algo, out=y24, ws=ws), reps,
                               warmup, flush if l2 == "flushed" else None)
                gbs = 8 * (1 << 24) / (ms * 1e-3) / 1e9
                rows.append({"config": "1", "n": 1 << 24, "dtype": "int32", "inclusive": False,
                             "algo": algo, "l2": l2, "ms": round(ms, 4), "GB/s": round(gbs, 1),
                             "frac_of_hbm": round(gbs / peak, 4)})
        del x24, y24, flush
        if cpu:
            from oracle import oracle as orc
            th = orc.max_threads()
            c1 = {}
            for scheme in ("ssa", "rts"):
                ms = _hampel_ms(lambda: orc.scan_omp(h24, scheme, th)[1], 5)
                c1[scheme] = {"ms": round(ms, 3),
                              "GB/s": round(8 * (1 << 24) / (ms * 1e-3) / 1e9, 2)}
            out["config1_cpu_baseline"] = {
                "value": max(v["GB/s"] for v in c1.values()), "unit": "GB/s", "cores": th,
                "kind": "port", "per_scheme": c1,
                "sample": "the full config (2^24 int32); OpenMP ports of scan_SSA_omp / "
                          "scan_RTS_omp (openmp/test_scan_CPU.cpp:85-163); Hampel mean of 5"}
    if config4:
        n = 1 << args.scan_log2n
        fp32_err = {}
        for dt, bpe in (("int32", 8), ("int64", 16), ("float32", 8)):
            if dt == "int32":
                h = edpp.gen_uniform_i32(n, 1, 0, 100)
            elif dt == "int64":
                h = edpp.gen_uniform_i64(n, 1, 0, 100)
            else:
                h = edpp.gen_uniform_f32(n, 1, -1.0, 1.0)
            x = torch.from_numpy(h).to(dev)
            y = torch.empty_like(x)
            ref = None
            if dt == "float32":
                from oracle import oracle as orc
                ref = torch.from_numpy(orc.scan(h, True)).to(dev)  # f64 accumulation
            for inc in ((False, True) if dt != "float32" else (True,)):
                for algo in ("lookback", "rts", "ssa"):
                    ws = edpp.workspace(edpp.scan_workspace_bytes(n, dt, algo), dev)
                    ms = _event_ms(lambda: edpp.scan(x, inclusive=inc, algo=algo, out=y, ws=ws),
                                   reps, warmup)
                    gbs = bpe * n / (ms * 1e-3) / 1e9
                    rows.append({"config": "4", "n": n, "dtype": dt, "inclusive": inc,
                                 "algo": algo, "ms": round(ms, 4), "GB/s": round(gbs, 1),
                                 "frac_of_hbm": round(gbs / peak, 4)})
                    if ref is not None:
                        err = (y.double() - ref).abs_() / ref.abs().clamp_min(FP32_EPS)
                        fp32_err[algo] = {"max_rel": float(err.max()),
                                          "mean_rel": float(err.mean()),
                                          "max_abs": float((y.double() - ref).abs().max())}
                        del err
                    del ws
            del x, y, ref
            torch.cuda.empty_cache()
        out["fp32_inclusive_error"] = {
            "n": n, "values": "uniform [-1,1], seed 1",
            "definition": f"|gpu - f64| / max(|f64|, {FP32_EPS}) over all n outputs, f64 = "
                          "sequential f64 accumulation of the same f32 inputs (the oracle)",
            "per_scheme": fp32_err}
        if cpu:
            from oracle import oracle as orc
            th = orc.max_threads()
            ns = min(n, 1 << 28)
            hs = edpp.gen_uniform_i32(ns, 1, 0, 100)
            c4 = {}
            for scheme in ("ssa", "rts"):
                ms = _hampel_ms(lambda: orc.scan_omp(hs, scheme, th)[1], 3)
                c4[scheme] = {"ms": round(ms, 3), "GB/s": round(8 * ns / (ms * 1e-3) / 1e9, 2)}
            out["config4_cpu_baseline"] = {
                "value": max(v["GB/s"] for v in c4.values()), "unit": "GB/s", "cores": th,
                "kind": "port", "per_scheme": c4,
                "sample": f"int32 exclusive at n=2^{ns.bit_length() - 1} of the 2^30 config; "
                          "OpenMP ports of scan_SSA_omp / scan_RTS_omp; Hampel mean of 3"}
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the scan workload")
    out["rows"] = rows
    return out


def run_scan_workload(args, rank, world):
    """--workload scan: configs 1 and 4 alone, as one JSON line."""
    import edpp
    edpp.lib()
    dev = _device(args)
    r = measure_scans(args, dev, args.steps, args.warmup, config4=not args.scan_config1_only,
                      cpu=not args.no_cpu)
    rows = r["rows"]
    head = [x for x in rows if x["config"] == "1" and x["algo"] == "lookback"
            and x["l2"] == "flushed"][0]
    if rank == 0:
        line = {"metric": METRIC, "workload_metric": "scan GB/s (8 B/elem int32)",
                "value": head["GB/s"], "unit": "GB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic",
                "config": {"workload": "scans: config 1 (2^24 int32 [0,15] seed 1) "
                                       "and config 4 (2^30, three schemes)"}}
        line.update(r)
        print(json.dumps(line), flush=True)
    return 0


def measure_split(args, dev, reps, warmup, buckets, kinds=("uniform", "zipf"), cpu=True):
    """Config 3: stable split of 2^28 (int32 key, int32 value = index) pairs,
    keys uniform over [0,2^31) or Zipf(1.0) buckets (seed 3).  cpu: the
    stable split restatement (counting sort; the reference has no CPU
    split) on a 2^24 sample at 256 buckets."""
    import torch

    import edpp
    peak, peak_kind = measured_peak_gbs()
    n = 1 << args.split_log2n
    vals = torch.arange(n, dtype=torch.int32, device=dev)
    ko = torch.empty(n, dtype=torch.int32, device=dev)
    vo = torch.empty_like(ko)
    ws = edpp.workspace(max(edpp.split_workspace_bytes(n, b, "soa") for b in buckets), dev)
    h_uniform = edpp.gen_keys_uniform(n, 3)
    uniform = torch.from_numpy(h_uniform).to(dev)
    rows = []
    for B in buckets:
        for kind in kinds:
            keys = uniform if kind == "uniform" else \
                torch.from_numpy(edpp.gen_keys_zipf(n, 3, B, 1.0)).to(dev)
            ms = _event_ms(lambda: edpp.split(keys, B, values=vals, keys_out=ko, values_out=vo,
                                              ws=ws), reps, warmup)
            gbs = 16 * n / (ms * 1e-3) / 1e9
            rows.append({"buckets": B, "keys": kind, "ms": round(ms, 4), "GB/s": round(gbs, 1),
                         "frac_of_hbm": round(gbs / peak, 4)})
            if kind != "uniform":
                del keys
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the split workload")
    out = {"workload": f"split 2^{args.split_log2n} KV (value = index), uniform / Zipf(1.0) keys, "
                       "seed 3", "n": n, "peak": peak, "peak_source": peak_kind, "rows": rows}
    del vals, ko, vo, ws, uniform
    torch.cuda.empty_cache()
    if cpu:
        import numpy as np

        from oracle import oracle as orc
        ns = min(n, 1 << 24)
        hk = h_uniform[:ns]
        hv = np.arange(ns, dtype=np.int32)
        ms = _hampel_ms(lambda: orc.split_timed(hk, 256, hv, "soa")[2], 3)
        out["cpu_baseline"] = {
            "value": round(16 * ns / (ms * 1e-3) / 1e9, 2), "unit": "GB/s", "cores": 1,
            "kind": "restatement",
            "sample": f"256 buckets, uniform keys, n=2^{ns.bit_length() - 1}; the reference has "
                      "no CPU split: a single-thread counting-sort restatement, labelled as such"}
    return out


def run_split_workload(args, rank, world):
    """--workload split: config 3 alone, as one JSON line."""
    import edpp
    edpp.lib()
    dev = _device(args)
    blist = [int(b) for b in args.split_buckets.split(",")] if args.split_buckets else \
        [2 ** k for k in range(1, 11)]
    r = measure_split(args, dev, args.steps, args.warmup, blist, cpu=not args.no_cpu)
    rows = r["rows"]
    head = ([x for x in rows if x["buckets"] == 256 and x["keys"] == "uniform"] or rows)[0]
    if rank == 0:
        line = {"metric": METRIC, "workload_metric": "stable split GB/s (16 B/pair)",
                "value": head["GB/s"], "unit": "GB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic",
                "config": {"workload": r["workload"]}}
        line.update({k: v for k, v in r.items() if k != "workload"})
        print(json.dumps(line), flush=True)
    return 0


def run_autotune_workload(args, rank, world):
    """Per-size-class autotuning of the plain primitives: for every size
    class, time each look-back tile shape and each slice length of the
    chunked reduce-then-scan (int32 and int64), and the gather's tiled form
    against its direct sweep, on seeded data; record the winners and write
    the table (--tune-out, default the committed
    efficient-dpp_gb300/tuning/plain_gb300.tsv).  Prints every variant's time."""
    import torch

    import edpp
    edpp.lib()
    dev = _device(args)
    if rank != 0:
        return 0
    edpp.lib().edpp_tune_clear()
    reps = max(3, args.steps)
    rows = []
    # timed cold: a buffer larger than L2 is overwritten before every timed
    # call, as the first touch of an array finds its data
    flush = torch.empty(64 << 20, dtype=torch.int32, device=dev)
    plan = [(edpp.TUNE_SCAN_LOOKBACK, "int32", range(16, 31, 2)),
            (edpp.TUNE_SCAN_LOOKBACK, "int64", range(16, 30, 2)),
            (edpp.TUNE_SCAN_RTS, "int32", range(20, 31)),
            (edpp.TUNE_SCAN_RTS, "int64", range(20, 30)),
            (edpp.TUNE_GATHER, "int32", (20, 22, 24, 25, 26, 27, 28))]
    for prim, dt, logs in plan:
        for lg in logs:
            n = 1 << lg
            tdt = getattr(torch, dt)
            if prim == edpp.TUNE_GATHER:
                x = torch.arange(n, dtype=tdt, device=dev)
                loc = torch.from_numpy(edpp.gen_permutation(n, 2)).to(dev)
                ws = edpp.workspace(edpp.gs_workspace_bytes("gather", n, 1, "tiled"), dev)
            else:
                x = torch.randint(0, 101, (n,), dtype=tdt, device=dev)
                loc = None
                algo = "lookback" if prim == edpp.TUNE_SCAN_LOOKBACK else "rts"
                ws = edpp.workspace(edpp.scan_workspace_bytes(n, dt, algo), dev)
            y = torch.empty_like(x)
            v, ms, each = edpp.autotune_plain(prim, x, y, ws, loc=loc, reps=reps, flush=flush)
            rows.append({"primitive": edpp.TUNE_NAMES[prim], "dtype": dt, "log2n": lg,
                         "best": v, "ms": [round(m, 4) for m in each]})
            del x, y, ws, loc
            torch.cuda.empty_cache()
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the autotune workload")
    out = args.tune_out or str(PKG / "tuning" / "plain_gb300.tsv")
    edpp.tune_save(out)
    print(json.dumps({"metric": METRIC, "workload_metric": "autotune table (ms per variant)",
                      "value": None, "unit": "ms", "n_gpus": world, "steps": reps,
                      "warmup": 1, "higher_is_better": False, "data": "synthetic",
                      "config": {"workload": "per-size-class autotune of the plain primitives"},
                      "table": out, "rows": rows}), flush=True)
    return 0


def run_radix_workload(args, rank, world):
    """LSD radix sort on the stable split (8-bit digits): 2^k uniform int32 keys
    (seed 3), keys only and with int32 values, against torch.sort(stable=True)
    on the same data (CUB's radix sort, the comparison of
    obsolete/CUDA/radixSortCUB.cu).  torch orders signed keys; the split sorts
    the bit pattern, so keys are drawn from [0, 2^31) where both agree."""
    import torch

    import edpp
    edpp.lib()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    peak, peak_kind = measured_peak_gbs()
    n = 1 << args.radix_log2n
    keys = torch.from_numpy(edpp.gen_keys_uniform(n, 3)).to(dev)
    vals = torch.arange(n, dtype=torch.int32, device=dev)
    ko = torch.empty_like(keys)
    vo = torch.empty_like(vals)
    rows = []
    for with_vals in (False, True):
        ws = edpp.workspace(edpp.lib().edpp_radix_sort_workspace_size(n, int(with_vals)), dev)
        ms = _event_ms(lambda: edpp.radix_sort(keys, vals if with_vals else None, 0, 31, ko,
                                               vo if with_vals else None, ws),
                       args.steps, args.warmup)
        ms_t = _event_ms(lambda: torch.sort(keys, stable=True), args.steps, args.warmup)
        ref_k, ref_i = torch.sort(keys, stable=True)
        ok = bool(torch.equal(ko, ref_k)) and (not with_vals or bool(torch.equal(vo, ref_i.int())))
        rows.append({"values": with_vals, "ms": round(ms, 4), "Mkeys/s": round(n / ms / 1e3, 1),
                     "torch_sort_ms": round(ms_t, 4), "identical_to_torch": ok})
        del ws
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the radix workload")
    head = rows[1]
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload_metric": "radix sort Mkeys/s (31-bit keys, 4 passes)",
                          "value": head["Mkeys/s"], "unit": "Mkeys/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"],
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "int32", "data": "synthetic", "peak": peak,
                          "peak_source": peak_kind,
                          "config": {"workload": f"radix sort 2^{args.radix_log2n} uniform keys "
                                                 "[0,2^31), seed 3, bits 0..31"},
                          "rows": rows}), flush=True)
    return 0


def run_join_workload(args, rank, world):
    """Hash join match count, partitioned (split both sides, shared-memory
    table per partition) and non-partitioned (one device table), |R| = 2^k
    keys and |S| in {2^k, 2^(k-4)}, uniform over [0, 2^k) (seeds 7, 8)."""
    import torch

    import edpp
    edpp.lib()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    peak, peak_kind = measured_peak_gbs()
    k = args.join_log2n
    rows = []
    r = torch.from_numpy(edpp.gen_uniform_i32(1 << k, 7, 0, (1 << k) - 1)).to(dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    for s_log2 in (k, k - 4):
        s = torch.from_numpy(edpp.gen_uniform_i32(1 << s_log2, 8, 0, (1 << k) - 1)).to(dev)
        for part in (True, False):
            nbytes = (edpp.lib().edpp_hash_join_workspace_size(r.numel(), s.numel(), 0) if part
                      else edpp.lib().edpp_hash_join_np_workspace_size(s.numel()))
            ws = edpp.workspace(nbytes, dev)
            ms = _event_ms(lambda: edpp.hash_join_count(r, s, ws=ws, partitioned=part, count=cnt),
                           args.steps, args.warmup)
            tuples = r.numel() + s.numel()
            rows.append({"r": r.numel(), "s": s.numel(),
                         "form": "partitioned" if part else "non-partitioned",
                         "ms": round(ms, 4), "Mtuples/s": round(tuples / (ms * 1e-3) / 1e6, 1),
                         "matches": int(cnt.item())})
            del ws
        del s
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the join workload")
    head = max(rows, key=lambda x: x["Mtuples/s"] if x["s"] == x["r"] else 0)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload_metric": "join Mtuples/s ((|R|+|S|)/t)",
                          "value": head["Mtuples/s"], "unit": "Mtuples/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"],
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "int32", "data": "synthetic", "peak": peak,
                          "peak_source": peak_kind,
                          "config": {"workload": f"hash join count, |R|=2^{k}, |S|=2^{k} and "
                                                 f"2^{k - 4}, keys uniform [0,2^{k})"},
                          "rows": rows}), flush=True)
    return 0


def run_access_workload(args, rank, world):
    """Access-pattern sweeps: scale with column / row / mixed / vector maps
    (local 512, grid 32768, repeat 1..20 as the reference's access test),
    block-order sweep (chunks 8 KB..8 MB, interleaved or shuffled order,
    cold or after a cache-heat pass), single-block matrix scans (tiles 1..49)."""
    import numpy as np
    import torch

    import edpp
    edpp.lib()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    peak, peak_kind = measured_peak_gbs()
    local, grid = 512, 32768
    repeats = [1, 2, 4, 8, 12, 16, 20]
    nmax = local * grid * max(repeats)
    a = torch.arange(nmax, dtype=torch.int32, device=dev)
    b = torch.empty_like(a)
    scale = []
    for pattern in ("column", "row", "mixed", "vec"):
        for rep in repeats:
            ms = _event_ms(lambda: edpp.access_scale(a, b, rep, pattern, local, grid),
                           args.steps, args.warmup)
            gbs = 8 * local * grid * rep / (ms * 1e-3) / 1e9
            scale.append({"pattern": pattern, "repeat": rep, "ms": round(ms, 4),
                          "GB/s": round(gbs, 1), "frac_of_hbm": round(gbs / peak, 4)})
    del b
    length = 1 << args.access_wg_log2n
    data = a[:length]
    wg = []
    for order_kind in ("interleaved", "random"):
        for loaded in (False, True):
            for kb in (8192, 1024, 128, 8):
                g = length * 4 // (kb * 1024)
                order = np.arange(g, dtype=np.int32)
                if order_kind == "random":
                    order = np.random.default_rng(9).permutation(g).astype(np.int32)
                d_order = torch.from_numpy(order).to(dev)
                out = torch.zeros(g, dtype=torch.int64, device=dev)
                tick = torch.zeros(1, dtype=torch.int32, device=dev)
                for lsz in (1, 256):
                    # "loaded": the input was just written by the heat pass
                    pre = (lambda: edpp.cache_heat(data, 512, 32768)) if loaded else None

                    def call():
                        if pre is not None:
                            pre()
                        edpp.access_wg(data, d_order, lsz, out=out, ticket=tick)
                    if loaded:
                        # time the sweep alone, after the heat pass
                        ms_h = _event_ms(pre, 2, 1)
                        ms = _event_ms(call, 2, 1) - ms_h
                    else:
                        ms = _event_ms(call, 2, 1)
                    wg.append({"order": order_kind, "loaded": loaded, "chunk_kb": kb,
                               "blocks": g, "threads": lsz, "ms": round(ms, 4),
                               "GB/s": round(4 * length / (max(ms, 1e-6) * 1e-3) / 1e9, 1)})
    del a
    lscan = []
    src = torch.from_numpy(edpp.gen_uniform_i32(512 * 49, 7, 0, 15)).to(dev)
    dst = torch.empty_like(src)
    for scheme in ("lm", "reg", "lm_reg", "warp"):
        for tile in (1, 2, 4, 8, 16, 24, 32, 49):
            reps = 200
            ms = _event_ms(lambda: edpp.local_scan(src, tile, scheme, repeat=reps, out=dst), 2, 1)
            lscan.append({"scheme": scheme, "tile": tile, "us_per_launch": round(ms * 1e3 / reps, 2)})
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault in the access workload")
    head = max(scale, key=lambda x: x["GB/s"])
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload_metric": "scale GB/s (8 B/elem), best map",
                          "value": head["GB/s"], "unit": "GB/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"],
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "int32", "data": "synthetic", "peak": peak,
                          "peak_source": peak_kind,
                          "config": {"workload": "access-pattern sweeps (scale 512x32768xR, "
                                                 f"block-order 2^{args.access_wg_log2n}, "
                                                 "matrix scans 512xT)"},
                          "scale": scale, "block_order": wg, "local_scan": lscan}), flush=True)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="edpp", choices=["edpp", "reference"])
    ap.add_argument("--log2n", type=int, default=28)
    ap.add_argument("--ref-n", type=int, default=0,
                    help="reference arm size (default: 2^log2n, the GPU arm's size)")
    ap.add_argument("--cpu-sample", type=int, default=1 << 26)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default run: skip the config 1/3/4/5 keys (scan, split, batch, serve)")
    ap.add_argument("--extras-serve-requests", type=int, default=200,
                    help="default run: requests per rate of the serving sweep")
    ap.add_argument("--method", default="tiled", choices=["partition", "sweep", "tiled"],
                    help="gather/scatter schedule of the timed step")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip timing the other gather/scatter schedule")
    ap.add_argument("--workload", default="gs_stream",
                    choices=["gs_stream", "batch", "serve", "scan", "split", "join", "access",
                             "radix", "autotune"],
                    help="gs_stream: multi-pass gather/scatter + STREAM (default); "
                         "batch: 4096 uneven segments, batched vs plain; "
                         "serve: Poisson request stream through the server")
    ap.add_argument("--rates", default="100,300,1000,3000", help="serve: request rates (1/s)")
    ap.add_argument("--serve-requests", type=int, default=400)
    ap.add_argument("--serve-payloads", type=int, default=48)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--pool-gb", type=float, default=40.0)
    ap.add_argument("--batch-log2-total", type=int, default=30,
                    help="batch: cap on the total elements (2^30 in the config)")
    ap.add_argument("--scan-log2n", type=int, default=30)
    ap.add_argument("--split-log2n", type=int, default=28)
    ap.add_argument("--split-buckets", default="", help="split: comma list (default 2..1024)")
    ap.add_argument("--join-log2n", type=int, default=26)
    ap.add_argument("--radix-log2n", type=int, default=28)
    ap.add_argument("--access-wg-log2n", type=int, default=26)
    ap.add_argument("--scan-config1-only", action="store_true",
                    help="scan: only the config-1 rows")
    ap.add_argument("--autotune", action="store_true",
                    help="batch: run the autotuner and record its choice")
    ap.add_argument("--tune-out", default="",
                    help="autotune: where to write the plain primitives' table")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)

    rank, world, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batch":
        return run_batch_workload(args, rank, world)
    if args.workload == "serve":
        return run_serve_workload(args, rank, world)
    if args.workload == "scan":
        return run_scan_workload(args, rank, world)
    if args.workload == "split":
        return run_split_workload(args, rank, world)
    if args.workload == "join":
        return run_join_workload(args, rank, world)
    if args.workload == "radix":
        return run_radix_workload(args, rank, world)
    if args.workload == "access":
        return run_access_workload(args, rank, world)
    if args.workload == "autotune":
        return run_autotune_workload(args, rank, world)

    import numpy as np
    import torch

    import edpp
    edpp.lib()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = 1 << args.log2n

    # inputs (host, seeded) -> device
    h_loc = edpp.gen_permutation(n, 2)
    h_in = np.arange(n, dtype=np.int32)
    h_a = np.arange(n, dtype=np.float32)
    h_b = (np.arange(n, dtype=np.float32) + 10).astype(np.float32)
    d_loc = torch.from_numpy(h_loc).to(dev)
    d_in = torch.from_numpy(h_in).to(dev)
    d_a = torch.from_numpy(h_a).to(dev)
    d_b = torch.from_numpy(h_b).to(dev)
    d_out = torch.empty(n, dtype=torch.int32, device=dev)
    d_fout = torch.empty(n, dtype=torch.float32, device=dev)
    # one workspace serves every pass count (allocated outside the timed region)
    ws = edpp.workspace(max(edpp.gs_workspace_bytes(k, n, p, m) for k in ("gather", "scatter")
                            for p in PASSES for m in ("partition", "tiled")), dev)

    def run_call(name, p, method=args.method):
        if name == "gather":
            edpp.gather(d_in, d_loc, p, out=d_out, method=method, ws=ws)
        elif name == "scatter":
            edpp.scatter(d_in, d_loc, p, out=d_out, method=method, ws=ws)
        else:
            edpp.stream(name, d_a, d_b, 3.0, out=d_fout)

    calls = step_calls()
    step_bytes = sum(call_bytes(name, n) for name, _ in calls)
    launches_per_step = sum(call_launches(name, p, args.method) for name, p in calls)

    for _ in range(args.warmup):
        for c in calls:
            run_call(*c)
    torch.cuda.synchronize()
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault during warm-up")

    # ---- device-timed region -------------------------------------------
    ev = {c: [] for c in calls}
    stream = torch.cuda.current_stream()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for _ in range(args.steps):
            for c in calls:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                run_call(*c)
                e1.record(stream)
                ev[c].append((e0, e1))
        t_end.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms_total = t_start.elapsed_time(t_end)
    ms_total = max_over_ranks(ms_total, world)
    ms_step = ms_total / args.steps
    value = world * step_bytes * args.steps / (ms_total * 1e-3) / 1e9
    per_call_ms = {c: statistics.mean(a.elapsed_time(b) for a, b in ev[c]) for c in calls}
    if edpp.sync_status() != edpp.EDPP_OK:
        raise SystemExit("device fault during the timed region")

    peak, peak_kind = measured_peak_gbs()
    primitives = {}
    for (name, p), ms in per_call_ms.items():
        key = f"{name}_p{p}" if p else name
        gbs = call_bytes(name, n) / (ms * 1e-3) / 1e9
        primitives[key] = {"ms": round(ms, 4), "GB/s": round(gbs, 1),
                           "frac_of_hbm": round(gbs / peak, 4)}
        if name in ("gather", "scatter"):
            # the reference's own figure: n * 4 bytes / time in GiB/s
            # (cuda/util/utility.cuh:15-17, opencl/test/test_gather.cpp:50)
            primitives[key]["reference_formula_GiB/s"] = round(n * 4 / (ms * 1e-3) / 2**30, 1)
    dom = max(per_call_ms, key=lambda c: per_call_ms[c])
    dom_name = f"{dom[0]}_p{dom[1]}" if dom[1] else dom[0]
    # The dominant call of the step: its algorithmic bytes over its CUDA-event
    # duration (all launches of the call, which run back to back on the stream).
    achieved = call_bytes(dom[0], n) / (per_call_ms[dom] * 1e-3) / 1e9
    # DRAM bytes of one such call from an ncu capture of the tiled schedule
    # (profiles/traffic.json); the rate they imply shows how close the call's
    # kernels run to the HBM roofline on the bytes they must move.
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists() and args.method == "tiled" and n == 1 << 28:
        try:
            traffic = json.loads(tf.read_text()).get(dom_name)
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "traffic_gbs": None if traffic is None else
                round(traffic / (per_call_ms[dom] * 1e-3) / 1e9, 1),
                "traffic_frac": None if traffic is None else
                round(traffic / (per_call_ms[dom] * 1e-3) / 1e9 / peak, 4),
                "kernel": dom_name,
                "launches_per_call": call_launches(dom[0], dom[1], args.method),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s"}

    # ---- the other schedule, per call, for comparison (not in `value`) ------
    compare = None
    if not args.no_compare:
        compare = {}
        for other in ("sweep", "partition", "tiled"):
            if other == args.method:
                continue
            cm = {}
            for c in calls:
                if c[0] not in ("gather", "scatter"):
                    continue
                run_call(*c, method=other)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(args.steps):
                    run_call(*c, method=other)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / args.steps
                cm[f"{c[0]}_p{c[1]}"] = {"ms": round(ms, 4),
                                         "GB/s": round(call_bytes(c[0], n) / (ms * 1e-3) / 1e9, 1)}
            compare[other] = cm

    # ---- end to end: host buffers through the C ABI ------------------------
    e2e = None
    if not args.no_e2e:
        p_loc = torch.from_numpy(h_loc).pin_memory()
        p_in = torch.from_numpy(h_in).pin_memory()
        p_a = torch.from_numpy(h_a).pin_memory()
        p_b = torch.from_numpy(h_b).pin_memory()
        p_out = torch.empty(n, dtype=torch.int32).pin_memory()
        p_fout = torch.empty(n, dtype=torch.float32).pin_memory()
        h2d = 4 * 4 * n
        d2h = 4 * n * len(calls)

        # Copies overlap compute: inputs arrive on an H2D stream (loc/in first,
        # then a/b), every call writes its own device output, and a D2H
        # stream reads each output back as soon as its call is done.  Events
        # keep every input alive until its last reader and every output until
        # its copy is done; the timed region covers all three streams.
        h2d_s = torch.cuda.Stream(device=dev)
        d2h_s = torch.cuda.Stream(device=dev)
        gs_calls = [c for c in calls if c[0] in ("gather", "scatter")]
        st_calls = [c for c in calls if c[0] not in ("gather", "scatter")]
        d_outs = {c: torch.empty(n, dtype=torch.int32, device=dev) for c in gs_calls}
        f_outs = {c: torch.empty(n, dtype=torch.float32, device=dev) for c in st_calls}
        ev = lambda: torch.cuda.Event()

        def e2e_step(prev):
            # prev: (loc/in free, a/b free, {call: its output copied}) of the last step
            if prev is not None:
                h2d_s.wait_event(prev[0])
            with torch.cuda.stream(h2d_s):
                d_loc.copy_(p_loc, non_blocking=True)
                d_in.copy_(p_in, non_blocking=True)
                e_gs_in = ev(); e_gs_in.record(h2d_s)
                if prev is not None:
                    h2d_s.wait_event(prev[1])
                d_a.copy_(p_a, non_blocking=True)
                d_b.copy_(p_b, non_blocking=True)
                e_st_in = ev(); e_st_in.record(h2d_s)
            copied = {}
            stream.wait_event(e_gs_in)
            for c in calls:
                if c == st_calls[0]:
                    stream.wait_event(e_st_in)
                if prev is not None:
                    stream.wait_event(prev[2][c])  # this output's last copy is done
                name, p = c
                if c in d_outs:
                    (edpp.gather if name == "gather" else edpp.scatter)(
                        d_in, d_loc, p, out=d_outs[c], method=args.method, ws=ws)
                else:
                    edpp.stream(name, d_a, d_b, 3.0, out=f_outs[c])
                e = ev(); e.record(stream)
                if c == gs_calls[-1]:
                    e_gs_free = e
                d2h_s.wait_event(e)
                with torch.cuda.stream(d2h_s):
                    if c in d_outs:
                        p_out.copy_(d_outs[c], non_blocking=True)
                    else:
                        p_fout.copy_(f_outs[c], non_blocking=True)
                    copied[c] = ev(); copied[c].record(d2h_s)
            e_st_free = ev(); e_st_free.record(stream)
            return (e_gs_free, e_st_free, copied)

        e2e_step(None)
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h2d_s.wait_event(e0)
        d2h_s.wait_event(e0)
        prev = None
        for _ in range(args.steps):
            prev = e2e_step(prev)
        for e in prev[2].values():
            stream.wait_event(e)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks(e0.elapsed_time(e1), world)
        # the last step's outputs, read back through the overlapped copies
        ok = bool(torch.equal(torch.from_numpy(p_fout.numpy()).to(dev), f_outs[st_calls[-1]]))
        if not ok:
            raise SystemExit("end-to-end output copy mismatch")
        e2e = {"value": round(world * step_bytes * args.steps / (e2e_ms * 1e-3) / 1e9, 3),
               "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": round(e2e_ms / args.steps, 3)}
        del p_loc, p_in, p_a, p_b, p_out, p_fout, d_outs, f_outs

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_sample)

    # ---- the other configurations, each as its own key of the same line -------
    # (not part of `value`, which stays the config-2 step above)
    extras = {}
    if not args.no_extras:
        del d_loc, d_in, d_a, d_b, d_out, d_fout, ws
        torch.cuda.empty_cache()
        reps = max(3, min(args.steps, 5))
        with_cpu = rank == 0 and world == 1 and not args.no_cpu
        scans = measure_scans(args, dev, reps, args.warmup, cpu=with_cpu)
        c1 = [r for r in scans["rows"] if r["config"] == "1"]
        c4 = [r for r in scans["rows"] if r["config"] == "4"]
        extras["config1_scan"] = {
            "workload": "int32 exclusive scan, 2^24 values uniform in [0,15], seed 1",
            "rows": c1, "cpu_baseline": scans.get("config1_cpu_baseline")}
        extras["config4_scan"] = {
            "workload": f"global scans at 2^{args.scan_log2n}: int32/int64 exclusive and "
                        "inclusive (values in [0,100]), f32 inclusive ([-1,1]), seed 1, "
                        "look-back / reduce-then-scan / scan-then-propagate",
            "rows": c4, "fp32_inclusive_error": scans.get("fp32_inclusive_error"),
            "cpu_baseline": scans.get("config4_cpu_baseline")}
        extras["config3_split"] = measure_split(args, dev, reps, args.warmup,
                                                [2 ** k for k in range(1, 11)], cpu=with_cpu)
        extras["config5_batch"] = measure_batch(args, dev, world, reps, args.warmup)
        if rank == 0:
            extras["config5_serve"] = measure_serve(
                args, dev, [float(x) for x in args.rates.split(",")], args.extras_serve_requests)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32+f32", "data": "synthetic",
            "config": step_config(n, world),
            "gather_scatter_method": args.method,
            "primitives": primitives,
            "compare": compare,
            "roofline": roofline,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
