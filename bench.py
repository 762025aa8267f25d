#!/usr/bin/env python3
"""Walker-step benchmark (one JSON line on rank 0).

Default workload: weighted DeepWalk (static alias sampling), walk length 80,
4,194,304 walkers (one per vertex) on a seeded R-MAT scale-22 graph (edge
factor 16, a/b/c = 0.57/0.19/0.19, undirected, lognormal(0,1) float32
weights); every step rebuilds the alias tables on the GPU and walks all
walkers (the reference includes the alias build in its timings).

value : walker-steps/s with the graph resident in HBM and paths written to HBM
        (kk_walk_device), device time from CUDA events on the engine's stream.
e2e   : the same walk through the public C-ABI call kk_walk_into: the start-vertex
        list is copied host->device and every path is copied device->host into
        pinned host memory, inside the timed region; K calls (the device loop's
        K), each call's time recorded in e2e.call_ms.
roofline: the walk kernel's bytes touched per walker-step at 32-byte sector
        granularity (sampling part only) over its CUDA-event duration, against
        the measured HBM copy bandwidth.
cpu_baseline / --impl reference: the CPU restatement of the reference's path
        (oracle/kk_oracle.c, pinned bit-for-bit to the reference) on all host
        cores, over a bounded sample of the same workload.

Multi-GPU (torchrun): weak scaling, each rank walks its own walker-id range on
its own replica of the graph; no collective on the data path.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "deepwalk-s22": dict(app="deepwalk", scale=22, weights=2, types=0, walk_length=80,
                         desc="weighted DeepWalk (alias sampling, alias build included), len 80, one walker per vertex, "
                              "R-MAT scale 22 ef16 lognormal(0,1) weights"),
    "node2vec-s16": dict(app="node2vec", scale=16, weights=1, types=0, walk_length=80, p=2.0, q=0.5,
                         desc="node2vec p=2 q=0.5 len 80, 65,536 walkers, R-MAT scale 16 ef16 uniform[1,5) weights"),
    "ppr-s24": dict(app="ppr", scale=24, weights=0, types=0, terminate_prob=1.0 / 80,
                    desc="PPR terminate 1/80, unweighted, one walker per vertex, R-MAT scale 24 ef16"),
    "metapath-s22": dict(app="metapath", scale=22, weights=1, types=5, walk_length=80,
                         schemes=[[1, 2, 4, 8], [2, 8, 2, 16], [4, 1, 16, 4]], scheme_round_robin=True,
                         desc="metapath len 80, 3 schemes of 4 one-hot type masks round robin, R-MAT scale 22 ef16, "
                              "5 edge types, uniform[1,5) weights"),
    "node2vec-s24": dict(app="node2vec", scale=24, weights=1, types=0, walk_length=80, p=2.0, q=0.5,
                         desc="node2vec p=2 q=0.5 len 80, one walker per vertex, R-MAT scale 24 ef16 uniform[1,5)"),
    "node2vec-serve-s24": dict(app="node2vec", scale=24, weights=1, types=0, serve=3000,
                               desc="served node2vec request stream on a resident R-MAT scale 24 ef16 uniform[1,5) "
                                    "graph: per request p, q log-uniform [0.25, 4], length uniform [5, 200], "
                                    "walkers lognormal (median 4096, sigma 1) clipped to [1, 2^20], each request "
                                    "its own seed and walker-id range"),
    "metapath-batch-s22": dict(app="metapath", scale=22, weights=1, types=5, batch=16,
                               schemes=[[1, 2, 4, 8], [2, 8, 2, 16], [4, 1, 16, 4]], scheme_round_robin=True,
                               desc="16 metapath jobs (walkers 2^10..2^22, lengths 5..200, 3 schemes of 4 one-hot "
                                    "type masks round robin) in one batched launch vs one launch per job, R-MAT "
                                    "scale 22 ef16, 5 edge types, uniform[1,5) weights"),
}


def batch_jobs(wl):
    """The batched workload's jobs: walker counts 2^10..2^22, lengths 5..200 in a fixed shuffled order."""
    n = wl["batch"]
    jobs = []
    for k in range(n):
        walkers = 1 << (10 + round(12 * k / (n - 1)))
        length = 5 + (195 * ((7 * k) % n)) // (n - 1)
        job = dict(walker_num=walkers, seed=100 + k, walk_length=length, weighted=bool(wl["weights"]))
        for key in ("schemes", "scheme_round_robin", "p", "q"):
            if key in wl:
                job[key] = wl[key]
        jobs.append(job)
    return jobs

# Algorithmic bytes per walker-step (the roofline numerator): bytes touched at
# 32 B sector granularity by the reference's access pattern.  An int64 offset
# pair (16 B) spans 1.25 sectors on average (40 B); a 12 B alias bucket spans
# 1.25 sectors (40 B); the candidate's neighbour id is one sector (32 B); the
# 4 B path write is merged by L2 into full sectors (4 B).
#   alias DeepWalk: 40 + 40 + 32 + 4 = 116;  unweighted PPR: 40 + 32 + 4 = 76.
B_STEP = {"deepwalk": 40 + 40 + 32 + 4, "ppr": 40 + 32 + 4}


def design_bytes_per_step(app, best):
    """Bytes this engine's layout touches per step, at 32 B sectors, under the
    tuned options.  Alias DeepWalk: a cursor bucket (layout 0) carries the next
    vertex and its adjacency position, so a step reads one 32 B sector; index
    or 16 B neighbour buckets (layouts 1, 2) add the next vertex's offset pair
    (40 B, in L2 while the offsets fit).  Unweighted PPR: a cursor-adjacency
    entry (one sector) or the offset pair and the neighbour id.  Each adds the
    4 B path write."""
    if app == "deepwalk":
        return 32 + 4 if best.get("alias_layout", 2) == 0 else 32 + 40 + 4
    if app == "ppr":
        return 32 + 4 if best.get("cursor_adjacency", 0) else 40 + 32 + 4
    return None


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce(world, value, op):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def rank_walkers(rank, walkers):
    """Walker ids of a rank: every rank walks `walkers` walkers (weak scaling),
    rank r the global ids [r * walkers, (r + 1) * walkers).  The stream is
    keyed by the global id, so the ranks' paths together are the paths of one
    walk over all of them."""
    return rank * walkers, walkers


def walk_kwargs(wl):
    kw = {}
    for k in ("walk_length", "terminate_prob", "p", "q", "schemes", "scheme_round_robin"):
        if k in wl:
            kw[k] = wl[k]
    return kw


def cpu_sample(g, wl, walkers, threads, seed, target_s=10.0, chunks=16):
    """Times the oracle (CPU restatement) on a bounded sample of the workload,
    about target_s seconds of walking on `threads` host threads.

    Alias tables (weighted) are built once for the whole graph and their time
    is charged per walker (t_alias * sample/walkers); the walk runs `chunks`
    contiguous walker-id ranges spread over the id space, sized from a short
    calibration walk.
    """
    from oracle import pyoracle
    csr = pyoracle.CSR(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))
    weighted = g.get("w") is not None
    kw = walk_kwargs(wl)
    t_alias = 0.0
    if weighted:
        t0 = time.perf_counter()
        pyoracle.alias_build(csr, threads=threads)
        t_alias = time.perf_counter() - t0

    def run(n_per_chunk):
        steps, t_walk, n_done = 0, 0.0, 0
        for c in range(chunks):
            begin = (walkers // chunks) * c
            prm = pyoracle.make_params(wl["app"], seed=seed, walker_begin=begin, walker_num=n_per_chunk,
                                       weighted=weighted, **kw)
            _, _, st = pyoracle.walk(csr, prm, cap=1, threads=threads, with_paths=False)
            steps += st
            t_walk += pyoracle.last_timing()[1]
            n_done += n_per_chunk
        return steps, t_walk, n_done

    chunk = max(1, min(walkers // chunks, 256))
    steps, t_walk, n_done = run(chunk)
    for _ in range(2):  # grow the sample toward target_s (per-call costs make small runs misleading)
        if t_walk >= 0.5 * target_s or chunk >= walkers // chunks:
            break
        chunk = max(1, min(walkers // chunks, int(chunk * target_s / max(t_walk, 1e-6))))
        steps, t_walk, n_done = run(chunk)
    t_total = t_walk + t_alias * (n_done / walkers)
    return {
        "value": steps / t_total, "unit": "walker-steps/s", "cores": threads, "kind": "port",
        "seconds": t_total,
        "sample": "%d walkers in %d id ranges spread over %d (%d steps, %.2f s walking); alias build over the "
                  "full graph %.2f s charged pro rata" % (n_done, chunks, walkers, steps, t_walk, t_alias),
    }


def walk_kernel_name(app, best):
    """The walk kernel the engine launches under the tuned options."""
    if best.get("walk_schedule", 0) == 1:
        return "walk_pool_kernel"
    if best.get("walk_multi", 1) > 1 and app in ("deepwalk", "ppr"):
        return "walk_multi_kernel<%d>" % best["walk_multi"]
    return "walk_static_kernel"


def run_reference(args, wl, world, rank, local):
    """The reference's CPU path (its C restatement, pinned to the reference) on all host cores."""
    if rank != 0:
        return
    from oracle import pyoracle
    pyoracle.build()
    g = pyoracle.rmat_graph(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=wl["types"])
    walkers = g["V"] if wl["app"] != "node2vec" or wl["scale"] != 16 else 65536
    threads = os.cpu_count() or 1
    vals = []
    # each step: a bounded sample of ~2 s of walking, so the whole run stays
    # within a few minutes
    for _ in range(args.warmup):
        cpu_sample(g, wl, walkers, threads, seed=1, target_s=0.5, chunks=4)
    for _ in range(args.steps):
        vals.append(cpu_sample(g, wl, walkers, threads, seed=1, target_s=2.0))
    value = statistics.median(v["value"] for v in vals)
    line = {
        "impl": "reference", "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(v["seconds"] for v in vals), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
        "config": {"workload": args.workload, "desc": wl["desc"], "walkers": walkers},
        "cpu_baseline": dict(vals[-1], value=value),
        "e2e": {"value": value, "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def serve_requests(wl, V, seed=5):
    """The served workload's request stream (seeded)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(wl["serve"]):
        walkers = int(np.clip(round(rng.lognormal(np.log(4096), 1.0)), 1, 1 << 20))
        reqs.append(dict(walker_num=walkers, seed=1000 + i, walk_length=int(rng.integers(5, 201)),
                         p=float(np.exp(rng.uniform(np.log(0.25), np.log(4.0)))),
                         q=float(np.exp(rng.uniform(np.log(0.25), np.log(4.0)))),
                         walker_begin=int(rng.integers(0, V)), weighted=bool(wl["weights"])))
    return reqs


def run_serve_bench(args, wl, world, rank, local):
    """Served request stream (continuous batching on two slots) against plain
    per-request launches and device-side batches of the same requests.

    value = saturated serving throughput: every request submitted at once,
    walker-steps over first submit -> last paths on the host.  Latency: an
    open-loop Poisson stream at 70% of that throughput, p50/p99 of submit ->
    paths on the host.  plain: one kk_walk_device per request (alias tables
    kept, or rebuilt per call as the reference's random_walk does)."""
    import numpy as np
    import torch

    import knightking_gb300 as kk

    torch.cuda.set_device(local)
    engine = kk.WalkEngine(local)
    engine.generate_rmat(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=wl["types"])
    V, E, _, _ = engine.info()
    app = wl["app"]
    reqs = serve_requests(wl, V)
    total_req_steps_cap = sum(r["walker_num"] * r["walk_length"] for r in reqs)
    stream = torch.cuda.Stream()
    engine.set_stream(stream.cuda_stream)

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        steps = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return steps, e0.elapsed_time(e1)

    def plain(rs):
        steps = 0
        for r in rs:
            kw = dict(r)
            steps += engine.walk_device(app, kw.pop("walker_num"), paths="unpacked", **kw)[0]
        return steps

    def batched(rs):
        steps = 0
        for k in range(0, len(rs), 1024):
            steps += engine.batch_walk_device(app, rs[k:k + 1024], paths=True)
        return steps

    # tables resident (sorted adjacency, edge set, alias tables), then tune the
    # batch kernel on the whole stream
    engine.set_option("alias_cache", 1)
    from knightking_gb300 import tuning
    best, tune_table = tuning.autotune(engine, lambda: batched(reqs), tuning.space_for(app, bool(wl["weights"])),
                                      repeats=1)
    for _ in range(args.warmup):
        batched(reqs[:64])
        plain(reqs[:8])
    barrier(world)
    n_plain = min(len(reqs), 300)
    with ClockSampler(local) as clocks:
        time.sleep(0.5)
        b_steps, b_ms = timed(lambda: batched(reqs))
        p_steps, p_ms = timed(lambda: plain(reqs[:n_plain]))
        engine.set_option("alias_cache", 0)
        r_steps, r_ms = timed(lambda: plain(reqs[:12]))
        engine.set_option("alias_cache", 1)
        # saturated serving (after one untimed pass that fills the server's
        # pinned result pool)
        srv = engine.serve(app, slots=2, max_jobs=256, slot_bytes=2 << 30)
        for t in [srv.submit(**r) for r in reqs]:
            srv.poll(t, keep_paths=False)
        srv.reset_stats()
        t0 = time.perf_counter()
        tickets = [srv.submit(**r) for r in reqs]
        s_steps = 0
        for t in tickets:
            res = srv.poll(t, keep_paths=False)
            assert res.status == 0
            s_steps += res.total_steps
        s_s = time.perf_counter() - t0
        sat = srv.stats()
    served_value = s_steps / s_s
    # latency under an open-loop Poisson stream at 70% of the saturated rate
    rate = 0.7 * served_value / (s_steps / len(reqs))
    rng = np.random.default_rng(11)
    gaps = rng.exponential(1.0 / rate, len(reqs))
    srv.reset_stats()
    results = [None] * len(reqs)

    def poller(ts):
        for i, t in ts:
            results[i] = srv.poll(t, keep_paths=False)

    import threading
    t_start = time.perf_counter()
    due = t_start
    pending = []
    pollers = []
    for i, r in enumerate(reqs):
        due += gaps[i]
        d = due - time.perf_counter()
        if d > 0:
            time.sleep(d)
        pending.append((i, srv.submit(**r)))
        if len(pending) == 64:
            th = threading.Thread(target=poller, args=(pending,))
            th.start()
            pollers.append(th)
            pending = []
    if pending:
        th = threading.Thread(target=poller, args=(pending,))
        th.start()
        pollers.append(th)
    for th in pollers:
        th.join()
    open_s = time.perf_counter() - t_start
    lat = srv.stats()
    srv.stop()
    open_steps = sum(r.total_steps for r in results)

    # access counts of the stream (binary-search probe counts), for the byte model
    engine.set_option("walk_stats", 1)
    engine.set_option("node2vec_adjacency", 1)
    c_steps = batched(reqs[:1024])
    trials, queries, probes = engine.last_stats()
    engine.set_option("walk_stats", 0)
    engine.set_option("node2vec_adjacency", best.get("node2vec_adjacency", 0))
    T, Q, P = trials / c_steps, queries / c_steps, probes / c_steps
    b_step = 40 + T * (40 + 32) + P * 32 + 4
    design_b = 40 + T * 32 + Q * 32 + 4
    peak, peak_kind = load_peaks()
    batched_value = b_steps / (b_ms / 1e3)
    plain_value = p_steps / (p_ms / 1e3)
    rebuild_value = r_steps / (r_ms / 1e3)
    achieved = batched_value * b_step / 1e9
    ceiling = engine.gather_ceiling(4 << 30)
    if rank == 0:
        line = {
            "metric": "walker-steps/s", "value": served_value, "unit": "walker-steps/s", "n_gpus": world,
            "steps": 1, "warmup": args.warmup, "ms_per_step": s_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded R-MAT generated on the GPU, seeded request stream)",
            "config": {"workload": args.workload, "desc": wl["desc"], "vertices": V, "edges": E,
                       "requests": len(reqs), "walker_step_capacity": total_req_steps_cap,
                       "parallelism": "replicas", "l2": "inputs larger than L2", "slots": 2, "max_jobs": 256,
                       "tuned": best, "tuning_ms": [[c, ms] for c, ms in tune_table]},
            "served": {"value": served_value, "what": "all requests submitted at once; submit -> paths on host",
                       "batches": sat["batches"], "mean_batch_jobs": sat["mean_batch_jobs"],
                       "slot_time_ms": {"walk": sat["walk_ms"], "copy_to_pinned": sat["copy_ms"],
                                        "per_request_copies": sat["host_ms"]}},
            "latency": {"offered_rate_req_s": rate, "p50_ms": lat["p50_ms"], "p99_ms": lat["p99_ms"],
                        "mean_ms": lat["mean_ms"], "throughput": open_steps / open_s,
                        "what": "open-loop Poisson arrivals at 70% of the saturated rate"},
            "batched": {"value": batched_value, "unit": "walker-steps/s", "ms": b_ms,
                        "what": "kk_batch_walk_device, 1024 requests per launch, paths in HBM"},
            "plain": {"value": plain_value, "unit": "walker-steps/s", "requests": n_plain,
                      "what": "one kk_walk_device launch per request, alias tables kept"},
            "plain_rebuild": {"value": rebuild_value, "unit": "walker-steps/s", "requests": 12,
                              "what": "one launch per request, alias tables rebuilt per call (reference)"},
            "served_over_plain": served_value / plain_value,
            "batched_over_plain": batched_value / plain_value,
            "e2e": {"value": served_value, "unit": "walker-steps/s",
                    "h2d_bytes_per_step": len(reqs) * 120, "d2h_bytes_per_step": 4 * (s_steps + sum(
                        r["walker_num"] for r in reqs))},
            "gpu_launches": sat["batches"],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                         "bytes_per_step": b_step, "design_bytes_per_step": design_b,
                         "access_counts": {"trials_per_step": T, "queries_per_step": Q, "probes_per_step": P},
                         "kernel": "walk_batch_kernel (second order), from the batched throughput",
                         "gather": {"ceiling_reads_per_s": ceiling, "reads_per_step": T + Q,
                                    "achieved_reads_per_s": batched_value * (T + Q),
                                    "frac": batched_value * (T + Q) / ceiling,
                                    "what": "alias buckets + edge-set sectors per step (batched throughput) vs "
                                            "kk_gather_ceiling (4 GiB, this GPU, this run)"}},
            "cpu_baseline": None, "clocks": clocks.summary(),
        }
        print(json.dumps(line))


def run_batch_bench(args, wl, world, rank, local):
    """Batched jobs in one launch vs one launch per job (the reference runs one
    random_walk() call per job), same jobs, same graph, timed back to back."""
    import torch

    import knightking_gb300 as kk

    torch.cuda.set_device(local)
    engine = kk.WalkEngine(local)
    engine.generate_rmat(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=wl["types"])
    V, E, _, _ = engine.info()
    jobs = batch_jobs(wl)
    for j in jobs:
        j["walker_begin"] = rank * (1 << 22)
    app = wl["app"]
    stream = torch.cuda.Stream()
    engine.set_stream(stream.cuda_stream)

    def batched():
        return engine.batch_walk_device(app, jobs, paths=True)

    def plain():
        steps = 0
        for j in jobs:
            kw = dict(j)
            steps += engine.walk_device(app, kw.pop("walker_num"), paths="unpacked", **kw)[0]
        return steps

    def timed(fn, k):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        steps = sum(fn() for _ in range(k))
        e1.record(stream)
        torch.cuda.synchronize()
        return steps, e0.elapsed_time(e1)

    for _ in range(args.warmup):
        batched()
        plain()
    barrier(world)
    with ClockSampler(local) as clocks:
        time.sleep(0.5)
        l0 = engine.launch_count()
        b_steps, b_ms = timed(batched, args.steps)
        b_launches = engine.launch_count() - l0
        p_steps, p_ms = timed(plain, args.steps)
    b_ms = allreduce(world, b_ms, "max")
    p_ms = allreduce(world, p_ms, "max")
    value = allreduce(world, float(b_steps), "sum") / (b_ms / 1e3)
    plain_value = allreduce(world, float(p_steps), "sum") / (p_ms / 1e3)
    # e2e: the batch through the C-ABI call kk_batch_walk, every job's lengths,
    # offsets and packed paths copied into host memory (pinned blocks the
    # library hands out); one untimed call first fills the pinned pool
    engine.batch_walk(app, jobs, keep_paths=False)
    t0 = time.perf_counter()
    e_steps = 0
    d2h = 0
    e2e_runs = max(1, args.steps)  # the same K as the device-timed loop
    for _ in range(e2e_runs):
        res = engine.batch_walk(app, jobs, keep_paths=False)
        e_steps += sum(r["total_steps"] for r in res)
        d2h += sum(r["walker_num"] * 12 + r["vertices"] * 4 for r in res)
    e2e_s = allreduce(world, time.perf_counter() - t0, "max")
    e2e_value = allreduce(world, float(e_steps), "sum") / e2e_s
    cpu = None
    if rank == 0 and not args.no_cpu:
        g = engine.download_graph()
        cpu = cpu_sample(g, dict(wl, walk_length=max(j["walk_length"] for j in jobs)), V, os.cpu_count() or 1,
                         seed=1)
    if rank == 0:
        line = {
            "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": b_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded R-MAT generated on the GPU)",
            "config": {"workload": args.workload, "desc": wl["desc"], "vertices": V, "edges": E,
                       "jobs": [[j["walker_num"], j["walk_length"]] for j in jobs],
                       "walker_steps_per_step": b_steps / args.steps, "parallelism": "replicas",
                       "l2": "inputs larger than L2"},
            "plain": {"value": plain_value, "unit": "walker-steps/s", "ms_per_step": p_ms / args.steps,
                      "what": "one kk_walk_device launch per job, alias tables rebuilt per job"},
            "batched_over_plain": value / plain_value,
            "e2e": {"value": e2e_value, "unit": "walker-steps/s", "h2d_bytes_per_step": 64 * len(jobs),
                    "d2h_bytes_per_step": d2h // e2e_runs},
            "gpu_launches": b_launches,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    engine.close()


def run_ours(args, wl, world, rank, local):
    import numpy as np
    import torch

    import knightking_gb300 as kk

    torch.cuda.set_device(local)
    engine = kk.WalkEngine(local)
    engine.generate_rmat(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=wl["types"])
    V, E, _, _ = engine.info()
    walkers = V if not (wl["app"] == "node2vec" and wl["scale"] == 16) else 65536
    walker_begin, walkers = rank_walkers(rank, walkers)
    kw = walk_kwargs(wl)
    stream = torch.cuda.Stream()
    engine.set_stream(stream.cuda_stream)
    app = wl["app"]

    def step():
        # paths are written to HBM as the walk produces them (no compaction pass)
        steps, _, _, _ = engine.walk_device(app, walkers, paths="unpacked", seed=1, walker_begin=walker_begin, **kw)
        return steps

    # warm-up; it also runs the engine's autotuner (knightking_gb300.tuning):
    # alias-table layout, node2vec adjacency test, walk block size, L2 fetch
    # hint and walk schedule, each picked by the event time of alias build + walk
    from knightking_gb300 import tuning
    best, tune_table = tuning.autotune(engine, step, tuning.space_for(app, bool(wl["weights"])))
    best_schedule = best.get("walk_schedule", 0)
    for _ in range(args.warmup):
        step()
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    total_steps = 0
    walk_ms = []
    alias_ms = []
    with ClockSampler(local) as clocks:
        time.sleep(0.5)  # nvidia-smi's first sample lands inside the timed region
        ev0.record(stream)
        l0 = engine.launch_count()
        for _ in range(args.steps):
            total_steps += step()
            a, w = engine.last_timing()
            alias_ms.append(a)
            walk_ms.append(w)
        ev1.record(stream)
        torch.cuda.synchronize()
        launches = engine.launch_count() - l0
    elapsed_ms = ev0.elapsed_time(ev1)
    barrier(world)
    elapsed_ms = allreduce(world, elapsed_ms, "max")
    all_steps = allreduce(world, float(total_steps), "sum")
    value = all_steps / (elapsed_ms / 1e3)

    # ---- e2e: public C-ABI call with host buffers and copies in the timed region ----
    # the start list lives in pinned host memory, as the step's inputs should
    start_pin = torch.empty(walkers, dtype=torch.int32, pin_memory=True)
    start = start_pin.numpy().view(np.uint32)
    start[:] = np.arange(walkers, dtype=np.uint32) % np.uint32(V)
    cap_per = (wl.get("walk_length", 0) + 1) if "walk_length" in wl else 0
    if cap_per == 0:
        cap_vertices = int(total_steps // args.steps) + walkers + 1024
    else:
        cap_vertices = walkers * cap_per
    h_len = torch.empty(walkers, dtype=torch.int32, pin_memory=True)
    h_off = torch.empty(walkers, dtype=torch.int64, pin_memory=True)
    h_vert = torch.empty(cap_vertices, dtype=torch.int32, pin_memory=True)
    e2e_steps = 0
    e2e_runs = max(1, args.steps)  # the same K as the device-timed loop
    engine.walk_into(app, walkers, h_len.data_ptr(), h_off.data_ptr(), h_vert.data_ptr(), cap_vertices, seed=1,
                     walker_begin=walker_begin, start=start, **kw)
    barrier(world)
    t0 = time.perf_counter()
    d2h = 0
    call_ms = []
    for _ in range(e2e_runs):
        tc = time.perf_counter()
        st = engine.walk_into(app, walkers, h_len.data_ptr(), h_off.data_ptr(), h_vert.data_ptr(), cap_vertices,
                              seed=1, walker_begin=walker_begin, start=start, **kw)
        call_ms.append(round((time.perf_counter() - tc) * 1e3, 3))
        e2e_steps += st
        d2h += walkers * 4 + walkers * 8 + (st + walkers) * 4
    e2e_s = time.perf_counter() - t0
    e2e_s = allreduce(world, e2e_s, "max")
    e2e_value = allreduce(world, float(e2e_steps), "sum") / e2e_s

    # ---- roofline of the walk kernel ----
    peak, peak_kind = load_peaks()
    steps_per_launch = total_steps / args.steps
    b_step = B_STEP.get(app)
    design_b = design_bytes_per_step(app, best)
    counts = None
    if app in ("node2vec", "metapath"):
        # one counted walk after the timed region (same paths): trials per step
        # and the probes a binary search of the query targets' adjacency takes
        # give the byte model of a rejection-sampled step
        engine.set_option("walk_stats", 1)
        adj = best.get("node2vec_adjacency", 0)
        if app == "node2vec":
            engine.set_option("node2vec_adjacency", 1)
        st_steps = step()
        trials, queries, probes = engine.last_stats()
        engine.set_option("walk_stats", 0)
        if app == "node2vec":
            engine.set_option("node2vec_adjacency", adj)
        T, Q, P = trials / st_steps, queries / st_steps, probes / st_steps
        counts = {"trials_per_step": T, "queries_per_step": Q, "probes_per_step": P}
        if app == "node2vec":
            # offsets 40 + T x (bucket 40 + neighbour 32) + probes x 32 + path 4
            b_step = 40 + T * (40 + 32) + P * 32 + 4
            # this engine: offsets 40 + T x one 32 B bucket + one edge-set sector per query + path 4
            design_b = 40 + T * 32 + Q * 32 + 4
        else:
            # vertex mask 32 + offsets 40 + T x (bucket 40 + type 32) + neighbour 32 + path 4
            b_step = 32 + 40 + T * (40 + 32) + 32 + 4
            # this engine: mask 32 + offsets 40 + T x (bucket 32 + type 32) + path 4
            design_b = 32 + 40 + T * (32 + 32) + 4
    mean_walk_ms = statistics.mean(walk_ms)
    roof = None
    if b_step is not None:
        achieved = steps_per_launch * b_step / (mean_walk_ms / 1e3) / 1e9
        traffic = None
        tf = os.path.join(ROOT, "profiles", "traffic_%s.json" % args.workload)
        if os.path.exists(tf):
            with open(tf) as f:
                per_kernel = json.load(f)["dram_bytes_per_step"]
            # ncu's DRAM bytes per step of the kernel this run launched
            b = per_kernel.get(walk_kernel_name(app, best)) if isinstance(per_kernel, dict) else per_kernel
            traffic = b * steps_per_launch if b is not None else None
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_kind": peak_kind, "bytes_per_step": b_step,
                "design_bytes_per_step": design_b, "access_counts": counts,
                "kernel": walk_kernel_name(app, best) + (" (second order)" if app == "node2vec" else " (first order)"),
                "kernel_ms": mean_walk_ms, "alias_build_ms": statistics.mean(alias_ms)}

    # ---- the random-gather ceiling: dependent random 32 B reads per second
    # over 4 GiB, measured on this GPU now; each step of these walks makes
    # reads_per_step such reads into structures far larger than L2 ----
    ceiling = engine.gather_ceiling(4 << 30)
    if app == "deepwalk":
        rps = 1.0  # one alias bucket (index or cursor layout); offsets of S22 sit in L2
    elif app == "ppr":
        rps = 1.0 if best.get("cursor_adjacency", 0) else 2.0  # cursor adjacency entry, or offsets + neighbour
    elif counts is not None and app == "node2vec":
        rps = counts["trials_per_step"] + counts["queries_per_step"]  # buckets + edge-set sectors
    elif counts is not None:
        rps = counts["trials_per_step"]  # buckets (edge types ride in them)
    else:
        rps = None
    steps_per_s_kernel = steps_per_launch / (mean_walk_ms / 1e3)
    gather = None
    if rps is not None:
        gather = {"ceiling_reads_per_s": ceiling, "reads_per_step": rps,
                  "achieved_reads_per_s": steps_per_s_kernel * rps,
                  "frac": steps_per_s_kernel * rps / ceiling, "kernel": roof["kernel"] if roof else None,
                  "what": "walk kernel's dependent random reads vs kk_gather_ceiling (4 GiB, this GPU, this run)"}
    if roof is not None:
        roof["gather"] = gather

    cpu = None
    if rank == 0 and not args.no_cpu:
        g = engine.download_graph()
        cpu = cpu_sample(g, wl, walkers, os.cpu_count() or 1, seed=1)

    if rank == 0:
        line = {
            "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded R-MAT generated on the GPU)",
            "config": {"workload": args.workload, "desc": wl["desc"], "vertices": V, "edges": E,
                       "walkers_per_gpu": walkers, "walker_steps_per_step": steps_per_launch,
                       "l2": "inputs larger than L2 (graph + alias tables > 129 MB)", "parallelism": "replicas",
                       "walk_schedule": "pool" if best_schedule == 1 else "one walker per thread",
                       "tuned": best,
                       "tuning_ms": [[cfg, ms] for cfg, ms in tune_table]},
            "e2e": {"value": e2e_value, "unit": "walker-steps/s", "h2d_bytes_per_step": walkers * 4 + 256,
                    "d2h_bytes_per_step": d2h // e2e_runs, "call_ms": call_ms},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    engine.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="deepwalk-s22", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--scale", type=int, default=None, help="override the R-MAT scale (profiling on a small case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = dict(WORKLOADS[args.workload])
    if args.scale is not None:
        wl["scale"] = args.scale
        wl["desc"] += " (scale overridden to %d)" % args.scale
        args.workload += "@s%d" % args.scale
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, wl, world, rank, local)
    elif "batch" in wl:
        run_batch_bench(args, wl, world, rank, local)
    elif "serve" in wl:
        run_serve_bench(args, wl, world, rank, local)
    else:
        run_ours(args, wl, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
