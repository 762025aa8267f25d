#!/usr/bin/env python3
"""Walker-step benchmark (one JSON line on rank 0).

Default workload (node2vec-serve-s24): a served node2vec request stream on a
resident R-MAT scale-24 weighted graph (edge factor 16, a/b/c = 0.57/0.19/0.19,
undirected, uniform [1,5) float32 weights): 3000 requests, per request p and q
log-uniform in [0.25, 4], length uniform in [5, 200], walkers lognormal (median
4096) clipped to [1, 2^20].  A step is one pass of the whole stream.

value : walker-steps/s of the stream through the batched kernel
        (kk_batch_walk_device, 1024 requests per launch from request tables
        built before the timed region, paths in HBM), device time from CUDA
        events on the engine's stream; the plain one-launch-per-request kernel
        is timed beside it (batched_over_plain).
e2e   : the same stream through the serving C-ABI (kk_serve_submit/poll,
        driven by the library's own client kk_serve_replay): job records
        host->device, every path device->host into pinned memory, inside the
        timed region (served_over_plain); p50/p99 latency of open-loop Poisson
        streams at 30%, 50% and 70% of that rate.
roofline: the walk kernel's bytes touched per walker-step at 32-byte sector
        granularity (the reference's access pattern) over its CUDA-event
        duration per launch, against the measured HBM copy bandwidth; beside it
        the fraction of the measured random-gather ceiling.
parity: the benchmarked walks' paths against the oracle (the C restatement,
        pinned bit for bit to the reference), walker for walker, on the
        benchmarked graph.
cpu_baseline / --impl reference: the oracle on all host cores over a bounded
        sample of the same workload.

The default run also measures weighted DeepWalk on R-MAT scale 22 (alias build
inside every step; e2e through kk_walk_into) and reports it under "also".
Other workloads: --workload (single walks, batches of jobs, and ingest-s22, the
load of a binary edge file into a CSR in HBM, in edges/s).

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

import numpy as np

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
    "ingest-s22": dict(app=None, scale=22, weights=1, types=0, ingest=True,
                       desc="graph ingestion: binary Edge<float> file (src u32, dst u32, weight f32 per record) of "
                            "the R-MAT scale 22 ef16 uniform[1,5) graph, each undirected edge once in a seeded "
                            "shuffled order, loaded with --make-undirected into a CSR in HBM"),
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


def oracle_cap(app, wl, gpu_lens=None):
    """Path capacity (vertices per walker) for an oracle walk of the workload."""
    if "walk_length" in wl:
        return wl["walk_length"] + 1
    return int(gpu_lens.max()) + 1 if gpu_lens is not None and len(gpu_lens) else 4096


def host_graph(engine, app, threads):
    """The engine's graph on the host for the oracle (bit-identical to the
    device's: the same seeded generator, downloaded), with the weight alias
    tables built once by the oracle.  Returns (csr, alias, alias_seconds)."""
    from oracle import pyoracle
    g = engine.download_graph()
    csr = pyoracle.CSR(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))
    alias, t_alias = None, 0.0
    if csr.w is not None:
        t0 = time.perf_counter()
        alias = pyoracle.alias_build(csr, threads=threads)
        t_alias = time.perf_counter() - t0
    return csr, alias, t_alias


def count_mismatches(lens_a, verts_a, lens_b, verts_b):
    """Walkers whose paths differ between two packed path sets of the same walkers."""
    lens_a = np.asarray(lens_a, np.int64)
    lens_b = np.asarray(lens_b, np.int64)
    if len(lens_a) != len(lens_b):
        return max(len(lens_a), len(lens_b))
    oa = np.zeros(len(lens_a) + 1, np.int64)
    ob = np.zeros(len(lens_b) + 1, np.int64)
    np.cumsum(lens_a, out=oa[1:])
    np.cumsum(lens_b, out=ob[1:])
    if np.array_equal(lens_a, lens_b) and len(verts_a) == len(verts_b):
        diff = np.asarray(verts_a) != np.asarray(verts_b)
        if not diff.any():
            return 0
        per = np.add.reduceat(diff.astype(np.int64), oa[:-1]) if len(diff) else np.zeros(0)
        return int(((per > 0) & (lens_a > 0)).sum())
    bad = 0
    for i in range(len(lens_a)):
        if lens_a[i] != lens_b[i] or not np.array_equal(verts_a[oa[i]:oa[i + 1]], verts_b[ob[i]:ob[i + 1]]):
            bad += 1
    return bad


def oracle_paths(csr, alias, app, threads, cap, **prm_kw):
    """The oracle's paths (lens, flat vertices, steps) of one walk; a path
    longer than cap raises."""
    from oracle import pyoracle
    prm = pyoracle.make_params(app, **prm_kw)
    return pyoracle.walk(csr, prm, cap=cap, threads=threads, alias=alias)


def parity_ranges(engine, csr, alias, wl, walkers, threads, chunks=16, per=8192):
    """Bit-for-bit parity of the benchmarked walk on the benchmarked graph:
    `chunks` walker-id ranges of `per` walkers spread over the id space, each
    walked by the engine (kk_walk, paths to the host) and by the oracle."""
    app = wl["app"]
    kw = walk_kwargs(wl)
    weighted = csr.w is not None
    checked = mism = steps = 0
    for c in range(chunks):
        begin = (walkers // chunks) * c
        n = min(per, walkers - begin)
        if n <= 0:
            continue
        ps = engine.walk(app, n, seed=1, walker_begin=begin, weighted=weighted, **kw)
        try:
            lens, verts, st = oracle_paths(csr, alias, app, threads, oracle_cap(app, wl, ps.path_length), seed=1,
                                           walker_begin=begin, walker_num=n, weighted=weighted, **kw)
            mism += count_mismatches(ps.path_length, ps.vertices, lens, verts)
        except RuntimeError:
            mism += n
            st = 0
        checked += n
        steps += st
        del ps
    return {"walkers_checked": checked, "mismatches": mism, "steps_checked": steps,
            "what": "%d walker-id ranges of %d walkers spread over %d: kk_walk paths vs the oracle (pinned to "
                    "the reference), bit for bit" % (chunks, per, walkers)}


def cpu_sample(csr, alias, t_alias, wl, walkers, threads, seed, target_s=10.0, chunks=16):
    """Times the oracle (CPU restatement) on a bounded sample of the workload,
    about target_s seconds of walking on `threads` host threads, without path
    output (the reference's pure-performance mode).

    Alias tables (weighted) are built once for the whole graph (t_alias) and
    their time is charged per walker (t_alias * sample/walkers); the walk runs
    `chunks` contiguous walker-id ranges spread over the id space, sized from
    a short calibration walk.
    """
    from oracle import pyoracle
    weighted = csr.w is not None
    kw = walk_kwargs(wl)

    def run(n_per_chunk):
        steps, t_walk, n_done = 0, 0.0, 0
        for c in range(chunks):
            begin = (walkers // chunks) * c
            prm = pyoracle.make_params(wl["app"], seed=seed, walker_begin=begin, walker_num=n_per_chunk,
                                       weighted=weighted, **kw)
            _, _, st = pyoracle.walk(csr, prm, cap=1, threads=threads, with_paths=False, alias=alias)
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


def cpu_sample_requests(csr, alias, t_alias, reqs, first, threads, target_s=10.0):
    """Times the oracle on a bounded sample of the served request stream: the
    requests from position `first` on, each as one plain node2vec() call
    (src/apps/node2vec.hpp:108-202) run one after the other, until about
    target_s seconds of walking.  The reference's random_walk rebuilds the
    whole graph's alias tables in every call (include/walk.hpp:538-652); here
    they are built once and charged to the sample pro rata by walker-steps
    against the whole stream (a CPU baseline favourable to the CPU)."""
    from oracle import pyoracle
    steps, t_walk, n = 0, 0.0, 0
    i = first
    while t_walk < target_s and n < len(reqs):
        r = reqs[i % len(reqs)]
        prm = pyoracle.make_params("node2vec", seed=r["seed"], walker_begin=r["walker_begin"],
                                   walker_num=r["walker_num"], walk_length=r["walk_length"], p=r["p"], q=r["q"],
                                   weighted=r["weighted"])
        _, _, st = pyoracle.walk(csr, prm, cap=1, threads=threads, with_paths=False, alias=alias)
        steps += st
        t_walk += pyoracle.last_timing()[1]
        n += 1
        i += 1
    stream_cap = sum(r["walker_num"] * r["walk_length"] for r in reqs)
    charged = t_alias * min(1.0, steps / max(stream_cap, 1))
    t_total = t_walk + charged
    return {
        "value": steps / t_total, "unit": "walker-steps/s", "cores": threads, "kind": "port",
        "seconds": t_total,
        "sample": "%d requests of the stream from request %d, each one node2vec() call in turn (%d steps, %.2f s "
                  "walking); alias build over the full graph %.2f s, charged %.3f s pro rata by steps (the "
                  "reference rebuilds it in every call)" % (n, first, steps, t_walk, t_alias, charged),
        "alias_build_s_per_call": t_alias,
    }, i


def walk_kernel_name(app, best):
    """The walk kernel the engine launches under the tuned options."""
    if best.get("walk_schedule", 0) == 1:
        return "walk_pool_kernel"
    if best.get("walk_multi", 1) > 1 and app in ("deepwalk", "ppr"):
        return "walk_multi_kernel<%d>" % best["walk_multi"]
    return "walk_static_kernel"


def run_reference(args, wl, world, rank, local):
    """The reference's CPU path (its C restatement, pinned to the reference)
    on all host cores, on the workload's graph generated on the CPU."""
    if rank != 0:
        return
    from oracle import pyoracle
    pyoracle.build()
    threads = os.cpu_count() or 1
    if "ingest" in wl:
        return run_reference_ingest(args, wl, world, threads)
    t0 = time.perf_counter()
    g = pyoracle.rmat_graph(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=wl["types"],
                            threads=threads)
    csr = pyoracle.CSR(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))
    del g
    t_gen = time.perf_counter() - t0
    alias, t_alias = None, 0.0
    if csr.w is not None:
        t0 = time.perf_counter()
        alias = pyoracle.alias_build(csr, threads=threads)
        t_alias = time.perf_counter() - t0
    vals = []
    if "serve" in wl:
        reqs = serve_requests(wl, csr.V)
        pos = 0
        for _ in range(args.warmup):
            _, pos = cpu_sample_requests(csr, alias, t_alias, reqs, pos, threads, target_s=0.3)
        for _ in range(args.steps):
            v, pos = cpu_sample_requests(csr, alias, t_alias, reqs, pos, threads, target_s=2.0)
            vals.append(v)
        walkers = None
    else:
        walkers = csr.V if wl["app"] != "node2vec" or wl["scale"] != 16 else 65536
        # each step: a bounded sample of ~2 s of walking, so the whole run stays
        # within a few minutes
        for _ in range(args.warmup):
            cpu_sample(csr, alias, t_alias, wl, walkers, threads, seed=1, target_s=0.5, chunks=4)
        for _ in range(args.steps):
            vals.append(cpu_sample(csr, alias, t_alias, wl, walkers, threads, seed=1, target_s=2.0))
    value = statistics.median(v["value"] for v in vals)
    line = {
        "impl": "reference", "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(v["seconds"] for v in vals), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
        "config": {"workload": args.workload, "desc": wl["desc"], "vertices": csr.V, "edges": csr.E,
                   "graph_generation_s": t_gen},
        "cpu_baseline": dict(vals[-1], value=value),
        "e2e": {"value": value, "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if walkers is not None:
        line["config"]["walkers"] = walkers
    print(json.dumps(line), flush=True)


def run_reference_ingest(args, wl, world, threads):
    """The reference's loader restated on the CPU (ingest_oracle) on the same
    file as the GPU arm's, a few whole-file steps (each takes seconds)."""
    import tempfile

    from oracle import pyoracle
    g = pyoracle.rmat_graph(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=0, threads=threads)
    V = g["V"]
    rec = ingest_records(V, g["off"], g["nbr"], g["w"])
    del g
    path = os.path.join(tempfile.gettempdir(), "kk_ingest_ref_s%d_%d.bin" % (wl["scale"], os.getpid()))
    rec.tofile(path)
    E = 2 * len(rec)
    del rec
    steps = min(args.steps, 3)
    try:
        ingest_oracle(V, path)
        secs = []
        for _ in range(steps):
            t0 = time.perf_counter()
            ingest_oracle(V, path)
            secs.append(time.perf_counter() - t0)
    finally:
        os.unlink(path)
    value = E / statistics.median(secs)
    line = {
        "impl": "reference", "metric": "edges/s", "value": value, "unit": "edges/s", "n_gpus": world,
        "steps": steps, "warmup": 1, "ms_per_step": 1e3 * statistics.median(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded R-MAT)",
        "config": {"workload": args.workload, "desc": wl["desc"], "vertices": V, "edges": E},
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": 1, "kind": "port",
                         "sample": "the whole file: read, mirror, stable sort by source, offsets (numpy)"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def serve_requests(wl, V, seed=5):
    """The served workload's request stream (seeded)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(wl["serve"]):
        walkers = int(np.clip(round(rng.lognormal(np.log(4096), 1.0)), 1, 1 << 20))
        reqs.append(dict(walker_num=walkers, seed=1000 + i, walk_length=int(rng.integers(5, 201)),
                         p=float(np.exp(rng.uniform(np.log(0.25), np.log(4.0)))),
                         q=float(np.exp(rng.uniform(np.log(0.25), np.log(4.0)))),
                         walker_begin=int(rng.integers(0, V)), weighted=bool(wl["weights"])))
    return reqs


def parity_requests(results, csr, alias, reqs, threads, what):
    """Each served (or batched) request's paths against the oracle's node2vec
    walk of the same request; results[i] is (lens, verts) of reqs[i]."""
    checked = mism = steps = 0
    for (lens_g, verts_g), r in zip(results, reqs):
        lens, verts, st = oracle_paths(csr, alias, "node2vec", threads, r["walk_length"] + 1, seed=r["seed"],
                                       walker_begin=r["walker_begin"], walker_num=r["walker_num"],
                                       walk_length=r["walk_length"], p=r["p"], q=r["q"], weighted=r["weighted"])
        mism += count_mismatches(lens_g, verts_g, lens, verts)
        checked += r["walker_num"]
        steps += st
    return {"requests": len(reqs), "walkers_checked": checked, "mismatches": mism, "steps_checked": steps,
            "what": what}


def n2v_outlier(p, q):
    """Whether node2vec (p, q) is in the outlier regime: the overflow
    1/p - max(1, 1/q), computed in double and rounded to float as
    src/apps/node2vec.hpp:126-139 does, is positive."""
    ub = np.float32(max(1.0 / float(np.float32(q)), 1.0))
    return float(np.float32(1.0 / float(np.float32(p)) - float(ub))) > 0.0


SERVE_JOB_BYTES = 80  # one BatchJob record (walk.cuh), uploaded per job slot of a batch
LATENCY_LOADS = (0.3, 0.5, 0.7)  # open-loop offered load, fraction of the saturated served rate
LATENCY_HEAD = 0.5  # the load of the line's headline p50/p99


def run_serve_bench(args, wl, world, rank, local):
    """North-star workload: the served node2vec request stream on a resident
    R-MAT scale-24 weighted graph.

    value  : K passes of the whole stream through kk_batch_walk_device (1024
             requests per launch, paths in HBM), CUDA events on the engine's
             stream; the plain one-launch-per-request kernel is timed beside it.
    e2e    : K passes through the serving API (kk_serve_submit / kk_serve_poll
             from kk_serve_replay, the library's client): the K passes' requests
             submitted at once as one stream, each job record copied to the
             device and its paths copied back into pinned host memory; submit
             of the first -> paths of the last on the host.  One pass driven
             request by request from Python is reported beside it.
    latency: open-loop Poisson streams at 30%, 50% and 70% of the saturated
             rate, p50/p99 of submit -> paths on the host.
    parity : the first requests' served paths (and their kk_batch_walk paths)
             against the oracle, walker for walker."""
    import torch

    import knightking_gb300 as kk

    torch.cuda.set_device(local)
    engine = kk.WalkEngine(local)
    engine.generate_rmat(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"], types=wl["types"])
    V, E, _, _ = engine.info()
    app = wl["app"]
    reqs = serve_requests(wl, V)
    stream_cap = sum(r["walker_num"] * r["walk_length"] for r in reqs)
    stream = torch.cuda.Stream()
    engine.set_stream(stream.cuda_stream)
    kernel_ms = []

    def batched(rs, record=False):
        steps = 0
        for k in range(0, len(rs), 1024):
            steps += engine.batch_walk_device(app, rs[k:k + 1024], paths=True)
            if record:
                kernel_ms.append((engine.last_timing()[1], steps))
        return steps

    # the stream's job tables (kk_walk_opts arrays, 1024 requests each), built
    # once as a caller of the C-ABI would hold them
    tables = [engine.job_table(app, reqs[k:k + 1024]) for k in range(0, len(reqs), 1024)]

    def batched_tables(record=False):
        steps = 0
        for t in tables:
            steps += engine.batch_walk_device(app, t, paths=True)
            if record:
                kernel_ms.append((engine.last_timing()[1], steps))
        return steps

    def plain(rs):
        steps = 0
        for r in rs:
            kw = dict(r)
            steps += engine.walk_device(app, kw.pop("walker_num"), paths="unpacked", **kw)[0]
        return steps

    # the plain leg's requests as kk_walk_opts, built once like the batches' tables
    plain_opts = [engine.make_opts(app, r["walker_num"], **{k: v for k, v in r.items() if k != "walker_num"})
                  for r in reqs[:300]]

    def plain_prebuilt(n):
        return sum(engine.walk_device(app, 0, paths="unpacked", opts=o)[0] for o in plain_opts[:n])

    def timed(fn, k=1):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        steps = sum(fn() for _ in range(k))
        e1.record(stream)
        torch.cuda.synchronize()
        return steps, e0.elapsed_time(e1)

    # tables resident (sorted adjacency, edge set, alias tables), then tune the
    # batch kernel on the whole stream
    engine.set_option("alias_cache", 1)
    from knightking_gb300 import tuning
    best, tune_table = tuning.autotune(engine, lambda: batched(reqs),
                                      tuning.space_for(app, bool(wl["weights"]), batch=True),
                                      repeats=1)
    for _ in range(args.warmup):
        batched(reqs)
    plain(reqs[:8])
    barrier(world)
    n_plain = min(len(reqs), 300)
    srv = engine.serve(app, slots=2, max_jobs=256, slot_bytes=2 << 30)
    for t in [srv.submit(**r) for r in reqs]:  # fills the server's pinned result pool
        srv.poll(t, keep_paths=False)
    with ClockSampler(local) as clocks:
        time.sleep(0.5)
        l0 = engine.launch_count()
        kernel_ms.clear()
        b_steps, b_ms = timed(lambda: batched_tables(record=True), args.steps)
        launches = engine.launch_count() - l0
        p_steps, p_ms = timed(lambda: plain_prebuilt(n_plain))
        engine.set_option("alias_cache", 0)
        r_steps, r_ms = timed(lambda: plain_prebuilt(12))
        engine.set_option("alias_cache", 1)
        # e2e: K saturated passes through the server, every request of a
        # pass submitted at once by the library's own client (kk_serve_replay:
        # kk_serve_submit from one host thread, kk_serve_poll and
        # kk_paths_free of every result from another)
        # the K passes go in as one stream (K x 3000 requests, all at once),
        # so the server stays saturated across pass boundaries
        srv.reset_stats()
        _, s_steps, s_s = srv.replay(reqs * args.steps, np.zeros(len(reqs) * args.steps))
        sat = srv.stats()
        # one pass driven from Python (submit and poll per request through ctypes)
        t0 = time.perf_counter()
        py_steps = 0
        for t in [srv.submit(**r) for r in reqs]:
            res = srv.poll(t, keep_paths=False)
            assert res.status == 0
            py_steps += res.total_steps
        py_s = time.perf_counter() - t0
    b_ms = allreduce(world, b_ms, "max")
    value = allreduce(world, float(b_steps), "sum") / (b_ms / 1e3)
    served_value = allreduce(world, float(s_steps), "sum") / allreduce(world, s_s, "max")
    # latency under open-loop Poisson streams at 30%, 50% and 70% of the
    # saturated served rate, three passes of the stream each (the first pass
    # warms the server up and is not counted), kk_serve_replay keeping the
    # arrival schedule
    steps_per_req = s_steps / args.steps / len(reqs)
    curve = []
    for frac in LATENCY_LOADS:
        rate = frac * served_value / steps_per_req
        rng = np.random.default_rng(11)
        n_open = 3 * len(reqs)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n_open))
        lat_ms, o_steps, o_s = srv.replay([reqs[i % len(reqs)] for i in range(n_open)], arrivals)
        kept = lat_ms[len(reqs):]
        curve.append({"load": frac, "offered_req_s": rate, "offered_steps_s": rate * steps_per_req,
                      "p50_ms": float(np.percentile(kept, 50)), "p99_ms": float(np.percentile(kept, 99)),
                      "mean_ms": float(kept.mean()), "throughput": o_steps / o_s, "requests": int(len(kept))})
    head = next(c for c in curve if c["load"] == LATENCY_HEAD)
    # the parity sample: the stream's first requests up to >= 131072 walkers,
    # served with their paths kept, and the same requests through kk_batch_walk
    n_par, acc = 0, 0
    while n_par < len(reqs) and acc < 131072:
        acc += reqs[n_par]["walker_num"]
        n_par += 1
    par_reqs = reqs[:n_par]
    served_paths = []
    for t in [srv.submit(**r) for r in par_reqs]:
        res = srv.poll(t, keep_paths=True)
        assert res.status == 0
        served_paths.append((np.array(res.paths.path_length), np.array(res.paths.vertices)))
    srv.stop()
    batch_paths = [(np.array(ps.path_length), np.array(ps.vertices)) for ps in engine.batch_walk(app, par_reqs)]

    # access counts of the stream (binary-search probe counts), for the byte model
    engine.set_option("walk_stats", 1)
    engine.set_option("node2vec_adjacency", 1)
    c_steps = batched(reqs[:1024])
    trials, queries, probes = engine.last_stats()
    engine.set_option("walk_stats", 0)
    engine.set_option("node2vec_adjacency", best.get("node2vec_adjacency", 0))
    T, Q, P = trials / c_steps, queries / c_steps, probes / c_steps
    # return-edge lookups of the outlier bound: one per step of a request in
    # the outlier regime (1/p > max(1, 1/q)), from the requests' own step counts
    per_job = engine.batch_walk(app, reqs[:1024], keep_paths=False)
    out_steps = sum(res["total_steps"] for res, r in zip(per_job, reqs[:1024]) if n2v_outlier(r["p"], r["q"]))
    R = out_steps / max(1, sum(res["total_steps"] for res in per_job))
    b_step = 40 + T * (40 + 32) + P * 32 + 4
    design_b = 40 + T * 32 + Q * 32 + R * 64 + 4
    peak, peak_kind = load_peaks()
    plain_value = p_steps / (p_ms / 1e3)
    rebuild_value = r_steps / (r_ms / 1e3)
    # the walk kernel's own launches: steps and CUDA-event time per launch
    launch_steps = []
    prev = 0
    for ms, cum in kernel_ms:
        if cum < prev:
            prev = 0
        launch_steps.append((ms, cum - prev))
        prev = cum
    k_ms = sum(ms for ms, _ in launch_steps)
    k_steps = sum(st for _, st in launch_steps)
    mean_launch_ms = k_ms / len(launch_steps)
    steps_per_launch = k_steps / len(launch_steps)
    achieved = steps_per_launch * b_step / (mean_launch_ms / 1e3) / 1e9
    kernel_rate = k_steps / (k_ms / 1e3)
    ceiling = engine.gather_ceiling(4 << 30)
    traffic = traffic_for(args.workload, "walk_batch_kernel", steps_per_launch)

    parity = cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        csr, alias, t_alias = host_graph(engine, app, threads)
        parity = {
            "served": parity_requests(served_paths, csr, alias, par_reqs, threads,
                                      "served paths (kk_serve_poll) of the stream's first requests vs the oracle's "
                                      "node2vec walks of the same requests, bit for bit"),
            "batched": parity_requests(batch_paths, csr, alias, par_reqs, threads,
                                       "the same requests through kk_batch_walk vs the oracle"),
        }
        parity["walkers_checked"] = parity["served"]["walkers_checked"] + parity["batched"]["walkers_checked"]
        parity["mismatches"] = parity["served"]["mismatches"] + parity["batched"]["mismatches"]
        if not args.no_cpu:
            cpu, _ = cpu_sample_requests(csr, alias, t_alias, reqs, n_par, threads)
        del csr, alias
    engine.close()
    if rank != 0:
        return None
    d2h = 0
    for r in reqs:
        d2h += r["walker_num"] * (4 + 8 + 4)
    d2h = args.steps * d2h + 4 * s_steps
    line = {
        "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": b_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT generated on the GPU, seeded request stream)",
        "config": {"workload": args.workload, "desc": wl["desc"], "vertices": V, "edges": E,
                   "requests": len(reqs), "walker_step_capacity": stream_cap,
                   "walker_steps_per_step": b_steps / args.steps,
                   "step": "one pass of the whole request stream",
                   "parallelism": "replicas", "l2": "inputs larger than L2 (graph, alias tables, edge set)",
                   "slots": 2, "max_jobs": 256, "tuned": best,
                   "tuning_ms": [[c, ms] for c, ms in tune_table]},
        "batched": {"value": value, "unit": "walker-steps/s", "ms_per_pass": b_ms / args.steps,
                    "what": "kk_batch_walk_device, 1024 requests per launch, paths in HBM (the line's value)"},
        "plain": {"value": plain_value, "unit": "walker-steps/s", "requests": n_plain,
                  "what": "one kk_walk_device launch per request, alias tables kept"},
        "plain_rebuild": {"value": rebuild_value, "unit": "walker-steps/s", "requests": 12,
                          "what": "one launch per request, alias tables rebuilt per call (as the reference's "
                                  "random_walk does)"},
        "served": {"value": served_value, "unit": "walker-steps/s",
                   "what": "kk_serve_*, the K passes' requests submitted at once as one stream; submit -> paths "
                           "on the host (the line's e2e)",
                   "client": "kk_serve_replay (the library's client: submit from one host thread, poll and "
                             "free from another)",
                   "python_client": {"value": py_steps / py_s, "unit": "walker-steps/s",
                                     "what": "one pass submitted and polled request by request from Python "
                                             "through ctypes"},
                   "batches": sat["batches"], "mean_batch_jobs": sat["mean_batch_jobs"],
                   "slot_time_ms": {"walk_seen_ended": sat["walk_ms"], "then_last_copies_issued": sat["copy_ms"],
                                    "after_last_copies_issued": sat["host_ms"]}},
        "batched_over_plain": value / plain_value,
        "served_over_plain": served_value / plain_value,
        "latency": {"load": head["load"], "offered_rate_req_s": head["offered_req_s"], "p50_ms": head["p50_ms"],
                    "p99_ms": head["p99_ms"], "mean_ms": head["mean_ms"], "throughput": head["throughput"],
                    "curve": curve,
                    "what": "open-loop Poisson arrivals (kk_serve_replay) at a stated fraction of the saturated "
                            "served rate; submit -> paths on the host; the headline fields at load %.1f, the curve "
                            "at every load" % LATENCY_HEAD},
        "e2e": {"value": served_value, "unit": "walker-steps/s",
                "h2d_bytes_per_step": (sat["batches"] // max(args.steps, 1)) * 1024 * SERVE_JOB_BYTES,
                "d2h_bytes_per_step": d2h // args.steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "bytes_per_step": b_step, "design_bytes_per_step": design_b,
                     "access_counts": {"trials_per_step": T, "queries_per_step": Q, "probes_per_step": P,
                                       "return_edge_lookups_per_step": R},
                     "kernel": "walk_batch_kernel (second order)", "kernel_ms": mean_launch_ms,
                     "launches": len(launch_steps), "steps_per_launch": steps_per_launch,
                     "gather": {"ceiling_reads_per_s": ceiling, "reads_per_step": T + Q + R,
                                "achieved_reads_per_s": kernel_rate * (T + Q + R),
                                "frac": kernel_rate * (T + Q + R) / ceiling,
                                "what": "alias buckets + edge-set sectors of the adjacency queries + return-edge "
                                        "lookups of the outlier bound, per step of the walk kernel's launches, vs "
                                        "kk_gather_ceiling (4 GiB, this GPU, this run)"}},
        "parity": parity,
        "cpu_baseline": cpu, "clocks": clocks.summary(),
    }
    return line


def traffic_for(workload, kernel, steps_per_launch):
    """ncu's DRAM bytes per walker-step of `kernel` (profiles/traffic_<workload>.json,
    captured on a smaller case of the same kernel) scaled to a full launch."""
    tf = os.path.join(ROOT, "profiles", "traffic_%s.json" % workload.split("@")[0])
    if not os.path.exists(tf):
        return None
    with open(tf) as f:
        per_kernel = json.load(f)["dram_bytes_per_step"]
    b = per_kernel.get(kernel) if isinstance(per_kernel, dict) else per_kernel
    return b * steps_per_launch if b is not None else None


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
    cpu = parity = None
    if rank == 0:
        threads = os.cpu_count() or 1
        csr, alias, t_alias = host_graph(engine, app, threads)
        parity = parity_jobs(engine, csr, alias, app, jobs, threads)
        if not args.no_cpu:
            cpu = cpu_sample(csr, alias, t_alias, dict(wl, walk_length=max(j["walk_length"] for j in jobs)), V,
                             threads, seed=1)
        del csr, alias
    engine.close()
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
            "parity": parity,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        return line
    return None


def parity_jobs(engine, csr, alias, app, jobs, threads, per=8192):
    """Every job of a batch through kk_batch_walk (paths to the host) against
    the oracle's walk of the same job, on each job's first `per` walkers."""
    res = engine.batch_walk(app, jobs)
    checked = mism = 0
    weighted = csr.w is not None
    for ps, j in zip(res, jobs):
        n = min(per, j["walker_num"])
        kw = {k: j[k] for k in ("walk_length", "terminate_prob", "p", "q", "schemes", "scheme_round_robin") if k in j}
        lens, verts, _ = oracle_paths(csr, alias, app, threads, j.get("walk_length", 4095) + 1, seed=j["seed"],
                                      walker_begin=j.get("walker_begin", 0), walker_num=n, weighted=weighted, **kw)
        tot = int(np.asarray(ps.path_length[:n], np.int64).sum())
        mism += count_mismatches(ps.path_length[:n], ps.vertices[:tot], lens, verts)
        checked += n
    del res
    return {"jobs": len(jobs), "walkers_checked": checked, "mismatches": mism,
            "what": "each job's first %d walkers through kk_batch_walk vs the oracle's walk of the job, bit for "
                    "bit" % per}


def run_ours(args, wl, world, rank, local):
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
        # ncu's DRAM bytes per step of the kernel this run launched
        traffic = traffic_for(args.workload, walk_kernel_name(app, best), steps_per_launch)
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

    cpu = parity = None
    if rank == 0:
        threads = os.cpu_count() or 1
        csr, alias, t_alias = host_graph(engine, app, threads)
        parity = parity_ranges(engine, csr, alias, wl, walkers, threads)
        if not args.no_cpu:
            cpu = cpu_sample(csr, alias, t_alias, wl, walkers, threads, seed=1)
        del csr, alias
    engine.close()

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
            "parity": parity,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        return line
    return None


DEFAULT_WORKLOAD = "node2vec-serve-s24"
SECOND_WORKLOAD = "deepwalk-s22"


INGEST_RECORD = np.dtype([("src", "<u4"), ("dst", "<u4"), ("w", "<f4")])


def ingest_records(V, off, nbr, w, seed=7):
    """The ingestion file's records: each undirected edge of a symmetric CSR
    once (source < destination), in a seeded shuffled order."""
    src = np.repeat(np.arange(V, dtype=np.uint32), np.diff(off))
    keep = src < nbr
    perm = np.random.default_rng(seed).permutation(int(keep.sum()))
    rec = np.empty(len(perm), dtype=INGEST_RECORD)
    rec["src"] = src[keep][perm]
    rec["dst"] = nbr[keep][perm]
    rec["w"] = w[keep][perm]
    return rec


def ingest_oracle(V, path):
    """The reference's loader (include/graph.hpp:408-530, --make-undirected at
    :430-443) restated on the CPU: read the records, follow each by its mirror,
    stable sort by source (file order within a source), offsets by counting."""
    from oracle import graphs
    rec = np.fromfile(path, dtype=INGEST_RECORD)
    src = np.empty(2 * len(rec), np.uint32)
    dst = np.empty(2 * len(rec), np.uint32)
    src[0::2], src[1::2] = rec["src"], rec["dst"]
    dst[0::2], dst[1::2] = rec["dst"], rec["src"]
    return graphs.csr_file_order(V, src, dst, w=np.repeat(rec["w"], 2))


def run_ingest_bench(args, wl, world, rank, local):
    """Graph ingestion, the step before the walk: kk_graph_load_binary of a
    binary Edge<float> file with --make-undirected into a CSR in HBM.

    value : CSR edges per second of the call's device part, from the file's
            records in HBM (read and copied in overlapped blocks) to the CSR:
            split and mirror, the stable radix sort by source carrying each
            edge's destination and weight, offsets from the sorted sources,
            unpack (kk_graph_load_timing), K calls.
    e2e   : CSR edges per second of the whole call, file (in the page cache)
            to CSR in HBM.
    parity: the loaded CSR (offsets, neighbours, weights) against the oracle's
            restatement of the reference's loader, array for array.
    cpu_baseline: that restatement (numpy, one core) timed on the same file."""
    import tempfile

    import torch

    import knightking_gb300 as kk

    torch.cuda.set_device(local)
    engine = kk.WalkEngine(local)
    engine.generate_rmat(wl["scale"], 16, seed=wl["scale"], weights=wl["weights"])
    V, _, _, _ = engine.info()
    g = engine.download_graph()
    rec = ingest_records(V, g["off"], g["nbr"], g["w"])
    del g
    path = os.path.join(tempfile.gettempdir(), "kk_ingest_s%d_r%d_%d.bin" % (wl["scale"], rank, os.getpid()))
    rec.tofile(path)
    file_bytes = rec.nbytes
    del rec
    steps = min(args.steps, 5)  # a call takes about a second
    try:
        for _ in range(args.warmup):
            engine.load_graph(V, path, load_as_undirected=True, kind="f32")
        barrier(world)
        total_s, device_s = [], []
        with ClockSampler(local) as clocks:
            l0 = engine.launch_count()
            for _ in range(steps):
                t0 = time.perf_counter()
                engine.load_graph(V, path, load_as_undirected=True, kind="f32")
                total_s.append(time.perf_counter() - t0)
                device_s.append(engine.load_timing()[1] / 1e3)
            launches = engine.launch_count() - l0
        _, E, _, _ = engine.info()
        t_all = allreduce(world, sum(total_s), "max")
        t_dev = allreduce(world, sum(device_s), "max")
        value = allreduce(world, float(E * steps), "sum") / t_dev
        e2e_value = allreduce(world, float(E * steps), "sum") / t_all
        parity = cpu = None
        if rank == 0:
            got = engine.download_graph()
            t0 = time.perf_counter()
            ref = ingest_oracle(V, path)
            t_cpu = time.perf_counter() - t0
            parity = {"edges": int(E),
                      "mismatches": int(np.count_nonzero(ref["off"] != got["off"])
                                        + np.count_nonzero(ref["nbr"].view(np.uint32) != got["nbr"])
                                        + np.count_nonzero(ref["w"].view(np.uint32) != got["w"].view(np.uint32))),
                      "what": "offsets, neighbours and weights of the loaded CSR vs the oracle's restatement of "
                              "the reference's loader, bit for bit"}
            cpu = {"value": E / t_cpu, "unit": "edges/s", "cores": 1, "kind": "port", "seconds": t_cpu,
                   "sample": "the whole file: read, mirror, stable sort by source, offsets (numpy)"}
    finally:
        os.unlink(path)
    engine.close()
    if rank != 0:
        return None
    return {
        "metric": "edges/s", "value": value, "unit": "edges/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_all / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded R-MAT generated on the GPU, written as "
                                                     "a binary edge file)",
        "config": {"workload": args.workload, "desc": wl["desc"], "vertices": V, "edges": E,
                   "file_records": E // 2, "file_bytes": file_bytes, "parallelism": "replicas",
                   "l2": "inputs larger than L2"},
        "device": {"ms_per_call": 1e3 * t_dev / steps,
                   "what": "from the records in HBM: split and mirror, stable radix sort by source carrying "
                           "destination and weight, offsets from the sorted sources, unpack"},
        "e2e": {"value": e2e_value, "unit": "edges/s", "h2d_bytes_per_step": E * 12, "d2h_bytes_per_step": 0,
                "what": "the whole kk_graph_load_binary call: file (page cache) -> CSR in HBM"},
        "gpu_launches": launches,
        "roofline": None,
        "parity": parity,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
    }


def run_workload(args, wl, world, rank, local):
    if "ingest" in wl:
        return run_ingest_bench(args, wl, world, rank, local)
    if "batch" in wl:
        return run_batch_bench(args, wl, world, rank, local)
    if "serve" in wl:
        return run_serve_bench(args, wl, world, rank, local)
    return run_ours(args, wl, world, rank, local)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=None, choices=sorted(WORKLOADS),
                    help="default: %s, with %s measured in the same run under the key 'also'"
                         % (DEFAULT_WORKLOAD, SECOND_WORKLOAD))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--scale", type=int, default=None, help="override the R-MAT scale (profiling on a small case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    default_run = args.workload is None and args.scale is None
    args.workload = args.workload or DEFAULT_WORKLOAD
    wl = dict(WORKLOADS[args.workload])
    if args.scale is not None:
        wl["scale"] = args.scale
        wl["desc"] += " (scale overridden to %d)" % args.scale
        args.workload += "@s%d" % args.scale
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, wl, world, rank, local)
    else:
        line = run_workload(args, wl, world, rank, local)
        if default_run and args.impl == "ours":
            # the second workload (weighted DeepWalk, alias build in every step)
            # in the same run, reported inside the same line
            a2 = argparse.Namespace(**vars(args))
            a2.workload = SECOND_WORKLOAD
            second = run_workload(a2, dict(WORKLOADS[SECOND_WORKLOAD]), world, rank, local)
            if line is not None:
                line["also"] = {SECOND_WORKLOAD: second}
        if rank == 0 and line is not None:
            print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
