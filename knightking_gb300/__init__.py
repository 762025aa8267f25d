"""knightking_gb300: KnightKing's walker-step path on one GB300 GPU.

Python mirror of the reference's interface (include/walk.hpp, src/apps/*.hpp)
over the C-ABI in include/knightking_gb300.h:

    engine = WalkEngine()                        # WalkEngine<edge_data_t, S>()
    engine.load_graph(v_num, "graph.bin", kind="f32", load_as_undirected=False)
    conf = WalkConfig(); conf.set_output_file("out", True); conf.set_walk_rate(0.5)
    paths = deepwalk(engine, walker_num, walk_length, conf)       # deepwalk.hpp:30
    paths = ppr(engine, walker_num, terminate_prob, None, conf)   # ppr.hpp:30
    paths = node2vec(engine, Node2vecConf(p, q, walker_num, walk_length), conf)
    paths = metapath(engine, schemes, walker_num, walk_length, conf)

Every walk returns a PathSet (host arrays in walker-id order).  Errors raise
KKError with the engine's message; the reference asserts or exits instead.
There is no CPU fallback: without the CUDA library the import raises.
"""

import ctypes
import os

import numpy as np

from . import _capi
from ._capi import KKError, lib, library_path  # noqa: F401

__all__ = ["WalkEngine", "WalkConfig", "PathSet", "Node2vecConf", "KKError", "deepwalk", "ppr", "node2vec",
           "metapath", "read_metapath_schemes", "EDGE_KINDS", "library_path"]

EDGE_KINDS = {"none": 0, "unweighted": 0, "f32": 1, "meta": 2, "meta_f32": 3}


class WalkConfig:
    """WalkConfig (include/walk.hpp:105-145)."""

    def __init__(self):
        self.output_file_flag = False
        self.output_path_prefix = None
        self.print_with_head_info = False
        self.output_consumer_flag = False
        self.output_consumer_func = None
        self.rate = 1.0

    def set_output_file(self, output_path_prefix, with_head_info=False):
        if output_path_prefix is None:
            raise KKError(_capi.KK_ERR_INVALID_CONFIG, "output_path_prefix is None")
        self.output_file_flag = True
        self.output_path_prefix = str(output_path_prefix)
        self.print_with_head_info = bool(with_head_info)

    def set_output_consumer(self, func):
        if func is None:
            raise KKError(_capi.KK_ERR_INVALID_CONFIG, "output consumer is None")
        self.output_consumer_flag = True
        self.output_consumer_func = func

    def set_walk_rate(self, rate):
        if not (0 < rate <= 1):
            raise KKError(_capi.KK_ERR_INVALID_CONFIG, "rate must be in (0, 1]")
        self.rate = float(rate)


class Node2vecConf:
    """Node2vecConf (src/apps/node2vec.hpp:35-41)."""

    def __init__(self, p, q, walker_num, walk_length):
        self.p = float(p)
        self.q = float(q)
        self.walker_num = int(walker_num)
        self.walk_length = int(walk_length)


class PathSet:
    """Paths of one walk in walker-id order (PathSet, include/path.hpp:46-84).

    walker_id[i], path_length[i] and the vertices vertices[offset[i] : offset[i] + path_length[i]].
    """

    def __init__(self, walker_begin, epoch_walkers, length, offset, vertices, total_steps):
        self.walker_begin = int(walker_begin)
        self.epoch_walkers = int(epoch_walkers)
        self.path_length = length
        self.offset = offset
        self.vertices = vertices
        self.total_steps = int(total_steps)

    @property
    def path_num(self):
        return len(self.path_length)

    @property
    def walker_id(self):
        return np.arange(self.walker_begin, self.walker_begin + self.path_num, dtype=np.uint32)

    def path(self, i):
        o = int(self.offset[i])
        return self.vertices[o:o + int(self.path_length[i])]

    def dump(self, output_path, fopen_mode="w", with_head_info=False, seg_num=1):
        """PathSet::dump text (include/path.hpp:85-109) in the reference's segment order."""
        p = _capi.KKPaths()
        p.walker_num = self.path_num
        p.walker_begin = self.walker_begin
        p.epoch_walkers = self.epoch_walkers
        p.total_steps = self.total_steps
        length = np.ascontiguousarray(self.path_length, dtype=np.uint32)
        offset = np.ascontiguousarray(self.offset, dtype=np.uint64)
        verts = np.ascontiguousarray(self.vertices, dtype=np.uint32)
        p.length = length.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        p.offset = offset.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        p.vertices = verts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        st = lib().kk_paths_dump(ctypes.byref(p), str(output_path).encode(), fopen_mode.encode(),
                                 int(with_head_info), int(seg_num))
        _capi.check(st, None)


class WalkEngine:
    """WalkEngine (include/walk.hpp:365-421) on CUDA device `device`."""

    def __init__(self, device=0):
        self._lib = lib()
        self._h = ctypes.c_void_p()
        _capi.check(self._lib.kk_engine_create(ctypes.byref(self._h), int(device)), None)
        self.seg_num = 1

    def close(self):
        if self._h:
            self._lib.kk_engine_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        _capi.check(st, self._h)

    def set_stream(self, stream_ptr):
        """Issue the engine's work on a CUDA stream given by address (0: own stream)."""
        self._check(self._lib.kk_engine_set_stream(self._h, ctypes.c_void_p(stream_ptr or None)))

    def set_option(self, name, value):
        """Tuning knob (see kk_engine_set_option): walk_schedule, walk_blocks_per_sm, trial_limit."""
        self._check(self._lib.kk_engine_set_option(self._h, name.encode(), int(value)))

    def set_concurrency(self, worker_num):
        """The GPU needs no thread count; it sets the segment count used by dumps
        so the text matches the reference run with that many workers."""
        self.seg_num = max(1, int(worker_num))

    # ---- graph (GraphEngine::load_graph, include/graph.hpp:408-530) ----
    def load_graph(self, v_num, graph_path, load_as_undirected=False, kind="f32"):
        """load_graph (include/graph.hpp:408-530): kind is a binary Edge<T> kind
        ("unweighted", "f32", "meta", "meta_f32") or a text edge list ("text",
        "text_f32")."""
        if kind in ("text", "text_f32"):
            self._check(self._lib.kk_graph_load_text(self._h, int(v_num), str(graph_path).encode(),
                                                     int(kind == "text_f32"), int(bool(load_as_undirected))))
            return
        self._check(self._lib.kk_graph_load_binary(self._h, int(v_num), str(graph_path).encode(),
                                                   EDGE_KINDS[kind], int(bool(load_as_undirected))))

    def load_timing(self):
        """(total_ms, device_ms) of the last load_graph from a file: the whole
        call and its device part (columns to HBM, sort by source, offsets)."""
        total = ctypes.c_double()
        dev = ctypes.c_double()
        self._check(self._lib.kk_graph_load_timing(self._h, ctypes.byref(total), ctypes.byref(dev)))
        return total.value, dev.value

    def load_arrays(self, v_num, off, nbr, w=None, etype=None):
        off = np.ascontiguousarray(off, dtype=np.int64)
        nbr = np.ascontiguousarray(nbr, dtype=np.uint32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        etype = None if etype is None else np.ascontiguousarray(etype, dtype=np.uint8)
        self._check(self._lib.kk_graph_load_arrays(self._h, int(v_num), int(off[-1]), _capi.ptr(off),
                                                   _capi.ptr(nbr), _capi.ptr(w), _capi.ptr(etype)))

    def generate_rmat(self, scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=None, weights=0, types=0):
        """Seeded R-MAT graph in HBM (weights: 0 none, 1 uniform [1,5), 2 lognormal(0,1))."""
        seed = scale if seed is None else seed
        self._check(self._lib.kk_graph_generate_rmat(self._h, int(scale), int(edge_factor), float(a), float(b),
                                                     float(c), int(seed), int(weights), int(types)))

    def info(self):
        V = ctypes.c_uint32()
        E = ctypes.c_uint64()
        hw = ctypes.c_int()
        ht = ctypes.c_int()
        self._check(self._lib.kk_graph_info(self._h, ctypes.byref(V), ctypes.byref(E), ctypes.byref(hw),
                                            ctypes.byref(ht)))
        return V.value, E.value, bool(hw.value), bool(ht.value)

    def get_vertex_num(self):
        return self.info()[0]

    def get_edge_num(self):
        return self.info()[1]

    def download_graph(self):
        V, E, hw, ht = self.info()
        off = np.empty(V + 1, np.int64)
        nbr = np.empty(E, np.uint32)
        w = np.empty(E, np.float32) if hw else None
        t = np.empty(E, np.uint8) if ht else None
        self._check(self._lib.kk_graph_download(self._h, _capi.ptr(off), _capi.ptr(nbr), _capi.ptr(w), _capi.ptr(t)))
        return {"V": V, "off": off, "nbr": nbr, "w": w, "type": t}

    def sort_adjacency(self):
        self._check(self._lib.kk_graph_sort_adjacency(self._h))

    def alias_tables(self):
        """(p, p_idx, q_idx, sum) of the weight alias tables (include/walk.hpp:538-652)."""
        V, E, hw, _ = self.info()
        p = np.empty(E, np.float32)
        pi = np.empty(E, np.uint32)
        qi = np.empty(E, np.uint32)
        s = np.empty(V, np.float32)
        self._check(self._lib.kk_alias_build(self._h, _capi.ptr(p), _capi.ptr(pi), _capi.ptr(qi), _capi.ptr(s)))
        return p, pi, qi, s

    # ---- walks (WalkEngine::random_walk, include/walk.hpp:423-436) ----
    def make_opts(self, app, walker_num, seed=1, walker_begin=0, walk_length=80, terminate_prob=1.0 / 80, p=1.0,
                  q=1.0, weighted=None, schemes=None, scheme_round_robin=False, start=None, rate=1.0):
        if weighted is None:
            weighted = self.info()[2]
        return _capi.make_opts(app, walker_num, seed, walker_begin, walk_length, terminate_prob, p, q, weighted,
                               schemes, scheme_round_robin, start, rate)

    def walk(self, app, walker_num, walk_conf=None, **kw):
        if walk_conf is not None:
            kw.setdefault("rate", walk_conf.rate)
        opts = self.make_opts(app, walker_num, **kw)
        out = ctypes.POINTER(_capi.KKPaths)()
        self._check(self._lib.kk_walk(self._h, ctypes.byref(opts), ctypes.byref(out)))
        # the arrays view the library's pinned block and return it when dropped
        paths = PathSet(*_capi.paths_to_numpy_owned(out))
        if walk_conf is not None:
            if walk_conf.output_file_flag:
                paths.dump(walk_conf.output_path_prefix + ".0", "w", walk_conf.print_with_head_info, self.seg_num)
            if walk_conf.output_consumer_flag:
                walk_conf.output_consumer_func(paths)
        return paths

    def job_table(self, app, jobs):
        """The kk_walk_opts array of a batch, built once (batch_walk_device and
        batch_walk take it in place of the list of job dicts)."""
        return JobTable(app, *self._job_array(app, jobs))

    def _job_array(self, app, jobs):
        if isinstance(jobs, JobTable):
            if jobs.app != app:
                raise ValueError("job table built for another app")
            return jobs.arr, jobs.keep
        arr = (_capi.KKWalkOpts * len(jobs))()
        keep = []
        for i, job in enumerate(jobs):
            job = dict(job)
            o = self.make_opts(app, job.pop("walker_num"), **job)
            keep.append(o)
            ctypes.memmove(ctypes.byref(arr[i]), ctypes.byref(o), ctypes.sizeof(o))
        return arr, keep

    def batch_walk(self, app, jobs, keep_paths=True):
        """Many jobs of one app in one launch (kk_batch_walk); jobs are dicts of
        make_opts keywords with walker_num.  Returns one PathSet per job, or
        with keep_paths=False, per job a dict of walker_num, total_steps and
        vertices, the paths (in pinned host memory when the call returns)
        handed back to the library's pool without a copy."""
        arr, keep = self._job_array(app, jobs)
        outs = (ctypes.POINTER(_capi.KKPaths) * len(jobs))()
        self._check(self._lib.kk_batch_walk(self._h, arr, len(jobs), outs))
        res = []
        owned = [False] * len(jobs)
        try:
            for k, p in enumerate(outs):
                if keep_paths:
                    # views of the pinned block, returned when the arrays are dropped
                    res.append(PathSet(*_capi.paths_to_numpy_owned(p)))
                    owned[k] = True
                else:
                    c = p.contents
                    res.append({"walker_num": int(c.walker_num), "total_steps": int(c.total_steps),
                                "vertices": int(c.total_steps) + int(c.walker_num)})
        finally:
            for k, p in enumerate(outs):
                if p and not owned[k]:
                    self._lib.kk_paths_free(p)
        return res

    def batch_submit(self, app, jobs):
        """kk_batch_submit: queues the batch and returns at once; the returned
        handle's wait() gives what batch_walk would have returned.  The engine
        takes no other call until then."""
        arr, keep = self._job_array(app, jobs)
        h = ctypes.c_void_p()
        self._check(self._lib.kk_batch_submit(self._h, arr, len(jobs), ctypes.byref(h)))
        return SubmittedBatch(self, h, len(jobs), keep)

    def batch_walk_device(self, app, jobs, paths=True):
        """kk_batch_walk_device: paths stay in HBM; returns the total walker-steps."""
        arr, keep = self._job_array(app, jobs)
        steps = ctypes.c_uint64()
        dl = ctypes.c_void_p()
        dv = ctypes.c_void_p()
        self._check(self._lib.kk_batch_walk_device(self._h, arr, len(jobs), ctypes.byref(steps), ctypes.byref(dl),
                                                   ctypes.byref(dv) if paths else None))
        return steps.value

    def walk_device(self, app, walker_num, paths=True, opts=None, **kw):
        """Walk with results left in HBM; returns (total_steps, d_length, d_offset, d_vertices) pointers.
        paths: True packed, "unpacked" as the walk wrote them (no compaction pass), False not stored.
        opts: a kk_walk_opts from make_opts, used as it is (walker_num and kw are then ignored)."""
        if opts is None:
            opts = self.make_opts(app, walker_num, **kw)
        steps = ctypes.c_uint64()
        dl = ctypes.c_void_p()
        do = ctypes.c_void_p()
        dv = ctypes.c_void_p()
        self._check(self._lib.kk_walk_device(self._h, ctypes.byref(opts), ctypes.byref(steps), ctypes.byref(dl),
                                             ctypes.byref(do) if paths is True else None,
                                             ctypes.byref(dv) if paths else None))
        return steps.value, dl.value, do.value, dv.value

    def walk_into(self, app, walker_num, h_length, h_offset, h_vertices, cap, **kw):
        """Walk into caller-owned host buffers given as raw addresses (e.g. pinned
        tensors' data_ptr()); cap is the vertex capacity of h_vertices."""
        opts = self.make_opts(app, walker_num, **kw)
        steps = ctypes.c_uint64()
        self._check(self._lib.kk_walk_into(self._h, ctypes.byref(opts), ctypes.c_void_p(h_length),
                                           ctypes.c_void_p(h_offset), ctypes.c_void_p(h_vertices),
                                           ctypes.c_uint64(cap), ctypes.byref(steps)))
        return steps.value

    def serve(self, app, weighted=None, slots=2, max_jobs=256, slot_bytes=1 << 30, graphs=True):
        """Starts a Server (continuous batching) that owns this engine until
        stopped; graphs: each slot replays a captured CUDA graph per batch."""
        return Server(self, app, weighted, slots, max_jobs, slot_bytes, graphs)

    def last_stats(self):
        """(trials, queries, probes) of the last walk (walk_stats option)."""
        t, q, p = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._lib.kk_last_walk_stats(self._h, ctypes.byref(t), ctypes.byref(q), ctypes.byref(p)))
        return t.value, q.value, p.value

    def last_timing(self):
        a = ctypes.c_float()
        w = ctypes.c_float()
        self._check(self._lib.kk_last_walk_timing(self._h, ctypes.byref(a), ctypes.byref(w)))
        return a.value, w.value

    def gather_ceiling(self, nbytes=4 << 30):
        """Dependent random 32 B reads per second over an nbytes buffer (the
        random-gather ceiling of this GPU)."""
        r = ctypes.c_double()
        self._check(self._lib.kk_gather_ceiling(self._h, ctypes.c_uint64(nbytes), ctypes.byref(r)))
        return r.value

    def launch_count(self):
        """Kernels the library has launched on this engine's streams so far
        (captured CUDA-graph replays of a serving slot not counted)."""
        c = ctypes.c_uint64()
        self._check(self._lib.kk_engine_launch_count(self._h, ctypes.byref(c)))
        return c.value


# ---- the apps' entry points (src/apps/*.hpp) ----

def deepwalk(graph, walker_num, walk_length, walk_conf=None, seed=1, **kw):
    """deepwalk() (src/apps/deepwalk.hpp:30-47)."""
    return graph.walk("deepwalk", walker_num, walk_conf, walk_length=walk_length, seed=seed, **kw)


def ppr(graph, walker_num, terminate_prob, start_vertices=None, walk_conf=None, seed=1, **kw):
    """ppr() (src/apps/ppr.hpp:30-64)."""
    return graph.walk("ppr", walker_num, walk_conf, terminate_prob=terminate_prob, start=start_vertices, seed=seed,
                      **kw)


def node2vec(graph, conf, walk_conf=None, seed=1, **kw):
    """node2vec() (src/apps/node2vec.hpp:108-202); sorts the adjacency in place first."""
    return graph.walk("node2vec", conf.walker_num, walk_conf, walk_length=conf.walk_length, p=conf.p, q=conf.q,
                      seed=seed, **kw)


def metapath(graph, schemes, walker_num, walk_length, walk_conf=None, seed=1, **kw):
    """metapath() (src/apps/metapath.hpp:70-128).  schemes: per scheme, per state,
    either a list of allowed-type booleans (the reference's vector<vector<vector<bool>>>)
    or an int type mask."""
    masks = []
    for sc in schemes:
        row = []
        for st in sc:
            if isinstance(st, (list, tuple, np.ndarray)):
                m = 0
                for k, allowed in enumerate(st):
                    if allowed:
                        m |= 1 << k
                row.append(m)
            else:
                row.append(int(st))
        masks.append(row)
    return graph.walk("metapath", walker_num, walk_conf, walk_length=walk_length, schemes=masks, seed=seed, **kw)


def text_to_binary(text_path, binary_path, weighted=False):
    """gconverter (src/tools/gconverter.cpp:69-100): text edge list -> binary
    Edge<T> file; returns the edge count."""
    n = ctypes.c_uint64()
    st = lib().kk_text_to_binary(str(text_path).encode(), str(binary_path).encode(), int(bool(weighted)),
                                 ctypes.byref(n))
    _capi.check(st, None)
    return n.value


def read_metapath_scheme_masks(path):
    """The scheme file as per-state edge-type masks (kk_read_metapath_schemes):
    a list of schemes, each a list of masks (bit t = type t allowed)."""
    o = _capi.KKWalkOpts()
    _capi.check(lib().kk_read_metapath_schemes(str(path).encode(), ctypes.byref(o)), None)
    return [[int(o.scheme_mask[s][j]) for j in range(o.scheme_len[s])] for s in range(o.n_schemes)]


def read_metapath_schemes(path):
    """read_metapath_schemes (src/apps/metascheme.hpp:69-98)."""
    with open(path) as f:
        toks = f.read().split()
    it = iter(toks)
    n, states = int(next(it)), int(next(it))
    schemes = []
    for _ in range(n):
        ln = int(next(it))
        schemes.append([[int(next(it)) != 0 for _ in range(states)] for _ in range(ln)])
    return schemes


def _here():
    return os.path.dirname(os.path.abspath(__file__))


class ServeResult:
    """One served request: its PathSet, status, queueing and total latency."""

    def __init__(self, paths, status, queue_ms, latency_ms, batch_jobs):
        self.paths = paths
        self.status = status
        self.queue_ms = queue_ms
        self.latency_ms = latency_ms
        self.batch_jobs = batch_jobs


class SubmittedBatch:
    """A batch queued by WalkEngine.batch_submit."""

    def __init__(self, engine, handle, n, keep):
        self._engine = engine
        self._h = handle
        self._n = n
        self._keep = keep

    def wait(self):
        """kk_batch_wait: one PathSet per job, in job order."""
        if self._h is None:
            raise ValueError("batch already waited for")
        lib = self._engine._lib
        outs = (ctypes.POINTER(_capi.KKPaths) * self._n)()
        st = lib.kk_batch_wait(self._h, outs)
        self._h = None
        self._engine._check(st)
        res, owned = [], [False] * self._n
        try:
            for k, p in enumerate(outs):
                res.append(PathSet(*_capi.paths_to_numpy_owned(p)))
                owned[k] = True
        finally:
            for k, p in enumerate(outs):
                if p and not owned[k]:
                    lib.kk_paths_free(p)
        return res


class JobTable:
    """A batch's job records in the C-ABI's layout (WalkEngine.job_table)."""

    def __init__(self, app, arr, keep):
        self.app = app
        self.arr = arr
        self.keep = keep

    def __len__(self):
        return len(self.arr)


class Server:
    """Continuous batching of walk requests (kk_serve_*).  submit() and poll()
    may be called from several threads; the engine is the server's until stop()."""

    def __init__(self, engine, app, weighted=None, slots=2, max_jobs=256, slot_bytes=1 << 30, graphs=True):
        self._engine = engine
        self._lib = engine._lib
        self.app = app
        if weighted is None:
            weighted = engine.info()[2]
        self.weighted = bool(weighted)
        o = _capi.KKServeOpts()
        o.app = _capi.APPS[app]
        o.weighted = int(self.weighted)
        o.slots = int(slots)
        o.max_jobs = int(max_jobs)
        o.slot_bytes = int(slot_bytes)
        o.launch_mode = 0 if graphs else 1
        h = ctypes.c_void_p()
        engine._check(self._lib.kk_serve_start(engine._h, ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def submit(self, walker_num, **kw):
        """Queues a request (make_opts keywords); returns its ticket."""
        kw.setdefault("weighted", self.weighted)
        opts = self._engine.make_opts(self.app, walker_num, **kw)
        t = ctypes.c_uint64()
        st = self._lib.kk_serve_submit(self._h, ctypes.byref(opts), ctypes.byref(t))
        if st != _capi.KK_OK:
            raise KKError(st, "request refused")
        return t.value

    def poll(self, ticket, timeout_ms=-1, keep_paths=True):
        """The request's ServeResult, or None if it is not done within
        timeout_ms.  keep_paths=False frees the paths unread (result.paths is
        then None and result.total_steps still counts them)."""
        r = _capi.KKServeResult()
        st = self._lib.kk_serve_poll(self._h, ctypes.c_uint64(ticket), int(timeout_ms), ctypes.byref(r))
        if st == _capi.KK_ERR_TIMEOUT:
            return None
        if st != _capi.KK_OK:
            raise KKError(st, "unknown ticket")
        paths = None
        total_steps = 0
        if r.paths:
            try:
                total_steps = r.paths.contents.total_steps
                if keep_paths:
                    paths = PathSet(*_capi.paths_to_numpy(r.paths.contents))
            finally:
                self._lib.kk_paths_free(r.paths)
        res = ServeResult(paths, r.status, r.queue_ms, r.latency_ms, r.batch_jobs)
        res.total_steps = int(total_steps)
        return res

    def replay(self, requests, arrival_s):
        """Open-loop client in the library (kk_serve_replay): request i (a dict
        of submit() keywords) is submitted arrival_s[i] seconds after the
        call starts while a library thread polls and frees every result.
        Returns (latency_ms per request, walker-steps, elapsed seconds)."""
        requests = [dict(r, weighted=r.get("weighted", self.weighted)) for r in requests]
        arr, keep = self._engine._job_array(self.app, requests)
        arrival = np.ascontiguousarray(arrival_s, dtype=np.float64)
        if len(arrival) != len(requests):
            raise ValueError("one arrival time per request")
        lat = np.zeros(len(requests), np.float64)
        steps = ctypes.c_uint64()
        elapsed = ctypes.c_double()
        st = self._lib.kk_serve_replay(self._h, arr, arrival.ctypes.data, len(requests), lat.ctypes.data,
                                       ctypes.byref(steps), ctypes.byref(elapsed))
        del keep
        if st != _capi.KK_OK:
            raise KKError(st, "replay failed")
        return lat, int(steps.value), float(elapsed.value)

    def stats(self):
        s = _capi.KKServeStats()
        self._lib.kk_serve_stats_get(self._h, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def reset_stats(self):
        self._lib.kk_serve_stats_reset(self._h)

    def stop(self):
        if self._h:
            self._lib.kk_serve_stop(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()
