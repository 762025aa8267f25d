"""ORACLE / TEST INFRASTRUCTURE ONLY: ctypes front end of liboracle.so.

liboracle.so is the plain-C restatement of KnightKing's walker-step path
(kk_oracle.c).  tests/, __graft_entry__.smoke() and bench.py's CPU legs use it as
the checker and as the CPU baseline; the product never imports it.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "kk_ref")
REF_STOCK_BIN = os.path.join(HERE, "_ref", "kk_ref_stock")

APP = {"deepwalk": 0, "ppr": 1, "node2vec": 2, "metapath": 3, "tagwalk": 4, "dynwalk": 5}
MAX_SCHEMES = 16
MAX_SCHEME_LEN = 16


class Graph(ctypes.Structure):
    _fields_ = [
        ("V", ctypes.c_uint32),
        ("E", ctypes.c_uint64),
        ("off", ctypes.c_void_p),
        ("nbr", ctypes.c_void_p),
        ("w", ctypes.c_void_p),
        ("etype", ctypes.c_void_p),
    ]


class WalkParams(ctypes.Structure):
    _fields_ = [
        ("app", ctypes.c_int),
        ("weighted", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("walker_begin", ctypes.c_uint32),
        ("walker_num", ctypes.c_uint32),
        ("walk_length", ctypes.c_uint32),
        ("terminate_prob", ctypes.c_float),
        ("p", ctypes.c_float),
        ("q", ctypes.c_float),
        ("n_schemes", ctypes.c_int),
        ("scheme_len", ctypes.c_int * MAX_SCHEMES),
        ("scheme_mask", (ctypes.c_uint8 * MAX_SCHEME_LEN) * MAX_SCHEMES),
        ("scheme_round_robin", ctypes.c_int),
        ("tag_num", ctypes.c_int),
        ("vertex_tag_weight", ctypes.c_float),
        ("outlier_amplifier", ctypes.c_float),
        ("order", ctypes.c_int),
        ("outlier", ctypes.c_int),
        ("vertex_tag", ctypes.c_void_p),
        ("start", ctypes.c_void_p),
        ("n_start", ctypes.c_uint32),
    ]


_lib = None


def build(force=False):
    """Compile liboracle.so with its Makefile (gcc only; make rebuilds it when
    a source is newer)."""
    subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []) + ["liboracle.so"], check=True)
    return LIB_PATH


def ref_root():
    """Where the reference's sources lie: the oracle Makefile's REF_ROOT
    (environment variable KK_REFERENCE_ROOT, else the recipe's default)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "ref-root"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def build_ref():
    """Compile the reference's own engine (only where its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.ko_walk.restype = ctypes.c_int
        _lib.ko_walk.argtypes = [ctypes.POINTER(Graph), ctypes.POINTER(WalkParams), ctypes.c_uint32,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
        _lib.ko_walk_alias.restype = ctypes.c_int
        _lib.ko_walk_alias.argtypes = [ctypes.POINTER(Graph), ctypes.POINTER(WalkParams), ctypes.c_uint32,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib.ko_alias_build.restype = None
        _lib.ko_alias_build.argtypes = [ctypes.POINTER(Graph), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int]
        _lib.ko_sort_adjacency.restype = None
        _lib.ko_sort_adjacency.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]
        _lib.ko_last_timing.restype = None
        _lib.ko_last_timing.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class CSR:
    """Host CSR with the oracle's element types (keeps arrays alive)."""

    def __init__(self, V, off, nbr, w=None, etype=None):
        self.V = int(V)
        self.off = np.ascontiguousarray(off, dtype=np.int64)
        self.nbr = np.ascontiguousarray(nbr, dtype=np.uint32)
        self.w = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        self.etype = None if etype is None else np.ascontiguousarray(etype, dtype=np.uint8)
        self.E = int(self.off[-1])

    @staticmethod
    def from_dict(g):
        return CSR(g["V"], g["off"], g["nbr"] if "nbr" in g else g["dst"], g.get("w"), g.get("type"))

    def c(self):
        return Graph(self.V, self.E, _ptr(self.off), _ptr(self.nbr), _ptr(self.w), _ptr(self.etype))

    def sorted_copy(self):
        """Adjacency sorted by neighbour, as node2vec() sorts it (src/apps/node2vec.hpp:122-125)."""
        c = CSR(self.V, self.off.copy(), self.nbr.copy(),
                None if self.w is None else self.w.copy(), None if self.etype is None else self.etype.copy())
        lib().ko_sort_adjacency(c.V, _ptr(c.off), _ptr(c.nbr), _ptr(c.w), _ptr(c.etype))
        return c


def alias_build(csr, threads=0):
    E, V = csr.E, csr.V
    p = np.zeros(E, np.float32)
    pi = np.zeros(E, np.uint32)
    qi = np.zeros(E, np.uint32)
    s = np.zeros(V, np.float32)
    g = csr.c()
    lib().ko_alias_build(ctypes.byref(g), _ptr(p), _ptr(pi), _ptr(qi), _ptr(s), threads)
    return p, pi, qi, s


def make_params(app, seed=1, walker_begin=0, walker_num=0, walk_length=80, terminate_prob=1.0 / 80, p=1.0, q=1.0,
                weighted=False, schemes=None, scheme_round_robin=False, tag_num=4, vertex_tag_weight=0.5,
                outlier_amplifier=4.0, order=1, outlier=False, vertex_tag=None, start=None):
    prm = WalkParams()
    prm.app = APP[app]
    prm.weighted = int(bool(weighted))
    prm.seed = seed
    prm.walker_begin = walker_begin
    prm.walker_num = walker_num
    prm.walk_length = walk_length
    prm.terminate_prob = terminate_prob
    prm.p = p
    prm.q = q
    keep = []
    if schemes is not None:
        prm.n_schemes = len(schemes)
        for i, sc in enumerate(schemes):
            prm.scheme_len[i] = len(sc)
            for j, m in enumerate(sc):
                prm.scheme_mask[i][j] = int(m)
    prm.scheme_round_robin = int(bool(scheme_round_robin))
    prm.tag_num = tag_num
    prm.vertex_tag_weight = vertex_tag_weight
    prm.outlier_amplifier = outlier_amplifier
    prm.order = order
    prm.outlier = int(bool(outlier))
    if vertex_tag is not None:
        vt = np.ascontiguousarray(vertex_tag, dtype=np.int32)
        keep.append(vt)
        prm.vertex_tag = vt.ctypes.data
    if start is not None:
        st = np.ascontiguousarray(start, dtype=np.uint32)
        keep.append(st)
        prm.start = st.ctypes.data
        prm.n_start = len(st)
    prm._keep = keep
    return prm


def walk(csr, prm, cap, threads=0, with_paths=True, alias=None):
    """Returns (lens, flat_paths, total_steps); flat_paths concatenates each walker's path.
    alias: the (p, p_idx, q_idx, sum) of alias_build(csr), reused instead of
    building the tables in the call."""
    n = prm.walker_num
    lens = np.zeros(n, np.uint32)
    buf = np.zeros(n * cap, np.uint32) if with_paths else None
    steps = ctypes.c_uint64(0)
    g = csr.c()
    a = [None] * 4 if alias is None else [_ptr(x) for x in alias]
    st = lib().ko_walk_alias(ctypes.byref(g), ctypes.byref(prm), cap, _ptr(lens), _ptr(buf), threads,
                             ctypes.byref(steps), *a)
    if st != 0:
        raise RuntimeError("ko_walk failed with status %d" % st)
    if not with_paths:
        return lens, None, steps.value
    idx = np.arange(cap)[None, :] < lens[:, None].astype(np.int64)
    flat = buf.reshape(n, cap)[idx]
    return lens, flat, steps.value


def rmat_graph(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=None, weights=0, types=0, threads=0):
    """The project's seeded R-MAT graph on the CPU (same definition as
    oracle/graphs.py and the product's generator): C draws, numpy dedupe.
    weights: 0 none, 1 uniform [1,5), 2 lognormal(0,1); types: type count."""
    seed = scale if seed is None else seed
    L = lib()
    m = edge_factor << scale
    keys = np.empty(m, np.uint64)
    L.ko_rmat_draw.restype = None
    L.ko_rmat_draw.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                               ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int]
    L.ko_rmat_draw(scale, m, int(np.floor(a * 4294967296.0)), int(np.floor((a + b) * 4294967296.0)),
                   int(np.floor((a + b + c) * 4294967296.0)), seed, keys.ctypes.data, threads)
    L.ko_radix_sort_u64.restype = None
    L.ko_radix_sort_u64.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    tmp = np.empty(m, np.uint64)
    L.ko_radix_sort_u64(m, keys.ctypes.data, tmp.ctypes.data, 64, threads)
    keep = np.empty(m, bool)
    keep[0] = True
    np.not_equal(keys[1:], keys[:-1], out=keep[1:])
    keys = keys[keep]
    if len(keys) and keys[-1] == np.uint64(0xFFFFFFFFFFFFFFFF):
        keys = keys[:-1]
    u = (keys >> np.uint64(32)).astype(np.uint32)
    v = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    del keys
    sh = np.uint64(scale)
    mirrored = np.concatenate([(u.astype(np.uint64) << sh) | v, (v.astype(np.uint64) << sh) | u])
    if len(tmp) < len(mirrored):
        tmp = np.empty(len(mirrored), np.uint64)
    L.ko_radix_sort_u64(len(mirrored), mirrored.ctypes.data, tmp.ctypes.data, 2 * scale, threads)
    del tmp
    src = (mirrored >> sh).astype(np.uint32)
    dst = (mirrored & np.uint64((1 << scale) - 1)).astype(np.uint32)
    del mirrored
    V = 1 << scale
    off = np.zeros(V + 1, np.int64)
    np.cumsum(np.bincount(src, minlength=V), out=off[1:])
    w = np.empty(len(dst), np.float32) if weights else None
    t = np.empty(len(dst), np.uint8) if types else None
    if weights or types:
        L.ko_pair_data.restype = None
        L.ko_pair_data.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                   ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ko_pair_data(len(dst), src.ctypes.data, dst.ctypes.data, seed + 1000, weights, types, _ptr(w), _ptr(t),
                       threads)
    return {"V": V, "off": off, "nbr": dst, "w": w, "type": t}


def last_timing():
    a = ctypes.c_double(0)
    w = ctypes.c_double(0)
    lib().ko_last_timing(ctypes.byref(a), ctypes.byref(w))
    return a.value, w.value
