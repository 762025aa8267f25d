"""ctypes bindings of the C-ABI (include/knightking_gb300.h).

The CUDA library is loaded from knightking_gb300/lib/ (built in-tree by
knightking_gb300/build.py).  If it is missing or cannot be loaded this module
raises: there is no CPU fallback.
"""

import atexit
import ctypes
import os

import numpy as np

KK_OK = 0
KK_ERR_INVALID_CONFIG = 1
KK_ERR_OOM = 2
KK_ERR_IO = 3
KK_ERR_TRIAL_LIMIT = 4
KK_ERR_TIMEOUT = 5
KK_ERR_CUDA = 6
KK_ERR_NO_GRAPH = 7
KK_ERR_PATH_CAPACITY = 8

APPS = {"deepwalk": 0, "ppr": 1, "node2vec": 2, "metapath": 3}
MAX_SCHEMES = 16
MAX_SCHEME_LEN = 16

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "lib", "libknightking_gb300.so")


class KKError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("kk status %d: %s" % (status, message))
        self.status = status
        self.message = message


class KKWalkOpts(ctypes.Structure):
    _fields_ = [
        ("app", ctypes.c_int),
        ("weighted", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("walker_num", ctypes.c_uint32),
        ("walker_begin", ctypes.c_uint32),
        ("walk_length", ctypes.c_uint32),
        ("terminate_prob", ctypes.c_float),
        ("p", ctypes.c_float),
        ("q", ctypes.c_float),
        ("n_schemes", ctypes.c_int),
        ("scheme_len", ctypes.c_int * MAX_SCHEMES),
        ("scheme_mask", (ctypes.c_uint8 * MAX_SCHEME_LEN) * MAX_SCHEMES),
        ("scheme_round_robin", ctypes.c_int),
        ("start", ctypes.POINTER(ctypes.c_uint32)),
        ("n_start", ctypes.c_uint32),
        ("rate", ctypes.c_double),
    ]


class KKPaths(ctypes.Structure):
    _fields_ = [
        ("walker_num", ctypes.c_uint32),
        ("walker_begin", ctypes.c_uint32),
        ("epoch_walkers", ctypes.c_uint32),
        ("total_steps", ctypes.c_uint64),
        ("length", ctypes.POINTER(ctypes.c_uint32)),
        ("offset", ctypes.POINTER(ctypes.c_uint64)),
        ("vertices", ctypes.POINTER(ctypes.c_uint32)),
        ("owner", ctypes.c_void_p),
    ]


class KKServeOpts(ctypes.Structure):
    _fields_ = [
        ("app", ctypes.c_int),
        ("weighted", ctypes.c_int),
        ("slots", ctypes.c_int),
        ("max_jobs", ctypes.c_uint32),
        ("slot_bytes", ctypes.c_uint64),
        ("launch_mode", ctypes.c_int),
    ]


class KKServeResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("paths", ctypes.POINTER(KKPaths)),
        ("queue_ms", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
        ("batch_jobs", ctypes.c_uint32),
    ]


class KKServeStats(ctypes.Structure):
    _fields_ = [
        ("completed", ctypes.c_uint64),
        ("failed", ctypes.c_uint64),
        ("batches", ctypes.c_uint64),
        ("walker_steps", ctypes.c_uint64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("mean_batch_jobs", ctypes.c_double),
        ("walk_ms", ctypes.c_double),
        ("copy_ms", ctypes.c_double),
        ("host_ms", ctypes.c_double),
    ]


_lib = None

_P = ctypes.c_void_p
_SIGS = {
    "kk_engine_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "kk_engine_destroy": (None, [_P]),
    "kk_engine_set_stream": (ctypes.c_int, [_P, _P]),
    "kk_engine_set_option": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int64]),
    "kk_last_error": (ctypes.c_char_p, [_P]),
    "kk_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "kk_graph_load_binary": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "kk_graph_load_arrays": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint64, _P, _P, _P, _P]),
    "kk_graph_load_text": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
    "kk_graph_load_timing": (ctypes.c_int, [_P, _P, _P]),
    "kk_text_to_binary": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, _P]),
    "kk_read_metapath_schemes": (ctypes.c_int, [ctypes.c_char_p, _P]),
    "kk_graph_generate_rmat": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_uint64, ctypes.c_int, ctypes.c_int]),
    "kk_graph_info": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "kk_graph_download": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "kk_graph_sort_adjacency": (ctypes.c_int, [_P]),
    "kk_alias_build": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "kk_alias_build_noalloc": (ctypes.c_int, [ctypes.c_uint32, _P, _P, _P, _P, _P, _P, _P]),
    "kk_walk": (ctypes.c_int, [_P, _P, _P]),
    "kk_walk_deepwalk": (ctypes.c_int, [_P, _P, _P]),
    "kk_walk_ppr": (ctypes.c_int, [_P, _P, _P]),
    "kk_walk_node2vec": (ctypes.c_int, [_P, _P, _P]),
    "kk_walk_metapath": (ctypes.c_int, [_P, _P, _P]),
    "kk_walk_into": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_uint64, _P]),
    "kk_batch_walk": (ctypes.c_int, [_P, _P, ctypes.c_int, _P]),
    "kk_batch_walk_device": (ctypes.c_int, [_P, _P, ctypes.c_int, _P, _P, _P]),
    "kk_batch_submit": (ctypes.c_int, [_P, _P, ctypes.c_int, _P]),
    "kk_batch_wait": (ctypes.c_int, [_P, _P]),
    "kk_walk_device": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "kk_last_walk_timing": (ctypes.c_int, [_P, _P, _P]),
    "kk_engine_launch_count": (ctypes.c_int, [_P, _P]),
    "kk_gather_ceiling": (ctypes.c_int, [_P, ctypes.c_uint64, _P]),
    "kk_last_walk_stats": (ctypes.c_int, [_P, _P, _P, _P]),
    "kk_philox_blocks": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint32, _P, _P]),
    "kk_serve_start": (ctypes.c_int, [_P, _P, _P]),
    "kk_serve_submit": (ctypes.c_int, [_P, _P, _P]),
    "kk_serve_poll": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_int, _P]),
    "kk_serve_stats_get": (ctypes.c_int, [_P, _P]),
    "kk_serve_stats_reset": (ctypes.c_int, [_P]),
    "kk_serve_stop": (ctypes.c_int, [_P]),
    "kk_serve_replay": (ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, _P, _P, _P]),
    "kk_paths_free": (None, [_P]),
    "kk_paths_dump": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]),
}


def library_path():
    return _LIB_PATH


def lib():
    """The loaded CUDA library (builds it in-tree first if it is missing or stale)."""
    global _lib
    if _lib is None:
        from . import build as _build
        try:
            _build.build()
        except (OSError, RuntimeError) as exc:
            if not os.path.exists(_LIB_PATH):
                raise ImportError("knightking_gb300: CUDA library missing and the build failed: %s" % exc)
        if not os.path.exists(_LIB_PATH):
            raise ImportError("knightking_gb300: CUDA library %s not built" % _LIB_PATH)
        L = ctypes.CDLL(_LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def check(status, handle):
    if status != KK_OK:
        L = lib()
        msg = L.kk_last_error(handle).decode() if handle else ""
        if not msg:
            msg = L.kk_status_string(status).decode()
        raise KKError(status, msg)


def make_opts(app, walker_num, seed, walker_begin, walk_length, terminate_prob, p, q, weighted, schemes,
              scheme_round_robin, start, rate):
    o = KKWalkOpts()
    o.app = APPS[app] if isinstance(app, str) else int(app)
    o.weighted = int(bool(weighted))
    o.seed = int(seed)
    o.walker_num = int(walker_num)
    o.walker_begin = int(walker_begin)
    o.walk_length = int(walk_length)
    o.terminate_prob = float(terminate_prob)
    o.p = float(p)
    o.q = float(q)
    if schemes is not None:
        if len(schemes) > MAX_SCHEMES:
            raise KKError(KK_ERR_INVALID_CONFIG, "at most 16 schemes")
        o.n_schemes = len(schemes)
        for i, sc in enumerate(schemes):
            if len(sc) > MAX_SCHEME_LEN:
                raise KKError(KK_ERR_INVALID_CONFIG, "scheme longer than 16 states")
            o.scheme_len[i] = len(sc)
            for j, m in enumerate(sc):
                o.scheme_mask[i][j] = int(m)
    o.scheme_round_robin = int(bool(scheme_round_robin))
    if start is not None:
        st = np.ascontiguousarray(start, dtype=np.uint32)
        o._start = st
        o.start = st.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        o.n_start = len(st)
    o.rate = float(rate)
    return o


_exiting = False


def _mark_exit():
    global _exiting
    _exiting = True


atexit.register(_mark_exit)


class _PathsOwner:
    """Owns a kk_paths: returns it to the library (kk_paths_free) once the last
    numpy array viewing it is gone.  At interpreter exit it leaves the memory
    alone: the library may already be unloading."""

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        if not _exiting and self.ptr:
            lib().kk_paths_free(self.ptr)
            self.ptr = None


def _view(addr, ctype, count, owner, dtype):
    """A numpy array over count elements at addr, keeping owner alive."""
    if count == 0:
        return np.zeros(0, dtype)
    buf = (ctype * count).from_address(addr)
    buf._owner = owner
    return np.frombuffer(buf, dtype=dtype)


def paths_to_numpy_owned(pp):
    """Like paths_to_numpy for a POINTER(KKPaths) whose ownership passes to
    the result: packed paths (every kk_walk and kk_batch_walk result) are
    returned as views of the library's pinned block, freed when the last view
    is gone; other layouts are copied and freed at once."""
    p = pp.contents
    n = int(p.walker_num)
    total = int(p.total_steps) + n
    owner = _PathsOwner(pp)
    length = _view(ctypes.addressof(p.length.contents), ctypes.c_uint32, n, owner, np.uint32) if n else \
        np.zeros(0, np.uint32)
    offset = _view(ctypes.addressof(p.offset.contents), ctypes.c_uint64, n, owner, np.uint64) if n else \
        np.zeros(0, np.uint64)
    # the library hands out packed paths or fixed-capacity slots (offset i *
    # cap); of those layouts, only packed paths end at total with offset 0 first
    packed = n == 0 or (int(offset[0]) == 0 and int(offset[n - 1]) + int(length[n - 1]) == total)
    if packed:
        verts = _view(ctypes.addressof(p.vertices.contents), ctypes.c_uint32, total, owner, np.uint32) if total \
            else np.zeros(0, np.uint32)
        return int(p.walker_begin), int(p.epoch_walkers), length, offset, verts, int(p.total_steps)
    out = paths_to_numpy(p)
    del length, offset
    return out


def paths_to_numpy(p):
    """A kk_paths as numpy arrays, packed: walker i's vertices at the prefix
    sum of the lengths (paths with gaps between walkers are compacted)."""
    n = p.walker_num
    length = np.ctypeslib.as_array(p.length, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
    offset = np.ctypeslib.as_array(p.offset, shape=(n,)).copy() if n else np.zeros(0, np.uint64)
    total = int(p.total_steps) + n
    packed = np.zeros(n, np.uint64)
    if n:
        np.cumsum(length[:-1], out=packed[1:])
    if n == 0 or np.array_equal(offset, packed):
        verts = np.ctypeslib.as_array(p.vertices, shape=(total,)).copy() if total else np.zeros(0, np.uint32)
    else:
        extent = int((offset + length.astype(np.uint64)).max())
        raw = np.ctypeslib.as_array(p.vertices, shape=(max(extent, 1),))
        idx = np.repeat(offset.astype(np.int64) - packed.astype(np.int64), length) + np.arange(total, dtype=np.int64)
        verts = raw[idx].copy()
        offset = packed
    return p.walker_begin, p.epoch_walkers, length, offset, verts, p.total_steps
