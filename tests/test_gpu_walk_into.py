"""kk_walk_into's two copy-out modes.  Streamed (walks whose path lengths are
known before they run): one launch per epoch, every segment of walkers copied
out as soon as its last walker finishes.  Metapath: one launch, then packed and
copied out.  Chunked (into_stream 0,
graphs with dead ends): chunk c + 1 walks while chunk c's paths are packed and
copied out.  Whatever the mode, the lengths, offsets and vertices in the
caller's buffers are the paths kk_walk returns, and both equal the oracle's
(the C restatement pinned to the reference), walker for walker."""

import numpy as np
import pytest

from oracle import graphs as G

pytestmark = pytest.mark.gpu

N = 600_000  # > 2 x 2^18 walkers: several chunks


@pytest.fixture(scope="module")
def engine():
    import knightking_gb300 as kk
    e = kk.WalkEngine(0)
    yield e
    e.close()


def _load(engine, seed, weighted, types=False):
    g = G.random_undirected(400, 5000, seed=seed, weight="unif" if weighted else None,
                            types="uniform" if types else None)
    csr = G.csr_file_order(400, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(400, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    return csr


def _oracle(oracle_lib, csr, app, n, weighted, kw):
    """The oracle's walk of the same walkers (lengths, packed vertices, steps)."""
    V = len(csr["off"]) - 1
    ocsr = oracle_lib.CSR(V, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    if app == "node2vec":
        ocsr = ocsr.sorted_copy()
    kw = {k: v for k, v in kw.items() if k != "rate"}
    prm = oracle_lib.make_params(app, walker_num=n, weighted=weighted, **kw)
    return oracle_lib.walk(ocsr, prm, cap=kw.get("walk_length", 400) + 1)


def _into(engine, app, n, cap, **kw):
    h_len = np.zeros(n, np.uint32)
    h_off = np.zeros(n, np.uint64)
    h_vert = np.zeros(cap, np.uint32)
    steps = engine.walk_into(app, n, h_len.ctypes.data, h_off.ctypes.data, h_vert.ctypes.data, cap, **kw)
    return steps, h_len, h_off, h_vert


CASES = [
    ("deepwalk", True, False, dict(walk_length=10, seed=3)),
    ("deepwalk", False, False, dict(walk_length=7, seed=4, walker_begin=1000)),
    ("ppr", False, False, dict(terminate_prob=0.15, seed=5)),
    ("node2vec", True, False, dict(walk_length=6, p=2.0, q=0.5, seed=6)),
    ("metapath", True, True, dict(walk_length=6, schemes=[[1, 2, 4, 8], [2, 8, 2, 16]], seed=7)),
]


@pytest.mark.parametrize("chunks,cursor,stream", [(1, 0, 1), (4, 1, 1), (3, 0, 0), (4, 1, 0)])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_walk_into_equals_walk(engine, oracle_lib, case, chunks, cursor, stream):
    app, weighted, types, kw = CASES[case]
    csr = _load(engine, 20 + case, weighted, types)
    ref = engine.walk(app, N, weighted=weighted, **kw)
    if chunks == 1:
        lens, verts, steps = _oracle(oracle_lib, csr, app, N, weighted, kw)
        np.testing.assert_array_equal(ref.path_length, lens)
        np.testing.assert_array_equal(ref.vertices, verts)
    engine.set_option("into_chunks", chunks)
    engine.set_option("cursor_adjacency", cursor)
    engine.set_option("into_stream", stream)
    try:
        steps, h_len, h_off, h_vert = _into(engine, app, N, len(ref.vertices) + 16, weighted=weighted, **kw)
    finally:
        engine.set_option("into_chunks", 6)
        engine.set_option("cursor_adjacency", 0)
        engine.set_option("into_stream", 1)
    assert steps == ref.total_steps
    np.testing.assert_array_equal(h_len, ref.path_length)
    total = int(h_len.sum(dtype=np.uint64))
    assert total == len(ref.vertices)
    np.testing.assert_array_equal(h_vert[:total], ref.vertices)
    np.testing.assert_array_equal(h_off[1:], np.cumsum(h_len.astype(np.uint64))[:-1])
    assert h_off[0] == 0


@pytest.mark.parametrize("stream", [1, 0])
def test_walk_into_epochs_and_small_capacity(engine, oracle_lib, stream):
    """Epochs (rate 0.5), streamed or in chunks, and a buffer one vertex short
    fails cleanly (before any copy in the streamed mode)."""
    import knightking_gb300 as kk
    csr = _load(engine, 31, True)
    kw = dict(walk_length=9, seed=11, rate=0.5)
    ref = engine.walk("deepwalk", N, weighted=True, **kw)
    lens, verts, _ = _oracle(oracle_lib, csr, "deepwalk", N, True, kw)
    np.testing.assert_array_equal(ref.path_length, lens)
    np.testing.assert_array_equal(ref.vertices, verts)
    total = len(ref.vertices)
    engine.set_option("into_stream", stream)
    try:
        steps, h_len, h_off, h_vert = _into(engine, "deepwalk", N, total, weighted=True, **kw)
        assert steps == ref.total_steps
        np.testing.assert_array_equal(h_len, ref.path_length)
        np.testing.assert_array_equal(h_vert, ref.vertices)
        with pytest.raises(kk.KKError):
            _into(engine, "deepwalk", N, total - 1, weighted=True, **kw)
        # the engine stays usable after the refused call
        steps2, h_len2, _, h_vert2 = _into(engine, "deepwalk", N, total, weighted=True, **kw)
        np.testing.assert_array_equal(h_vert2, ref.vertices)
    finally:
        engine.set_option("into_stream", 1)


@pytest.mark.parametrize("layout", [0, 2])
def test_walk_into_streamed_large_walk(engine, oracle_lib, layout):
    """A walk of 2^21 walkers over a graph with isolated vertices: 256
    segments of 8192 walkers, some holding only one-vertex paths; cursor and
    16 B neighbour buckets."""
    g = G.random_undirected(3000, 20000, seed=41, weight="unif")
    csr = G.csr_file_order(4000, g["src"], g["dst"], w=g.get("w"))  # vertices 3000.. are isolated
    engine.load_arrays(4000, csr["off"], csr["nbr"], csr.get("w"))
    n = 1 << 21
    kw = dict(walk_length=5, seed=13)
    ref = engine.walk("deepwalk", n, weighted=True, **kw)
    if layout == 0:
        lens, verts, _ = _oracle(oracle_lib, csr, "deepwalk", n, True, kw)
        np.testing.assert_array_equal(ref.path_length, lens)
        np.testing.assert_array_equal(ref.vertices, verts)
    engine.set_option("alias_layout", layout)
    try:
        steps, h_len, h_off, h_vert = _into(engine, "deepwalk", n, len(ref.vertices), weighted=True, **kw)
    finally:
        engine.set_option("alias_layout", 2)
    assert steps == ref.total_steps
    np.testing.assert_array_equal(h_len, ref.path_length)
    np.testing.assert_array_equal(h_vert, ref.vertices)
    np.testing.assert_array_equal(h_off[1:], np.cumsum(h_len.astype(np.uint64))[:-1])
