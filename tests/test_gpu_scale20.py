"""GPU parity at scale: R-MAT scale 20 (1,048,576 vertices, ~33 M directed
edges) generated on the device, checked walker for walker against the oracle
(the C restatement pinned to the reference) on walker-id ranges spread over
the id space.

The smaller test graphs never reach the paths these graphs take: hub rows
above the block-row class (degree > 16,384; the first ids of an R-MAT graph
are its largest hubs, and range 0 starts on them), the whole-graph alias
build over every degree class at once, offsets and tables far larger than
L2, the edge set of a graph of this size, and the served request mix.

Covered: the alias tables of the whole graph index for index and 0 ulp
(include/walk.hpp:538-652); DeepWalk on lognormal weights (src/apps/
deepwalk.hpp:30-47) under every alias layout; PPR with the cursor adjacency
(src/apps/ppr.hpp:30-64); node2vec in and out of the outlier regime
(src/apps/node2vec.hpp:108-202) with the edge set; metapath with three
schemes (src/apps/metapath.hpp:32-128); a batch of requests of the served
mix through kk_batch_walk.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402  (the bench's own parity helpers)

pytestmark = pytest.mark.gpu

SCALE = 20
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def engine():
    import knightking_gb300
    e = knightking_gb300.WalkEngine(0)
    yield e
    e.close()


def _load(engine, oracle_lib, weights, types=0):
    engine.generate_rmat(SCALE, 16, seed=SCALE, weights=weights, types=types)
    csr, alias, _ = bench.host_graph(engine, "x", THREADS)
    deg = np.diff(csr.off)
    assert deg.max() > 16384, "the scale-20 graph must hold hub rows above the block-row class"
    return csr, alias


def _ranges(engine, csr, alias, wl, chunks=8, per=4096):
    res = bench.parity_ranges(engine, csr, alias, wl, csr.V, THREADS, chunks=chunks, per=per)
    assert res["walkers_checked"] == chunks * per
    assert res["mismatches"] == 0, res
    return res


def test_alias_tables_whole_graph(engine, oracle_lib):
    csr, alias = _load(engine, oracle_lib, weights=2)
    p, pi, qi, s = engine.alias_tables()
    op, opi, oqi, osum = alias
    np.testing.assert_array_equal(pi, opi)
    np.testing.assert_array_equal(qi, oqi)
    np.testing.assert_array_equal(p.view(np.uint32), np.asarray(op).view(np.uint32))
    np.testing.assert_array_equal(s.view(np.uint32), np.asarray(osum).view(np.uint32))


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_deepwalk_lognormal(engine, oracle_lib, layout):
    csr, alias = _load(engine, oracle_lib, weights=2)
    engine.set_option("alias_layout", layout)
    try:
        _ranges(engine, csr, alias, dict(bench.WORKLOADS["deepwalk-s22"]))
    finally:
        engine.set_option("alias_layout", 2)


def test_ppr_cursor_adjacency(engine, oracle_lib):
    csr, alias = _load(engine, oracle_lib, weights=0)
    engine.set_option("cursor_adjacency", 1)
    try:
        _ranges(engine, csr, alias, dict(bench.WORKLOADS["ppr-s24"]))
    finally:
        engine.set_option("cursor_adjacency", 0)


@pytest.mark.parametrize("p,q", [(2.0, 0.5), (0.5, 2.0)])
def test_node2vec(engine, oracle_lib, p, q):
    csr, alias = _load(engine, oracle_lib, weights=1)
    wl = dict(bench.WORKLOADS["node2vec-s24"], p=p, q=q)
    _ranges(engine, csr, alias, wl, chunks=6, per=2048)


def test_metapath(engine, oracle_lib):
    csr, alias = _load(engine, oracle_lib, weights=1, types=5)
    _ranges(engine, csr, alias, dict(bench.WORKLOADS["metapath-s22"]))


def test_node2vec_batch_of_served_requests(engine, oracle_lib):
    """48 requests of the served mix (p, q log-uniform [0.25, 4], lengths
    5..200, lognormal walker counts capped at 8192 here) in one batch."""
    csr, alias = _load(engine, oracle_lib, weights=1)
    reqs = bench.serve_requests(dict(bench.WORKLOADS["node2vec-serve-s24"]), csr.V)[:48]
    for r in reqs:
        r["walker_num"] = min(r["walker_num"], 8192)
    assert any(bench.n2v_outlier(r["p"], r["q"]) for r in reqs)
    out = engine.batch_walk("node2vec", reqs)
    res = bench.parity_requests([(ps.path_length, ps.vertices) for ps in out], csr, alias, reqs, THREADS,
                                "batch vs oracle")
    assert res["mismatches"] == 0, res
