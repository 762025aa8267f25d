"""node2vec batches against the oracle, job by job.

Every job of a node2vec batch (kk_batch_walk, the kernel the serving slots
replay) must have the oracle's paths: the C restatement pinned to the
reference's node2vec (src/apps/node2vec.hpp:108-202, include/walk.hpp:
1082-1381).  Covered: every alias layout, weighted and unweighted, jobs in and
out of the outlier regime (1/p > max(1, 1/q)), undirected graphs and a
directed graph where the previous vertex is often not a neighbour (the
return-edge lookup misses the edge set and falls back to std::lower_bound's
binary search, which may find no edge), and the edge set against the binary
search of the sorted adjacency.
"""

import numpy as np
import pytest

from oracle import graphs as G

pytestmark = pytest.mark.gpu

JOBS = [dict(walker_num=300, seed=1, walk_length=20, p=2.0, q=0.5),
        dict(walker_num=7, seed=2, walk_length=50, p=0.25, q=4.0, walker_begin=1000),
        dict(walker_num=0, seed=3, walk_length=10, p=1.0, q=1.0),
        dict(walker_num=513, seed=4, walk_length=5, p=0.5, q=2.0),
        dict(walker_num=64, seed=5, walk_length=33, p=3.0, q=0.3, walker_begin=77),
        dict(walker_num=900, seed=6, walk_length=41, p=0.3, q=0.6, walker_begin=5),
        dict(walker_num=1000, seed=7, walk_length=12, p=0.26, q=0.27, walker_begin=123456)]


@pytest.fixture(scope="module")
def engine():
    import knightking_gb300 as kk
    e = kk.WalkEngine(0)
    yield e
    e.close()


def _graph(kind, weighted, seed):
    if kind == "undirected":
        g = G.random_undirected(400, 6000, seed=seed, weight="unif" if weighted else None)
        return G.csr_file_order(400, g["src"], g["dst"], w=g.get("w"))
    rng = np.random.default_rng(seed)
    V = 300
    src = rng.integers(0, V, size=4000)
    dst = rng.integers(0, V, size=4000)
    keep = src != dst
    pairs = np.unique(np.stack([src[keep], dst[keep]], 1), axis=0)
    w = (1.0 + 4.0 * rng.random(len(pairs))).astype(np.float32) if weighted else None
    return G.csr_file_order(V, pairs[:, 0].astype(np.uint32), pairs[:, 1].astype(np.uint32), w=w)


def _oracle_job(oracle_lib, csr, job, weighted):
    V = len(csr["off"]) - 1
    ocsr = oracle_lib.CSR(V, csr["off"], csr["nbr"], csr.get("w")).sorted_copy()
    prm = oracle_lib.make_params("node2vec", seed=job["seed"], walker_begin=job.get("walker_begin", 0),
                                 walker_num=job["walker_num"], walk_length=job["walk_length"], p=job["p"],
                                 q=job["q"], weighted=weighted)
    return oracle_lib.walk(ocsr, prm, cap=job["walk_length"] + 1)


@pytest.mark.parametrize("adjacency", [0, 1])
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("kind,weighted", [("undirected", True), ("undirected", False), ("directed", True),
                                           ("directed", False)])
def test_node2vec_batch_matches_oracle(engine, oracle_lib, kind, weighted, layout, adjacency):
    if not weighted and layout != 2:
        pytest.skip("alias layouts only matter with weights")
    csr = _graph(kind, weighted, 21)
    V = len(csr["off"]) - 1
    engine.load_arrays(V, csr["off"], csr["nbr"], csr.get("w"))
    jobs = [dict(j, weighted=weighted) for j in JOBS]
    engine.set_option("alias_layout", layout)
    engine.set_option("node2vec_adjacency", adjacency)
    try:
        got = engine.batch_walk("node2vec", jobs)
        engine.set_option("cursor_adjacency", 1)
        got_c = engine.batch_walk("node2vec", jobs) if not weighted else got
    finally:
        engine.set_option("alias_layout", 2)
        engine.set_option("node2vec_adjacency", 0)
        engine.set_option("cursor_adjacency", 0)
    for job, ps, pc in zip(jobs, got, got_c):
        lens, verts, steps = _oracle_job(oracle_lib, csr, job, weighted)
        np.testing.assert_array_equal(ps.path_length, lens)
        np.testing.assert_array_equal(ps.vertices, verts)
        assert ps.total_steps == steps
        np.testing.assert_array_equal(pc.path_length, lens)
        np.testing.assert_array_equal(pc.vertices, verts)


def test_node2vec_batch_trial_limit(engine, oracle_lib):
    """A trial limit of 1 ends the walks of rejecting jobs with
    KK_ERR_TRIAL_LIMIT; the engine recovers and walks the oracle's paths."""
    import knightking_gb300 as kk
    csr = _graph("undirected", True, 23)
    engine.load_arrays(400, csr["off"], csr["nbr"], csr["w"])
    jobs = [dict(walker_num=2000, seed=3, walk_length=40, p=4.0, q=4.0, weighted=True)]
    engine.set_option("trial_limit", 1)
    try:
        with pytest.raises(kk.KKError) as err:
            engine.batch_walk("node2vec", jobs)
        assert err.value.status == kk._capi.KK_ERR_TRIAL_LIMIT
    finally:
        engine.set_option("trial_limit", 1 << 24)
    ps = engine.batch_walk("node2vec", jobs)[0]
    lens, verts, _ = _oracle_job(oracle_lib, csr, jobs[0], True)
    np.testing.assert_array_equal(ps.path_length, lens)
    np.testing.assert_array_equal(ps.vertices, verts)
