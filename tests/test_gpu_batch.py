"""Batched walks (kk_batch_walk): every job of a batch has exactly the paths it
has when run alone through kk_walk and the oracle's paths (the C restatement
pinned to the reference).

Jobs in one batch differ in seed, walker range, walk length, node2vec (p, q)
(in and out of the outlier regime) and metapath schemes."""

import numpy as np
import pytest

from oracle import graphs as G

pytestmark = pytest.mark.gpu


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


def _check(engine, app, jobs, oracle_lib=None, csr=None):
    """Both batch schedules (one walker per thread, the persistent pool) and
    uniform picks with and without the cursor adjacency."""
    batch = engine.batch_walk(app, jobs)
    engine.set_option("walk_schedule", 1)
    try:
        pooled = engine.batch_walk(app, jobs)
    finally:
        engine.set_option("walk_schedule", 0)
    engine.set_option("cursor_adjacency", 1)
    try:
        cursored = engine.batch_walk(app, jobs)
    finally:
        engine.set_option("cursor_adjacency", 0)
    for a, b, c in zip(batch, pooled, cursored):
        np.testing.assert_array_equal(a.path_length, b.path_length)
        np.testing.assert_array_equal(a.vertices, b.vertices)
        np.testing.assert_array_equal(a.path_length, c.path_length)
        np.testing.assert_array_equal(a.vertices, c.vertices)
    assert len(batch) == len(jobs)
    for job, got in zip(jobs, batch):
        kw = dict(job)
        n = kw.pop("walker_num")
        alone = engine.walk(app, n, **kw)
        np.testing.assert_array_equal(got.path_length, alone.path_length)
        np.testing.assert_array_equal(got.vertices, alone.vertices)
        assert got.walker_begin == alone.walker_begin
        assert got.total_steps == alone.total_steps
        if oracle_lib is not None:
            ocsr = oracle_lib.CSR(400, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
            if app == "node2vec":
                ocsr = ocsr.sorted_copy()
            prm = oracle_lib.make_params(app, walker_num=n, **kw)
            lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=kw["walk_length"] + 1)
            np.testing.assert_array_equal(got.path_length, lens)
            np.testing.assert_array_equal(got.vertices, verts)


@pytest.mark.parametrize("weighted", [True, False])
def test_node2vec_batch_equals_single_jobs(engine, oracle_lib, weighted):
    csr = _load(engine, 3, weighted)
    jobs = [dict(walker_num=300, seed=1, walk_length=20, p=2.0, q=0.5, weighted=weighted),
            dict(walker_num=7, seed=2, walk_length=50, p=0.25, q=4.0, weighted=weighted, walker_begin=1000),
            dict(walker_num=0, seed=3, walk_length=10, p=1.0, q=1.0, weighted=weighted),
            dict(walker_num=513, seed=4, walk_length=5, p=0.5, q=2.0, weighted=weighted),
            dict(walker_num=64, seed=5, walk_length=33, p=3.0, q=0.3, weighted=weighted, walker_begin=77)]
    _check(engine, "node2vec", jobs, oracle_lib, csr)


@pytest.mark.parametrize("weighted", [True, False])
def test_metapath_batch_equals_single_jobs(engine, oracle_lib, weighted):
    csr = _load(engine, 4, weighted, types=True)
    jobs = [dict(walker_num=400, seed=7, walk_length=30, weighted=weighted, schemes=[[1, 2, 4, 8], [2, 8, 2, 16]]),
            dict(walker_num=129, seed=8, walk_length=12, weighted=weighted, schemes=[[3, 12]],
                 scheme_round_robin=True),
            dict(walker_num=1000, seed=9, walk_length=60, weighted=weighted,
                 schemes=[[31], [1, 2], [4, 16, 8]], scheme_round_robin=True)]
    _check(engine, "metapath", jobs, oracle_lib, csr)


@pytest.mark.parametrize("weighted,layout", [(True, 2), (True, 0), (True, 1), (False, 2)])
def test_deepwalk_batch_equals_single_jobs(engine, oracle_lib, weighted, layout):
    """Every alias layout: 16 B neighbour buckets (the default), cursor and index buckets."""
    csr = _load(engine, 5, weighted)
    jobs = [dict(walker_num=n, seed=s, walk_length=l, weighted=weighted, walker_begin=b)
            for n, s, l, b in ((1, 1, 80, 0), (1024, 2, 5, 10), (333, 3, 200, 5000), (2048, 4, 17, 0))]
    engine.set_option("alias_layout", layout)
    try:
        _check(engine, "deepwalk", jobs, oracle_lib, csr)
    finally:
        engine.set_option("alias_layout", 2)


def test_batch_rejects_mixed_apps_and_ppr(engine):
    import knightking_gb300 as kk
    _load(engine, 6, True)
    with pytest.raises(kk.KKError):
        engine.batch_walk("deepwalk", [dict(walker_num=3, weighted=True), dict(walker_num=3, weighted=False)])
    with pytest.raises(kk.KKError):
        engine.batch_walk("ppr", [dict(walker_num=3, terminate_prob=0.1)])


def test_batch_results_from_pooled_blocks_across_calls(engine):
    """kk_batch_walk hands its results out in pooled pinned blocks: blocks
    returned by one call (kk_paths_free) carry the next call's paths, and the
    counts-only form frees them without reading."""
    _load(engine, 7, True)
    jobs = [dict(walker_num=n, seed=s, walk_length=l, weighted=True, walker_begin=b)
            for n, s, l, b in ((5000, 11, 40, 0), (0, 12, 9, 0), (777, 13, 3, 123), (1, 14, 100, 9))]
    first = engine.batch_walk("deepwalk", jobs)
    counts = engine.batch_walk("deepwalk", jobs, keep_paths=False)
    again = engine.batch_walk("deepwalk", jobs)
    for a, b, c, job in zip(first, again, counts, jobs):
        np.testing.assert_array_equal(a.path_length, b.path_length)
        np.testing.assert_array_equal(a.vertices, b.vertices)
        assert c["walker_num"] == job["walker_num"] == a.path_num
        assert c["total_steps"] == a.total_steps
        assert c["vertices"] == len(a.vertices)


@pytest.mark.parametrize("app", ["node2vec", "metapath"])
def test_submitted_batch_equals_batch_walk(engine, oracle_lib, app):
    """kk_batch_submit / kk_batch_wait: the engine refuses other calls while
    the batch is outstanding, and the waited-for paths equal kk_batch_walk's
    and the oracle's; metapath runs with parking, as kk_batch_walk does."""
    import knightking_gb300 as kk
    csr = _load(engine, 8, True, types=app == "metapath")
    if app == "node2vec":
        jobs = [dict(walker_num=n, seed=s, walk_length=l, p=p, q=q, weighted=True, walker_begin=b)
                for n, s, l, p, q, b in ((300, 1, 20, 2.0, 0.5, 0), (0, 2, 10, 1.0, 1.0, 0),
                                         (900, 3, 60, 0.25, 4.0, 50), (17, 4, 5, 0.5, 0.5, 333))]
    else:
        jobs = [dict(walker_num=700, seed=7, walk_length=30, weighted=True, schemes=[[1, 2, 4, 8], [2, 8, 2, 16]]),
                dict(walker_num=64, seed=8, walk_length=12, weighted=True, schemes=[[3, 12]],
                     scheme_round_robin=True)]
    ref = engine.batch_walk(app, jobs)
    b = engine.batch_submit(app, jobs)
    with pytest.raises(kk.KKError):
        engine.walk(app, 4, **{k: v for k, v in jobs[0].items() if k != "walker_num"})
    with pytest.raises(kk.KKError):
        engine.batch_submit(app, jobs)
    got = b.wait()
    with pytest.raises(ValueError):
        b.wait()
    assert len(got) == len(jobs)
    for job, g, r in zip(jobs, got, ref):
        np.testing.assert_array_equal(g.path_length, r.path_length)
        np.testing.assert_array_equal(g.vertices, r.vertices)
        assert g.total_steps == r.total_steps
        kw = dict(job)
        n = kw.pop("walker_num")
        ocsr = oracle_lib.CSR(400, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
        if app == "node2vec":
            ocsr = ocsr.sorted_copy()
        lens, verts, _ = oracle_lib.walk(ocsr, oracle_lib.make_params(app, walker_num=n, **kw),
                                         cap=kw["walk_length"] + 1)
        np.testing.assert_array_equal(g.path_length, lens)
        np.testing.assert_array_equal(g.vertices, verts)
    # the engine serves calls again
    assert engine.walk(app, 4, **{k: v for k, v in jobs[0].items() if k != "walker_num"}).total_steps >= 0
