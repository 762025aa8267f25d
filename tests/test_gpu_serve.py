"""Serving (kk_serve_*): continuous batching of requests from several client
threads on two slots.  Every request's paths equal those of the same request
run alone through kk_walk (bit-identical), whatever else shared its batch and
whichever slot ran it, and equal the oracle's (the C restatement pinned to the
reference); the server reports its latency statistics."""

import threading

import numpy as np
import pytest

from oracle import graphs as G

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]


@pytest.fixture(scope="module")
def engine():
    import knightking_gb300 as kk
    e = kk.WalkEngine(0)
    yield e
    e.close()


def _load(engine, seed, types=False):
    g = G.random_undirected(600, 8000, seed=seed, weight="unif", types="uniform" if types else None)
    csr = G.csr_file_order(600, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(600, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    return csr


def _oracle(oracle_lib, csr, app, r):
    ocsr = oracle_lib.CSR(600, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    if app == "node2vec":
        ocsr = ocsr.sorted_copy()
    kw = dict(r)
    prm = oracle_lib.make_params(app, weighted=True, **kw)
    return oracle_lib.walk(ocsr, prm, cap=r["walk_length"] + 1)


def _requests(app, n, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        r = dict(walker_num=int(np.clip(rng.lognormal(np.log(64), 1.0), 1, 2000)), seed=int(rng.integers(1, 2**40)),
                 walk_length=int(rng.integers(5, 120)), walker_begin=int(rng.integers(0, 1 << 20)))
        if app == "node2vec":
            r["p"] = float(np.exp(rng.uniform(np.log(0.25), np.log(4))))
            r["q"] = float(np.exp(rng.uniform(np.log(0.25), np.log(4))))
        if app == "metapath":
            r["schemes"] = [[1 << int(t) for t in rng.integers(0, 5, int(rng.integers(1, 5)))] for _ in range(3)]
        reqs.append(r)
    return reqs


def _serve_all(engine, app, reqs, clients=4, **server_kw):
    results = [None] * len(reqs)
    srv = engine.serve(app, **server_kw)
    try:
        def client(k):
            tickets = [(i, srv.submit(**reqs[i])) for i in range(k, len(reqs), clients)]
            for i, t in tickets:
                results[i] = srv.poll(t)
        th = [threading.Thread(target=client, args=(k,)) for k in range(clients)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        stats = srv.stats()
    finally:
        srv.stop()
    return results, stats


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("app", ["node2vec", "deepwalk", "metapath"])
def test_served_requests_equal_alone(engine, oracle_lib, app, graphs):
    """Slots replaying captured CUDA graphs, and slots launching on their streams."""
    csr = _load(engine, 11, types=app == "metapath")
    reqs = _requests(app, 60, seed=5)
    results, stats = _serve_all(engine, app, reqs, slots=2, max_jobs=16, slot_bytes=8 << 20, graphs=graphs)
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["batches"] >= 2
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for r, res in zip(reqs, results):
        assert res.status == 0
        kw = dict(r)
        alone = engine.walk(app, kw.pop("walker_num"), **kw)
        np.testing.assert_array_equal(res.paths.path_length, alone.path_length)
        np.testing.assert_array_equal(res.paths.vertices, alone.vertices)
        assert res.paths.total_steps == alone.total_steps
        assert res.latency_ms >= res.queue_ms >= 0
        if graphs:
            lens, verts, steps = _oracle(oracle_lib, csr, app, r)
            np.testing.assert_array_equal(res.paths.path_length, lens)
            np.testing.assert_array_equal(res.paths.vertices, verts)


def test_server_refuses_bad_requests(engine):
    import knightking_gb300 as kk
    _load(engine, 12)
    with engine.serve("node2vec", slots=1, max_jobs=4, slot_bytes=1 << 20) as srv:
        with pytest.raises(kk.KKError):
            srv.submit(100000, walk_length=80, p=1.0, q=1.0)      # larger than a slot
        with pytest.raises(kk.KKError):
            srv.submit(10, walk_length=80, p=0.0, q=1.0)           # p must be > 0
        t = srv.submit(10, walk_length=10, p=1.0, q=2.0)
        assert srv.poll(t).status == 0
        with pytest.raises(kk.KKError):
            srv.poll(t)                                             # handed out once


def test_replay_client_keeps_schedule_and_counts_every_step(engine):
    """kk_serve_replay (the library's open-loop client): every request
    completes with a latency, the walker-steps equal those of the same
    requests run alone (and so do the server's own statistics, which count
    the completed requests' steps from their paths), an arrival schedule that
    spreads the requests over 0.2 s is kept (the call lasts at least that
    long), and a schedule that runs backwards or a refused request is
    reported."""
    import knightking_gb300 as kk
    _load(engine, 13)
    reqs = _requests("node2vec", 80, seed=9)
    alone = sum(engine.walk("node2vec", dict(r)["walker_num"], **{k: v for k, v in r.items() if k != "walker_num"})
                .total_steps for r in reqs)
    with engine.serve("node2vec", slots=2, max_jobs=16, slot_bytes=8 << 20) as srv:
        lat, steps, elapsed = srv.replay(reqs, np.zeros(len(reqs)))
        assert steps == alone
        assert np.all(lat > 0)
        st = srv.stats()
        assert st["walker_steps"] == alone and st["completed"] == len(reqs) and st["failed"] == 0
        arrivals = np.linspace(0.0, 0.2, len(reqs))
        lat, steps, elapsed = srv.replay(reqs, arrivals)
        assert steps == alone and np.all(lat > 0)
        assert elapsed >= 0.2
        with pytest.raises(kk.KKError):
            srv.replay(reqs[:3], [0.0, 0.2, 0.1])
        bad = [dict(reqs[0]), dict(reqs[1], p=0.0), dict(reqs[2])]
        with pytest.raises(kk.KKError):
            srv.replay(bad, np.zeros(3))
        # the server still serves after the refused request
        lat, steps, _ = srv.replay(reqs[:4], np.zeros(4))
        assert np.all(lat > 0)


@pytest.mark.parametrize("graphs", [True, False])
def test_failed_request_fails_alone(engine, oracle_lib, graphs):
    """Each request of a batch is handed out with its own outcome as soon as
    its own walkers end: with a trial limit of 1, requests whose scheme
    allows one edge type per step (most steps need more trials) fail with
    KK_ERR_TRIAL_LIMIT, while the requests that shared their batches, whose
    scheme allows every type (every trial accepted), come back with the
    oracle's paths."""
    csr = _load(engine, 14, types=True)
    good = [dict(walker_num=40 + i, seed=100 + i, walk_length=12 + i, walker_begin=50 * i, schemes=[[31, 31, 31]])
            for i in range(24)]
    bad = [dict(walker_num=30 + i, seed=300 + i, walk_length=15, walker_begin=2000 + 50 * i, schemes=[[1], [2]])
           for i in range(8)]
    reqs = []
    for i in range(8):
        reqs += good[3 * i:3 * i + 3] + [bad[i]]
    engine.set_option("trial_limit", 1)
    try:
        results, stats = _serve_all(engine, "metapath", reqs, clients=2, slots=2, max_jobs=16,
                                    slot_bytes=8 << 20, graphs=graphs)
    finally:
        engine.set_option("trial_limit", 1 << 24)
    assert stats["completed"] == len(good) and stats["failed"] == len(bad)
    for r, res in zip(reqs, results):
        if r["schemes"] == [[1], [2]]:
            assert res.status == 4 and res.paths is None  # KK_ERR_TRIAL_LIMIT
        else:
            assert res.status == 0
            lens, verts, steps = _oracle(oracle_lib, csr, "metapath", r)
            np.testing.assert_array_equal(res.paths.path_length, lens)
            np.testing.assert_array_equal(res.paths.vertices, verts)
    # the server's engine serves again at the usual limit
    results, stats = _serve_all(engine, "metapath", bad[:2], clients=1, slots=1, max_jobs=4, slot_bytes=8 << 20)
    assert all(res.status == 0 for res in results)


def test_request_of_no_walkers_is_served(engine):
    """A request of zero walkers shares a batch with others and comes back at
    once, empty; the others keep their paths."""
    _load(engine, 15)
    reqs = _requests("node2vec", 12, seed=21)
    reqs.insert(5, dict(walker_num=0, seed=7, walk_length=30, walker_begin=3, p=1.0, q=2.0))
    results, stats = _serve_all(engine, "node2vec", reqs, clients=1, slots=1, max_jobs=32, slot_bytes=8 << 20)
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert results[5].status == 0 and results[5].paths.path_num == 0
    for r, res in zip(reqs, results):
        if r["walker_num"]:
            kw = dict(r)
            alone = engine.walk("node2vec", kw.pop("walker_num"), **kw)
            np.testing.assert_array_equal(res.paths.vertices, alone.vertices)
