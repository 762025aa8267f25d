"""Regrouped walks (option regroup_interval = k): the walk runs in phases of k
steps and each phase takes its walkers sorted by the vertex they stand on.
The stream is keyed by (walker, step), so the paths must stay the reference's:

* every golden fixture of the built-in apps (the reference's own paths) with
  k = 1 and k = 3, covering isolated vertices, zero length and immediate
  termination;
* R-MAT scale-16 walks of DeepWalk, PPR (also with the cursor adjacency),
  node2vec and metapath (parking off, so it regroups) against the oracle on
  walker-id ranges, k in {1, 5, 16};
* kk_walk_into (streamed segments) regrouped against the oracle.
"""

import os
import sys

import numpy as np
import pytest

from cases import Case, case_ids, walk_kwargs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402  (the bench's own parity helpers)

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
APP_CASES = [c for c in case_ids() if not c.startswith(("case_alias", "case_t200", "case_dyn"))]


@pytest.fixture(scope="module")
def engine():
    import knightking_gb300
    e = knightking_gb300.WalkEngine(0)
    yield e
    e.close()


@pytest.fixture
def regroup(engine):
    def set_k(k, park=20):
        engine.set_option("regroup_interval", k)
        engine.set_option("walk_park", park)
    yield set_k
    engine.set_option("regroup_interval", 0)
    engine.set_option("walk_park", 20)


@pytest.mark.parametrize("k", [1, 3])
@pytest.mark.parametrize("name", APP_CASES)
def test_golden_paths_regrouped(engine, regroup, name, k):
    case = Case(name)
    g = case.graph()
    engine.load_arrays(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))
    regroup(k, park=0)
    kw = walk_kwargs(case)
    n = kw.pop("walker_num")
    ps = engine.walk(case.cmd, n, **kw)
    np.testing.assert_array_equal(ps.path_length, case.lens)
    np.testing.assert_array_equal(ps.vertices, case.verts)


WL = {
    "deepwalk": (dict(app="deepwalk", walk_length=80), dict(weights=2)),
    "ppr": (dict(app="ppr", terminate_prob=1.0 / 80), dict(weights=0)),
    "node2vec": (dict(app="node2vec", walk_length=80, p=2.0, q=0.5), dict(weights=1)),
    "node2vec_outlier": (dict(app="node2vec", walk_length=40, p=0.5, q=2.0), dict(weights=1)),
    "metapath": (dict(app="metapath", walk_length=80, schemes=[[1, 2, 4, 8], [2, 8, 2, 16], [4, 1, 16, 4]],
                      scheme_round_robin=True), dict(weights=1, types=5)),
}


@pytest.mark.parametrize("k", [1, 5, 16])
@pytest.mark.parametrize("which", sorted(WL))
def test_rmat16_regrouped_matches_oracle(engine, oracle_lib, regroup, which, k):
    wl, gen = WL[which]
    engine.generate_rmat(16, 16, seed=16, **gen)
    csr, alias, _ = bench.host_graph(engine, wl["app"], THREADS)
    regroup(k, park=0)
    res = bench.parity_ranges(engine, csr, alias, wl, csr.V, THREADS, chunks=4, per=4096)
    assert res["walkers_checked"] == 4 * 4096
    assert res["mismatches"] == 0, res


def test_ppr_cursor_adjacency_regrouped(engine, oracle_lib, regroup):
    wl, gen = WL["ppr"]
    engine.generate_rmat(16, 16, seed=16, **gen)
    csr, alias, _ = bench.host_graph(engine, "ppr", THREADS)
    regroup(4)
    engine.set_option("cursor_adjacency", 1)
    try:
        res = bench.parity_ranges(engine, csr, alias, wl, csr.V, THREADS, chunks=4, per=4096)
    finally:
        engine.set_option("cursor_adjacency", 0)
    assert res["mismatches"] == 0, res


@pytest.mark.parametrize("app", ["deepwalk", "node2vec"])
def test_walk_into_regrouped_matches_oracle(engine, oracle_lib, regroup, app):
    wl, gen = WL[app]
    engine.generate_rmat(16, 16, seed=16, **gen)
    csr, alias, _ = bench.host_graph(engine, app, THREADS)
    n = csr.V
    L = wl["walk_length"]
    kw = {k: v for k, v in wl.items() if k != "app"}
    h_len = np.zeros(n, np.uint32)
    h_off = np.zeros(n, np.uint64)
    h_vert = np.zeros(n * (L + 1), np.uint32)
    regroup(8)
    steps = engine.walk_into(app, n, h_len.ctypes.data, h_off.ctypes.data, h_vert.ctypes.data, len(h_vert), seed=3,
                             weighted=True, **kw)
    lens, verts, st = bench.oracle_paths(csr, alias, app, THREADS, L + 1, seed=3, walker_begin=0, walker_num=n,
                                         weighted=True, **kw)
    assert steps == st
    np.testing.assert_array_equal(h_len, lens)
    np.testing.assert_array_equal(h_vert[:int(h_len.sum())], verts)
