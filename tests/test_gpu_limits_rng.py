"""Device-side random stream and loop bounds.

* The device's Philox4x32-10 (the generator every walk draws from, replacing
  the reference's mt19937 of include/util.hpp:45-70) reproduces the published
  Random123 known answers and the oracle's generator on random counters.
* The rejection-trial bound: the reference's trial loop has no bound
  (include/walk.hpp:979-1041); the engine stops a walker whose step takes
  more than trial_limit trials and reports KK_ERR_TRIAL_LIMIT.  A metapath
  walk whose allowed edge type is rare runs the bound out; the engine stays
  usable and its next walk equals the oracle's.
"""

import ctypes

import numpy as np
import pytest

from oracle import graphs as G
from test_rng_kat_cpu import KAT, oracle_blocks, seed_of

pytestmark = pytest.mark.gpu


def device_blocks(kk, seed, ctr):
    ctr = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros_like(ctr)
    st = kk.lib().kk_philox_blocks(ctypes.c_uint64(seed), len(ctr), ctr.ctypes.data, out.ctypes.data)
    assert st == 0
    return out


def test_device_generator_matches_known_answers():
    import knightking_gb300 as kk
    for ctr, key, want in KAT:
        got = device_blocks(kk, seed_of(key), [ctr])[0]
        assert [int(x) for x in got] == list(want)


def test_device_generator_matches_oracle(oracle_lib):
    import knightking_gb300 as kk
    rng = np.random.default_rng(4)
    ctr = rng.integers(0, 1 << 32, size=(100000, 4), dtype=np.uint64).astype(np.uint32)
    for seed in (0, 1, 0xFFFFFFFFFFFFFFFF, 1234567890123):
        np.testing.assert_array_equal(device_blocks(kk, seed, ctr), oracle_blocks(oracle_lib, seed, ctr))


def _rare_type_graph():
    """Undirected graph, type 0 on most edges and type 4 on about 2%."""
    g = G.random_undirected(400, 8000, seed=61, weight="unif")
    rng = np.random.default_rng(62)
    t = np.where(rng.random(len(g["src"])) < 0.02, 4, 0).astype(np.uint8)
    return G.csr_file_order(400, g["src"], g["dst"], w=g["w"], type=t)


@pytest.mark.parametrize("park", [0, 20])
def test_trial_limit_is_reported_and_the_engine_recovers(oracle_lib, park):
    import knightking_gb300 as kk
    csr = _rare_type_graph()
    engine = kk.WalkEngine(0)
    try:
        engine.load_arrays(400, csr["off"], csr["nbr"], csr["w"], csr["type"])
        kw = dict(walk_length=20, schemes=[[1 << 4, 1 << 4]], weighted=True)
        engine.set_option("walk_park", park)
        engine.set_option("trial_limit", 2)
        with pytest.raises(kk.KKError) as err:
            engine.walk("metapath", 4000, seed=3, **kw)
        assert err.value.status == kk._capi.KK_ERR_TRIAL_LIMIT
        engine.set_option("trial_limit", 1 << 24)
        ps = engine.walk("metapath", 4000, seed=3, **kw)
        prm = oracle_lib.make_params("metapath", seed=3, walker_num=4000, **kw)
        lens, verts, steps = oracle_lib.walk(oracle_lib.CSR(400, csr["off"], csr["nbr"], csr["w"], csr["type"]), prm,
                                             cap=64)
        np.testing.assert_array_equal(ps.path_length, lens)
        np.testing.assert_array_equal(ps.vertices, verts)
        assert ps.total_steps == steps and steps > 0
    finally:
        engine.close()
