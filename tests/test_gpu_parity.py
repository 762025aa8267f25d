"""GPU parity: the CUDA walker-step path against the reference's own outputs.

* every golden fixture (paths of the reference's engine with the Philox hook):
  bit-identical paths per walker id; alias tables index for index, 0 ulp;
* R-MAT scale 16 (the node2vec configuration and its siblings): the device
  generator reproduces the graph (SHA-256) and the walks reproduce the
  reference's path digest over all 65,536 walkers;
* fresh seeds and graphs beyond the fixtures, against the CPU oracle (itself
  pinned to the reference by tests/test_oracle_golden.py).
All calls go through the C-ABI (knightking_gb300 -> libknightking_gb300.so).
"""

import hashlib
import json
import os

import numpy as np
import pytest

from cases import GOLDEN, Case, case_ids, walk_kwargs
from oracle import graphs as G

pytestmark = pytest.mark.gpu

# tag walks and the dynamic walk have user hooks: their own tests run them
APP_CASES = [c for c in case_ids() if not c.startswith(("case_alias", "case_t200", "case_dyn"))]


@pytest.fixture(scope="module")
def kk():
    import knightking_gb300
    return knightking_gb300


@pytest.fixture(scope="module")
def engine(kk):
    e = kk.WalkEngine(0)
    yield e
    e.close()


def load_case(engine, case):
    g = case.graph()
    engine.load_arrays(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))


def gpu_walk(engine, case):
    kw = walk_kwargs(case)
    n = kw.pop("walker_num")
    return engine.walk(case.cmd, n, **kw)


@pytest.mark.parametrize("name", APP_CASES)
def test_paths_match_reference(engine, name):
    case = Case(name)
    load_case(engine, case)
    ps = gpu_walk(engine, case)
    np.testing.assert_array_equal(ps.path_length, case.lens)
    np.testing.assert_array_equal(ps.vertices, case.verts)
    assert ps.total_steps == int(case.lens.sum()) - len(case.lens)


@pytest.mark.parametrize("name", case_ids("case_alias"))
def test_alias_tables_match_reference(engine, name):
    case = Case(name)
    load_case(engine, case)
    p, pi, qi, s = engine.alias_tables()
    d = case.d
    np.testing.assert_array_equal(pi, d["alias_pidx"])
    np.testing.assert_array_equal(qi, d["alias_qidx"])
    np.testing.assert_array_equal(p.view(np.uint32), d["alias_p"].view(np.uint32))
    np.testing.assert_array_equal(s.view(np.uint32), d["alias_sum"].view(np.uint32))


def _csr_digest(g):
    h = hashlib.sha256()
    for k in ("off", "nbr", "w", "type"):
        if g.get(k) is not None:
            h.update(np.ascontiguousarray(g[k]).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", case_ids("rmat16_"))
def test_rmat16_matches_reference_digest(engine, name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    gen = json.loads(str(d["rmat"]))
    engine.generate_rmat(gen["scale"], gen["edge_factor"], gen["a"], gen["b"], gen["c"], seed=gen["seed"],
                         weights=1 if gen.get("weights") else 0, types=5 if gen.get("types") else 0)
    g = engine.download_graph()
    assert _csr_digest(g) == str(d["graph_sha256"]), "device R-MAT differs from the fixture's graph"
    params = json.loads(str(d["params"]))
    cmd = str(d["cmd"])
    kw = dict(seed=params["seed"], weighted=str(d["kind"]) != "none")
    if "len" in params:
        kw["walk_length"] = params["len"]
    if "term" in params:
        kw["terminate_prob"] = float(np.float32(params["term"]))
    if cmd == "node2vec":
        kw["p"], kw["q"] = params["p"], params["q"]
    if cmd == "metapath":
        kw["schemes"] = params["schemes"]
    ps = engine.walk(cmd, params["walkers"], **kw)
    assert ps.total_steps == int(d["total_steps"])
    nh = len(d["head_lens"])
    np.testing.assert_array_equal(ps.path_length[:nh], d["head_lens"])
    np.testing.assert_array_equal(ps.vertices[:int(d["head_lens"].sum())], d["head_verts"])
    assert G.paths_digest(ps.path_length, ps.vertices) == str(d["paths_sha256"])


# ---- beyond the fixtures: against the pinned CPU oracle ----

FRESH = [
    ("deepwalk", dict(weight="unif"), dict(walk_length=40)),
    ("deepwalk", dict(), dict(walk_length=40)),
    ("ppr", dict(weight="int5"), dict(terminate_prob=0.02)),
    ("ppr", dict(), dict(terminate_prob=0.2)),
    ("node2vec", dict(weight="unif"), dict(walk_length=30, p=0.4, q=1.7)),
    ("node2vec", dict(weight="unif"), dict(walk_length=30, p=3.0, q=0.3)),
    ("node2vec", dict(), dict(walk_length=30, p=0.2, q=0.9)),
    ("metapath", dict(weight="unif", types="uniform"), dict(walk_length=30, schemes=[[3, 6, 12], [17, 8]])),
    ("metapath", dict(types="uniform"), dict(walk_length=30, schemes=[[1, 2, 4, 8, 16]])),
]


@pytest.mark.parametrize("i", range(len(FRESH)))
@pytest.mark.parametrize("seed,schedule,layout", [(7, 0, 0), (1234567890123, 1, 1), (99, 1, 0), (5, 0, 1)])
def test_fresh_walks_match_oracle(engine, oracle_lib, i, seed, schedule, layout):
    """Both walk schedules (one walker per thread, persistent walker pool),
    both alias-table layouts (cursor buckets where allowed, index buckets),
    both node2vec adjacency tests (edge set, binary search) and uniform picks
    with and without the cursor adjacency."""
    app, gkw, wkw = FRESH[i]
    g = G.random_undirected(500, 6000, seed=seed % 1000 + i, **gkw)
    csr = G.csr_file_order(500, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    weighted = "w" in csr
    n = 1500
    engine.set_option("walk_schedule", schedule)
    engine.set_option("alias_layout", layout)
    engine.set_option("node2vec_adjacency", layout)
    engine.set_option("cursor_adjacency", 1 - layout)
    try:
        ps = engine.walk(app, n, seed=seed, weighted=weighted, walker_begin=77, **wkw)
    finally:
        engine.set_option("walk_schedule", 0)
        engine.set_option("alias_layout", 2)
        engine.set_option("node2vec_adjacency", 0)
        engine.set_option("cursor_adjacency", 0)
    ocsr = oracle_lib.CSR(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    if app == "node2vec":
        ocsr = ocsr.sorted_copy()
    prm = oracle_lib.make_params(app, seed=seed, walker_begin=77, walker_num=n, weighted=weighted, **wkw)
    lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=4096)
    np.testing.assert_array_equal(ps.path_length, lens)
    np.testing.assert_array_equal(ps.vertices, verts)
    assert ps.total_steps == steps


@pytest.mark.parametrize("app", ["deepwalk", "ppr", "node2vec"])
def test_dead_ends_and_isolated_starts_match_oracle(kk, engine, oracle_lib, app):
    """A directed graph with dead ends (vertices without out-edges that walks
    reach) and isolated start vertices: paths end early there, so the engine
    cannot know their lengths before the walk and packs them afterwards; on
    the same graph made undirected (isolated starts only) the walk writes
    them packed.  Both match the oracle, through kk_walk and kk_walk_into."""
    rng = np.random.default_rng(5)
    V = 300
    src = rng.integers(0, V, size=2400)
    dst = rng.integers(0, V, size=2400)
    keep = (src % 7 != 0) & (src != dst)  # sources divisible by 7 have no out-edges
    for directed in (True, False):
        s, d = src[keep], dst[keep]
        if not directed:
            s, d = np.concatenate([s, d]), np.concatenate([d, s])
            iso = (s % 11 == 5) | (d % 11 == 5)  # these vertices end up isolated
            s, d = s[~iso], d[~iso]
        pairs = np.unique(np.stack([s, d], 1), axis=0)
        csr = G.csr_file_order(V, pairs[:, 0].astype(np.uint32), pairs[:, 1].astype(np.uint32))
        engine.load_arrays(V, csr["off"], csr["nbr"])
        kw = dict(walk_length=12) if app != "ppr" else dict(terminate_prob=0.1)
        if app == "node2vec":
            kw.update(p=2.0, q=0.5)
        n = 2000
        ps = engine.walk(app, n, seed=9, **kw)
        ocsr = oracle_lib.CSR(V, csr["off"], csr["nbr"])
        if app == "node2vec":
            ocsr = ocsr.sorted_copy()
        prm = oracle_lib.make_params(app, seed=9, walker_num=n, weighted=False, **kw)
        lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=4096)
        np.testing.assert_array_equal(ps.path_length, lens)
        np.testing.assert_array_equal(ps.vertices, verts)
        h_len = np.zeros(n, np.uint32)
        h_off = np.zeros(n, np.uint64)
        h_vert = np.zeros(len(verts), np.uint32)
        assert engine.walk_into(app, n, h_len.ctypes.data, h_off.ctypes.data, h_vert.ctypes.data, len(verts),
                                seed=9, **kw) == steps
        np.testing.assert_array_equal(h_len, lens)
        np.testing.assert_array_equal(h_vert, verts)


@pytest.mark.parametrize("multi", [2, 4])
@pytest.mark.parametrize("i", [0, 1, 2, 3])
def test_multi_walker_kernel_matches_oracle(engine, oracle_lib, i, multi):
    """Several walkers per thread (DeepWalk and PPR), both alias layouts."""
    app, gkw, wkw = FRESH[i]
    g = G.random_undirected(500, 6000, seed=40 + i, **gkw)
    csr = G.csr_file_order(500, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    weighted = "w" in csr
    n = 1500
    ocsr = oracle_lib.CSR(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    prm = oracle_lib.make_params(app, seed=31, walker_begin=9, walker_num=n, weighted=weighted, **wkw)
    lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=4096)
    engine.set_option("walk_multi", multi)
    try:
        for layout in (0, 1):
            engine.set_option("alias_layout", layout)
            engine.set_option("cursor_adjacency", layout)
            ps = engine.walk(app, n, seed=31, weighted=weighted, walker_begin=9, **wkw)
            np.testing.assert_array_equal(ps.path_length, lens)
            np.testing.assert_array_equal(ps.vertices, verts)
            assert ps.total_steps == steps
    finally:
        engine.set_option("walk_multi", 1)
        engine.set_option("alias_layout", 2)
        engine.set_option("cursor_adjacency", 0)


def test_ppr_start_list_matches_oracle(engine, oracle_lib):
    g = G.random_undirected(300, 3000, seed=3, weight="int5")
    csr = G.csr_file_order(300, g["src"], g["dst"], w=g["w"])
    engine.load_arrays(300, csr["off"], csr["nbr"], csr["w"])
    start = np.array([5, 17, 17, 250, 3], np.uint32)
    ps = engine.walk("ppr", 1000, seed=9, terminate_prob=0.05, start=start)
    prm = oracle_lib.make_params("ppr", seed=9, walker_num=1000, terminate_prob=0.05, weighted=True, start=start)
    lens, verts, _ = oracle_lib.walk(oracle_lib.CSR(300, csr["off"], csr["nbr"], csr["w"]), prm, cap=4096)
    np.testing.assert_array_equal(ps.path_length, lens)
    np.testing.assert_array_equal(ps.vertices, verts)


def test_epochs_give_the_same_paths_and_dump(kk, engine, tmp_path):
    """WalkConfig rate (-r) splits walkers into epochs (include/walk.hpp:804-844):
    paths per walker do not change, and the dump equals the reference's text."""
    d = np.load(os.path.join(GOLDEN, "dump_deepwalk_head1.npz"))
    params = json.loads(str(d["params"]))
    V = int(d["V"])
    csr = G.csr_file_order(V, d["src"], d["dst"], w=d["w"])
    engine.load_arrays(V, csr["off"], csr["nbr"], csr["w"])
    conf = kk.WalkConfig()
    conf.set_walk_rate(params["rate"])
    conf.set_output_file(str(tmp_path / "walks"), True)
    engine.set_concurrency(params["threads"])
    ps = kk.deepwalk(engine, params["walkers"], params["len"], conf, seed=params["seed"])
    engine.set_concurrency(1)
    np.testing.assert_array_equal(ps.path_length, d["lens"])
    np.testing.assert_array_equal(ps.vertices, d["verts"])
    assert (tmp_path / "walks.0").read_text() == str(d["text"])


def test_binary_file_load_matches_file_order(kk, engine, tmp_path):
    g = G.random_undirected(200, 2000, seed=11, weight="int5")
    f = tmp_path / "g.bin"
    G.write_edge_file(f, g, "f32")
    engine.load_graph(200, f, kind="f32")
    dg = engine.download_graph()
    csr = G.csr_file_order(200, g["src"], g["dst"], w=g["w"])
    np.testing.assert_array_equal(dg["off"], csr["off"])
    np.testing.assert_array_equal(dg["nbr"], csr["nbr"])
    np.testing.assert_array_equal(dg["w"], csr["w"])
    # --make-undirected on a directed file: edges mirrored one by one (include/graph.hpp:430-443)
    half = {"V": 200, "src": g["src"][0::2], "dst": g["dst"][0::2], "w": g["w"][0::2]}
    G.write_edge_file(f, half, "f32")
    engine.load_graph(200, f, load_as_undirected=True, kind="f32")
    dg2 = engine.download_graph()
    np.testing.assert_array_equal(dg2["nbr"], csr["nbr"])
    # the call's timing: the whole call, and the device part inside it
    total_ms, device_ms = engine.load_timing()
    assert 0.0 < device_ms <= total_ms


def test_binary_file_load_in_parallel_and_refusals(kk, engine, tmp_path):
    """A file of more than 2^16 records is read and split by several host
    threads: the CSR still keeps file order within each source, with and
    without --make-undirected (include/graph.hpp:309-330, :430-443).  A record
    whose endpoint is >= v_num, or in a typed file whose type is outside
    [0, 8), is refused; the engine keeps its graph and loads the next file.
    Untyped records are split on the device, typed ones on the host: both
    paths are covered, unweighted too."""
    rng = np.random.default_rng(5)
    V, n = 5000, 300_000
    g = {"V": V, "src": rng.integers(0, V, n).astype(np.uint32), "dst": rng.integers(0, V, n).astype(np.uint32),
         "w": rng.random(n, dtype=np.float32)}
    f = tmp_path / "big.bin"
    G.write_edge_file(f, g, "f32")
    engine.load_graph(V, f, kind="f32")
    dg = engine.download_graph()
    csr = G.csr_file_order(V, g["src"], g["dst"], w=g["w"])
    np.testing.assert_array_equal(dg["off"], csr["off"])
    np.testing.assert_array_equal(dg["nbr"], csr["nbr"])
    np.testing.assert_array_equal(dg["w"], csr["w"])
    engine.load_graph(V, f, load_as_undirected=True, kind="f32")
    dg2 = engine.download_graph()
    s2 = np.empty(2 * n, np.uint32)
    d2 = np.empty(2 * n, np.uint32)
    s2[0::2], s2[1::2] = g["src"], g["dst"]
    d2[0::2], d2[1::2] = g["dst"], g["src"]
    csr2 = G.csr_file_order(V, s2, d2, w=np.repeat(g["w"], 2))
    np.testing.assert_array_equal(dg2["off"], csr2["off"])
    np.testing.assert_array_equal(dg2["nbr"], csr2["nbr"])
    np.testing.assert_array_equal(dg2["w"], csr2["w"])
    bad = dict(g, dst=g["dst"].copy())
    bad["dst"][n - 7] = V
    G.write_edge_file(f, bad, "f32")
    with pytest.raises(kk.KKError):
        engine.load_graph(V, f, kind="f32")
    typed = dict(g, type=rng.integers(0, 8, n).astype(np.int32))
    typed["type"][n // 3] = 9
    G.write_edge_file(f, typed, "meta")
    with pytest.raises(kk.KKError):
        engine.load_graph(V, f, kind="meta")
    # a refused file leaves the engine's graph as it was
    np.testing.assert_array_equal(engine.download_graph()["nbr"], csr2["nbr"])
    G.write_edge_file(f, g, "f32")
    engine.load_graph(V, f, kind="f32")
    np.testing.assert_array_equal(engine.download_graph()["nbr"], csr["nbr"])
    # unweighted records, and typed ones (split on the host), in file order
    G.write_edge_file(f, g, "none")
    engine.load_graph(V, f, load_as_undirected=True, kind="unweighted")
    dg3 = engine.download_graph()
    np.testing.assert_array_equal(dg3["off"], csr2["off"])
    np.testing.assert_array_equal(dg3["nbr"], csr2["nbr"])
    assert dg3["w"] is None
    typed["type"][n // 3] = 4
    G.write_edge_file(f, typed, "meta")
    engine.load_graph(V, f, kind="meta")
    dg4 = engine.download_graph()
    csr4 = G.csr_file_order(V, g["src"], g["dst"], type=typed["type"])
    np.testing.assert_array_equal(dg4["nbr"], csr4["nbr"])
    np.testing.assert_array_equal(dg4["type"], csr4["type"])


@pytest.mark.parametrize("undirected", [False, True])
def test_text_file_load_matches_file_order(kk, engine, tmp_path, undirected):
    """Text edge lists (read_edge_txt, include/storage.hpp:107-115) build the
    same CSR as the binary file, in file order, mirrored edge by edge for
    --make-undirected; metapath types come from binary files only."""
    g = G.random_undirected(300, 3000, seed=13, weight="unif")
    src, dst, w = (g["src"][0::2], g["dst"][0::2], g["w"][0::2]) if undirected else (g["src"], g["dst"], g["w"])
    f = tmp_path / "g.txt"
    with open(f, "w") as out:
        out.write("% a comment\n")
        for i in range(len(src)):
            out.write("%d %d %.9g\n" % (src[i], dst[i], w[i]))
    engine.load_graph(300, f, load_as_undirected=undirected, kind="text_f32")
    dg = engine.download_graph()
    csr = G.csr_file_order(300, g["src"], g["dst"], w=g["w"])
    np.testing.assert_array_equal(dg["off"], csr["off"])
    np.testing.assert_array_equal(dg["nbr"], csr["nbr"])
    np.testing.assert_array_equal(dg["w"], csr["w"])
    # and it walks like the arrays it equals
    a = engine.walk("deepwalk", 500, seed=5, walk_length=20)
    engine.load_arrays(300, csr["off"], csr["nbr"], csr["w"])
    b = engine.walk("deepwalk", 500, seed=5, walk_length=20)
    np.testing.assert_array_equal(a.vertices, b.vertices)


def test_invalid_configs_raise(kk, engine):
    g = G.random_undirected(50, 200, seed=1)
    csr = G.csr_file_order(50, g["src"], g["dst"])
    engine.load_arrays(50, csr["off"], csr["nbr"])
    with pytest.raises(kk.KKError):
        engine.walk("node2vec", 10, p=0.0, q=1.0)
    with pytest.raises(kk.KKError):
        engine.walk("deepwalk", 10, weighted=True)
    with pytest.raises(kk.KKError):
        engine.walk("metapath", 10, schemes=[[1]])
    with pytest.raises(kk.KKError):
        engine.walk("ppr", 10, terminate_prob=0.0)
    with pytest.raises(kk.KKError, match="start vertex"):
        engine.walk("deepwalk", 10, start=[0, 3, 50])
    # the engine stays usable after the failed call
    assert engine.walk("deepwalk", 10, start=[0, 3, 49]).total_steps > 0


def _compare_alias(engine, oracle_lib, V, off, nbr, w):
    p, pi, qi, s = engine.alias_tables()
    op, opi, oqi, osum = oracle_lib.alias_build(oracle_lib.CSR(V, off, nbr, w))
    np.testing.assert_array_equal(pi, opi)
    np.testing.assert_array_equal(qi, oqi)
    np.testing.assert_array_equal(p.view(np.uint32), op.view(np.uint32))
    np.testing.assert_array_equal(s.view(np.uint32), osum.view(np.uint32))


@pytest.mark.parametrize("streams", [1, 2, 3])
@pytest.mark.parametrize("weights", [1, 2])
def test_alias_tables_match_oracle_rmat16(engine, oracle_lib, weights, streams):
    """R-MAT scale 16 has no hub above degree 16384: with alias_streams 2 the
    side stream runs the light classes alone."""
    engine.generate_rmat(16, 16, seed=3, weights=weights)
    g = engine.download_graph()
    engine.set_option("alias_streams", streams)
    try:
        _compare_alias(engine, oracle_lib, g["V"], g["off"], g["nbr"], g["w"])
    finally:
        engine.set_option("alias_streams", 3)


@pytest.mark.parametrize("hub_grid,streams", [(0, 1), (2, 1), (0, 2), (0, 3), (2, 3), (0, 4), (2, 4)])
@pytest.mark.parametrize("dist", ["lognormal", "pareto", "uniform", "equal", "twovalue", "halves", "wide", "tiny",
                                  "zeros"])
def test_alias_tables_match_oracle_hubs(engine, oracle_lib, dist, hub_grid, streams):
    """Every build class and both sides of every class boundary: hubs (40000,
    20000, 16385), 4097..16384 (block per vertex, queues in the scratch),
    2049..4096 (block per vertex, shared memory), 1..2048 (lane groups of 32,
    16, 8, 4 and 2), with rows of unequal degree side by side in a warp.
    The large rows' sums take the exact block scan; these weights exercise
    its rounding: halves (exact ties at every binade), wide (lognormal sigma
    4: terms far above and below the running sum), tiny (sums below 2^-103,
    the serial chain) and zeros (half the terms +0)."""
    rng = np.random.default_rng(17)
    degs = [40000, 20000, 16385, 16384, 12000, 5000, 4097, 4096, 3000, 2049, 2048, 1500, 1025, 1024, 600, 513, 512,
            300, 129, 128, 100, 33, 32, 31, 17, 16, 7, 1]
    degs += list(rng.integers(0, 40, size=2000)) + list(rng.integers(100, 600, size=60))
    degs += list(rng.integers(900, 1100, size=20)) + list(rng.integers(2000, 4200, size=6))
    V = 60000
    degs = np.array(degs + [0] * (V - len(degs)), np.int64)
    off = np.zeros(V + 1, np.int64)
    np.cumsum(degs, out=off[1:])
    E = int(off[-1])
    nbr = rng.integers(0, V, size=E).astype(np.uint32)
    if dist == "lognormal":
        w = rng.lognormal(0.0, 1.0, size=E)
    elif dist == "pareto":
        w = rng.pareto(1.2, size=E) + 0.01
    elif dist == "uniform":
        w = 1.0 + 4.0 * rng.random(E)
    elif dist == "equal":
        w = np.full(E, 0.3)
    elif dist == "twovalue":
        w = np.where(rng.random(E) < 0.9, 1.0, 50.0)
    elif dist == "halves":
        w = 0.5 * rng.integers(1, 9, size=E)
    elif dist == "wide":
        w = rng.lognormal(0.0, 4.0, size=E)
    elif dist == "tiny":
        w = 1e-33 * rng.lognormal(0.0, 1.0, size=E)
    else:
        w = np.where(rng.random(E) < 0.5, 0.0, rng.lognormal(0.0, 1.0, size=E))
        w[off[:-1][degs > 0]] = 1.0  # no all-zero row (its 0/0 average is NaN)
    w = w.astype(np.float32)
    engine.load_arrays(V, off, nbr, w)
    engine.set_option("alias_hub_grid", hub_grid)
    engine.set_option("alias_streams", streams)
    engine.set_option("alias_small_lanes", int(streams == 4))
    try:
        _compare_alias(engine, oracle_lib, V, off, nbr, w)
    finally:
        engine.set_option("alias_hub_grid", 0)
        engine.set_option("alias_streams", 3)
        engine.set_option("alias_small_lanes", 0)


@pytest.mark.parametrize("park", [8, 31, 32])
@pytest.mark.parametrize("i", [7, 8])
def test_parked_walks_match_oracle(engine, oracle_lib, i, park):
    """Parking (walk_park): walkers of thinned-out warps stop at a step
    boundary and later launches resume them; paths, steps and the trial
    count equal the oracle's and the unparked walk's.  park 32 parks a
    walker as soon as any lane of its warp has ended."""
    app, gkw, wkw = FRESH[i]
    g = G.random_undirected(500, 6000, seed=300 + i, **gkw)
    csr = G.csr_file_order(500, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    weighted = "w" in csr
    n = 20000
    engine.set_option("walk_stats", 1)
    try:
        engine.set_option("walk_park", 0)
        plain = engine.walk(app, n, seed=21, weighted=weighted, **wkw)
        t_plain = engine.last_stats()[0]
        engine.set_option("walk_park", park)
        ps = engine.walk(app, n, seed=21, weighted=weighted, **wkw)
        t_park = engine.last_stats()[0]
    finally:
        engine.set_option("walk_park", 20)
        engine.set_option("walk_stats", 0)
    ocsr = oracle_lib.CSR(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    prm = oracle_lib.make_params(app, seed=21, walker_begin=0, walker_num=n, weighted=weighted, **wkw)
    lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=4096)
    np.testing.assert_array_equal(ps.path_length, lens)
    np.testing.assert_array_equal(ps.vertices, verts)
    assert ps.total_steps == steps == plain.total_steps
    assert t_park == t_plain


@pytest.mark.parametrize("name", APP_CASES)
def test_paths_match_reference_parked(engine, name):
    """The reference's own paths with parking on (metapath parks; the other
    apps have no rejection trials of the first order and do not)."""
    case = Case(name)
    load_case(engine, case)
    engine.set_option("walk_park", 24)
    try:
        ps = gpu_walk(engine, case)
    finally:
        engine.set_option("walk_park", 20)
    np.testing.assert_array_equal(ps.path_length, case.lens)
    np.testing.assert_array_equal(ps.vertices, case.verts)


@pytest.mark.parametrize("multi,schedule", [(1, 0), (2, 0), (4, 0), (1, 1)])
@pytest.mark.parametrize("i", [0, 2, 4])
def test_neighbour_buckets_match_oracle(engine, oracle_lib, i, multi, schedule):
    """alias_layout 2 (16 B buckets holding p and the two neighbours) in the
    one-walker, multi-walker and pool kernels: weighted DeepWalk, PPR and
    node2vec (whose hooks need index buckets where they read the edge)."""
    app, gkw, wkw = FRESH[i]
    g = G.random_undirected(500, 6000, seed=400 + i, **gkw)
    csr = G.csr_file_order(500, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    n = 3000
    engine.set_option("alias_layout", 2)
    engine.set_option("walk_multi", multi)
    engine.set_option("walk_schedule", schedule)
    try:
        ps = engine.walk(app, n, seed=31, weighted=True, walker_begin=5, **wkw)
    finally:
        engine.set_option("alias_layout", 2)
        engine.set_option("walk_multi", 1)
        engine.set_option("walk_schedule", 0)
    ocsr = oracle_lib.CSR(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    if app == "node2vec":
        ocsr = ocsr.sorted_copy()
    prm = oracle_lib.make_params(app, seed=31, walker_begin=5, walker_num=n, weighted=True, **wkw)
    lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=4096)
    np.testing.assert_array_equal(ps.path_length, lens)
    np.testing.assert_array_equal(ps.vertices, verts)
    assert ps.total_steps == steps


@pytest.mark.parametrize("i", [0, 2, 4, 7])
def test_epoch_split_matches_single_epoch(engine, i):
    """kk_walk with epochs (rate 0.37): DeepWalk and node2vec into one pooled
    block sized by walk_length + 1, PPR and metapath through per-epoch host
    chunks; every path equals the single-epoch walk's."""
    app, gkw, wkw = FRESH[i]
    g = G.random_undirected(500, 6000, seed=500 + i, **gkw)
    csr = G.csr_file_order(500, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))
    engine.load_arrays(500, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    weighted = "w" in csr
    one = engine.walk(app, 5000, seed=17, weighted=weighted, **wkw)
    import knightking_gb300 as kk
    conf = kk.WalkConfig()
    conf.set_walk_rate(0.37)
    many = engine.walk(app, 5000, walk_conf=conf, seed=17, weighted=weighted, **wkw)
    np.testing.assert_array_equal(many.path_length, one.path_length)
    np.testing.assert_array_equal(many.vertices, one.vertices)
    assert many.total_steps == one.total_steps


@pytest.mark.parametrize("p,q,lo,hi", [(2.0, 0.5, 0.35, 0.56), (0.5, 2.0, 0.35, 0.56)])
def test_node2vec_asks_only_queries_that_can_matter(engine, oracle_lib, p, q, lo, hi):
    """The adjacency question is skipped for the return edge and for darts at
    or below min(1, 1/q), where either answer accepts.  With p = 2, q = 0.5
    the reference asks for darts above lb = 0.5 of ub = 2 (3/4 of the trials)
    and this engine for darts above 1 (1/2); with p = 0.5, q = 2 both ask for
    darts above 0.5 of ub = 1 (1/2).  Paths are the same with the access
    counts on and off, and equal the oracle's; the counted binary-search
    probes cover every question the reference asks."""
    g = G.random_undirected(400, 6000, seed=77, weight="unif")
    csr = G.csr_file_order(400, g["src"], g["dst"], w=g["w"])
    engine.load_arrays(400, csr["off"], csr["nbr"], csr["w"])
    n, L = 20000, 20
    a = engine.walk("node2vec", n, seed=5, walk_length=L, p=p, q=q, weighted=True)
    engine.set_option("walk_stats", 1)
    engine.set_option("node2vec_adjacency", 1)
    try:
        b = engine.walk("node2vec", n, seed=5, walk_length=L, p=p, q=q, weighted=True)
        trials, queries, probes = engine.last_stats()
    finally:
        engine.set_option("walk_stats", 0)
        engine.set_option("node2vec_adjacency", 0)
    np.testing.assert_array_equal(a.vertices, b.vertices)
    ocsr = oracle_lib.CSR(400, csr["off"], csr["nbr"], csr["w"]).sorted_copy()
    prm = oracle_lib.make_params("node2vec", seed=5, walker_num=n, walk_length=L, p=p, q=q, weighted=True)
    lens, verts, steps = oracle_lib.walk(ocsr, prm, cap=L + 1)
    np.testing.assert_array_equal(a.vertices, verts)
    assert lo < queries / trials < hi
    assert probes > queries
