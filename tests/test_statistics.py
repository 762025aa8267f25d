"""Statistical checks: empirical transition frequencies of node2vec, PPR and
metapath walks against exact transition probabilities computed in FP64.

They restate the reference's checkers (src/tests/test_walk.hpp:152-186,
src/tests/test_node2vec.cpp:45-149, src/tests/test_metapath.cpp:46-196) as
chi-square tests: per context (current vertex, plus the previous vertex for
node2vec or the scheme state for metapath) the observed next-vertex counts
against count * P_exact.  The CPU tests run the oracle (the reference's
algorithm, pinned to its outputs); the GPU tests run the CUDA engine on fresh
seeds.  Contexts with few visits are pooled by requiring expected counts >= 5.
"""

import numpy as np
import pytest

from oracle import graphs as G

scipy_stats = pytest.importorskip("scipy.stats")

V = 40
E_UND = 240  # undirected pairs * 2 directed


def _graph(seed, weight="int5", types=None):
    g = G.random_undirected(V, E_UND, seed=seed, weight=weight, types=types)
    return G.csr_file_order(V, g["src"], g["dst"], w=g.get("w"), type=g.get("type"))


def _sorted(csr):
    """CSR with each adjacency sorted by neighbour (node2vec's order)."""
    off, nbr = csr["off"], csr["nbr"]
    out = dict(csr)
    out["nbr"] = nbr.copy()
    for key in ("w", "type"):
        if key in csr:
            out[key] = csr[key].copy()
    for v in range(V):
        a, b = int(off[v]), int(off[v + 1])
        order = np.argsort(nbr[a:b], kind="stable")
        out["nbr"][a:b] = nbr[a:b][order]
        for key in ("w", "type"):
            if key in csr:
                out[key][a:b] = csr[key][a:b][order]
    return out


def _chi2(observed, expected):
    """Pooled chi-square over contexts: cells with expected >= 5; returns the p-value."""
    obs, exp = np.asarray(observed, float), np.asarray(expected, float)
    keep = exp >= 5
    chi = float((((obs - exp) ** 2) / np.where(keep, exp, 1))[keep].sum())
    dof = max(int(keep.sum()) - 1, 1)
    return float(scipy_stats.chi2.sf(chi, dof))


def _paths(lens, verts):
    out, o = [], 0
    for n in lens:
        out.append(verts[o:o + int(n)])
        o += int(n)
    return out


def node2vec_check(csr, paths, p, q):
    """node2vec second-order transitions: P(x | t, v) ~ w(v, x) * alpha(t, x)."""
    off, nbr, w = csr["off"], csr["nbr"], csr["w"].astype(np.float64)
    adj = [set(nbr[off[v]:off[v + 1]].tolist()) for v in range(V)]
    counts = {}
    for pth in paths:
        for i in range(2, len(pth)):
            key = (int(pth[i - 2]), int(pth[i - 1]))
            c = counts.setdefault(key, {})
            c[int(pth[i])] = c.get(int(pth[i]), 0) + 1
    obs, exp = [], []
    for (t, v), c in counts.items():
        n = sum(c.values())
        xs = nbr[off[v]:off[v + 1]]
        ws = w[off[v]:off[v + 1]]
        alpha = np.array([1.0 / p if x == t else (1.0 if x in adj[t] else 1.0 / q) for x in xs.tolist()])
        pr = ws * alpha
        pr /= pr.sum()
        for x, px in zip(xs.tolist(), pr):
            obs.append(c.get(x, 0))
            exp.append(n * px)
    return _chi2(obs, exp)


def first_order_check(csr, paths, weighted):
    """PPR / DeepWalk transitions: P(x | v) ~ w(v, x) (or uniform)."""
    off, nbr = csr["off"], csr["nbr"]
    counts = np.zeros(int(off[-1]), np.int64)
    visits = np.zeros(V, np.int64)
    pos = {}
    for v in range(V):
        for e in range(int(off[v]), int(off[v + 1])):
            pos[(v, int(nbr[e]))] = e
    for pth in paths:
        for i in range(1, len(pth)):
            counts[pos[(int(pth[i - 1]), int(pth[i]))]] += 1
            visits[int(pth[i - 1])] += 1
    exp = np.zeros_like(counts, dtype=float)
    for v in range(V):
        a, b = int(off[v]), int(off[v + 1])
        ws = csr["w"][a:b].astype(np.float64) if weighted else np.ones(b - a)
        exp[a:b] = visits[v] * ws / ws.sum()
    return _chi2(counts, exp)


def ppr_length_check(lens, term):
    """Geometric walk lengths (no isolated vertices): P(steps = k) = (1-t)^k t."""
    steps = np.asarray(lens, np.int64) - 1
    kmax = 60
    obs = np.array([(steps == k).sum() for k in range(kmax)] + [(steps >= kmax).sum()], float)
    pk = np.array([(1 - term) ** k * term for k in range(kmax)] + [(1 - term) ** kmax])
    return _chi2(obs, len(steps) * pk)


def metapath_check(csr, paths, scheme):
    """Metapath transitions (one scheme, round robin): P(x | v, state) ~ w(v, x) * [type allowed]."""
    off, nbr, w, ty = csr["off"], csr["nbr"], csr["w"].astype(np.float64), csr["type"]
    L = len(scheme)
    counts = {}
    for pth in paths:
        for i in range(1, len(pth)):
            key = (int(pth[i - 1]), (i - 1) % L)
            c = counts.setdefault(key, {})
            c[int(pth[i])] = c.get(int(pth[i]), 0) + 1
    obs, exp = [], []
    for (v, s), c in counts.items():
        n = sum(c.values())
        a, b = int(off[v]), int(off[v + 1])
        allowed = np.array([(scheme[s] >> int(t)) & 1 for t in ty[a:b]], float)
        pr = w[a:b] * allowed
        pr /= pr.sum()
        for x, px in zip(nbr[a:b].tolist(), pr):
            obs.append(c.get(x, 0))
            exp.append(n * px)
    return _chi2(obs, exp)


# ---- the oracle (the reference's algorithm), on the CPU ----

def _oracle_walk(oracle_lib, csr, app, n, **kw):
    ocsr = oracle_lib.CSR(V, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    prm = oracle_lib.make_params(app, walker_num=n, weighted="w" in csr, **kw)
    lens, verts, _ = oracle_lib.walk(ocsr, prm, cap=512)
    return lens, verts


@pytest.mark.parametrize("p,q", [(2.0, 0.5), (0.5, 2.0), (0.3, 0.6)])
def test_oracle_node2vec_transitions(oracle_lib, p, q):
    csr = _sorted(_graph(21))
    lens, verts = _oracle_walk(oracle_lib, csr, "node2vec", 20000, seed=3, walk_length=30, p=p, q=q)
    assert node2vec_check(csr, _paths(lens, verts), p, q) > 1e-4


def test_oracle_ppr_transitions_and_lengths(oracle_lib):
    csr = _graph(22)
    lens, verts = _oracle_walk(oracle_lib, csr, "ppr", 40000, seed=5, terminate_prob=0.1)
    assert first_order_check(csr, _paths(lens, verts), True) > 1e-4
    assert ppr_length_check(lens, np.float32(0.1)) > 1e-4


def test_oracle_metapath_transitions(oracle_lib):
    csr = _graph(23, weight="unif", types="uniform")
    scheme = [0b00111, 0b11000, 0b01110]
    lens, verts = _oracle_walk(oracle_lib, csr, "metapath", 20000, seed=7, walk_length=24, schemes=[scheme],
                               scheme_round_robin=True)
    assert metapath_check(csr, _paths(lens, verts), scheme) > 1e-4


def test_chi2_detects_a_wrong_distribution(oracle_lib):
    """The check has power: node2vec paths tested against the wrong (p, q) fail."""
    csr = _sorted(_graph(21))
    lens, verts = _oracle_walk(oracle_lib, csr, "node2vec", 20000, seed=3, walk_length=30, p=2.0, q=0.5)
    assert node2vec_check(csr, _paths(lens, verts), 0.5, 2.0) < 1e-6


# ---- the CUDA engine, fresh seeds ----

@pytest.fixture(scope="module")
def engine():
    import knightking_gb300 as kk
    e = kk.WalkEngine(0)
    yield e
    e.close()


def _gpu_walk(engine, csr, app, n, **kw):
    engine.load_arrays(V, csr["off"], csr["nbr"], csr.get("w"), csr.get("type"))
    ps = engine.walk(app, n, weighted="w" in csr, **kw)
    return ps.path_length, ps.vertices


@pytest.mark.gpu
@pytest.mark.parametrize("p,q", [(2.0, 0.5), (0.5, 2.0), (0.3, 0.6)])
def test_gpu_node2vec_transitions(engine, p, q):
    csr = _sorted(_graph(31))
    lens, verts = _gpu_walk(engine, csr, "node2vec", 40000, seed=11, walk_length=30, p=p, q=q)
    assert node2vec_check(csr, _paths(lens, verts), p, q) > 1e-4


@pytest.mark.gpu
def test_gpu_ppr_transitions_and_lengths(engine):
    csr = _graph(32)
    lens, verts = _gpu_walk(engine, csr, "ppr", 60000, seed=13, terminate_prob=0.1)
    assert first_order_check(csr, _paths(lens, verts), True) > 1e-4
    assert ppr_length_check(lens, np.float32(0.1)) > 1e-4


@pytest.mark.gpu
def test_gpu_metapath_transitions(engine):
    csr = _graph(33, weight="unif", types="uniform")
    scheme = [0b00111, 0b11000, 0b01110]
    lens, verts = _gpu_walk(engine, csr, "metapath", 30000, seed=17, walk_length=24, schemes=[scheme],
                            scheme_round_robin=True)
    assert metapath_check(csr, _paths(lens, verts), scheme) > 1e-4
