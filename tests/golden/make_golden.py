"""Generate the golden fixtures in this directory from the reference itself.

Runs KnightKing's own engine and apps (compiled from the reference sources by
``make -C oracle ref`` into oracle/_ref/kk_ref, with the single-rank MPI shim
and the Philox RNG hook) on seeded synthetic graphs, and stores graph, parameters
and the reference's outputs as compressed .npz files:

* ``case_*.npz``   small graphs (tests' generator style, karate, edge cases):
  full paths (lengths + vertices in walker-id order) or full alias tables;
* ``rmat16_*.npz`` R-MAT scale 16 (65,536 vertices): the graph is regenerated
  from its seed at test time (oracle/graphs.py and the product's generator
  compute the same graph), so the fixture stores the graph's SHA-256, the
  SHA-256 of all paths and the first 64 walkers' paths;
* ``dump_*.npz``   the text written by PathSet::dump (include/path.hpp:85-109)
  with epoch splitting (-r), for the path-export format.

Run here (where the reference sources are):  python tests/golden/make_golden.py
The tests never run the reference; they read these files.
"""

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import graphs as G  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
KARATE = os.path.join(O.ref_root(), "dataset", "karate.txt")  # the oracle recipe's REF_ROOT

SCHEMES = [  # 3 schemes x 4 states over 5 edge types, as type masks
    [0b00001, 0b00010, 0b00100, 0b01000],
    [0b00010, 0b01000, 0b00010, 0b10000],
    [0b00100, 0b00001, 0b10000, 0b00100],
]
SCHEMES_MULTI = [  # masks allowing several types per state
    [0b00011, 0b00110, 0b01100],
    [0b11000, 0b10001, 0b00101, 0b01010, 0b11111],
]


def write_schemes(path, schemes, ntypes=5):
    with open(path, "w") as f:
        f.write("%d %d\n" % (len(schemes), ntypes))
        for sc in schemes:
            f.write("%d\n" % len(sc))
            for m in sc:
                f.write(" ".join(str((m >> k) & 1) for k in range(ntypes)) + " \n")


def run_ref(args):
    r = subprocess.run([O.REF_BIN] + [str(a) for a in args], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("kk_ref failed: %s\n%s" % (" ".join(map(str, args)), r.stderr))


def graph_arrays(g):
    out = {"V": np.uint32(g["V"]), "src": g["src"].astype(np.uint32), "dst": g["dst"].astype(np.uint32)}
    if "w" in g:
        out["w"] = g["w"].astype(np.float32)
    if "type" in g:
        out["type"] = np.asarray(g["type"]).astype(np.uint8)
    return out


def ref_walk(tmp, g, kind, cmd, params, extra=()):
    gfile = os.path.join(tmp, "graph.bin")
    G.write_edge_file(gfile, g, kind)
    out = os.path.join(tmp, "paths.bin")
    args = [cmd, "--graph", gfile, "--v", g["V"], "--kind", kind, "--out", out, "--seed", params["seed"],
            "--walkers", params["walkers"]]
    for k in ("len", "term", "p", "q", "tag-num", "vtw", "amp", "order", "variant", "threads", "rate"):
        if k in params:
            args += ["--" + k, params[k]]
    if "schemes" in params:
        sfile = os.path.join(tmp, "schemes.txt")
        write_schemes(sfile, params["schemes"])
        args += ["--schemes", sfile]
    if "vertex_tag" in params:
        vfile = os.path.join(tmp, "vtag.bin")
        np.asarray(params["vertex_tag"], dtype=np.int32).tofile(vfile)
        args += ["--vtag", vfile]
    args += list(extra)
    run_ref(args)
    return G.read_paths(out)


def save_case(name, g, kind, cmd, params, lens, verts):
    p = {k: v for k, v in params.items() if k != "vertex_tag"}
    arrays = graph_arrays(g)
    if "vertex_tag" in params:
        arrays["vertex_tag"] = np.asarray(params["vertex_tag"], dtype=np.int32)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), kind=np.array(kind), cmd=np.array(cmd),
                        params=np.array(json.dumps(p)), lens=lens, verts=verts, **arrays)
    print("%-34s walkers=%-6d steps=%d" % (name, len(lens), int(lens.sum()) - len(lens)))


def karate():
    rows = np.loadtxt(KARATE)
    return {"V": 34, "src": rows[:, 0].astype(np.uint32), "dst": rows[:, 1].astype(np.uint32),
            "w": rows[:, 2].astype(np.float32)}


def tag_graph(v, e, seed, weighted, T):
    g = G.random_undirected(v, e, seed, weight="int5" if weighted else None, types="uniform", ntypes=T)
    order = np.lexsort((g["dst"], g["type"], g["src"]))  # grouped by (src, tag)
    for k in ("src", "dst", "w", "type"):
        if k in g:
            g[k] = g[k][order]
    return g


def small_cases(tmp):
    cases = []
    kar = karate()
    cases += [
        ("case_karate_deepwalk_w", kar, "f32", "deepwalk", dict(seed=3, walkers=200, len=30)),
        ("case_karate_deepwalk_u", kar, "none", "deepwalk", dict(seed=4, walkers=200, len=30)),
        ("case_karate_ppr_w", kar, "f32", "ppr", dict(seed=5, walkers=300, term=0.05)),
        ("case_karate_node2vec_w_p2q05", kar, "f32", "node2vec", dict(seed=6, walkers=200, len=30, p=2.0, q=0.5)),
        ("case_karate_node2vec_w_p025q2", kar, "f32", "node2vec", dict(seed=7, walkers=200, len=30, p=0.25, q=2.0)),
    ]
    gu = G.random_undirected(300, 3000, seed=101)
    gi = G.random_undirected(300, 3000, seed=102, weight="int5")
    gf = G.random_undirected(200, 2400, seed=103, weight="unif")
    cases += [
        ("case_u300_deepwalk", gu, "none", "deepwalk", dict(seed=11, walkers=600, len=20)),
        ("case_u300_ppr", gu, "none", "ppr", dict(seed=12, walkers=600, term=0.0125)),
        ("case_u300_node2vec_p2q05", gu, "none", "node2vec", dict(seed=13, walkers=600, len=20, p=2.0, q=0.5)),
        ("case_u300_node2vec_p05q2", gu, "none", "node2vec", dict(seed=14, walkers=600, len=20, p=0.5, q=2.0)),
        ("case_u300_node2vec_p025q4", gu, "none", "node2vec", dict(seed=15, walkers=600, len=20, p=0.25, q=4.0)),
        ("case_u300_node2vec_p1q1", gu, "none", "node2vec", dict(seed=16, walkers=600, len=20, p=1.0, q=1.0)),
        ("case_i300_deepwalk", gi, "f32", "deepwalk", dict(seed=21, walkers=600, len=20)),
        ("case_i300_ppr", gi, "f32", "ppr", dict(seed=22, walkers=600, term=0.05)),
        ("case_i300_node2vec_p2q05", gi, "f32", "node2vec", dict(seed=23, walkers=600, len=20, p=2.0, q=0.5)),
        ("case_i300_node2vec_p05q2", gi, "f32", "node2vec", dict(seed=24, walkers=600, len=20, p=0.5, q=2.0)),
        ("case_f200_deepwalk", gf, "f32", "deepwalk", dict(seed=31, walkers=400, len=25)),
        ("case_f200_node2vec_p03q3", gf, "f32", "node2vec", dict(seed=32, walkers=400, len=25, p=0.3, q=3.0)),
        ("case_f200_node2vec_p4q025", gf, "f32", "node2vec", dict(seed=33, walkers=400, len=25, p=4.0, q=0.25)),
    ]
    # metapath, random scheme per walker (src/apps/metapath.hpp:91-95)
    gm = G.random_undirected(300, 4000, seed=41, weight="int5", types="uniform")
    gmu = G.random_undirected(300, 4000, seed=42, types="uniform")
    cases += [
        ("case_m300_metapath_w", gm, "meta_f32", "metapath", dict(seed=43, walkers=600, len=20, schemes=SCHEMES)),
        ("case_m300_metapath_u", gmu, "meta", "metapath", dict(seed=44, walkers=600, len=20, schemes=SCHEMES_MULTI)),
    ]
    # tag walks: the generic hooks with custom functors (bounds, outlier, 2nd order)
    T = 4
    vt = np.random.default_rng(51).integers(0, T, size=200).astype(np.int32)
    gtu = tag_graph(200, 2400, 52, False, T)
    gtw = tag_graph(200, 2400, 53, True, T)
    base = dict(walkers=400, len=20, **{"tag-num": T, "vtw": 0.5, "amp": 4.0}, vertex_tag=vt)
    cases += [
        ("case_t200_bound_o1_u", gtu, "tag", "tagwalk", dict(seed=54, order=1, variant="bound", **base)),
        ("case_t200_bound_o2_w", gtw, "tag_f32", "tagwalk", dict(seed=55, order=2, variant="bound", **base)),
        ("case_t200_outlier_o1_w", gtw, "tag_f32", "tagwalk", dict(seed=56, order=1, variant="outlier", **base)),
        ("case_t200_outlier_o2_u", gtu, "tag", "tagwalk", dict(seed=57, order=2, variant="outlier", **base)),
        ("case_t200_outlier_o2_w", gtw, "tag_f32", "tagwalk", dict(seed=58, order=2, variant="outlier", **base)),
    ]
    # the dynamic walk of src/examples/dynamic_walk.cpp:52-93 (return edge
    # doubled): the example's own 34 walkers on karate, and a random graph
    cases += [
        ("case_dyn_karate", kar, "f32", "dynwalk", dict(seed=8, walkers=34, len=80)),
        ("case_dyn_f200", gf, "f32", "dynwalk", dict(seed=35, walkers=400, len=25)),
    ]
    # edge cases: isolated and degree-1 vertices, walkers not a multiple of V,
    # a single walker, zero length, immediate termination
    gs = G.random_undirected(400, 500, seed=61, weight="int5")
    cases += [
        ("case_sparse_deepwalk_w", gs, "f32", "deepwalk", dict(seed=62, walkers=1001, len=15)),
        ("case_sparse_ppr_u", gs, "none", "ppr", dict(seed=63, walkers=999, term=0.1)),
        ("case_sparse_node2vec_w", gs, "f32", "node2vec", dict(seed=64, walkers=1001, len=15, p=0.5, q=2.0)),
        ("case_single_walker", gi, "f32", "node2vec", dict(seed=65, walkers=1, len=50, p=2.0, q=0.5)),
        ("case_zero_length", gi, "f32", "deepwalk", dict(seed=66, walkers=300, len=0)),
        ("case_terminate_all", gu, "none", "ppr", dict(seed=67, walkers=300, term=1.0)),
    ]
    for name, g, kind, cmd, params in cases:
        lens, verts = ref_walk(tmp, g, kind, cmd, params)
        save_case(name, g, kind, cmd, params, lens, verts)

    # alias tables, index for index (include/walk.hpp:538-652)
    for name, g in (("alias_i300", gi), ("alias_f200", gf), ("alias_karate", kar)):
        gfile = os.path.join(tmp, "graph.bin")
        G.write_edge_file(gfile, g, "f32")
        out = os.path.join(tmp, "alias.bin")
        run_ref(["alias", "--graph", gfile, "--v", g["V"], "--kind", "f32", "--out", out])
        p, pi, qi, s = G.read_alias(out)
        np.savez_compressed(os.path.join(OUT, "case_%s.npz" % name), kind=np.array("f32"), cmd=np.array("alias"),
                            params=np.array("{}"), alias_p=p, alias_pidx=pi, alias_qidx=qi, alias_sum=s,
                            **graph_arrays(g))
        print("%-34s edges=%d" % ("case_" + name, len(p)))


def dump_cases(tmp):
    """PathSet text dump with epochs: -r 0.3, 3 worker threads, with and without head info."""
    gi = G.random_undirected(120, 800, seed=71, weight="int5")
    for head in (0, 1):
        gfile = os.path.join(tmp, "graph.bin")
        G.write_edge_file(gfile, gi, "f32")
        prefix = os.path.join(tmp, "dump_out")
        if os.path.exists(prefix + ".0"):
            os.remove(prefix + ".0")
        params = dict(seed=72, walkers=100, len=10, rate=0.3, threads=3, head=head)
        run_ref(["deepwalk", "--graph", gfile, "--v", gi["V"], "--kind", "f32", "--out", os.path.join(tmp, "p.bin"),
                 "--seed", 72, "--walkers", 100, "--len", 10, "--rate", 0.3, "--threads", 3, "--dump", prefix,
                 "--head", head])
        with open(prefix + ".0") as f:
            text = f.read()
        lens, verts = G.read_paths(os.path.join(tmp, "p.bin"))
        np.savez_compressed(os.path.join(OUT, "dump_deepwalk_head%d.npz" % head), kind=np.array("f32"),
                            cmd=np.array("deepwalk"), params=np.array(json.dumps(params)), text=np.array(text),
                            lens=lens, verts=verts, **graph_arrays(gi))
        print("%-34s bytes=%d" % ("dump_deepwalk_head%d" % head, len(text)))


def csr_digest(csr_dict):
    import hashlib
    h = hashlib.sha256()
    for k in ("off", "nbr", "w", "type"):
        if k in csr_dict and csr_dict[k] is not None:
            h.update(np.ascontiguousarray(csr_dict[k]).tobytes())
    return h.hexdigest()


def rmat_cases(tmp):
    """R-MAT scale 16: the node2vec parity config and its siblings."""
    specs = [
        ("rmat16_node2vec_p2q05", dict(weights=True), "f32", "node2vec",
         dict(seed=1, walkers=65536, len=80, p=2.0, q=0.5)),
        ("rmat16_node2vec_p05q2", dict(weights=True), "f32", "node2vec",
         dict(seed=2, walkers=65536, len=40, p=0.5, q=2.0)),
        ("rmat16_deepwalk_w", dict(weights=True), "f32", "deepwalk", dict(seed=3, walkers=65536, len=80)),
        ("rmat16_ppr_u", dict(), "none", "ppr", dict(seed=4, walkers=65536, term=1.0 / 80)),
        ("rmat16_metapath_w", dict(weights=True, types=True), "meta_f32", "metapath",
         dict(seed=5, walkers=65536, len=80, schemes=SCHEMES)),
    ]
    graphs = {}
    for name, gkw, kind, cmd, params in specs:
        key = tuple(sorted(gkw.items()))
        if key not in graphs:
            graphs[key] = G.rmat(16, 16, 0.57, 0.19, 0.19, seed=16, **gkw)
        g = graphs[key]
        csr = {"off": g["off"], "nbr": g["dst"].astype(np.uint32), "w": g.get("w"), "type": g.get("type")}
        lens, verts = ref_walk(tmp, g, kind, cmd, params)
        n_head = 64
        head_len = lens[:n_head]
        head_verts = verts[:int(head_len.sum())]
        gen = dict(scale=16, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=16, **gkw)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), kind=np.array(kind), cmd=np.array(cmd),
                            params=np.array(json.dumps(params)), rmat=np.array(json.dumps(gen)),
                            graph_sha256=np.array(csr_digest(csr)), paths_sha256=np.array(G.paths_digest(lens, verts)),
                            total_steps=np.uint64(int(lens.sum()) - len(lens)), head_lens=head_len,
                            head_verts=head_verts, E=np.uint64(len(g["dst"])))
        print("%-34s E=%d steps=%d" % (name, len(g["dst"]), int(lens.sum()) - len(lens)))


def main():
    O.build_ref()
    with tempfile.TemporaryDirectory() as tmp:
        small_cases(tmp)
        dump_cases(tmp)
        rmat_cases(tmp)


if __name__ == "__main__":
    main()
