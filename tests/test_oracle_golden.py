"""Pins the CPU oracle (oracle/kk_oracle.c) to the reference's own outputs.

Every fixture in tests/golden/ was produced by KnightKing's engine itself,
compiled from the reference sources with a Philox RNG hook
(tests/golden/make_golden.py).  The oracle must reproduce each one bit for bit:
paths per walker id, alias tables index for index, the R-MAT scale-16 digests.
"""

import json

import numpy as np
import pytest

from cases import Case, case_ids, walk_kwargs
from oracle import graphs as G


def oracle_csr(oracle, case):
    g = case.graph()
    csr = oracle.CSR(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))
    if case.cmd == "node2vec":
        csr = csr.sorted_copy()
    return csr


@pytest.mark.parametrize("name", [c for c in case_ids() if not c.startswith("case_alias")])
def test_oracle_paths_match_reference(oracle_lib, name):
    case = Case(name)
    csr = oracle_csr(oracle_lib, case)
    prm = oracle_lib.make_params(case.cmd, **walk_kwargs(case))
    lens, verts, steps = oracle_lib.walk(csr, prm, cap=case.cap(), threads=4)
    np.testing.assert_array_equal(lens, case.lens)
    np.testing.assert_array_equal(verts, case.verts)
    assert steps == int(case.lens.sum()) - len(case.lens)


@pytest.mark.parametrize("name", case_ids("case_alias"))
def test_oracle_alias_tables_match_reference(oracle_lib, name):
    case = Case(name)
    csr = oracle_csr(oracle_lib, case)
    p, pi, qi, s = oracle_lib.alias_build(csr, threads=3)
    d = case.d
    # index for index, and probabilities to the bit (0 ulp)
    np.testing.assert_array_equal(pi, d["alias_pidx"])
    np.testing.assert_array_equal(qi, d["alias_qidx"])
    np.testing.assert_array_equal(p.view(np.uint32), d["alias_p"].view(np.uint32))
    np.testing.assert_array_equal(s.view(np.uint32), d["alias_sum"].view(np.uint32))


@pytest.mark.parametrize("name", case_ids("rmat16_"))
def test_oracle_rmat16_digest_matches_reference(oracle_lib, name):
    d = np.load("%s/%s.npz" % (__import__("cases").GOLDEN, name))
    gen = json.loads(str(d["rmat"]))
    g = G.rmat(gen["scale"], gen["edge_factor"], gen["a"], gen["b"], gen["c"], seed=gen["seed"],
               weights=gen.get("weights", False), types=gen.get("types", False))
    csr_d = {"off": g["off"], "nbr": g["dst"].astype(np.uint32), "w": g.get("w"), "type": g.get("type")}
    import hashlib
    h = hashlib.sha256()
    for k in ("off", "nbr", "w", "type"):
        if csr_d[k] is not None:
            h.update(np.ascontiguousarray(csr_d[k]).tobytes())
    assert h.hexdigest() == str(d["graph_sha256"]), "R-MAT generator changed"
    params = json.loads(str(d["params"]))
    cmd = str(d["cmd"])
    kw = dict(seed=params["seed"], walker_num=params["walkers"], weighted=str(d["kind"]) != "none")
    if "len" in params:
        kw["walk_length"] = params["len"]
    if "term" in params:
        kw["terminate_prob"] = float(np.float32(params["term"]))
    if cmd == "node2vec":
        kw["p"], kw["q"] = params["p"], params["q"]
    if cmd == "metapath":
        kw["schemes"] = params["schemes"]
    csr = oracle_lib.CSR(g["V"], g["off"], g["dst"], g.get("w"), g.get("type"))
    prm = oracle_lib.make_params(cmd, **kw)
    cap = 2048 if cmd == "ppr" else params["len"] + 1
    lens, verts, steps = oracle_lib.walk(csr, prm, cap=cap, threads=0)
    assert steps == int(d["total_steps"])
    nh = len(d["head_lens"])
    np.testing.assert_array_equal(lens[:nh], d["head_lens"])
    np.testing.assert_array_equal(verts[:int(d["head_lens"].sum())], d["head_verts"])
    assert G.paths_digest(lens, verts) == str(d["paths_sha256"])
