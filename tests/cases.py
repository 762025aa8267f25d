"""Loads the golden fixtures (tests/golden/*.npz) into graph + parameters.

Shared by the oracle tests (CPU) and the CUDA parity tests (GPU): both rebuild
the same CSR from the stored edge list and map the stored parameters onto their
own API.
"""

import glob
import json
import os

import numpy as np

from oracle import graphs as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_files(prefix="case_"):
    return sorted(glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def case_ids(prefix="case_"):
    return [os.path.basename(f)[:-4] for f in case_files(prefix)]


class Case:
    def __init__(self, name):
        self.name = name
        d = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
        self.d = d
        self.kind = str(d["kind"])
        self.cmd = str(d["cmd"])
        self.params = json.loads(str(d["params"]))
        self.lens = d["lens"] if "lens" in d else None
        self.verts = d["verts"] if "verts" in d else None

    def graph(self):
        """CSR in file order per source, like include/graph.hpp:309-330."""
        d = self.d
        V = int(d["V"])
        data = {}
        if "w" in d:
            data["w"] = d["w"]
        if "type" in d:
            data["type"] = d["type"]
        g = G.csr_file_order(V, d["src"], d["dst"], **data)
        g["weighted"] = self.kind in ("f32", "meta_f32", "tag_f32")
        return g

    @property
    def weighted(self):
        return self.kind in ("f32", "meta_f32", "tag_f32")

    @property
    def walkers(self):
        return int(self.params["walkers"])

    def cap(self):
        if self.lens is not None and len(self.lens):
            return int(self.lens.max()) + 1
        return 2


def walk_kwargs(case):
    """Keyword arguments shared by the oracle's make_params and the product API."""
    p = case.params
    app = case.cmd
    kw = dict(seed=int(p["seed"]), walker_num=int(p["walkers"]), weighted=case.weighted)
    if app in ("deepwalk", "node2vec", "metapath", "tagwalk", "dynwalk"):
        kw["walk_length"] = int(p["len"])
    if app == "ppr":
        kw["terminate_prob"] = float(np.float32(p["term"]))
    if app == "node2vec":
        kw["p"] = float(p["p"])
        kw["q"] = float(p["q"])
    if app == "metapath":
        kw["schemes"] = p["schemes"]
    if app == "tagwalk":
        kw["tag_num"] = int(p["tag-num"])
        kw["vertex_tag_weight"] = float(p["vtw"])
        kw["outlier_amplifier"] = float(p["amp"])
        kw["order"] = int(p["order"])
        kw["outlier"] = p["variant"] == "outlier"
        kw["vertex_tag"] = case.d["vertex_tag"]
    return kw
