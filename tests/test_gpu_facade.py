"""The reference's dynamic-walk example (src/examples/dynamic_walk.cpp:30-93)
ported onto the C++ classes WalkEngine / WalkConfig / PathSet
(include/knightking_gb300/walk_engine.cuh) by changing its includes and
turning its lambdas into functors (knightking_gb300/examples/dynamic_walk.cu).

The port runs as a program (its entry point called with an argv) on a binary
Edge<real_t> file, writes its paths through WalkConfig::set_output_file, and
the text must equal the reference's own paths for the same configuration
(tests/golden/case_dyn_*.npz, made by the reference's engine with the Philox
hook) and the oracle's, walker for walker.
"""

import ctypes
import os

import numpy as np
import pytest

from cases import Case
from oracle import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def example():
    import knightking_gb300 as kk
    path = os.path.join(os.path.dirname(kk.library_path()), "libkk_example_dynamic_walk.so")
    L = ctypes.CDLL(path)
    L.kk_example_dynamic_walk.restype = ctypes.c_int
    L.kk_example_dynamic_walk.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
    return L


def run(example, args):
    argv = [b"dynamic_walk"] + [str(a).encode() for a in args]
    arr = (ctypes.c_char_p * len(argv))(*argv)
    return example.kk_example_dynamic_walk(len(argv), arr)


def read_dump(path):
    lens, verts = [], []
    with open(path) as f:
        for line in f:
            vs = [int(x) for x in line.split()]
            lens.append(len(vs))
            verts += vs
    return np.array(lens, np.uint32), np.array(verts, np.uint32)


def oracle_walk(oracle_lib, g, n, length, seed):
    csr = G.csr_file_order(g["V"], g["src"], g["dst"], w=g["w"])
    prm = oracle_lib.make_params("dynwalk", seed=seed, walker_num=n, walk_length=length, weighted=True)
    return oracle_lib.walk(oracle_lib.CSR(g["V"], csr["off"], csr["nbr"], csr["w"]), prm, cap=length + 1)


@pytest.mark.parametrize("name,rate", [("case_dyn_karate", None), ("case_dyn_f200", None), ("case_dyn_f200", 0.3)])
def test_dynamic_walk_port_matches_reference(example, oracle_lib, tmp_path, name, rate):
    case = Case(name)
    d = case.d
    g = {"V": int(d["V"]), "src": d["src"], "dst": d["dst"], "w": d["w"]}
    gfile = tmp_path / "graph.bin"
    G.write_edge_file(gfile, g, "f32")
    p = case.params
    args = ["-v", g["V"], "-g", gfile, "-o", tmp_path / "walks", "-l", p["len"], "-w", p["walkers"], "--seed",
            p["seed"]]
    if rate is not None:
        args += ["-r", rate]
    assert run(example, args) == 0
    lens, verts = read_dump(tmp_path / "walks.0")
    np.testing.assert_array_equal(lens, case.lens)
    np.testing.assert_array_equal(verts, case.verts)
    olens, overts, _ = oracle_walk(oracle_lib, g, int(p["walkers"]), int(p["len"]), int(p["seed"]))
    np.testing.assert_array_equal(lens, olens)
    np.testing.assert_array_equal(verts, overts)


def test_dynamic_walk_port_make_undirected_and_errors(example, oracle_lib, tmp_path):
    """--make-undirected on the half edge list gives the undirected graph's
    walk; a missing graph file fails with status 1 (kk::Error), not an exit."""
    case = Case("case_dyn_f200")
    d = case.d
    half = {"V": int(d["V"]), "src": d["src"][0::2], "dst": d["dst"][0::2], "w": d["w"][0::2]}
    gfile = tmp_path / "half.bin"
    G.write_edge_file(gfile, half, "f32")
    p = case.params
    assert run(example, ["-v", half["V"], "-g", gfile, "--make-undirected", "-o", tmp_path / "u", "-l", p["len"],
                         "-w", p["walkers"], "--seed", p["seed"]]) == 0
    lens, verts = read_dump(tmp_path / "u.0")
    np.testing.assert_array_equal(lens, case.lens)
    np.testing.assert_array_equal(verts, case.verts)
    assert run(example, ["-v", 10, "-g", tmp_path / "missing.bin"]) == 1
    assert run(example, ["-v", 10]) == 2
