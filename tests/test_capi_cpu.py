"""CPU checks of the C-ABI boundary: the library builds and loads without a GPU,
exports every function include/*.h declares, and its host-only code (the
PathSet::dump writer, argument checks) behaves like the reference."""

import ctypes
import glob
import json
import os
import re

import numpy as np
import pytest

from cases import GOLDEN

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(kk_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def kk():
    import knightking_gb300
    return knightking_gb300


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("kk_engine_create", "kk_graph_load_binary", "kk_walk", "kk_walk_node2vec", "kk_alias_build",
                 "kk_paths_dump", "kk_walk_into", "kk_walk_device"):
        assert must in names


def test_library_exports_every_declared_symbol(kk):
    lib = ctypes.CDLL(kk.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(kk):
    lib = kk.lib()
    assert lib.kk_status_string(0) == b"ok"
    assert lib.kk_status_string(8) == b"path capacity exceeded"


def test_null_arguments_are_rejected_without_a_gpu(kk):
    lib = kk.lib()
    assert lib.kk_engine_create(None, 0) == 1
    assert lib.kk_walk(None, None, None) == 1
    assert lib.kk_paths_dump(None, b"x", b"w", 0, 1) == 1


@pytest.mark.parametrize("head", [0, 1])
def test_dump_matches_reference_text(kk, tmp_path, head):
    """PathSet::dump (include/path.hpp:85-109) with -r 0.3 and 3 worker threads."""
    d = np.load(os.path.join(GOLDEN, "dump_deepwalk_head%d.npz" % head))
    params = json.loads(str(d["params"]))
    lens, verts = d["lens"], d["verts"]
    offset = np.zeros(len(lens), np.uint64)
    offset[1:] = np.cumsum(lens[:-1].astype(np.uint64))
    per = int(params["walkers"] * params["rate"])
    ps = kk.PathSet(0, per, lens, offset, verts, int(lens.sum()) - len(lens))
    out = tmp_path / "dump.0"
    ps.dump(out, "w", bool(head), seg_num=params["threads"])
    assert out.read_text() == str(d["text"])


def test_walk_config_mirrors_reference_checks(kk):
    conf = kk.WalkConfig()
    with pytest.raises(kk.KKError):
        conf.set_walk_rate(0.0)
    with pytest.raises(kk.KKError):
        conf.set_walk_rate(1.5)
    conf.set_walk_rate(0.25)
    assert conf.rate == 0.25
    with pytest.raises(kk.KKError):
        conf.set_output_file(None)


def test_read_metapath_schemes(kk, tmp_path):
    f = tmp_path / "s.txt"
    f.write_text("2 3\n2\n1 0 0 \n0 1 1 \n1\n0 0 1 \n")
    sc = kk.read_metapath_schemes(f)
    assert sc == [[[True, False, False], [False, True, True]], [[False, False, True]]]
