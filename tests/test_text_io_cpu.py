"""Host-only file formats (no GPU): gconverter's text -> binary edge files and
metapath scheme files, through the C-ABI library."""

import numpy as np
import pytest

import knightking_gb300 as kk
from oracle import graphs as G


def _edges(seed, weighted):
    g = G.random_undirected(300, 2000, seed=seed, weight="unif" if weighted else None)
    return g["src"], g["dst"], g.get("w")


@pytest.mark.parametrize("weighted", [False, True])
def test_text_to_binary_matches_edge_records(tmp_path, weighted):
    src, dst, w = _edges(3, weighted)
    txt = tmp_path / "g.txt"
    with open(txt, "w") as f:
        f.write("# comment line\n")
        for i in range(len(src)):
            if weighted:
                f.write("%d %d %.9g\n" % (src[i], dst[i], w[i]))
            else:
                f.write("%d\t%d\n" % (src[i], dst[i]))
    out = tmp_path / "g.bin"
    n = kk.text_to_binary(txt, out, weighted)
    assert n == len(src)
    if weighted:
        rec = np.dtype([("s", "<u4"), ("d", "<u4"), ("w", "<f4")])
    else:
        rec = np.dtype([("s", "<u4"), ("d", "<u4")])
    got = np.fromfile(out, dtype=rec)
    np.testing.assert_array_equal(got["s"], src)
    np.testing.assert_array_equal(got["d"], dst)
    if weighted:
        np.testing.assert_array_equal(got["w"], w)


def test_text_to_binary_rejects_malformed_lines(tmp_path):
    txt = tmp_path / "bad.txt"
    txt.write_text("1 2\n3 x\n")
    with pytest.raises(kk.KKError):
        kk.text_to_binary(txt, tmp_path / "bad.bin", False)


def test_metapath_scheme_file(tmp_path):
    # the reference's write_metapath_schemes layout (src/apps/metascheme.hpp:100-116)
    p = tmp_path / "schemes.txt"
    p.write_text("2 5\n3\n1 0 0 0 0 \n0 1 1 0 0 \n0 0 0 0 1 \n1\n1 1 1 1 1 \n")
    masks = kk.read_metapath_scheme_masks(p)
    assert masks == [[0b00001, 0b00110, 0b10000], [0b11111]]
    nested = kk.read_metapath_schemes(p)
    assert [[sum(1 << t for t, on in enumerate(st) if on) for st in sc] for sc in nested] == masks
