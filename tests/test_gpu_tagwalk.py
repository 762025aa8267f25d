"""User-defined hooks through the plugin API, against the reference.

knightking_gb300/examples/tagwalk.cu writes the bound and outlier tag walks
(after src/tests/test_bound.cpp and src/tests/test_outlier.cpp) as __device__
functors for TransitionConfig / SecondOrderTransitionConfig and runs them with
kk::random_walk.  The golden fixtures case_t200_* are the reference's own engine
running the same hooks (tests/golden/make_golden.py): the paths must match bit
for bit, covering per-vertex lower/upper bounds, the outlier appendix with its
search hook, weighted and unweighted, first and second order with a custom
query/response.
"""

import ctypes
import os

import numpy as np
import pytest

from cases import Case, case_ids, walk_kwargs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kk():
    import knightking_gb300
    return knightking_gb300


@pytest.fixture(scope="module")
def example(kk):
    kk.lib()
    path = os.path.join(os.path.dirname(kk.library_path()), "libkk_example_tagwalk.so")
    L = ctypes.CDLL(path)
    L.kk_example_tagwalk.restype = ctypes.c_int
    L.kk_example_tagwalk.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    return L


@pytest.fixture(scope="module")
def engine(kk):
    e = kk.WalkEngine(0)
    yield e
    e.close()


@pytest.mark.parametrize("park", [0, 20])
@pytest.mark.parametrize("name", case_ids("case_t200"))
def test_tagwalk_hooks_match_reference(kk, example, engine, name, park):
    """park 20: first-order tag walks (rejection trials) park the walkers of
    thinned-out warps and resume them in later launches (walk_park)."""
    from knightking_gb300 import _capi
    case = Case(name)
    g = case.graph()
    engine.load_arrays(g["V"], g["off"], g["nbr"], g.get("w"), g.get("type"))
    kw = walk_kwargs(case)
    opts = engine.make_opts("deepwalk", kw["walker_num"], seed=kw["seed"], walk_length=kw["walk_length"],
                            weighted=kw["weighted"])
    vtag = np.ascontiguousarray(kw["vertex_tag"], dtype=np.int32)
    out = ctypes.POINTER(_capi.KKPaths)()
    engine.set_option("walk_park", park)
    try:
        st = example.kk_example_tagwalk(engine._h, ctypes.byref(opts), vtag.ctypes.data, kw["tag_num"],
                                        kw["vertex_tag_weight"], kw["outlier_amplifier"], kw["order"],
                                        int(kw["outlier"]), ctypes.byref(out))
    finally:
        engine.set_option("walk_park", 20)
    assert st == 0, _capi.lib().kk_last_error(engine._h)
    try:
        _, _, lens, _, verts, steps = _capi.paths_to_numpy(out.contents)
    finally:
        _capi.lib().kk_paths_free(out)
    np.testing.assert_array_equal(lens, case.lens)
    np.testing.assert_array_equal(verts, case.verts)
