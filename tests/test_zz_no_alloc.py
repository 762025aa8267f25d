"""kk_alias_build_noalloc: alias tables from a call that allocates no device memory.

Callers that cannot call cudaMalloc (a serving process whose device memory
belongs to its own pool, or a latency-critical path where allocation and the
synchronisation of cudaFree are not allowed) hand the entry point their own
device buffers; it keeps its queue scratch in a fixed array inside the
library.  These tests check its tables bit for bit against kk_alias_build's
and against the oracle's restatement of the reference's alias build
(include/walk.hpp:538-652), on two calls in a row with different graphs (the
scratch keeps the previous call's contents); that a call leaves the device's
free memory unchanged; that a degree above the scratch limit is refused; and,
where two GPUs are visible, that a call on the second device works after one
on the first.  The buffers here are allocated by the test (with torch), not by
the entry point.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_DEGREE = 16384


def _graph(seed, head_degrees, V=20000):
    rng = np.random.default_rng(seed)
    degs = np.zeros(V, np.int64)
    degs[:len(head_degrees)] = head_degrees
    degs[len(head_degrees):4000] = rng.integers(0, 60, size=4000 - len(head_degrees))
    off = np.zeros(V + 1, np.int64)
    np.cumsum(degs, out=off[1:])
    E = int(off[-1])
    nbr = rng.integers(0, V, size=E).astype(np.uint32)
    w = rng.lognormal(0.0, 1.0, size=E).astype(np.float32)
    return V, off, nbr, w


def _noalloc(lib, torch, V, off, w):
    E = int(off[-1])
    d_off = torch.from_numpy(off).cuda()
    d_w = torch.from_numpy(w).cuda()
    d_p = torch.empty(E, dtype=torch.float32, device="cuda")
    d_pi = torch.empty(E, dtype=torch.int32, device="cuda")
    d_qi = torch.empty(E, dtype=torch.int32, device="cuda")
    d_sum = torch.zeros(V, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = lib.kk_alias_build_noalloc(V, d_off.data_ptr(), d_w.data_ptr(), d_p.data_ptr(), d_pi.data_ptr(),
                                    d_qi.data_ptr(), d_sum.data_ptr(), None)
    torch.cuda.synchronize()
    return st, d_p.cpu().numpy(), d_pi.cpu().numpy().view(np.uint32), d_qi.cpu().numpy().view(np.uint32), \
        d_sum.cpu().numpy()


def test_noalloc_alias_matches_kk_alias_build_on_two_calls():
    torch = pytest.importorskip("torch")
    import knightking_gb300 as kk
    from oracle import pyoracle
    lib = kk.lib()
    engine = kk.WalkEngine(0)
    try:
        # degrees in shared-memory queues (<= 512), in scratch slices, at the limit
        for seed, head in ((5, [MAX_DEGREE, 9000, 700, 513, 512, 31]), (6, [2000, 600, 33, 1])):
            V, off, nbr, w = _graph(seed, head)
            engine.load_arrays(V, off, nbr, w)
            p, pi, qi, s = engine.alias_tables()
            st, p2, pi2, qi2, s2 = _noalloc(lib, torch, V, off, w)
            assert st == 0
            np.testing.assert_array_equal(pi2, pi)
            np.testing.assert_array_equal(qi2, qi)
            np.testing.assert_array_equal(p2.view(np.uint32), p.view(np.uint32))
            np.testing.assert_array_equal(s2.view(np.uint32), s.view(np.uint32))
            op, opi, oqi, osum = pyoracle.alias_build(pyoracle.CSR(V, off, nbr, w))
            np.testing.assert_array_equal(pi2, opi)
            np.testing.assert_array_equal(qi2, oqi)
            np.testing.assert_array_equal(p2.view(np.uint32), op.view(np.uint32))
            np.testing.assert_array_equal(s2.view(np.uint32), osum.view(np.uint32))
    finally:
        engine.close()


def test_noalloc_alias_allocates_no_device_memory():
    torch = pytest.importorskip("torch")
    import knightking_gb300 as kk
    lib = kk.lib()
    V, off, nbr, w = _graph(8, [MAX_DEGREE, 3000, 600, 40])
    E = int(off[-1])
    d_off = torch.from_numpy(off).cuda()
    d_w = torch.from_numpy(w).cuda()
    out = [torch.empty(E, dtype=t, device="cuda") for t in (torch.float32, torch.int32, torch.int32)]
    d_sum = torch.empty(V, dtype=torch.float32, device="cuda")
    args = (V, d_off.data_ptr(), d_w.data_ptr(), out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
            d_sum.data_ptr(), None)
    assert lib.kk_alias_build_noalloc(*args) == 0  # first call: per-device set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.kk_alias_build_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_alias_rejects_degree_above_limit():
    torch = pytest.importorskip("torch")
    import knightking_gb300 as kk
    V, off, _, w = _graph(7, [MAX_DEGREE + 1, 40])
    st, *_ = _noalloc(kk.lib(), torch, V, off, w)
    assert st == 1  # KK_ERR_INVALID_CONFIG


def test_noalloc_alias_on_a_second_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two visible GPUs")
    import knightking_gb300 as kk
    from oracle import pyoracle
    lib = kk.lib()
    V, off, nbr, w = _graph(9, [MAX_DEGREE, 4000, 513, 12])
    op, opi, oqi, _ = pyoracle.alias_build(pyoracle.CSR(V, off, nbr, w))
    for dev in (0, 1):
        with torch.cuda.device(dev):
            st, p2, pi2, qi2, _ = _noalloc(lib, torch, V, off, w)
            assert st == 0
            np.testing.assert_array_equal(pi2, opi)
            np.testing.assert_array_equal(qi2, oqi)
            np.testing.assert_array_equal(p2.view(np.uint32), op.view(np.uint32))
