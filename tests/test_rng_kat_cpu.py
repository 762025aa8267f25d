"""Known-answer checks of the random stream on the host.

Every draw of a walk is a word of Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
"Parallel Random Numbers: As Easy as 1, 2, 3", SC'11), keyed by the walk's
seed; it replaces the reference's per-thread mt19937 (include/util.hpp:45-70).
The three vectors below are the published Random123 known answers for
philox4x32_10 (counter, key -> output).  The oracle's C generator and the
Python generator of the synthetic graphs must both reproduce them; the
device generator is checked against the same vectors in test_gpu_limits_rng.py.
"""

import ctypes

import numpy as np

from oracle import graphs as G

# (counter words, key words (k0, k1), output words)
KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def seed_of(key):
    return key[0] | (key[1] << 32)


def oracle_blocks(oracle_lib, seed, ctr):
    ctr = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros_like(ctr)
    L = oracle_lib.lib()
    L.ko_philox_blocks.restype = None
    L.ko_philox_blocks.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    L.ko_philox_blocks(seed, len(ctr), ctr.ctypes.data, out.ctypes.data)
    return out


def test_oracle_generator_matches_known_answers(oracle_lib):
    for ctr, key, want in KAT:
        got = oracle_blocks(oracle_lib, seed_of(key), [ctr])[0]
        assert [int(x) for x in got] == list(want)


def test_graph_generator_matches_known_answers():
    for ctr, key, want in KAT:
        got = G.philox4x32_10(*[np.array([c], np.uint32) for c in ctr], seed_of(key))
        assert [int(x[0]) for x in got] == list(want)


def test_oracle_and_graph_generators_agree(oracle_lib):
    rng = np.random.default_rng(3)
    ctr = rng.integers(0, 1 << 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    seed = 0x0123456789ABCDEF
    a = oracle_blocks(oracle_lib, seed, ctr)
    b = np.stack(G.philox4x32_10(ctr[:, 0], ctr[:, 1], ctr[:, 2], ctr[:, 3], seed), axis=1)
    np.testing.assert_array_equal(a, b)
