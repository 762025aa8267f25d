"""ORACLE / TEST INFRASTRUCTURE ONLY: synthetic graphs and reference file formats.

Used by the golden-fixture script, the CPU tests and the checker side of the
GPU tests.  Nothing in the product imports this module.

* ``write_edge_file`` writes the reference's binary edge list: a packed array
  of ``Edge<T>`` records ``{u32 src; u32 dst; T data}`` (include/type.hpp:43-85,
  read by include/storage.hpp:35-55).
* ``csr_file_order`` builds the CSR the reference builds: edges grouped by
  source, file order kept within a source (include/graph.hpp:309-330).
* ``random_undirected`` follows the tests' generator (src/tests/test.hpp:49-99):
  distinct unordered pairs without self-loops, each written as (s,t) then
  (t,s) with the same data, in generation order.
* ``rmat`` is the project's seeded R-MAT definition, restated here with numpy;
  the CUDA generator in the product computes the same graph bit for bit:
    - M = edge_factor * 2**scale draws; draw i takes, for level l, the 32-bit
      word l%4 of Philox4x32-10(key=seed, counter=(i, 0, l//4, 3));
    - quadrant by integer thresholds floor(a*2^32), floor((a+b)*2^32),
      floor((a+b+c)*2^32): a -> (0,0), b -> (0,1), c -> (1,0), d -> (1,1);
      level 0 gives the most significant bit of (src, dst);
    - self-loops dropped, pairs made (min,max) and deduplicated, mirrored,
      sorted by (src, dst);
    - per unordered pair (u<v), Philox(key=seed, counter=(u, v, 0, 4)) gives
      word0 -> weight 1 + 4*(word0>>8)*2^-24 (uniform [1,5), float32 ops),
      word1 -> edge type floor(word1*ntypes / 2^32).
"""

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

STREAM_GRAPH = 3
STREAM_EDGE_DATA = 4

EDGE_DTYPES = {
    "none": np.dtype([("src", "<u4"), ("dst", "<u4")]),
    "f32": np.dtype([("src", "<u4"), ("dst", "<u4"), ("w", "<f4")]),
    "meta": np.dtype([("src", "<u4"), ("dst", "<u4"), ("type", "<i4")]),
    "meta_f32": np.dtype([("src", "<u4"), ("dst", "<u4"), ("w", "<f4"), ("type", "<i4")]),
    "tag": np.dtype([("src", "<u4"), ("dst", "<u4"), ("type", "<i4")]),
    "tag_f32": np.dtype([("src", "<u4"), ("dst", "<u4"), ("type", "<i4"), ("w", "<f4")]),
}


def philox4x32_10(c0, c1, c2, c3, seed):
    """Vectorised Philox4x32-10 (Salmon et al., SC'11).  Arrays of uint32."""
    c0 = np.asarray(c0, dtype=np.uint32).copy()
    c1 = np.asarray(c1, dtype=np.uint32).copy()
    c2 = np.asarray(c2, dtype=np.uint32).copy()
    c3 = np.asarray(c3, dtype=np.uint32).copy()
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    c0, c1, c2, c3 = c0.copy(), c1.copy(), c2.copy(), c3.copy()
    k0 = np.uint32(seed & 0xFFFFFFFF)
    k1 = np.uint32((seed >> 32) & 0xFFFFFFFF)
    with np.errstate(over="ignore"):
        for r in range(10):
            if r:
                k0 = np.uint32(k0 + W0)
                k1 = np.uint32(k1 + W1)
            p0 = M0 * c0.astype(np.uint64)
            p1 = M1 * c2.astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & MASK32).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & MASK32).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def unit_f32(word):
    """(word >> 8) * 2^-24 as float32 (exact)."""
    return (np.asarray(word, dtype=np.uint32) >> np.uint32(8)).astype(np.float32) * np.float32(2.0 ** -24)


def rmat_pairs(scale, edge_factor, a, b, c, seed):
    """Unordered, deduplicated R-MAT pairs (u < v) as a sorted uint64 key array."""
    m = edge_factor << scale
    ta = np.uint64(int(np.floor(a * 4294967296.0)))
    tab = np.uint64(int(np.floor((a + b) * 4294967296.0)))
    tabc = np.uint64(int(np.floor((a + b + c) * 4294967296.0)))
    idx = np.arange(m, dtype=np.uint64)
    src = np.zeros(m, dtype=np.uint64)
    dst = np.zeros(m, dtype=np.uint64)
    i32 = idx.astype(np.uint32)
    for blk in range((scale + 3) // 4):
        words = philox4x32_10(i32, 0, blk, STREAM_GRAPH, seed)
        for wi in range(4):
            lvl = blk * 4 + wi
            if lvl >= scale:
                break
            w = words[wi].astype(np.uint64)
            sbit = (w >= tab).astype(np.uint64)
            dbit = ((w >= ta) & (w < tab)) | (w >= tabc)
            src = (src << np.uint64(1)) | sbit
            dst = (dst << np.uint64(1)) | dbit.astype(np.uint64)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    lo = np.minimum(src, dst)
    hi = np.maximum(src, dst)
    return np.unique((lo << np.uint64(32)) | hi)


def pair_data(u, v, seed, ntypes=5):
    """Per unordered pair: uniform [1,5) float32 weight and an edge type."""
    w0, w1, _, _ = philox4x32_10(np.asarray(u, np.uint32), np.asarray(v, np.uint32), 0, STREAM_EDGE_DATA, seed)
    weight = np.float32(1.0) + unit_f32(w0) * np.float32(4.0)
    etype = ((w1.astype(np.uint64) * np.uint64(ntypes)) >> np.uint64(32)).astype(np.uint8)
    return weight.astype(np.float32), etype


def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=None, weights=False, types=False, ntypes=5):
    """Seeded R-MAT graph as a sorted, symmetric CSR dict (see module docstring)."""
    if seed is None:
        seed = scale
    keys = rmat_pairs(scale, edge_factor, a, b, c, seed)
    u = (keys >> np.uint64(32)).astype(np.uint32)
    v = (keys & MASK32).astype(np.uint32)
    src = np.concatenate([u, v])
    dst = np.concatenate([v, u])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    g = {"V": 1 << scale, "src": src, "dst": dst}
    if weights or types:
        lo = np.minimum(src, dst)
        hi = np.maximum(src, dst)
        w, t = pair_data(lo, hi, seed + 1000, ntypes)
        if weights:
            g["w"] = w
        if types:
            g["type"] = t
    g["off"] = offsets(g["V"], src)
    return g


def offsets(V, src):
    counts = np.bincount(src.astype(np.int64), minlength=V).astype(np.int64)
    off = np.zeros(V + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    return off


def csr_file_order(V, src, dst, **data):
    """CSR with file order kept per source (include/graph.hpp:309-330)."""
    order = np.argsort(src, kind="stable")
    out = {"V": V, "off": offsets(V, src), "nbr": dst[order].astype(np.int32)}
    for k, arr in data.items():
        if arr is not None:
            out[k] = np.asarray(arr)[order]
    return out


def random_undirected(v_num, e_num, seed, weight=None, types=None, ntypes=5):
    """Random simple undirected graph in the tests' file order.

    weight: None, "int5" (integers 1..5 stored as float, like
    src/tests/generator_helper.hpp:65-76) or "unif" (uniform [1,5) float32).
    types: None or "uniform" (int in [0, ntypes)).
    """
    assert e_num % 2 == 0
    rng = np.random.default_rng(seed)
    seen = set()
    pairs = []
    while len(pairs) < e_num // 2:
        s, t = (int(x) for x in rng.integers(0, v_num, size=2))
        if s == t:
            continue
        if s > t:
            s, t = t, s
        if (s, t) in seen:
            continue
        seen.add((s, t))
        pairs.append((s, t))
    pairs = np.array(pairs, dtype=np.uint32)
    n = len(pairs)
    src = np.empty(2 * n, np.uint32)
    dst = np.empty(2 * n, np.uint32)
    src[0::2], dst[0::2] = pairs[:, 0], pairs[:, 1]
    src[1::2], dst[1::2] = pairs[:, 1], pairs[:, 0]
    g = {"V": v_num, "src": src, "dst": dst}
    if weight == "int5":
        w = rng.integers(1, 6, size=n).astype(np.float32)
    elif weight == "unif":
        w = (np.float32(1.0) + rng.random(n, dtype=np.float32) * np.float32(4.0)).astype(np.float32)
    else:
        w = None
    if w is not None:
        g["w"] = np.repeat(w, 2)
    if types is not None:
        g["type"] = np.repeat(rng.integers(0, ntypes, size=n).astype(np.int32), 2)
    return g


def write_edge_file(path, g, kind):
    dt = EDGE_DTYPES[kind]
    rec = np.zeros(len(g["src"]), dtype=dt)
    rec["src"] = g["src"]
    rec["dst"] = g["dst"]
    if "w" in dt.names:
        rec["w"] = g["w"]
    if "type" in dt.names:
        rec["type"] = g["type"]
    rec.tofile(path)


def read_paths(path):
    """Read a "KKP1" path file: u32 n, u32 len[n], u32 vertices[sum(len)]."""
    raw = np.fromfile(path, dtype=np.uint8)
    assert raw[:4].tobytes() == b"KKP1"
    n = int(raw[4:8].view(np.uint32)[0])
    lens = raw[8:8 + 4 * n].view(np.uint32).copy()
    verts = raw[8 + 4 * n:].view(np.uint32).copy()
    assert len(verts) == int(lens.sum())
    return lens, verts


def read_alias(path):
    raw = np.fromfile(path, dtype=np.uint8)
    assert raw[:4].tobytes() == b"KKA1"
    V = int(raw[4:8].view(np.uint32)[0])
    E = int(raw[8:16].view(np.uint64)[0])
    o = 16
    p = raw[o:o + 4 * E].view(np.float32).copy(); o += 4 * E
    pi = raw[o:o + 4 * E].view(np.uint32).copy(); o += 4 * E
    qi = raw[o:o + 4 * E].view(np.uint32).copy(); o += 4 * E
    s = raw[o:o + 4 * V].view(np.float32).copy()
    return p, pi, qi, s


def paths_digest(lens, verts):
    """SHA-256 over the little-endian bytes of (lens, verts)."""
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(lens, dtype="<u4").tobytes())
    h.update(np.ascontiguousarray(verts, dtype="<u4").tobytes())
    return h.hexdigest()
