"""Two ranks on CPU (gloo), as bench.py runs N GPUs under torchrun: each rank
takes its walker-id range from bench.rank_walkers and walks it on its own
replica of the graph; times are reduced with MAX and steps with SUM, and no
data-path collective exists.  The ranks' paths, walked here by the oracle,
concatenate to the paths of one walk over all walkers."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

N_PER_RANK = 300


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _graph():
    from oracle import graphs as G
    g = G.random_undirected(200, 2000, seed=4, weight="unif")
    return G.csr_file_order(200, g["src"], g["dst"], w=g.get("w"))


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    from oracle import pyoracle
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    begin, num = bench.rank_walkers(rank, N_PER_RANK)
    csr = _graph()
    ocsr = pyoracle.CSR(200, csr["off"], csr["nbr"], csr["w"])
    prm = pyoracle.make_params("deepwalk", seed=7, walker_begin=begin, walker_num=num, weighted=True, walk_length=15)
    lens, verts, steps = pyoracle.walk(ocsr, prm, cap=64)
    bench.barrier(world)
    t_max = bench.allreduce(world, 1.0 + rank, "max")
    s_sum = bench.allreduce(world, float(steps), "sum")
    out.put((rank, begin, num, lens, verts, steps, t_max, s_sum))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_ranks_shard_walkers_and_reduce():
    from oracle import pyoracle
    pyoracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in range(2)], key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, b0, n0, l0, v0, s0, t0, sum0), (r1, b1, n1, l1, v1, s1, t1, sum1) = res
    assert (b0, n0, b1, n1) == (0, N_PER_RANK, N_PER_RANK, N_PER_RANK)
    assert t0 == t1 == 2.0                      # MAX over ranks
    assert sum0 == sum1 == float(s0 + s1)       # SUM over ranks
    csr = _graph()
    ocsr = pyoracle.CSR(200, csr["off"], csr["nbr"], csr["w"])
    prm = pyoracle.make_params("deepwalk", seed=7, walker_begin=0, walker_num=2 * N_PER_RANK, weighted=True,
                               walk_length=15)
    lens, verts, steps = pyoracle.walk(ocsr, prm, cap=64)
    np.testing.assert_array_equal(np.concatenate([l0, l1]), lens)
    np.testing.assert_array_equal(np.concatenate([v0, v1]), verts)
    assert s0 + s1 == steps
