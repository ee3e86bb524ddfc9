"""The replica (N>1) path of bench.py on CPU: two gloo ranks, no GPU.  Chains shard across ranks by
global chain id (one seed, a chain range per rank) with no data-path collective; only the final
figures are reduced (max time, summed ESS and gradient evaluations)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r pretends to have sampled for (10 + r) ms with ESS 100 (r + 1) and 1000 (r + 1) gradients
        res = bench.reduce_over_ranks(dist, 10.0 + rank, 100.0 * (rank + 1), 1000 * (rank + 1))
        out[rank] = (res, bench.replica_chains(rank, 1024))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_bench():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True,
                           start_method="spawn")
        res = dict(out)
    for rank in range(world):
        (ms, ess, grads), seed = res[rank]
        assert ms == 11.0 and ess == 300.0 and grads == 3000
    # one seed, disjoint global chain ranges: the ranks' chains are the single run's, split by chain
    assert res[0][1] == (1000, 0) and res[1][1] == (1000, 1024)
