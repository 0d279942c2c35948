"""The multi-GPU host logic on CPU ranks (gloo, world size 2): the LP shards
of the batched path are disjoint and cover every LP, and the timing reduction
returns the slowest rank's value (and the sum of the ranks' counts)."""
import os

import pytest


def _worker(rank, world, port, count, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from coolpdlp.distributed import dist_info, reduce_over_ranks, shard_indices
        ws, r, _ = dist_info()
        mine = shard_indices(count, r, ws)
        t_max = reduce_over_ranks(1.5 + r, "max")
        n_sum = reduce_over_ranks(len(mine), "sum")
        out.put((r, mine, t_max, n_sum))
    finally:
        dist.destroy_process_group()


def test_batch_sharding_over_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    count, world = 11, 2
    procs = [ctx.Process(target=_worker, args=(r, world, port, count, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shards = [set(m) for _, m, _, _ in res]
    assert shards[0].isdisjoint(shards[1])
    assert shards[0] | shards[1] == set(range(count))
    assert all(t == 2.5 for _, _, t, _ in res)          # the slowest rank's time
    assert all(n == count for _, _, _, n in res)


def test_shard_indices_single_rank_and_errors():
    from coolpdlp.distributed import reduce_over_ranks, shard_indices
    assert shard_indices(5, 0, 1) == [0, 1, 2, 3, 4]
    assert reduce_over_ranks(3.0) == 3.0
    with pytest.raises(ValueError):
        shard_indices(5, 2, 2)
