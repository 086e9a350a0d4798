"""Data-parallel helpers of the modelling sequence, two gloo ranks on the CPU
(the GPU runs use NCCL with the same calls)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from gigalens_gb300.cuda import distributed as D


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = {}
        out["rank_world"] = D.rank_world()
        # 13 chains over 2 ranks: 7 + 6, contiguous, covering everything once
        out["shard"] = D.shard_range(13)
        # mean of per-rank tensors
        t = torch.full((4,), float(rank + 1))
        out["mean"] = D.allreduce_mean_(t).tolist()
        # gather unequal shards in rank order
        lo, hi = D.shard_range(13)
        x = torch.arange(lo, hi, dtype=torch.float32)[:, None].repeat(1, 3)
        out["gather"] = D.gather_chains(x, dim=0)[:, 0].tolist()
        # samples (results, chains, d): gather along the chain axis
        s = torch.full((2, hi - lo, 3), float(rank))
        out["gather1"] = list(D.gather_chains(s, dim=1).shape)
        # global best: rank 1 holds the best chain
        z = torch.tensor([[rank * 10.0 + 1, 0.0], [rank * 10.0 + 2, 0.0]])
        logp = torch.tensor([float(rank), float("nan")]) if rank == 0 else torch.tensor([-1.0, 5.0])
        out["best"] = D.global_best(z, logp).tolist()
        # one chain over two ranks: rank 1's shard is empty and must not
        # raise or leave rank 0 waiting in the exchange
        lo1, hi1 = D.shard_range(1)
        z1 = torch.tensor([[7.0, 8.0]])[lo1:hi1]
        lp1 = torch.tensor([3.0])[lo1:hi1]
        out["shard1"] = (lo1, hi1)
        out["best1"] = D.global_best(z1, lp1).tolist()
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_two_rank_helpers():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0]["rank_world"] == (0, 2) and res[1]["rank_world"] == (1, 2)
    assert res[0]["shard"] == (0, 7) and res[1]["shard"] == (7, 13)
    for r in (0, 1):
        assert res[r]["mean"] == [1.5] * 4
        assert res[r]["gather"] == [float(i) for i in range(13)]
        assert res[r]["gather1"] == [2, 13, 3]
        assert res[r]["best"] == [12.0, 0.0]
        assert res[r]["best1"] == [7.0, 8.0]
    assert res[0]["shard1"] == (0, 1) and res[1]["shard1"] == (1, 1)


def test_single_process_is_identity():
    assert D.rank_world() == (0, 1)
    assert D.shard_range(13) == (0, 13)
    t = torch.ones(3)
    assert D.allreduce_mean_(t) is t and t.tolist() == [1.0] * 3
    x = torch.randn(5, 2)
    assert D.gather_chains(x) is x
    z = torch.tensor([[1.0], [2.0], [3.0]])
    assert D.global_best(z, torch.tensor([0.0, float("nan"), 1.0])).tolist() == [3.0]


@pytest.mark.parametrize("n,world", [(10, 3), (2, 4), (4096, 8)])
def test_shards_cover_once(n, world):
    seen = []
    for r in range(world):
        lo, hi = D.shard_range(n, r, world)
        seen.extend(range(lo, hi))
    assert seen == list(range(n))
