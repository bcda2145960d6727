"""The N>1 host path on CPU with two gloo ranks: shard placement and the timing
reduction that bench.py runs across ranks (no GPU, no data-path collective)."""
import os
import socket

import pytest

from eq_gb300 import shard
from eq_gb300 import workloads as wl


def test_balanced_shards_cover_and_balance():
    traps = wl.batched_uneven(3, 64)
    w = [t.n_nodes for t in traps]
    for world in (1, 2, 3, 8):
        sh = shard.balanced_shards(w, world)
        flat = sorted(i for s in sh for i in s)
        assert flat == list(range(len(traps)))
        loads = [sum(w[i] for i in s) for s in sh]
        assert max(loads) - min(loads) <= max(w)
        assert sh == shard.balanced_shards(w, world)  # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # weak scaling (bench.py's mode): every rank steps its own batch
        own = wl.batched_uneven(shard.rank_seed(3, rank), 16)
        nodes = sum(t.n_nodes for t in own)
        # strong scaling: one shared workload split into per-rank shards of whole traps
        common = wl.batched_uneven(3, 16)
        mine = shard.balanced_shards([t.n_nodes for t in common], world)[rank]
        fake_ms = 10.0 + 5.0 * rank
        dist.barrier()
        q.put((rank, shard.max_over_ranks(fake_ms), shard.sum_over_ranks(nodes), sorted(mine),
               [(t.nx, t.ny) for t in own], nodes))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_timing_and_place_traps():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res[0][1] == res[1][1] == 15.0  # max over ranks
    assert res[0][2] == res[1][2] == res[0][5] + res[1][5]  # global sum of the own batches
    # strong-scaling shards: disjoint, together the whole workload
    assert set(res[0][3]).isdisjoint(res[1][3])
    assert sorted(res[0][3] + res[1][3]) == list(range(16))
    # weak scaling: the ranks' batches are different draws
    assert res[0][4] != res[1][4]
