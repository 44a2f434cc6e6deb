"""Multi-process path of the batched form on CPU: world_size-2 gloo ranks shard the molecules by
cost, solve nothing on a GPU (each rank stands in a per-molecule result), and gather on rank 0."""
import os
import socket

import numpy as np
import pytest

from dftbplus_gb300.shard import share_cost, shard_by_cost


def test_shard_partition_and_balance():
    rng = np.random.default_rng(4096)
    n = 6 * rng.integers(2, 49, 4096)
    for world in (1, 2, 3, 8):
        shares = shard_by_cost(n, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(n)))
        costs = [share_cost(n, s) for s in shares]
        # greedy longest-first: max load within one largest item of the mean
        assert max(costs) - sum(costs) / world <= max(int(v) ** 3 for v in n)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n_orb, q):
    import torch.distributed as dist
    from dftbplus_gb300.shard import gather_to_root, shard_by_cost
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    share = shard_by_cost(n_orb, world)[rank]
    # stand-in for the per-molecule result of a batched SCC on this rank's GPU
    local = {"energy": [-float(n_orb[i]) for i in share], "rank": [rank] * len(share)}
    out = gather_to_root(local, share, len(n_orb))
    if rank == 0:
        q.put(out)
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_gather():
    mp = pytest.importorskip("torch.multiprocessing")
    n_orb = [6 * k for k in (2, 48, 17, 5, 30, 30, 9, 41, 3)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, n_orb, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out["energy"] == [-float(v) for v in n_orb]
    assert set(out["rank"]) == {0, 1}
