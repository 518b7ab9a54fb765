"""Host-side multi-rank logic on CPU: two gloo ranks split a 64-atmosphere
sweep disjointly, agree on the job time (maximum over ranks) and gather
their per-rank results in rank order."""
import os
import socket

import pytest

from sfsim_gb300 import config as C
from sfsim_gb300 import replicas


def test_shard_partition():
    items = list(range(64))
    parts = [replicas.shard(items, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == items
    assert all(set(a).isdisjoint(b) for i, a in enumerate(parts) for b in parts[i + 1:])
    with pytest.raises(ValueError):
        replicas.shard(items, 3, 3)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfgs = C.parameter_sweep(64)
    mine = replicas.shard_indices(len(cfgs), rank, world)
    radii = [cfgs[i].radius for i in mine]
    t = replicas.max_over_ranks(1.0 + rank)
    everything = replicas.gather_objects((rank, mine, radii))
    q.put((rank, t, everything))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cfgs = C.parameter_sweep(64)
    for rank, t, everything in results:
        assert t == 2.0
        assert [e[0] for e in everything] == [0, 1]
        got = sorted(i for e in everything for i in e[1])
        assert got == list(range(64))
        for r, idx, radii in everything:
            assert radii == [cfgs[i].radius for i in idx]
