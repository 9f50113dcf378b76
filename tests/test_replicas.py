"""The multi-rank path on CPU (gloo, world size 2): node shards cover the
batch, per-rank expansions of the shards (oracle) gathered equal the
expansion of the whole batch, and the step reduction takes the max time
and the summed units."""
import os
import socket
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from dynoplan_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import oracle_bind as ob
    from dynoplan_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = W.make_workload(1, scale=0.05)
    mine = replicas.shard(wl.nodes, rank, world)
    lo, _ = replicas.shard_bounds(len(wl.nodes), rank, world)
    r = ob.expand(wl.robot, wl.prims, wl.env, mine, wl.radius)
    rows = np.stack([r["node"].astype(np.int64) + lo, r["prim"].astype(np.int64), r["verdict"].astype(np.int64),
                     r["first_invalid"].astype(np.int64)], 1)
    gathered = [None] * world
    dist.all_gather_object(gathered, rows)
    t, u = replicas.reduce_step(0.5 + rank, 10.0 * (rank + 1))
    if rank == 0:
        np.save(os.path.join(out_dir, "gathered.npy"), np.concatenate(gathered))
        np.save(os.path.join(out_dir, "reduced.npy"), np.array([t, u]))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_bounds_cover():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_reduce_identity_without_group():
    assert replicas.reduce_step(1.5, 7) == (1.5, 7.0)


def test_two_gloo_ranks_match_single_expand(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import oracle_bind as ob
    from dynoplan_gb300 import workloads as W
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = np.load(tmp_path / "gathered.npy")
    wl = W.make_workload(1, scale=0.05)
    r = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
    want = np.stack([r["node"].astype(np.int64), r["prim"].astype(np.int64), r["verdict"].astype(np.int64),
                     r["first_invalid"].astype(np.int64)], 1)
    key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]
    assert got.shape == want.shape and np.array_equal(key(got), key(want))
    t, u = np.load(tmp_path / "reduced.npy")
    assert t == 1.5 and u == 30.0
