"""Chain sharding over ranks and the host-side reduction, with two gloo
ranks on the CPU (the multi-GPU path has no collective on the data path;
the final reduction is the only exchange)."""
import os
import socket

import numpy as np
import pytest

from w2dynamics_gb300 import shard


def test_chain_range_partitions():
    for n in (1, 7, 4096, 4099):
        for w in (1, 2, 3, 8):
            parts = [shard.chain_range(n, r, w) for r in range(w)]
            assert sum(c for _, c in parts) == n
            assert [f for f, _ in parts] == sorted(f for f, _ in parts)
            for (f0, c0), (f1, _) in zip(parts, parts[1:]):
                assert f0 + c0 == f1
            assert max(c for _, c in parts) - min(c for _, c in parts) <= 1


def test_shard_groups_keep_seeds():
    groups = [dict(beta=10.0, nchains=10, seed0=0), dict(beta=50.0, nchains=5, seed0=10)]
    seen = []
    for r in range(3):
        for g, sg in zip(groups, shard.shard_groups(groups, r, 3)):
            seen += [(g["beta"], sg["seed0"] + c) for c in range(sg["nchains"])]
    assert sorted(seen) == sorted([(10.0, s) for s in range(10)] + [(50.0, 10 + s) for s in range(5)])


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(rank)
    g = rng.standard_normal((3, 2, 5))
    sums = shard.reduce_group_sums(g, sign_sum=10.0 + rank, count=100 * (rank + 1))
    t = shard.max_over_ranks(1.5 + rank)
    if rank == 0:
        np.save(out, np.concatenate([sums[0].ravel(), [sums[1], sums[2], t]]))
    dist.destroy_process_group()


def test_reduction_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "r.npy")
    tmp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    exp = sum(np.random.default_rng(r).standard_normal((3, 2, 5)) for r in range(2)).ravel()
    assert np.allclose(got[:-3], exp)
    assert got[-3] == 21.0 and got[-2] == 300 and got[-1] == 2.5
