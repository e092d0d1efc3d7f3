"""Multi-rank host logic on CPU (gloo, world size 2): row sharding, ragged
balancing, and the FP64 all-reduce of the tap gradient of a data-parallel
backward pass (checked against the single-process FP64 oracle)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from matx_gb300.sharding import ragged_shard, reduce_tap_grad, row_shard


def test_row_shard_covers_batch():
    for batch in (1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            got = [row_shard(batch, r, world) for r in range(world)]
            assert sum(c for _, c in got) == batch
            assert [s for s, _ in got] == sorted(s for s, _ in got)
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
            for (s, c), (s2, _) in zip(got, got[1:]):
                assert s + c == s2


def test_ragged_shard_balances():
    rng = np.random.default_rng(0)
    work = np.exp(rng.uniform(np.log(1e3), np.log(1e6), 4096))
    parts = ragged_shard(work, 4)
    assert sorted(np.concatenate(parts).tolist()) == list(range(4096))
    loads = [work[p].sum() for p in parts]
    assert max(loads) / min(loads) < 1.01


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, x, gy, h, ret):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    start, count = row_shard(x.shape[0], rank, world)
    _, dh = oracle.resample_poly_bwd(gy[start:start + count], x[start:start + count], h, 3, 2)
    t = torch.from_numpy(dh.astype(np.float32))
    reduce_tap_grad(t)
    ret[rank] = t.numpy().copy()
    dist.barrier()
    dist.destroy_process_group()


def test_tap_grad_allreduce_world2():
    import oracle
    oracle.build()
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (6, 800))
    h = rng.standard_normal(31)
    gy = rng.standard_normal((6, 1200))
    _, full = oracle.resample_poly_bwd(gy, x, h, 3, 2)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    ret = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, x, gy, h, ret)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        assert np.allclose(ret[r], full, rtol=1e-5, atol=1e-6)
