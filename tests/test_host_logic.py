"""Host-side logic on the CPU: the reference-named module map, geometry
packing, and the multi-rank batch sharding over a gloo process group."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from fanbeamctrecon_tensorflowop_gb300 import utils
from fanbeamctrecon_tensorflowop_gb300.config import default_config
from fanbeamctrecon_tensorflowop_gb300.geometry import decode, fan_param16, param_set
from fanbeamctrecon_tensorflowop_gb300.sharding import max_over_ranks, shard_range


def test_load_op_library_names():
    assert utils.load_op_library("./FP/FP.so") is utils.FP_module
    assert utils.load_op_library("./BP/BP.so") is utils.BP_module
    assert utils.load_op_library("./FBP/FBP.so") is utils.FBP_module
    assert utils.load_op_library("./FBP_op.so") is utils.FDK_module
    assert callable(utils.FDK_module.BackProjection)
    with pytest.raises(ValueError):
        utils.load_op_library("./nope.so")


def test_param_set_follows_config_changes():
    c = default_config()
    c.DetectorShift = 2
    c.ProjectionsPerRotation = 100
    p = param_set(3, c)
    dcol = np.float32(c.FanAngle / c.DetectorColumnNumber)
    assert p[2] == 100 and p[9] == 2 and p[11] == 3
    assert p[10] == np.float32(-c.FanAngle / 2 - 2 * (c.FanAngle / c.DetectorColumnNumber))
    assert p[8] == dcol
    assert list(p[13:]) == [13, 14, 15]


def test_fan_param16_roundtrip():
    p = fan_param16(sdd=949.0, sid=541.0, n_views=984, n_cols=888, n=512, pixel_mm=0.7,
                    dcol_rad=1 / 949)
    g = decode(p)
    assert (g.n_views, g.n_cols, g.nx, g.ny) == (984, 888, 512, 512)
    assert abs(g.dx - 0.7) < 1e-6 and abs(g.dcol - 1 / 949) < 1e-9
    assert abs(g.left + 888 / 949 / 2) < 1e-6


@pytest.mark.parametrize("batch,world", [(32, 2), (7, 2), (1, 4), (0, 3), (10, 8)])
def test_shard_range_partitions(batch, world):
    spans = [shard_range(batch, r, world) for r in range(world)]
    covered = [i for a, b in spans for i in range(a, b)]
    assert covered == list(range(batch))
    sizes = [b - a for a, b in spans]
    assert max(sizes) - min(sizes) <= 1


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, batch, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    a, b = shard_range(batch, rank, world)
    owned = torch.zeros(batch, dtype=torch.int64)
    owned[a:b] = 1
    dist.all_reduce(owned)  # every slice owned exactly once
    t = max_over_ranks(float(rank + 1) * 0.5)
    q.put((rank, owned.tolist(), t))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_shard_and_reduce():
    world, batch = 2, 9
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, batch, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, owned, t in res:
        assert owned == [1] * batch
        assert t == 1.0  # max over ranks of (rank+1)/2


def _worker_op(rank, world, port, batch, q):
    """Each rank projects its own shard of a seeded batch (the FP64 oracle
    stands in for the operator: no GPU here) and the shards are gathered in
    rank order, as the replicas of a multi-GPU run split a batch."""
    import torch
    import torch.distributed as dist
    import oracle
    from fanbeamctrecon_tensorflowop_gb300.geometry import angle as _angle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle.build()
    p = fan_param16(sdd=949.0, sid=541.0, n_views=16, n_cols=40, n=24, pixel_mm=4.0,
                    dcol_rad=4.0 / 949.0)
    ang = _angle(16, 0.0)
    g = oracle.decode(p)
    imgs = np.random.default_rng(5).random((batch, 24, 24), dtype=np.float32)
    a, b = shard_range(batch, rank, world)
    mine = oracle.fp_fan(g, ang, imgs[a:b]) if b > a else np.zeros((0, 16, 40))
    # pad to the largest shard so every rank sends the same shape
    rows = shard_range(batch, 0, world)[1]
    buf = torch.zeros((rows, 16, 40), dtype=torch.float64)
    buf[: b - a] = torch.from_numpy(np.asarray(mine, np.float64))
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    if rank == 0:
        got = np.concatenate([parts[r][: shard_range(batch, r, world)[1]
                                        - shard_range(batch, r, world)[0]].numpy()
                              for r in range(world)])
        want = np.asarray(oracle.fp_fan(g, ang, imgs), np.float64)
        q.put((got.shape == want.shape, bool(np.array_equal(got, want))))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_run_their_shards():
    world, batch = 2, 5
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_op, args=(r, world, port, batch, q))
             for r in range(world)]
    for p in procs:
        p.start()
    same_shape, equal = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert same_shape and equal
