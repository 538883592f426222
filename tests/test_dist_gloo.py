"""Multi-rank shot sharding on CPU with gloo, world size 2.

Each rank stacks the (oracle-computed) images of its own shots; one
all-reduce must reproduce the single-rank stack of all shots, and the
misfit sum and the max-over-ranks timing reduce correctly."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from seismic_gb300 import dist as sdist


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, shots_img, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = sdist.shard(len(shots_img), rank, world)
        img = np.zeros_like(shots_img[0])
        f = np.zeros(1, np.float64)
        for i in mine:
            img += shots_img[i]
            f += float(i) + 0.5
        img_all, f_all = sdist.allreduce_sum([img, f])
        tmax = sdist.allreduce_max(float(rank + 1))
        q.put((rank, img_all, float(f_all[0]), tmax))
    finally:
        dist.destroy_process_group()


def test_shard_round_robin():
    assert sdist.shard(7, 0, 2) == [0, 2, 4, 6]
    assert sdist.shard(7, 1, 2) == [1, 3, 5]
    with pytest.raises(ValueError):
        sdist.shard(3, 2, 2)


def test_gloo_world2_stack_equals_serial():
    rng = np.random.default_rng(0)
    shots_img = [rng.standard_normal(64).astype(np.float32) for _ in range(5)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, shots_img, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    serial = np.zeros(64, np.float32)
    for i in (0, 2, 4):
        serial += shots_img[i]
    serial2 = np.zeros(64, np.float32)
    for i in (1, 3):
        serial2 += shots_img[i]
    for rank, img, f, tmax in res:
        np.testing.assert_allclose(img, serial + serial2, rtol=1e-6)
        assert f == sum(i + 0.5 for i in range(5))
        assert tmax == 2.0
