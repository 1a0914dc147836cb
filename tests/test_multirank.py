"""The path shards by frames / tiles with no collective on the data path:
two gloo ranks each render half of the samples of the small workload
(oracle, CPU) and the sum of their fixed-point images equals the
single-process image (integer accumulation is order-free)."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "tesina-rt_gb300"))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import pyoracle
    from rtgb import scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = scenes.workload_small()
    orc = pyoracle.Oracle()
    s = orc.new_scene(wl["scene"])
    s.build(30, 1, 0)
    n = 512 * 512
    per = n // world
    img, st = s.render(wl["camera"], 512, 512, 3, offset=rank * per, count=per, threads=2)
    t = torch.from_numpy(img.astype(np.int64))
    dist.all_reduce(t)
    rays = torch.tensor([st.primary_rays + st.secondary_rays], dtype=torch.int64)
    dist.all_reduce(rays)
    if rank == 0:
        np.save(out, t.numpy())
        np.save(out + ".rays.npy", rays.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_frame(tmp_path, orc):
    from rtgb import scenes
    out = str(tmp_path / "img.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    wl = scenes.workload_small()
    s = orc.new_scene(wl["scene"])
    s.build(30, 1, 0)
    img, st = s.render(wl["camera"], 512, 512, 3)
    assert np.array_equal(np.load(out), img.astype(np.int64))
    assert int(np.load(out + ".rays.npy")[0]) == st.primary_rays + st.secondary_rays
