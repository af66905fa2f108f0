"""Replicas on two ranks (gloo, CPU): each rank renders its shard of the
image's samples (its own RNG seeds, its share of the spp) — here with the
oracle, which computes what the GPU kernels compute bit for bit — and the
FP64 accumulations are merged with an all-reduce, as ``merge_from`` merges
lanes in the reference.  The merged image must equal the sum of the shards
computed in one process and hold exactly spp samples per pixel."""
import os
import socket

import numpy as np
import pytest

W, H, SPP, NPATHS = 24, 24, 6, 512


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard_render(rank: int, world: int):
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import replicas, scenes
    from oracle import pyoracle as po
    from tests.helpers import build, camera

    sm, osc = build(scenes.cornell_box())
    cam = camera(scenes.cornell_camera(), W, H)
    cfg = replicas.shard_config(rg.render_config(dof=0.0, max_depth=5, spp=SPP), rank, world, NPATHS)
    acc, _, _ = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, W * H), NPATHS, 200, threads=2,
                           want_slots=False)
    return acc, int(cfg.spp), int(cfg.seed_offset)


def _worker(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist
    from raccoongpurender_gb300 import replicas

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        acc, spp, seed = _shard_render(rank, world)
        np.save(os.path.join(out_dir, f"shard{rank}.npy"), acc)
        replicas.merge_sums(acc)
        np.save(os.path.join(out_dir, f"merged{rank}.npy"), acc)
        np.save(os.path.join(out_dir, f"meta{rank}.npy"), np.array([spp, seed]))
    finally:
        dist.destroy_process_group()


def test_two_replicas_merge(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    shards = [np.load(tmp_path / f"shard{r}.npy") for r in range(world)]
    merged = [np.load(tmp_path / f"merged{r}.npy") for r in range(world)]
    meta = [np.load(tmp_path / f"meta{r}.npy") for r in range(world)]
    assert [int(m[0]) for m in meta] == [3, 3]            # spp split
    assert int(meta[1][1]) - int(meta[0][1]) == NPATHS     # lane k seeded at k * path_count
    for m in merged:                                       # every rank holds the merged image
        np.testing.assert_array_equal(m, shards[0] + shards[1])
    assert (merged[0][:, 3] == SPP).all()                  # exactly spp samples per pixel
    # the shards are different samples of the same image
    assert not np.array_equal(shards[0], shards[1])
    m0 = shards[0][:, :3].sum() / shards[0][:, 3].sum()
    m1 = shards[1][:, :3].sum() / shards[1][:, 3].sum()
    assert abs(m0 / m1 - 1.0) < 0.2
