"""Sample shards across ranks (CPU, gloo, world size 2): disjoint sample streams
per rank, one all-reduce of the accumulators, max-over-ranks timing. The
shard images come from the oracle, which renders what the GPU kernels render
for the same sample keys."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    import trayracer_gb300 as tr
    from oracle import Oracle
    from trayracer_gb300.shards import max_over_ranks, reduce_accumulators, shard_settings

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    scene = tr.cornell_box(width=16, height=12)
    st = shard_settings(tr.settings_for(scene, multi_sample=2), rank)
    acc, _, _ = Oracle(scene).render(scene.camera, st, scene.width, scene.height)
    np.save(os.path.join(out_dir, f"shard{rank}.npy"), acc)
    t = torch.from_numpy(acc.astype(np.float32))
    reduce_accumulators(t)
    slowest = max_over_ranks(10.0 * (rank + 1))
    if rank == 0:
        np.save(os.path.join(out_dir, "merged.npy"), t.numpy())
        np.save(os.path.join(out_dir, "slowest.npy"), np.array([slowest]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sample_shards(tmp_path):
    import torch.multiprocessing as mp

    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    a0 = np.load(tmp_path / "shard0.npy")
    a1 = np.load(tmp_path / "shard1.npy")
    merged = np.load(tmp_path / "merged.npy")
    # distinct seeds: the shards' samples differ
    assert not np.allclose(a0[:, :3], a1[:, :3])
    # one sum of float4 accumulators makes the image of all samples
    np.testing.assert_allclose(merged, (a0 + a1).astype(np.float32), rtol=1e-6, atol=1e-6)
    assert np.all(merged[:, 3] == 4.0)
    assert float(np.load(tmp_path / "slowest.npy")[0]) == 20.0
