"""Multi-GPU sharding host logic, run as two gloo ranks on the CPU.

Each rank renders its own sample range (or its own views) of the same frame
with the oracle standing in for a GPU; one all-reduce of the accumulators
must give the single-process render."""
import os
import socket
import sys

import numpy as np
import pytest

from cudart_gb300.sharding import sample_range, view_shard

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sample_ranges_partition_the_samples():
    for spp in (1, 7, 64, 255):
        for world in (1, 2, 3, 8):
            got = [sample_range(spp, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == spp
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        sample_range(8, 2, 2)


def test_view_shards_partition_and_balance():
    rng = np.random.default_rng(1)
    work = [int(x) for x in rng.integers(1, 1000, 64)]
    for world in (1, 2, 4, 8):
        shards = [view_shard(work, r, world) for r in range(world)]
        flat = sorted(k for s in shards for k in s)
        assert flat == list(range(64))
        loads = [sum(work[k] for k in s) for s in shards]
        assert max(loads) - min(loads) <= max(work)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import torch.distributed as dist
    import oracle
    from cudart_gb300 import scenes
    from cudart_gb300.sharding import reduce_accumulators, sample_range, view_shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = scenes.cornell_box(width=24, height=16)
    o = oracle.OracleScene(sc)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    spp = 10
    s0, s1 = sample_range(spp, rank, world)
    _, mean, _ = o.render(cam, seed=3, spp=s1 - s0, spp0=s0, max_depth=5, threads=1)
    acc = torch.from_numpy(mean * (s1 - s0))           # FP64 sums of this rank's samples
    reduce_accumulators(acc)
    # batched views: whole views per rank, gathered ids must cover every view once
    work = [w * h * s for w, h, s in ((8, 8, 4), (16, 8, 2), (4, 4, 16), (12, 6, 3), (8, 4, 1))]
    mine = view_shard(work, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), acc.numpy())
        np.save(os.path.join(out_dir, "views.npy"), np.array(sorted(k for g in gathered for k in g)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sample_sharding_equals_single_render(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from cudart_gb300 import scenes
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    sc = scenes.cornell_box(width=24, height=16)
    o = oracle.OracleScene(sc)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    _, mean, _ = o.render(cam, seed=3, spp=10, max_depth=5, threads=1)
    got = np.load(tmp_path / "sum.npy")
    assert np.allclose(got, mean * 10, rtol=1e-12, atol=1e-12)
    assert np.load(tmp_path / "views.npy").tolist() == [0, 1, 2, 3, 4]
