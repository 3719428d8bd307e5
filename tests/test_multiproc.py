"""Multi-rank host paths on CPU with the gloo backend (world_size 2): the scene
partition is computed identically on every rank without communication and
covers every scene exactly once; the bench's barrier / max-over-ranks timing
works over gloo."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, counts, out_dir):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gaia_gb300.sharding import partition_scenes

    import bench

    parts = partition_scenes(counts, world)
    mine = torch.tensor(parts[rank] + [-1] * (len(counts) - len(parts[rank])), dtype=torch.int64)
    gathered = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine)
    bench.barrier(world)
    t = bench.allmax(world, float(rank + 1) * 1.5)
    np.save(os.path.join(out_dir, f"r{rank}.npy"),
            np.concatenate([torch.stack(gathered).numpy().ravel(), [t]]))
    dist.destroy_process_group()


def test_partition_over_gloo(tmp_path):
    import torch.multiprocessing as mp

    rng = np.random.Generator(np.random.PCG64(2))
    counts = [int(c) ** 3 for c in rng.integers(4, 25, size=37)]
    port = _free_port()
    mp.spawn(_worker, args=(2, port, counts, str(tmp_path)), nprocs=2, join=True)
    a = np.load(tmp_path / "r0.npy")
    b = np.load(tmp_path / "r1.npy")
    assert np.array_equal(a, b)  # every rank saw the same partition and the same max
    assert a[-1] == 3.0
    ids = a[:-1].astype(np.int64)
    ids = ids[ids >= 0]
    assert sorted(ids.tolist()) == list(range(len(counts)))


def test_partition_balance():
    from gaia_gb300.sharding import partition_scenes

    rng = np.random.Generator(np.random.PCG64(4))
    counts = [int(c) ** 3 for c in rng.integers(4, 25, size=512)]
    for world in (1, 2, 4, 8):
        parts = partition_scenes(counts, world)
        loads = [sum(counts[i] for i in p) for p in parts]
        assert sorted(i for p in parts for i in p) == list(range(512))
        assert max(loads) - min(loads) <= max(counts)


def test_write_shard(tmp_path, gaia_lib):
    from gaia_gb300 import VBDPhysics, scenes
    from gaia_gb300.sharding import write_shard

    mp, pp = scenes.batch_cubes(str(tmp_path / "all"), n_scenes=6, side_range=(3, 5), iterations=3)
    smp, spp = write_shard(mp, pp, [1, 4], str(tmp_path / "shard"))
    p = VBDPhysics()
    p.loadRunningparameters(smp, spp)
    assert p.numMeshes() == 2
    p.close()
