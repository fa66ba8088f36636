"""Two ranks (gloo, on the CPU) render disjoint sample ranges of one frame and combine them with
one all-reduce; the result equals a single-process render of all samples. The oracle stands in
for the GPU renderer here (same per-path streams); the sharding and the exchange are the
product's (x3dcore2_gb300.shard)."""
import os

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from x3dcore2_gb300 import shard


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests")]
    import torch.distributed as dist

    import golden_util as G
    import oracle_bind as ob
    from x3dcore2_gb300 import abi
    from x3dcore2_gb300 import shard as sh
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = G.load("cornell.npz")
    osc = ob.OracleScene(G.scene_from(d))
    first, count = sh.sample_range(7, rank, world)
    img = osc.render(abi.MODE_REF_LT1, 64, 48, count, seed=5, offset=first, threads=1)
    t = torch.from_numpy(img.copy())
    sh.combine(t, count, 7)
    if rank == 0:
        np.save(out, t.numpy())
    dist.destroy_process_group()


def test_sample_range_covers_all_samples():
    for spp in (1, 7, 64):
        for world in (1, 2, 3, 8):
            got = [shard.sample_range(spp, r, world) for r in range(world)]
            assert sum(c for _, c in got) == spp
            assert [f for f, _ in got] == [sum(c for _, c in got[:r]) for r in range(world)]
    with pytest.raises(ValueError):
        shard.sample_range(4, 2, 2)


def test_two_ranks_equal_one(tmp_path, oracle):
    import golden_util as G
    import oracle_bind as ob
    from x3dcore2_gb300 import abi
    out = str(tmp_path / "img.npy")
    port = 29500 + os.getpid() % 1000
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    combined = np.load(out)
    d = G.load("cornell.npz")
    single = ob.OracleScene(G.scene_from(d)).render(abi.MODE_REF_LT1, 64, 48, 7, seed=5, threads=1)
    assert np.allclose(combined, single, rtol=1e-5, atol=1e-6)
