"""Replica sharding host logic with world_size 2 over gloo (CPU): disjoint sample
ranges that cover the render, max-over-ranks timing, and the final accumulator sum,
which with the oracle as the per-rank renderer equals a single-process render."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from illume_gb300.sharding import shard_samples


def test_shard_ranges_cover_exactly_once():
    for spp in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                b, n = shard_samples(spp, r, world)
                seen += list(range(b, b + n))
            assert seen == list(range(spp))
    with pytest.raises(ValueError):
        shard_samples(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from illume_gb300 import synth
    from illume_gb300.sharding import max_over_ranks, reduce_sums, shard_samples
    from oracle import pyoracle
    sd = synth.cornell_scene(8, 8)
    b, n = shard_samples(6, rank, world)
    s, s2, rays = pyoracle.OracleScene(sd).render(8, 8, n, 5, sample_begin=b, precision=64, nthreads=1)
    tot, tot2 = reduce_sums(s, s2)
    t = max_over_ranks(float(rank + 1))
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), tot)
        np.save(os.path.join(out_dir, "tmax.npy"), np.array([t]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_render_equals_single_render(tmp_path):
    from illume_gb300 import synth
    from oracle import pyoracle
    pyoracle.build()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    tot = np.load(tmp_path / "sum.npy")
    assert float(np.load(tmp_path / "tmax.npy")[0]) == 2.0
    sd = synth.cornell_scene(8, 8)
    s, _, _ = pyoracle.OracleScene(sd).render(8, 8, 6, 5, precision=64, nthreads=1)
    np.testing.assert_allclose(tot, s, rtol=1e-12, atol=1e-12)
