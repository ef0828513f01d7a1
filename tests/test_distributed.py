"""Sample sharding with world-size-2 gloo ranks on the CPU (the GPU tests have one GPU).

The renderer inside each rank is the oracle in Philox replay mode, which traces the very
paths the GPU traces; the test checks the host logic: shard ranges, the film all-reduce
and the normalisation, against a single-process render of the same samples.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from nanogi_gb300.distributed import shard_range

W, H = 10, 8


@pytest.mark.parametrize("n,world", [(W * H * 7, 2), (W * H * 7 + 13, 2), (W * H * 2, 3), (5, 2), (0, 2),
                                     (W * H * 100 + 1, 4)])
def test_shards_partition_the_samples(n, world):
    ranges = [shard_range(n, W, H, world, r) for r in range(world)]
    pos = 0
    for off, cnt in ranges:
        assert off == pos and cnt >= 0
        pos += cnt
    assert pos == n
    for off, cnt in ranges[:-1]:
        assert off % (W * H) == 0 and cnt % (W * H) == 0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, out_path):
    import sys

    import torch
    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from nanogi_gb300 import scenegen
    from nanogi_gb300.distributed import render_sharded
    from oracle.oracle import OracleScene

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ora = OracleScene.from_desc(scenegen.cornell_box(), W / H)

    def raw(offset, count):
        if count == 0:
            return torch.zeros((H, W, 3), dtype=torch.float64)
        f = ora.render("ptdirect", num_samples=count, max_vertices=6, width=W, height=H, seed=5, sample_offset=offset,
                       rng_mode="replay", use_bvh=False, threads=1)
        return torch.from_numpy(f * (count / (W * H)))  # back to raw sums

    film = render_sharded(raw, n, W, H, rank, world)
    if rank == 0:
        np.save(out_path, film.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("n", [W * H * 6, W * H * 6 + 37])
def test_gloo_two_ranks_equal_single_process(tmp_path, n):
    import torch.multiprocessing as mp

    from nanogi_gb300 import scenegen
    from oracle.oracle import OracleScene

    out = str(tmp_path / "film.npy")
    mp.spawn(_worker, args=(2, _free_port(), n, out), nprocs=2, join=True)
    sharded = np.load(out)
    single = OracleScene.from_desc(scenegen.cornell_box(), W / H).render(
        "ptdirect", num_samples=n, max_vertices=6, width=W, height=H, seed=5, rng_mode="replay", use_bvh=False,
        threads=1)
    assert np.allclose(sharded, single, rtol=1e-12, atol=1e-15)


def _failing_worker(rank, world, port):
    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    if rank == 1:
        raise RuntimeError("rank 1 fails between steps")
    film = torch.zeros(4, dtype=torch.float64)
    dist.all_reduce(film)


def test_rank_failure_surfaces_on_the_host():
    """A rank that dies between steps ends the job with an error, not a hang."""
    import torch.multiprocessing as mp

    with pytest.raises(Exception):
        mp.spawn(_failing_worker, args=(2, _free_port()), nprocs=2, join=True)
