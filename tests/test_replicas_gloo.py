"""Multi-GPU path (replicas) covered on CPU: two gloo ranks shard a batch of maps,
each transforms its shard (the oracle stands in for the device transform), and the
gathered result equals the single-process transform; the timing reduction is the max."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

from fastsht_gb300.replicas import max_over_ranks, shard


def test_shard_covers_every_map_once():
    for nmaps in (0, 1, 7, 500, 1001):
        for world in (1, 2, 3, 8):
            parts = [shard(nmaps, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == nmaps
            for (a, b), (c, d) in zip(parts, parts[1:]):
                assert b == c
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, maps, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import OracleSHT
    nside, lmax = 8, 23
    a, b = shard(maps.shape[1], rank, world)
    o = OracleSHT(nside, lmax, fft_workers=1)
    alm = o.t2alm(np.asfortranarray(maps[:, a:b]))             # (b - a, L, L)
    sizes = [shard(maps.shape[1], r, world) for r in range(world)]
    L = lmax + 1
    big = max(s1 - s0 for s0, s1 in sizes)            # gloo gathers equal shapes: pad
    mine = torch.zeros((big, L, L), dtype=torch.float64)
    mine[:b - a] = torch.from_numpy(np.ascontiguousarray(alm))
    buf = [torch.zeros((big, L, L), dtype=torch.float64) for _ in sizes]
    dist.all_gather(buf, mine)
    t = max_over_ranks(10.0 * (rank + 1), dist)
    if rank == 0:
        full = torch.cat([x[:s1 - s0] for x, (s0, s1) in zip(buf, sizes)])
        np.savez(out_path, alm=full.numpy(), tmax=t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process(tmp_path):
    rng = np.random.default_rng(0)
    nside, lmax = 8, 23
    maps = np.asfortranarray(rng.standard_normal((12 * nside * nside, 5)))
    out = tmp_path / "r.npz"
    mp.start_processes(_rank_main, args=(2, _free_port(), maps, str(out)), nprocs=2,
                       join=True, start_method="spawn")
    from oracle import OracleSHT
    ref = OracleSHT(nside, lmax, fft_workers=1).t2alm(maps)
    got = np.load(out)
    # BLAS blocking differs with the batch width: equal to rounding, not bit for bit
    assert np.abs(got["alm"] - ref).max() <= 1e-13 * np.abs(ref).max()
    assert got["tmax"] == 20.0
