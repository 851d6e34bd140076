"""Multi-rank path on CPU: world_size 2 over gloo (127.0.0.1)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pyatmosphere_gb300.engine.shard import gather_measures, max_over_ranks, realisation_range


def test_realisation_ranges_partition_the_job():
    for total in [0, 1, 7, 256, 1001]:
        for world in [1, 2, 3, 8]:
            rs = [realisation_range(r, world, total) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total = 11
        first, last = realisation_range(rank, world, total)
        # stand-in for the engine's per-realisation measures: a deterministic
        # function of the realisation index (what counter-keyed draws give)
        local = torch.tensor([[r, r * 0.5 + 1] for r in range(first, last)], dtype=torch.float64)
        allm = gather_measures(local)
        t = max_over_ranks(0.1 * (rank + 1))
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([allm.numpy().ravel(), [t]]))
    finally:
        dist.destroy_process_group()


def test_gather_over_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for rank in range(2):
        v = np.load(tmp_path / f"rank{rank}.npy")
        allm, t = v[:-1].reshape(-1, 2), v[-1]
        np.testing.assert_array_equal(allm[:, 0], np.arange(11))
        assert t == pytest.approx(0.2)
