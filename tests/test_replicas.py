"""Replica sharding over ranks (gloo, world size 2, CPU): every rank solves
its slice of the wavelengths and the host gather rebuilds exactly the
unsharded result.  The per-rank solve is the FP64 oracle here (no GPU)."""
import math
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from wavefiber3d_gb300 import replicas


def test_shard_range_partitions():
    for n in (0, 1, 5, 25):
        for w in (1, 2, 3, 8):
            got = [i for r in range(w) for i in replicas.shard_range(n, r, w)]
            assert got == list(range(n))
    with pytest.raises(ValueError):
        replicas.shard_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import torch.distributed as dist

    import oracle
    from wavefiber3d_gb300 import api, geometry
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cloud = geometry.fibonacci_sphere(0.5e-6, 300)
    lams = [400e-9 + 50e-9 * i for i in range(5)]
    il = api.Illumination.__new__(api.Illumination)
    il.__init__(lams, [0.2], [0.4], api.PO_POL_TM, 1.55 + 0.1j, 1e-2)
    mine, idx = replicas.shard_illumination(il, rank, world)
    local = np.stack([oracle.solve_direct(cloud, oracle.make_illum(l, 0.2, 0.4, "M", 1.55 + 0.1j), 8, 16)
                      for l in mine.wavelengths_m]) if len(idx) else np.zeros((0, 8, 16))
    full = replicas.gather_patterns(local, len(lams), rank, world)
    if rank == 0:
        np.save(out_path, full)
    dist.destroy_process_group()


def test_two_rank_gather_matches_single_process(tmp_path):
    import oracle
    from wavefiber3d_gb300 import geometry
    out = tmp_path / "full.npy"
    mp.start_processes(_worker, args=(2, _free_port(), str(out)), nprocs=2, join=True, start_method="spawn")
    full = np.load(out)
    cloud = geometry.fibonacci_sphere(0.5e-6, 300)
    want = np.stack([oracle.solve_direct(cloud, oracle.make_illum(400e-9 + 50e-9 * i, 0.2, 0.4, "M", 1.55 + 0.1j),
                                         8, 16) for i in range(5)])
    assert np.array_equal(full, want)
