"""Multi-rank host logic on CPU (gloo, world size 2): profile sharding with no
data-path collective reproduces the single-process result, and the timing
reduction takes the maximum over ranks."""
import os
import socket

import numpy as np
import pytest

from crtmv3_gb300.replicas import max_over_ranks, shard_profiles


def test_shards_cover_the_batch():
    for n in (0, 1, 5, 2000, 2001):
        for w in (1, 2, 3, 8):
            r = [shard_profiles(n, k, w) for k in range(w)]
            assert r[0][0] == 0 and r[-1][1] == n
            assert all(r[k][1] == r[k + 1][0] for k in range(w - 1))
            sizes = [b - a for a, b in r]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_profiles(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, coeff_dir, out_dir):
    import torch.distributed as dist
    from crtmv3_gb300 import synthetic as sy
    from oracle.pyoracle import Oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    atm, sfc, geo, opt = sy.clear_sky_workload("mwsynth_c22", 7, 100, 5)
    a, b = shard_profiles(7, rank, world)
    idx = slice(a, b)
    _, bt = Oracle(coeff_dir, "mwsynth_c22").forward(atm.subset(idx), sfc.subset(idx),
                                                     geo.subset(idx), opt.subset(idx))
    np.save(os.path.join(out_dir, f"bt{rank}.npy"), bt)
    m = max_over_ranks(10.0 * (rank + 1), dist)
    np.save(os.path.join(out_dir, f"max{rank}.npy"), np.array([m]))
    dist.destroy_process_group()


def test_two_rank_gloo_sharding(coeff_dir, tmp_path):
    import torch.multiprocessing as mp
    from crtmv3_gb300 import synthetic as sy
    from oracle.pyoracle import Oracle
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), coeff_dir, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    bt = np.concatenate([np.load(tmp_path / f"bt{r}.npy") for r in range(world)])
    atm, sfc, geo, opt = sy.clear_sky_workload("mwsynth_c22", 7, 100, 5)
    _, ref = Oracle(coeff_dir, "mwsynth_c22").forward(atm, sfc, geo, opt)
    assert np.array_equal(bt, ref)
    assert all(float(np.load(tmp_path / f"max{r}.npy")[0]) == 20.0 for r in range(world))
