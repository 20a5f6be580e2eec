"""Trajectory sharding over ranks: each rank holds a slice of the ensemble and the only
collective is the final all-reduce of the density moments (gloo, 2 CPU processes)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, shards, out):
    import torch.distributed as dist

    import __graft_entry__
    gpe = __graft_entry__.load_package()
    from gpe_gb300 import twa
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mean, var = twa.allreduce_moments(shards[rank])
    out[rank] = (mean, var)
    dist.barrier()
    dist.destroy_process_group()


def test_allreduce_moments_two_ranks():
    rng = np.random.default_rng(0)
    full = (rng.standard_normal((16, 16, 40)) + 1j * rng.standard_normal((16, 16, 40))).astype(np.complex64)
    shards = [full[..., :17], full[..., 17:]]  # uneven split
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, shards, out), nprocs=2, join=True)
    n = np.abs(full.astype(np.complex128)) ** 2
    for r in range(2):
        mean, var = out[r]
        assert np.allclose(mean, n.mean(-1), rtol=1e-12)
        assert np.allclose(var, n.var(-1), rtol=1e-10)


def test_allreduce_moments_without_process_group():
    import __graft_entry__
    __graft_entry__.load_package()
    from gpe_gb300 import twa
    x = np.arange(24, dtype=np.complex128).reshape(2, 3, 4)
    mean, var = twa.allreduce_moments(x)
    n = np.abs(x) ** 2
    assert np.allclose(mean, n.mean(-1)) and np.allclose(var, n.var(-1))


def test_merged_moments_keep_a_small_spread_over_a_large_mean():
    """Densities ~1e6 with a spread of order 1: the one-pass s2/n - mean^2 loses about
    12 of its 16 digits there, the (count, mean, M2) merge keeps the variance to 1e-9."""
    import __graft_entry__
    __graft_entry__.load_package()
    from gpe_gb300 import twa
    rng = np.random.default_rng(5)
    dens = 1e6 + rng.standard_normal((8, 8, 300))
    fields = np.sqrt(dens).astype(np.complex128)
    parts = [twa.local_moments(fields[..., a:b]) for a, b in ((0, 17), (17, 160), (160, 300))]
    cnt, mean, m2 = twa.merge_moments(parts)
    n = np.abs(fields) ** 2
    assert cnt == 300
    assert np.allclose(mean, n.mean(-1), rtol=1e-14)
    assert np.allclose(m2 / cnt, n.var(-1), rtol=1e-9)
    one_pass = (n * n).mean(-1) - n.mean(-1) ** 2
    assert np.abs(one_pass / n.var(-1) - 1).max() > 1e-6  # the cancellation the merge avoids


def test_shard_range_covers_the_ensemble_once():
    import __graft_entry__
    __graft_entry__.load_package()
    from gpe_gb300 import twa
    for ntraj in (1, 7, 1024, 1025):
        for world in (1, 2, 3, 8):
            nxt = 0
            for r in range(world):
                first, count = twa.shard_range(ntraj, r, world)
                assert first == nxt and count >= 0
                nxt = first + count
            assert nxt == ntraj
            counts = [twa.shard_range(ntraj, r, world)[1] for r in range(world)]
            assert max(counts) - min(counts) <= 1
    with pytest.raises(ValueError):
        twa.shard_range(10, 2, 2)


def test_wigner_initial_slices_equal_the_full_draw():
    import __graft_entry__
    __graft_entry__.load_package()
    from gpe_gb300 import twa
    prm = twa.DampedDrivenParams()
    full = twa.wigner_initial(16, 0, 9, prm, seed=4)
    part = twa.wigner_initial(16, 3, 4, prm, seed=4)
    assert np.array_equal(full[:, :, 3:7], part)


def test_philox_restatement_offset_draws_the_slice():
    from oracle import gpe_oracle as O
    full = O.PhiloxNoise(11, 1, (6,), (8, 16))
    part = O.PhiloxNoise(11, 1, (2,), (8, 16), traj0=3)
    for h in (0, 5):
        assert np.array_equal(full(h)[:, 3:5], part(h))


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist

    import __graft_entry__
    __graft_entry__.load_package()
    from gpe_gb300 import twa
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    prm = twa.DampedDrivenParams()
    first, count = twa.shard_range(13, rank, world)
    fields = twa.wigner_initial(16, first, count, prm, seed=9)
    mean, var = twa.allreduce_moments(fields)
    out[rank] = (first, count, mean, var)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_plan_and_merged_moments_two_ranks():
    """The rank-aware plan (two gloo ranks): each rank builds its contiguous slice of a
    13-trajectory ensemble and the merged density moments equal the whole ensemble's."""
    import __graft_entry__
    __graft_entry__.load_package()
    from gpe_gb300 import twa
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_shard_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    full = twa.wigner_initial(16, 0, 13, twa.DampedDrivenParams(), seed=9)
    n = np.abs(full.astype(np.complex128)) ** 2
    assert [out[r][:2] for r in range(2)] == [(0, 7), (7, 6)]
    for r in range(2):
        assert np.allclose(out[r][2], n.mean(-1), rtol=1e-13)
        assert np.allclose(out[r][3], n.var(-1), rtol=1e-11)
    assert np.array_equal(out[0][3], out[1][3])  # every rank merges in rank order: the same bits
