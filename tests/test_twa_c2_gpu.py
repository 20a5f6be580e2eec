"""The batched truncated-Wigner configuration's statistics against the FP64 CPU ensemble:
the 64^2 group of the 1024-trajectory ensemble (342 trajectories, FP32 fields, Philox
noise, dt = 0.02) over the full 2000 steps, and the same trajectories advanced in FP64 by
the C oracle with the same initial states and Philox draws.  The per-site mean and
variance of |u|^2 over the trajectories agree to 1e-5 (FP32 arithmetic against FP64 on
identical dW), every trajectory to 1e-4."""
import pytest

pytestmark = pytest.mark.gpu


def test_c2_group_moments_match_fp64_cpu_ensemble(gpe, lib):
    import bench
    r = bench.twa_c2_statistics(gpe, steps=2000)
    print(r)
    assert r["rel_l2_mean_density_field"] <= 1e-5, r
    assert r["rel_l2_variance_field"] <= 1e-5, r
    assert r["max_rel_l2_per_trajectory"] <= 1e-4, r
