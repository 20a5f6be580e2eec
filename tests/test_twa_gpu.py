"""Truncated-Wigner ensembles: groups on grids of different sizes advanced by one CUDA
graph (gpe_ensemble_run), checked against plain stepping, against the FP64 oracle per
trajectory (replayed noise) and statistically (independent noise)."""
import math

import numpy as np
import pytest

from cases import c_order, jl

pytestmark = pytest.mark.gpu


def twa(gpe):
    return __import__("gpe_gb300.twa", fromlist=["Ensemble"])


def test_ensemble_graph_equals_plain_stepping(gpe, lib):
    """Graph replay (device step counter) reproduces un-captured stepping bit for bit,
    for resident (32^2, 64^2, 128^2 FP32) and two-pass (256^2) groups in one graph."""
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    sizes = [(32, 6), (64, 4), (128, 2), (256, 2)]
    nsteps = 40
    graph_its = [T.make_group(N, B, prm, nsteps, seed=N) for N, B in sizes]
    ens = T.Ensemble(graph_its)
    ens.run(nsteps, 10)
    assert ens.last_run_launches() > 0
    ens.close()
    for (N, B), git in zip(sizes, graph_its):
        it = T.make_group(N, B, prm, nsteps, seed=N)
        it.step(nsteps)
        a, b = git.get_fields()[0], it.get_fields()[0]
        assert np.array_equal(a, b), f"N={N}"
        assert git.state().steps == nsteps
        it.close()
        git.close()


def test_resident_and_two_pass_groups_agree(gpe, oracle, lib):
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    for N in (64, 128):
        a = T.make_group(N, 3, prm, 60, seed=5, resident=True)
        b = T.make_group(N, 3, prm, 60, seed=5, resident=False)
        a.step(60)
        b.step(60)
        fa, fb = a.get_fields()[0].astype(np.complex128), b.get_fields()[0].astype(np.complex128)
        assert oracle.rel_l2(fa, fb) <= 2e-5, N
        a.close()
        b.close()


def test_twa_group_per_trajectory_replay_parity(gpe, oracle, lib):
    """FP32 group with replayed noise against the FP64 oracle on the same u0 and xi."""
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    N, B, nsteps = 32, 4, 50
    prob = T.wigner_problem(N, B, prm, seed=3, dtype=np.complex64)
    rn = oracle.ReplayNoise(17, (1, B, N, N))
    xi32 = lambda h: rn(h).astype(np.complex64).astype(np.complex128)
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, nsteps * prm.dt), dt=prm.dt, nsaves=5,
                        noise_replay=lambda h: np.ascontiguousarray(xi32(h)))
    dV = (prm.L / N) ** 2
    u0c = c_order(prob.u0[0]).astype(np.complex128)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(prm.L, prm.L),
                               dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.5j * prm.gamma,
                               nonlin_g=np.array([[prm.g]]), pump_profile=np.ones((1, N, N), np.complex128),
                               pump_amp=lambda t: np.array([prm.F]), eta=np.array([math.sqrt(prm.gamma / (2 * dV))]))
    ots, ores = oracle.solve(orc, (0.0, nsteps * prm.dt), prm.dt, 5, xi_source=xi32)
    got = c_order(res[0]).astype(np.complex128)
    for b in range(B):
        e = oracle.rel_l2(got[:, b], ores[0][:, b])
        assert e <= 1e-5, (b, e)


def test_twa_density_statistics_match_fp64_ensemble(gpe, oracle, lib):
    """Philox ensemble (GPU, FP32) vs an independent FP64 oracle ensemble (numpy noise):
    the mean density and its variance agree within their standard errors."""
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    N, B, nsteps = 32, 512, 100
    it = T.make_group(N, B, prm, nsteps, seed=11)
    it.step(nsteps)
    n_gpu = np.abs(it.get_fields()[0].astype(np.complex128)) ** 2  # (N, N, B)
    it.close()
    dV = (prm.L / N) ** 2
    rng = np.random.default_rng(99)
    xi0 = (rng.standard_normal((B, N, N)) + 1j * rng.standard_normal((B, N, N))) * math.sqrt(0.5)
    u0c = 1.0 + xi0 / math.sqrt(2 * dV)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(prm.L, prm.L),
                               dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.5j * prm.gamma,
                               nonlin_g=np.array([[prm.g]]), pump_profile=np.ones((1, N, N), np.complex128),
                               pump_amp=lambda t: np.array([prm.F]), eta=np.array([math.sqrt(prm.gamma / (2 * dV))]))
    nrng = np.random.default_rng(7)
    ts, ores = oracle.solve(orc, (0.0, nsteps * prm.dt), prm.dt, 1, save_start=False,
                            xi_source=lambda h: oracle.complex_normal(nrng, (1, B, N, N)))
    n_cpu = np.abs(ores[0, -1]) ** 2  # (B, N, N)
    # trajectory-level means (spatial average per trajectory) are independent samples
    mg, mc = n_gpu.mean(axis=(0, 1)), n_cpu.mean(axis=(1, 2))
    se = math.sqrt(mg.var() / B + mc.var() / B)
    assert abs(mg.mean() - mc.mean()) <= 5 * se + 1e-12
    vg, vc = n_gpu.var(axis=-1).mean(), n_cpu.var(axis=0).mean()
    assert abs(vg - vc) <= 0.1 * vc


def test_momentum_statistics_match_numpy(gpe, lib):
    """n(k), G2(k,k'), g2 of a 1D noisy ensemble computed on the GPU agree with the same
    formulas evaluated in numpy on the fields (examples/truncated_wigner.jl:110-165)."""
    T = twa(gpe)
    N, B, L = 64, 256, 64.0
    dx = L / N
    rng = np.random.default_rng(2)
    u0 = (rng.standard_normal((N, B)) + 1j * rng.standard_normal((N, B))) / math.sqrt(2 * dx)
    hb = 0.6582
    gam = 0.047 / hb
    prob = gpe.GrossPitaevskiiProblem((np.asfortranarray(u0),), (L,),
                                      dispersion=lambda k, p: hb * k[0] ** 2 / (2 / 6) - 0.49 / hb - 0.5j * gam,
                                      nonlinearity=lambda u, p: 3e-4 / hb * (np.abs(u[0]) ** 2 - 1 / dx),
                                      pump=lambda r, p, t: 10.0 + 0 * r[0],
                                      position_noise_func=lambda u, r, p: math.sqrt(gam / (2 * dx)))
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 10.0), dt=0.05, nsaves=1, rng=5)
    it.step(200)
    nk, G2, g2 = T.momentum_statistics(it, 1 / L)
    sol = it.get_fields()[0]
    it.close()
    ft = np.fft.fftshift(np.fft.fft(sol, axis=0), axes=0) / N
    n_ref = (np.abs(ft) ** 2).mean(axis=1) - 1 / (2 * L)
    a = np.abs(ft) ** 2
    c = 1 / L
    G2_ref = (a @ a.T) / B - (1 + np.eye(N)) * c / 2 * (a.mean(1)[:, None] + a.mean(1)[None, :] - c / 2)
    assert np.allclose(nk, n_ref, rtol=1e-10, atol=1e-14)
    assert np.allclose(G2, G2_ref, rtol=1e-9, atol=1e-13 * np.abs(G2_ref).max())
    assert np.allclose(g2, G2_ref / np.outer(n_ref, n_ref), rtol=1e-8)


def test_alternative_tiling_matches_oracle(gpe, oracle, lib):
    """The second line tiling of FP32 one-component fields (gpe_set_variant 1) against the
    FP64 oracle on replayed noise (two-pass path, so both passes run the tiling)."""
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    N, B, nsteps = 64, 3, 30
    prob = T.wigner_problem(N, B, prm, seed=4, dtype=np.complex64)
    rn = oracle.ReplayNoise(23, (1, B, N, N))
    xi32 = lambda h: rn(h).astype(np.complex64).astype(np.complex128)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, nsteps * prm.dt), dt=prm.dt, nsaves=1,
                  noise_replay=lambda h: np.ascontiguousarray(xi32(h)), resident=False, variant=1)
    ts, res = it.solve()
    it.close()
    dV = (prm.L / N) ** 2
    u0c = c_order(prob.u0[0]).astype(np.complex128)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(prm.L, prm.L),
                               dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.5j * prm.gamma,
                               nonlin_g=np.array([[prm.g]]), pump_profile=np.ones((1, N, N), np.complex128),
                               pump_amp=lambda t: np.array([prm.F]), eta=np.array([math.sqrt(prm.gamma / (2 * dV))]))
    ots, ores = oracle.solve(orc, (0.0, nsteps * prm.dt), prm.dt, 1, xi_source=xi32)
    got = c_order(res[0]).astype(np.complex128)
    assert oracle.rel_l2(got, ores[0]) <= 1e-5


def test_variant_needs_fp32_one_component(gpe, lib):
    """The alternative tiling exists for FP32 one-component fields only; other handles
    refuse it with GPE_ERR_UNSUPPORTED and keep working.  The fine tiling (2) and the
    choice by size (-1) exist everywhere; other values are invalid."""
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    it = T.make_group(32, 2, prm, 10, seed=1, dtype=np.complex128)
    assert lib.gpe_set_variant(it.h, 1) == -2
    assert lib.gpe_set_variant(it.h, 3) == -1
    assert lib.gpe_set_variant(it.h, -2) == -1
    assert lib.gpe_set_variant(it.h, 2) == 0
    assert lib.gpe_set_variant(it.h, -1) == 0
    assert lib.gpe_set_variant(it.h, 0) == 0
    it.step(2)
    it.close()


@pytest.mark.parametrize("dtype,resident", [(np.complex64, True), (np.complex64, False), (np.complex128, False)],
                         ids=["f32-resident", "f32-two-pass", "f64-two-pass"])
def test_noise_offset_reproduces_the_slice(gpe, lib, dtype, resident):
    """A handle holding trajectories 3..5 of an ensemble (gpe_set_noise_offset, initial
    states drawn by global trajectory index) equals trajectories 3..5 of the whole 7-
    trajectory handle bit for bit: sharded ensembles reproduce the single-GPU run."""
    T = twa(gpe)
    prm = T.DampedDrivenParams()
    N, nsteps = 64, 30
    full = T.make_group(N, 7, prm, nsteps, seed=21, dtype=dtype, resident=resident)
    part = T.make_group(N, 3, prm, nsteps, seed=21, dtype=dtype, resident=resident, traj0=3)
    full.step(nsteps)
    part.step(nsteps)
    a, b = full.get_fields()[0], part.get_fields()[0]
    assert np.array_equal(a[:, :, 3:6], b)
    assert not np.array_equal(a[:, :, 0:3], b)
    full.close()
    part.close()


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128], ids=["f32", "f64"])
def test_philox_draws_have_gaussian_moments(gpe, lib, dtype):
    """Over 2^21 draws of the in-kernel generator (FP32 Box-Muller on the hardware log and
    sin/cos approximations, FP64 on the accurate routines): a noise-only 1D field from
    u = 0 after one step (dt = 2, eta = 1) is s = -i (xi_a + xi_b) for the two half steps'
    draws, complex normal with <|s|^2> = 2, <s^2> = 0, <|s|^4> = 8 if <|xi|^2> = 1,
    <xi^2> = 0 and <|xi|^4> = 2.  Bounds: 5 standard errors."""
    N, B = 1024, 1024
    prob = gpe.GrossPitaevskiiProblem((np.zeros((N, B), dtype),), (float(N),),
                                      position_noise_func=lambda u, r, p: 1.0)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 2.0), dt=2.0, nsaves=1, rng=20251204)
    it.step(1)
    s = it.get_fields()[0].astype(np.complex128).ravel()
    it.close()
    n = s.size
    m2 = np.mean(np.abs(s) ** 2)
    c2 = np.mean(s * s)
    m4 = np.mean(np.abs(s) ** 4)
    assert abs(m2 - 2.0) <= 5 * 2.0 / math.sqrt(n), m2            # var |s|^2 = 4
    assert abs(c2) <= 5 * math.sqrt(8.0 / n), c2                   # <|s^2|^2> = 8
    assert abs(m4 - 8.0) <= 5 * math.sqrt(384.0 - 64.0) / math.sqrt(n), m4  # <|s|^8> = 384
    # no correlation between neighbouring points or trajectories
    g = s.reshape(B, N)
    assert abs(np.mean(g[:, 1:] * np.conj(g[:, :-1]))) <= 5 * 2.0 / math.sqrt(n)
    assert abs(np.mean(g[1:] * np.conj(g[:-1]))) <= 5 * 2.0 / math.sqrt(n)
