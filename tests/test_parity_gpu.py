"""GPU parity: the package (libgpe through its C ABI) against the FP64 oracle on the
same inputs.

Tolerances (relative L2 over the saved trajectory and at every save):
* FP64 fields: 1e-10.
* FP32 fields: 1e-5, or 1.5x the error of the reference's own ComplexF32 arithmetic
  (oracle.solve_fp32: single-precision FFTs, FP64 tables) when that arithmetic cannot
  reach 1e-5 on the problem (self-focusing or long pumped runs).  The FP32 path is
  held to the reference's FP32 accuracy, never looser than 1e-5 where it reaches it.
"""
import numpy as np
import pytest

from cases import c_order, jl, kerr2d, polariton2d

pytestmark = pytest.mark.gpu

TOL = {np.complex128: 1e-10, np.complex64: 1e-5}
# FP64 fields run in native FP64 by default ("native"), with block floating point line
# transforms ("bfp") or in double-word arithmetic ("dw")
FP64_MODES = ["dw", "native", "bfp"]
PRECISIONS = [(np.complex128, "dw"), (np.complex128, "native"), (np.complex128, "bfp"), (np.complex64, "dw")]
PREC_IDS = ["c128-dw", "c128-native", "c128-bfp", "c64"]


def run_both(gpe, oracle, gpu_kw, orc, tspan, dt, nsaves, save_start=True, xi=None, rng=None, fp64="dw",
             resident=True):
    prob = gpe.GrossPitaevskiiProblem(**gpu_kw)
    kw = {"resident": resident}
    if xi is not None:
        kw["noise_replay"] = lambda h: np.ascontiguousarray(xi(h))
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), tspan, dt=dt, nsaves=nsaves, save_start=save_start, rng=rng,
                        fp64=fp64, **kw)
    ots, ores = oracle.solve(orc, tspan, dt, nsaves, save_start=save_start, xi_source=xi)
    return ts, res, ots, ores


def fp32_tol(oracle, orc, tspan, dt, nsaves, save_start=True, xi=None):
    """max(1e-5, 1.5 x the rel L2 error of the reference's FP32 arithmetic)."""
    ts, r32 = oracle.solve_fp32(orc, tspan, dt, nsaves, save_start=save_start, xi_source=xi)
    ts, r64 = oracle.solve(orc, tspan, dt, nsaves, save_start=save_start, xi_source=xi)
    err = max(oracle.rel_l2(r32[m].astype(np.complex128), r64[m]) for m in range(r64.shape[0]))
    return max(1e-5, 1.5 * err)


def assert_close(oracle, res, ores, tol, per_save=True):
    M = len(res)
    for m in range(M):
        got = c_order(res[m]).astype(np.complex128)
        ref = ores[m]
        assert got.shape == ref.shape, (got.shape, ref.shape)
        err = oracle.rel_l2(got, ref)
        assert err <= tol, f"component {m}: rel L2 {err:.3e} > {tol:g}"
        if per_save:
            for s in range(got.shape[0]):
                if np.linalg.norm(ref[s]) > 0:
                    e = oracle.rel_l2(got[s], ref[s])
                    assert e <= tol, f"component {m} save {s}: rel L2 {e:.3e} > {tol:g}"


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_kerr_plain_case(gpe, oracle, lib, dtype, fp64):
    """2D Kerr 128^2, L=8, g=-6, dt=0.01 on [0, 0.4] with 64 saves: dt resolves to
    0.00625 and 64 steps (src/fixed_time_stepping.jl:14-24)."""
    gpu_kw, orc = kerr2d(128, 8.0, -6.0, dtype)
    ts, res, ots, ores = run_both(gpe, oracle, gpu_kw, orc, (0.0, 0.4), 0.01, 64, fp64=fp64)
    assert np.array_equal(ts, ots)
    assert len(ts) == 65 and res[0].shape == (128, 128, 65)
    if dtype == np.complex128:
        assert_close(oracle, res, ores, TOL[dtype])
    else:
        # g = -6 self-focusing amplifies rounding: the reference's FP32 arithmetic
        # reaches ~1.3e-5 here
        tol = fp32_tol(oracle, orc, (0.0, 0.4), 0.01, 64)
        assert_close(oracle, res, ores, tol, per_save=False)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_polariton_matrix_dispersion_pump_ramp(gpe, oracle, lib, dtype, fp64):
    """Two components, 2x2 matrix dispersion table, diagonal nonlinearity, pump with a
    linear ramp sampled at the reference's shifted pump times."""
    gpu_kw, orc = polariton2d(N=128, L=256.0, A=5.0, ramp=20.0)
    gpu_kw["u0"] = tuple(u.astype(dtype) for u in gpu_kw["u0"])
    ts, res, ots, ores = run_both(gpe, oracle, gpu_kw, orc, (0.0, 10.0), 0.05, 10, fp64=fp64)
    assert np.array_equal(ts, ots)
    if dtype == np.complex128:
        assert_close(oracle, res, ores, TOL[dtype])
    else:
        # the reference's FP32 arithmetic reaches ~2.5e-5 on the photon field here
        assert_close(oracle, res, ores, fp32_tol(oracle, orc, (0.0, 10.0), 0.05, 10), per_save=False)


@pytest.mark.parametrize("resident", [True, False], ids=["resident", "two-pass"])
@pytest.mark.parametrize("fp64", FP64_MODES)
@pytest.mark.parametrize("N", [16, 32, 64, 256, 512, 1024])
def test_kerr_sizes(gpe, oracle, lib, N, fp64, resident):
    """Square grids up to 64^2 run in the resident plane kernel unless resident=False."""
    if resident is False and N > 64:
        pytest.skip("larger grids always take the two-pass path")
    gpu_kw, orc = kerr2d(N, 8.0, -2.0, np.complex128)
    ts, res, ots, ores = run_both(gpe, oracle, gpu_kw, orc, (0.0, 0.05), 0.005, 2, fp64=fp64, resident=resident)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("fp64", FP64_MODES)
def test_rectangular_and_batch(gpe, oracle, lib, fp64):
    L = (8.0, 4.0)
    X, Y = oracle.mesh(oracle.grids(L, (64, 32))[0])  # C order (32, 64)
    rng = np.random.default_rng(0)
    u0c = np.stack([np.exp(-(X - 4) ** 2 - (Y - 2) ** 2) * (1 + 0.2 * j) for j in range(3)]).astype(np.complex128)
    u0c = u0c + 0.01 * (rng.standard_normal(u0c.shape) + 1j * rng.standard_normal(u0c.shape))
    disp = lambda k, p: (k[0] ** 2 + 2 * k[1] ** 2) / 2 - 0.05j
    gkw = dict(u0=(jl(u0c),), lengths=L, dispersion=disp, nonlinearity=lambda u, p: (1.5 - 0.1j) * np.abs(u[0]) ** 2 + 0.3)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=L, dispersion=disp, nonlin_g=np.array([[1.5 - 0.1j]]),
                               nonlin_c=np.array([0.3]))
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, (0.0, 0.3), 0.01, 3, fp64=fp64)
    assert res[0].shape == (64, 32, 3, 4)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("fp64", FP64_MODES)
@pytest.mark.parametrize("kind", ["scalar", "diag"])
def test_potential_tables(gpe, oracle, lib, kind, fp64):
    N, L = 64, 10.0
    (X, Y), _ = (oracle.mesh(oracle.grids((L, L), (N, N))[0]), None)
    u0c = (np.exp(-((X - 5) ** 2 + (Y - 5) ** 2) / 2) + 0j)
    u1c = 0.5 * u0c * np.exp(1j * X)
    if kind == "scalar":
        pot = lambda r, p: 0.5 * ((r[0] - 5) ** 2 + (r[1] - 5) ** 2)
    else:
        pot = lambda r, p: [0.5 * ((r[0] - 5) ** 2 + (r[1] - 5) ** 2), 0.2 * (r[0] - 5) - 0.01j]
    disp = lambda k, p: [(k[0] ** 2 + k[1] ** 2) / 2, (k[0] ** 2 + k[1] ** 2) / 4]
    g = np.array([[1.0, 0.5], [0.5, 2.0]])
    gkw = dict(u0=(jl(u0c), jl(u1c)), lengths=(L, L), dispersion=disp, potential=pot,
               nonlinearity=lambda u, p: [np.abs(u[0]) ** 2 + 0.5 * np.abs(u[1]) ** 2,
                                          0.5 * np.abs(u[0]) ** 2 + 2 * np.abs(u[1]) ** 2])
    odisp = lambda k, p: np.stack([(k[0] ** 2 + k[1] ** 2) / 2, (k[0] ** 2 + k[1] ** 2) / 4])
    opot = pot if kind == "scalar" else (lambda r, p: np.stack([np.asarray(v) * np.ones_like(r[0]) for v in pot(r, p)]))
    orc = oracle.OracleProblem(u0=(u0c, u1c), lengths=(L, L), dispersion=odisp, potential=opot, nonlin_g=g)
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, (0.0, 0.2), 0.01, 4, fp64=fp64)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_noise_replay_2d(gpe, oracle, lib, dtype, fp64):
    """Replay mode feeds the same xi to both sides: identical dW."""
    N, L, B = 32, 16.0, 3
    rng = np.random.default_rng(11)
    u0c = (1.0 + 0.1 * (rng.standard_normal((B, N, N)) + 1j * rng.standard_normal((B, N, N))))
    eta = 0.3
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j
    gkw = dict(u0=(jl(u0c).astype(dtype),), lengths=(L, L), dispersion=disp,
               nonlinearity=lambda u, p: 0.01 * np.abs(u[0]) ** 2,
               pump=lambda r, p, t: 1.0 + 0 * r[0],
               position_noise_func=lambda u, r, p: eta)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(L, L), dispersion=disp, nonlin_g=np.array([[0.01]]),
                               pump_profile=np.ones((1, N, N), np.complex128), pump_amp=lambda t: np.array([1.0]),
                               eta=np.array([eta]))
    rn = oracle.ReplayNoise(5, (1, B, N, N))
    xi = (lambda h: rn(h).astype(np.complex64).astype(np.complex128)) if dtype == np.complex64 else rn
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, (0.0, 0.4), 0.02, 4, xi=xi, fp64=fp64)
    tol = TOL[dtype] if dtype == np.complex128 else fp32_tol(oracle, orc, (0.0, 0.4), 0.02, 4, xi=xi)
    assert_close(oracle, res, ores, tol, per_save=dtype == np.complex128)


@pytest.mark.parametrize("fp64", FP64_MODES)
def test_noise_philox_matches_restatement(gpe, oracle, lib, fp64):
    """Philox mode: the in-kernel draws equal the CPU restatement of Philox4x32-10 +
    Box-Muller, so FP64 results agree with the oracle to 1e-10."""
    N, L, B = 32, 16.0, 2
    u0c = np.ones((B, N, N), np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j
    eta = 0.25 - 0.1j
    gkw = dict(u0=(jl(u0c),), lengths=(L, L), dispersion=disp, position_noise_func=lambda u, r, p: eta)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(L, L), dispersion=disp, eta=np.array([eta]))
    seed = 0x1234_5678_9ABC
    xi = oracle.PhiloxNoise(seed, 1, (B,), (N, N))
    prob = gpe.GrossPitaevskiiProblem(**gkw)
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.02, nsaves=2, rng=seed, fp64=fp64)
    ots, ores = oracle.solve(orc, (0.0, 0.2), 0.02, 2, xi_source=xi)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("resident", [True, False], ids=["resident", "two-pass"])
def test_noise_philox_fp32_matches_restatement(gpe, oracle, lib, resident):
    """FP32 one-component fields draw one Philox block for the points x and x + n0/2 of a
    row (the row pass shares it between them); the draws equal the oracle's restatement
    up to the FP32 Box-Muller's hardware approximations (~2^-21), far below what a wrong
    block or word pair would give."""
    N, L, B = 64, 16.0, 2
    u0c = np.ones((B, N, N), np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j
    eta = 0.25 - 0.1j
    gkw = dict(u0=(jl(u0c).astype(np.complex64),), lengths=(L, L), dispersion=disp,
               position_noise_func=lambda u, r, p: eta)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(L, L), dispersion=disp, eta=np.array([eta]))
    seed = 0xC0FFEE
    xi = oracle.PhiloxNoise(seed, 1, (B,), (N, N), fp32=True)
    prob = gpe.GrossPitaevskiiProblem(**gkw)
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.02, nsaves=2, rng=seed, resident=resident)
    ots, ores = oracle.solve(orc, (0.0, 0.2), 0.02, 2, xi_source=xi)
    assert_close(oracle, res, ores, 1e-4)


def test_noise_philox_fp32_1d_matches_restatement(gpe, oracle, lib):
    """The same for a batch of 1D lines (the resident line kernel)."""
    N, L, B = 256, 32.0, 3
    u0c = np.ones((B, N), np.complex128)
    disp = lambda k, p: k[0] ** 2 / 2 - 0.1j
    gkw = dict(u0=(jl(u0c).astype(np.complex64),), lengths=(L,), dispersion=disp,
               position_noise_func=lambda u, r, p: 0.3)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(L,), dispersion=disp, eta=np.array([0.3]))
    seed = 99
    ts, res = gpe.solve(gpe.GrossPitaevskiiProblem(**gkw), gpe.StrangSplitting(), (0.0, 0.2), dt=0.02, nsaves=2,
                        rng=seed)
    ots, ores = oracle.solve(orc, (0.0, 0.2), 0.02, 2, xi_source=oracle.PhiloxNoise(seed, 1, (B,), (N,), fp32=True))
    assert_close(oracle, res, ores, 1e-4)


@pytest.mark.parametrize("fp64", FP64_MODES)
def test_1d_bistability_segment(gpe, oracle, lib, fp64):
    """1D driven-dissipative line (the reference's bistability problem), a short
    segment of its ramp: resident 1D kernel vs oracle."""
    w0, g, d, kz, gam, L, N = 1483.0, 0.01, 0.3, 27.0, 0.1, 256.0, 256
    wp = w0 + d
    disp = lambda k, p: -1j * gam / 2 + w0 * (1 + k[0] ** 2 / (2 * kz ** 2)) - wp
    Imax, tmax, width = 0.6, 3300.0, 50.0
    I = lambda t: max(-Imax * t * (t - tmax) * 4 / tmax ** 2, 0.0)
    x = np.arange(N) * (L / N)
    prof = np.exp(-((x - L / 2) ** 2) / width ** 2)
    gkw = dict(u0=(np.zeros(N, np.complex128),), lengths=(L,), dispersion=disp,
               nonlinearity=lambda u, p: g * np.abs(u[0]) ** 2,
               pump=lambda r, p, t: np.exp(-((r[0] - L / 2) ** 2) / width ** 2) * np.sqrt(I(t)))
    orc = oracle.OracleProblem(u0=(np.zeros(N, np.complex128),), lengths=(L,), dispersion=disp,
                               nonlin_g=np.array([[g]]), pump_profile=prof[None].astype(np.complex128),
                               pump_amp=lambda t: np.array([np.sqrt(I(t))]))
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, (0.0, 300.0), 0.05, 20, fp64=fp64)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("fp64", FP64_MODES)
def test_1d_batch_noise_replay(gpe, oracle, lib, fp64):
    """1D, 200 trajectories with position noise (the windowed-FT test's shape)."""
    N, L, B = 64, 20.0, 200
    hb = 0.6582
    gam, m, d0 = 0.1 / hb, hb ** 2 / 2.5, 0.49 / hb
    dL = L / N
    disp = lambda k, p: -1j * gam / 2 + hb * k[0] ** 2 / (2 * m) - d0
    eta = np.sqrt(gam / 2 / dL)
    u0c = np.zeros((B, N), np.complex128)
    gkw = dict(u0=(jl(u0c),), lengths=(L,), dispersion=disp, position_noise_func=lambda u, r, p: eta)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(L,), dispersion=disp, eta=np.array([eta]))
    xi = oracle.ReplayNoise(9, (1, B, N))
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, (0.0, 40.0), 4.0, 1, save_start=False, xi=xi, fp64=fp64)
    assert res[0].shape == (64, 200, 1)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("dtype,fp64", [(np.complex128, "native"), (np.complex64, "dw")], ids=["c128-native", "c64"])
def test_resume_is_bit_identical(gpe, oracle, lib, dtype, fp64):
    """Checkpoint (fields + gpe_state) and resume equals an uninterrupted run.  (The
    double-word state is rounded to FP64 when read out, so its checkpoints resume to
    within one FP64 rounding; see test_resume_double_word.)"""
    gpu_kw, _ = kerr2d(64, 8.0, -3.0, dtype)
    gpu_kw["position_noise_func"] = lambda u, r, p: 0.05
    prob = gpe.GrossPitaevskiiProblem(**gpu_kw)
    kw = dict(fp64=fp64)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=1, rng=77, **kw)
    it.step(20)
    full = it.get_fields()[0].copy()
    it.close()
    it1 = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=1, rng=77, **kw)
    it1.step(8)
    st = it1.state()
    f = it1.get_fields()
    it1.close()
    it2 = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=1, rng=77, **kw)
    it2.set_fields(f)
    it2.set_state(st)
    it2.step(12)
    resumed = it2.get_fields()[0]
    it2.close()
    assert np.array_equal(full, resumed)


def test_resume_double_word(gpe, oracle, lib):
    """Double-word state: a resumed run agrees with an uninterrupted one to 1e-13 (the
    checkpoint holds the FP64 rounding of the 48-bit state)."""
    gpu_kw, _ = kerr2d(64, 8.0, -3.0, np.complex128)
    gpu_kw["position_noise_func"] = lambda u, r, p: 0.05
    prob = gpe.GrossPitaevskiiProblem(**gpu_kw)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=1, rng=77)
    it.step(20)
    full = it.get_fields()[0].copy()
    it.close()
    it1 = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=1, rng=77)
    it1.step(8)
    st, f = it1.state(), it1.get_fields()
    it1.close()
    it2 = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=1, rng=77)
    it2.set_fields(f)
    it2.set_state(st)
    it2.step(12)
    resumed = it2.get_fields()[0]
    it2.close()
    assert oracle.rel_l2(resumed, full) <= 1e-13


@pytest.mark.parametrize("fp64", FP64_MODES)
def test_norm_matches_oracle(gpe, oracle, lib, fp64):
    gpu_kw, orc = kerr2d(64, 8.0, -3.0, np.complex128)
    prob = gpe.GrossPitaevskiiProblem(**gpu_kw)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.1), dt=0.01, nsaves=1, fp64=fp64)
    it.step(5)
    nrm = it.norm()
    u = c_order(it.get_fields()[0])
    it.close()
    ref = oracle.norm(u, (8.0, 8.0), 2)
    assert abs(nrm[0] - ref) <= 1e-12 * ref


@pytest.mark.parametrize("N,dtype,M", [(64, np.complex64, 1), (128, np.complex64, 1), (64, np.complex64, 2),
                                       (64, np.complex128, 1), (32, np.complex128, 2)])
def test_resident_plane_matches_two_pass(gpe, oracle, lib, N, dtype, M):
    """The resident plane kernel (whole trajectory in shared memory) and the two-pass HBM
    path agree: same half steps, pump, Philox noise and saves; only the FFT radix split
    differs (8 vs 16 points per thread), so they agree to rounding."""
    L = 16.0
    rng = np.random.default_rng(4)
    B = 3
    u0 = [jl(1.0 + 0.1 * (rng.standard_normal((B, N, N)) + 1j * rng.standard_normal((B, N, N)))).astype(dtype)
          for _ in range(M)]
    disp = (lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j) if M == 1 else \
        (lambda k, p: [[(k[0] ** 2 + k[1] ** 2) / 2 - 0.1j, 0.3], [0.3, (k[0] ** 2 + k[1] ** 2) / 4 - 0.05j]])
    nl = (lambda u, p: 0.01 * np.abs(u[0]) ** 2) if M == 1 else \
        (lambda u, p: [0.01 * np.abs(u[0]) ** 2, 0.02 * np.abs(u[1]) ** 2 + 0.01 * np.abs(u[0]) ** 2])
    pump = (lambda r, p, t: 1.0 + 0 * r[0]) if M == 1 else (lambda r, p, t: [min(t, 1.0) + 0 * r[0], 0])
    kw = dict(u0=tuple(u0), lengths=(L, L), dispersion=disp, nonlinearity=nl, pump=pump,
              position_noise_func=lambda u, r, p: 0.2)
    prob = gpe.GrossPitaevskiiProblem(**kw)
    out = {}
    for resident in (True, False):
        ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.4), dt=0.02, nsaves=4, rng=123, resident=resident)
        out[resident] = res
    tol = 2e-5 if dtype == np.complex64 else 1e-12
    for m in range(M):
        a, b = out[True][m].astype(np.complex128), out[False][m].astype(np.complex128)
        assert oracle.rel_l2(a, b) <= tol


@pytest.mark.parametrize("fp64", FP64_MODES)
@pytest.mark.parametrize("shape", [(32, 16, 16), (16, 32, 64)])
def test_3d_grids(gpe, oracle, lib, shape, fp64):
    """3D: x row pass, y forward / z forward-table-inverse / y inverse column passes."""
    nx, ny, nz = shape
    L = (8.0, 6.0, 5.0)
    X, Y, Z = oracle.mesh(oracle.grids(L, (nx, ny, nz))[0])  # C order (nz, ny, nx)
    u0c = (np.exp(-((X - 4) ** 2 + (Y - 3) ** 2 + (Z - 2.5) ** 2)) * np.exp(1j * X)).astype(np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2 + 2 * k[2] ** 2) / 2
    pot = lambda r, p: 0.1 * (r[2] - 2.5) ** 2
    gkw = dict(u0=(jl(u0c),), lengths=L, dispersion=disp, potential=pot,
               nonlinearity=lambda u, p: -1.5 * np.abs(u[0]) ** 2)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=L, dispersion=disp, potential=pot, nonlin_g=np.array([[-1.5]]))
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, (0.0, 0.2), 0.01, 4, fp64=fp64)
    assert res[0].shape == (nx, ny, nz, 5)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
@pytest.mark.parametrize("case", ["kerr2d", "polariton", "3d"])
def test_energy_matches_oracle(gpe, oracle, lib, case, dtype, fp64):
    if case == "kerr2d":
        gkw, orc = kerr2d(64, 8.0, -2.0, dtype)
        gkw["potential"] = orc.potential = (lambda r, p: 0.3 * ((r[0] - 4) ** 2 + (r[1] - 4) ** 2))
    elif case == "polariton":
        gkw, orc = polariton2d(N=64, L=128.0, A=5.0, ramp=20.0)
        gkw["u0"] = tuple(u.astype(dtype) for u in gkw["u0"])
    else:
        L = (8.0, 6.0, 5.0)
        X, Y, Z = oracle.mesh(oracle.grids(L, (32, 16, 16))[0])
        u0c = (np.exp(-((X - 4) ** 2 + (Y - 3) ** 2 + (Z - 2.5) ** 2)) * np.exp(1j * Y)).astype(np.complex128)
        disp = lambda k, p: (k[0] ** 2 + k[1] ** 2 + k[2] ** 2) / 2
        gkw = dict(u0=(jl(u0c).astype(dtype),), lengths=L, dispersion=disp,
                   nonlinearity=lambda u, p: 2.0 * np.abs(u[0]) ** 2 + 0.5)
        orc = oracle.OracleProblem(u0=(u0c,), lengths=L, dispersion=disp, nonlin_g=np.array([[2.0]]),
                                   nonlin_c=np.array([0.5]))
    prob = gpe.GrossPitaevskiiProblem(**gkw)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=2, fp64=fp64)
    it.step(7)
    e_gpu = it.energy()
    u = np.stack([c_order(f).astype(np.complex128) for f in it.get_fields()])
    it.close()
    oit = oracle.OracleIterator(orc, (0.0, 0.2), 0.01, 2)
    e_ref = oracle.energy(oit, u)
    tol = 1e-10 if dtype == np.complex128 else 1e-5
    scale = np.abs(e_ref).sum()
    assert np.all(np.abs(e_gpu - e_ref) <= tol * scale), (e_gpu, e_ref)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_nonfinite_upload_is_rejected_and_state_kept(gpe, lib, dtype, fp64):
    """A field with a NaN is refused (GPE_ERR_NONFINITE) after being staged on the
    device, and the handle keeps its previous state."""
    gkw, _ = kerr2d(32, 8.0, -1.0, dtype)
    it = gpe.init(gpe.GrossPitaevskiiProblem(**gkw), gpe.StrangSplitting(), (0.0, 0.1), dt=0.01, nsaves=1, fp64=fp64)
    it.step(3)
    before = it.get_fields()[0].copy()
    bad = before.copy()
    bad[5, 7] = np.nan
    with pytest.raises(Exception, match="NaN or Inf"):
        it.set_fields((bad,))
    assert np.array_equal(it.get_fields()[0], before)
    it.step(1)
    assert np.all(np.isfinite(it.get_fields()[0]))
    it.close()


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
@pytest.mark.parametrize("variant", [0, 2], ids=["default-tiling", "fine-tiling"])
@pytest.mark.parametrize("case", ["kerr", "polariton", "3d"])
def test_line_tilings_match_oracle(gpe, oracle, lib, case, variant, dtype, fp64):
    """Both line tilings of the two-pass passes (forced with gpe_set_variant) against the
    oracle, for one- and two-component 2D fields and a 3D grid."""
    if case == "kerr":
        gkw, orc = kerr2d(128, 8.0, -2.0, dtype)
        tspan, dt, ns = (0.0, 0.1), 0.005, 4
    elif case == "polariton":
        gkw, orc = polariton2d(N=128, L=256.0, A=5.0, ramp=20.0, dtype=dtype)
        tspan, dt, ns = (0.0, 2.0), 0.05, 4
    else:
        L = (8.0, 6.0, 5.0)
        X, Y, Z = oracle.mesh(oracle.grids(L, (32, 16, 16))[0])
        u0c = np.exp(-(X - 4) ** 2 - (Y - 3) ** 2 - (Z - 2.5) ** 2 + 0.2j * X).astype(np.complex128)
        disp = lambda k, p: (k[0] ** 2 + k[1] ** 2 + k[2] ** 2) / 2
        gkw = dict(u0=(jl(u0c).astype(dtype),), lengths=L, dispersion=disp,
                   nonlinearity=lambda u, p: 1.3 * np.abs(u[0]) ** 2)
        orc = oracle.OracleProblem(u0=(u0c,), lengths=L, dispersion=disp, nonlin_g=np.array([[1.3]]))
        tspan, dt, ns = (0.0, 0.1), 0.01, 2
    prob = gpe.GrossPitaevskiiProblem(**gkw)
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), tspan, dt=dt, nsaves=ns, fp64=fp64, resident=False,
                        variant=variant)
    ots, ores = oracle.solve(orc, tspan, dt, ns)
    if dtype == np.complex128:
        assert_close(oracle, res, ores, TOL[dtype])
    else:
        assert_close(oracle, res, ores, fp32_tol(oracle, orc, tspan, dt, ns), per_save=False)
