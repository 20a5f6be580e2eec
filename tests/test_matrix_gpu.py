"""GPU parity of the matrix nonlinearity family (an SMatrix-valued G whose cis is a 2x2
matrix exponential per point, src/kernels.jl:23-25,44) against the FP64 oracle: 1D, 2D
and 3D grids, scalar and matrix potentials, pumps, replayed and Philox noise, pointwise-
only problems, and graph replay against plain stepping."""
import numpy as np
import pytest

from cases import jl
from oracle import gpe_oracle as O
from test_parity_gpu import PREC_IDS, PRECISIONS, TOL, assert_close, fp32_tol, run_both

pytestmark = pytest.mark.gpu

# G = [[gc |u0|^2 + c00, k + gk |u1|^2], [k, gx |u1|^2 + gxc |u0|^2 + c11]]: cross-Kerr,
# a Rabi coupling k with a density-dependent part on one side (a non-Hermitian G), losses
GC, GX, GXC, GK, K, C00, C11 = 0.8, 0.5, 0.2, 0.05, 0.9, -0.03j, 0.1 - 0.02j


def gmat_closure(u, p):
    d0, d1 = np.abs(u[0]) ** 2, np.abs(u[1]) ** 2
    return [[GC * d0 + C00, K + GK * d1], [K + 0 * d0, GX * d1 + GXC * d0 + C11]]


def gmat_oracle(u):
    return np.asarray(gmat_closure(u, None), dtype=np.complex128)


def two_comp_u0(shape_c, lengths, batch=(), seed=0):
    dg, _ = O.grids(lengths, tuple(reversed(shape_c)))
    R = O.mesh(dg)
    r2 = sum((x - L / 2) ** 2 for x, L in zip(R, lengths))
    a = np.exp(-r2 / 2) * (1 + 0.2j * R[0])
    b = 0.6 * np.exp(-r2 / 3)
    if batch:
        rng = np.random.default_rng(seed)
        nb = int(np.prod(batch))
        a = np.stack([a * (1 + 0.1 * rng.standard_normal()) for _ in range(nb)]).reshape(batch + a.shape)
        b = np.stack([b * (1 + 0.1 * rng.standard_normal()) for _ in range(nb)]).reshape(batch + b.shape)
    return a.astype(np.complex128), b.astype(np.complex128)


def check(oracle, dtype, res, ores, orc, tspan, dt, nsaves, xi=None):
    if dtype == np.complex128:
        assert_close(oracle, res, ores, TOL[dtype])
    else:
        assert_close(oracle, res, ores, fp32_tol(oracle, orc, tspan, dt, nsaves, xi=xi), per_save=False)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_matrix_nonlinearity_2d_pump_scalar_potential(gpe, oracle, lib, dtype, fp64):
    N, L = 64, 12.0
    a, b = two_comp_u0((N, N), (L, L))
    disp = lambda k, p: [(k[0] ** 2 + k[1] ** 2) / 2 - 0.02j, 0.1 + 0 * k[0]]
    pot = lambda r, p: 0.05 * ((r[0] - L / 2) ** 2 + (r[1] - L / 2) ** 2) / L
    pump = lambda r, p, t: [0.3 * np.exp(-((r[0] - L / 2) ** 2 + (r[1] - L / 2) ** 2) / 4) * min(t / 0.2, 1.0), 0]
    gkw = dict(u0=(jl(a).astype(dtype), jl(b).astype(dtype)), lengths=(L, L), dispersion=disp, potential=pot,
               nonlinearity=gmat_closure, pump=pump)
    dg, _ = oracle.grids((L, L), (N, N))
    X, Y = oracle.mesh(dg)
    prof = np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / 4)
    odisp = lambda k, p: np.stack([(k[0] ** 2 + k[1] ** 2) / 2 - 0.02j, 0.1 + 0 * k[0]]).astype(np.complex128)
    orc = oracle.OracleProblem(u0=(a, b), lengths=(L, L), dispersion=odisp,
                               potential=lambda r, p: 0.05 * ((r[0] - L / 2) ** 2 + (r[1] - L / 2) ** 2) / L + 0j,
                               nonlin_matrix=gmat_oracle,
                               pump_profile=np.stack([prof, 0 * prof]).astype(np.complex128),
                               pump_amp=lambda t: np.array([0.3 * min(t / 0.2, 1.0), 0.0]))
    tspan, dt, ns = (0.0, 0.6), 0.02, 6
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, tspan, dt, ns, fp64=fp64)
    assert np.array_equal(ts, ots)
    check(oracle, dtype, res, ores, orc, tspan, dt, ns)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_matrix_nonlinearity_matrix_potential_noise_batch(gpe, oracle, lib, dtype, fp64):
    """Rectangular 64x32 grid, 2 trajectories, a 2x2 potential table composed after the
    nonlinear exponential (cis(-dt G) * exp(-i dt V)), replayed noise on both components."""
    L = (10.0, 6.0)
    B = 2
    a, b = two_comp_u0((32, 64), L, batch=(B,), seed=2)
    disp = lambda k, p: [[(k[0] ** 2 + k[1] ** 2) / 2, 0.3 + 0 * k[0]], [0.3 + 0 * k[0], 0.2 * k[0] ** 2 - 0.05j]]

    def pot(r, p):
        x = r[0] - L[0] / 2
        return [[0.02 * x ** 2, 0.1 + 0.05j + 0 * x], [0.1 - 0.05j + 0 * x, -0.01 * x ** 2]]

    eta = 0.05
    gkw = dict(u0=(jl(a).astype(dtype), jl(b).astype(dtype)), lengths=L, dispersion=disp, potential=pot,
               nonlinearity=gmat_closure, position_noise_func=lambda u, r, p: [eta, 0.5 * eta])
    arr = lambda f: (lambda q, p: np.asarray([[np.asarray(v, np.complex128) * np.ones_like(q[0]) for v in row]
                                              for row in f(q, p)]))
    orc = oracle.OracleProblem(u0=(a, b), lengths=L, dispersion=arr(disp), potential=arr(pot),
                               nonlin_matrix=gmat_oracle, eta=np.array([eta, 0.5 * eta]))
    rn = oracle.ReplayNoise(3, (2, B, 32, 64))
    xi = (lambda h: rn(h).astype(np.complex64).astype(np.complex128)) if dtype == np.complex64 else rn
    tspan, dt, ns = (0.0, 0.4), 0.02, 4
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, tspan, dt, ns, xi=xi, fp64=fp64)
    assert res[0].shape == (64, 32, B, ns + 1)
    check(oracle, dtype, res, ores, orc, tspan, dt, ns, xi=xi)


@pytest.mark.parametrize("fp64", ["dw", "native", "bfp"])
def test_matrix_nonlinearity_1d_philox(gpe, oracle, lib, fp64):
    """1D line with in-kernel Philox noise: the draws equal the oracle's restatement."""
    N, L, B = 256, 40.0, 3
    a, b = two_comp_u0((N,), (L,), batch=(B,), seed=5)
    disp = lambda k, p: [k[0] ** 2 / 2 - 0.05j, 0.3 + 0 * k[0]]
    gkw = dict(u0=(jl(a), jl(b)), lengths=(L,), dispersion=disp, nonlinearity=gmat_closure,
               position_noise_func=lambda u, r, p: [0.1, 0.1])
    orc = oracle.OracleProblem(u0=(a, b), lengths=(L,),
                               dispersion=lambda k, p: np.stack([k[0] ** 2 / 2 - 0.05j, 0.3 + 0 * k[0]]),
                               nonlin_matrix=gmat_oracle, eta=np.array([0.1, 0.1]))
    seed = 0xBEEF
    xi = oracle.PhiloxNoise(seed, 2, (B,), (N,))
    prob = gpe.GrossPitaevskiiProblem(**gkw)
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 1.0), dt=0.01, nsaves=5, rng=seed, fp64=fp64)
    ots, ores = oracle.solve(orc, (0.0, 1.0), 0.01, 5, xi_source=xi)
    assert_close(oracle, res, ores, 1e-10)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_matrix_nonlinearity_3d(gpe, oracle, lib, dtype, fp64):
    shape_c, L = (16, 16, 32), (8.0, 6.0, 5.0)
    a, b = two_comp_u0(shape_c, L)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2 + k[2] ** 2) / 2
    gkw = dict(u0=(jl(a).astype(dtype), jl(b).astype(dtype)), lengths=L, dispersion=disp, nonlinearity=gmat_closure)
    orc = oracle.OracleProblem(u0=(a, b), lengths=L, dispersion=lambda k, p: disp(k, p) + 0j,
                               nonlin_matrix=gmat_oracle)
    tspan, dt, ns = (0.0, 0.2), 0.01, 4
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, tspan, dt, ns, fp64=fp64)
    check(oracle, dtype, res, ores, orc, tspan, dt, ns)


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
def test_matrix_nonlinearity_pointwise_only(gpe, oracle, lib, dtype, fp64):
    """No dispersion: every step runs in one pointwise launch with in-launch saves."""
    N, L = 32, 8.0
    a, b = two_comp_u0((N, N), (L, L))
    gkw = dict(u0=(jl(a).astype(dtype), jl(b).astype(dtype)), lengths=(L, L), nonlinearity=gmat_closure,
               pump=lambda r, p, t: [0.1 + 0 * r[0], 0.05j + 0 * r[0]])
    orc = oracle.OracleProblem(u0=(a, b), lengths=(L, L), nonlin_matrix=gmat_oracle,
                               pump_profile=np.stack([np.full((N, N), 0.1), np.full((N, N), 0.05j)]).astype(np.complex128),
                               pump_amp=lambda t: np.array([1.0, 1.0]))
    tspan, dt, ns = (0.0, 1.0), 0.05, 5
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, tspan, dt, ns, fp64=fp64)
    check(oracle, dtype, res, ores, orc, tspan, dt, ns)


def test_matrix_nonlinearity_graph_equals_plain_stepping(gpe, lib):
    """Graph replay (device step counter) of the matrix pass chain equals plain stepping
    bit for bit."""
    N, L = 128, 12.0
    a, b = two_comp_u0((N, N), (L, L))
    kw = dict(u0=(jl(a).astype(np.complex64), jl(b).astype(np.complex64)), lengths=(L, L),
              dispersion=lambda k, p: [(k[0] ** 2 + k[1] ** 2) / 2, 0 * k[0]], nonlinearity=gmat_closure,
              position_noise_func=lambda u, r, p: [0.02, 0.02])
    its = [gpe.init(gpe.GrossPitaevskiiProblem(**kw), gpe.StrangSplitting(), (0.0, 0.6), dt=0.01, nsaves=1, rng=9)
           for _ in range(2)]
    assert lib.gpe_set_graph(its[0].h, 10) == 0
    its[0].step(30)
    its[1].step(30)
    for m in range(2):
        assert np.array_equal(its[0].get_fields()[m], its[1].get_fields()[m])
    for it in its:
        it.close()


def test_matrix_nonlinearity_rejects_diagonal_potential(gpe, lib):
    N, L = 32, 8.0
    a, b = two_comp_u0((N, N), (L, L))
    kw = dict(u0=(jl(a), jl(b)), lengths=(L, L), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
              nonlinearity=gmat_closure, potential=lambda r, p: [0 * r[0] + 0.1, 0 * r[0]])
    with pytest.raises(Exception, match="diagonal potential"):
        gpe.init(gpe.GrossPitaevskiiProblem(**kw), gpe.StrangSplitting(), (0.0, 0.1), dt=0.01, nsaves=1)
