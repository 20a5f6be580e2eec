"""Pins the FP64 oracle to the reference's own known-answer tests (test/*.jl),
restated from their mathematics.  CPU only."""
import math

import numpy as np
import pytest

from oracle import gpe_oracle as O


def test_free_propagation_is_exact_spectral(oracle=O):
    """test/free_propagation.jl:1-29: with only D = |k|^2/2 the split step is exact,
    so every save equals ifft(exp(-i |k|^2 t / 2) fft(u0)); scalar, vector and 1x1
    matrix dispersions agree (the three closure shapes)."""
    rng = np.random.default_rng(0)
    N = 64
    for trial in range(3):
        L = float(rng.integers(4, 11))
        dt = 0.3 * rng.random()
        nsaves = int(rng.integers(20, 60))
        dg, rg = O.grids((L, L), (N, N))
        X, Y = O.mesh(dg)
        u0 = (np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2)) * (X - L / 2 + 1j * (Y - L / 2)) ** (trial + 1)
              + np.exp(-((X - L / 3) ** 2 + (Y - L / 2) ** 2) / 2))
        KX, KY = O.mesh(rg)
        K2 = KX ** 2 + KY ** 2
        tspan = (0.0, nsaves * dt)
        forms = [lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                 lambda k, p: np.stack([(k[0] ** 2 + k[1] ** 2) / 2]),
                 lambda k, p: ((k[0] ** 2 + k[1] ** 2) / 2)[None, None]]
        sols = []
        for D in forms:
            ts, res = O.solve(O.OracleProblem(u0=(u0,), lengths=(L, L), dispersion=D), tspan, dt, nsaves)
            exact = np.stack([np.fft.ifft2(np.exp(-1j * K2 / 2 * t) * np.fft.fft2(u0)) for t in ts])
            assert O.rel_l2(res[0], exact) <= 1.49e-8
            sols.append(res[0])
        assert O.rel_l2(sols[0], sols[1]) <= 1e-14 and O.rel_l2(sols[0], sols[2]) <= 1e-14


def test_kerr_closure_shape_invariance():
    """test/kerr_propagation.jl:30-36: scalar / SVector / SMatrix{1,1} dispersion and
    nonlinearity give the same solution (rel L2 <= sqrt(eps))."""
    N, L, g = 64, 10.0, -1.3
    dg, _ = O.grids((L, L), (N, N))
    X, Y = O.mesh(dg)
    u0 = np.exp(-((X - 5) ** 2 + (Y - 5) ** 2)) * np.exp(1j * X)
    Ds = [lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2, lambda k, p: np.stack([(k[0] ** 2 + k[1] ** 2) / 2]),
          lambda k, p: ((k[0] ** 2 + k[1] ** 2) / 2)[None, None]]
    Gs = [lambda u: g * np.abs(u) ** 2 / 2, lambda u: np.stack([g * np.abs(u[0]) ** 2 / 2]),
          lambda u: g * np.abs(u) ** 2 / 2]
    base = None
    for D in Ds:
        for G in Gs:
            prob = O.OracleProblem(u0=(u0,), lengths=(L, L), dispersion=D, nonlin_fn=G)
            ts, res = O.solve(prob, (0.0, 0.05), 0.002, 10)
            if base is None:
                base = res
            assert O.rel_l2(res, base) <= 1.49e-8


def bistability_problem():
    w0, g, d, kz, gam = 1483.0, 0.01, 0.3, 27.0, 0.1
    wp = w0 + d
    L, N = 256.0, 256
    Imax, width, tmax = 0.6, 50.0, 3300.0
    I = lambda t: max(-Imax * t * (t - tmax) * 4 / tmax ** 2, 0.0)
    x = O.direct_grid(L, N)
    prof = np.exp(-((x - L / 2) ** 2) / width ** 2)
    prob = O.OracleProblem(u0=(np.zeros(N, np.complex128),), lengths=(L,),
                           dispersion=lambda k, p: -1j * gam / 2 + w0 * (1 + k[0] ** 2 / (2 * kz ** 2)) - wp,
                           nonlin_g=np.array([[g]]), pump_profile=prof[None].astype(np.complex128),
                           pump_amp=lambda t: np.array([math.sqrt(I(t))]))
    return prob, I, (d, g, gam), tmax


def test_bistability_cycle():
    """test/bistability_cycle.jl:37-65: the peak density follows the bistability curve
    n (gamma^2/4 + (g n - delta)^2) = I(t); mean error over saves 140..400 <= 3e-3."""
    prob, I, (d, g, gam), tmax = bistability_problem()
    ts, res = O.solve(prob, (0.0, tmax), 0.05, 512)
    err = []
    for n, t in enumerate(ts):
        nmax = np.max(np.abs(res[0, n]) ** 2)
        err.append(abs(nmax * (gam ** 2 / 4 + (g * nmax - d) ** 2) - I(t)))
    err = np.array(err)
    assert err[139:400].sum() / len(ts) <= 3e-3


def test_exciton_polariton_steady_state():
    """test/exciton_polariton_test.jl:15-53: at the pump centre the steady state obeys
    two analytic relations within 3e-2."""
    hb = 0.654
    Om = 5.07 / 2 / hb
    gx = 0.0015 / hb
    gc = 0.07 / 0.6571 / hb
    wx, wc = 1484.44 / hb, 1482.76 / hb
    m = hb ** 2 / (2 * 2e-1)
    wp = wc
    dx, dc = wp - wx, wp - wc
    A, w, g = 2.0, 100.0, 1e-2 / hb
    L, N = 256.0, 128

    def disp(k, p):
        k2 = k[0] ** 2 + k[1] ** 2
        one = np.ones_like(k2)
        return np.array([[hb * k2 / (2 * m) - dc - 1j * gc, Om * one], [Om * one, (-dx - 1j * gx) * one]])

    dg, _ = O.grids((L, L), (N, N))
    X, Y = O.mesh(dg)
    prof = A * np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / w ** 2)
    z = np.zeros((N, N), np.complex128)
    prob = O.OracleProblem(u0=(z, z.copy()), lengths=(L, L), dispersion=disp,
                           nonlin_g=np.array([[0, 0], [0, g]], np.complex128),
                           pump_profile=np.stack([prof, 0 * prof]).astype(np.complex128),
                           pump_amp=lambda t: np.array([1.0, 0.0]))
    ts, res = O.solve(prob, (0.0, 100.0), 0.1, 256)
    nx = abs(res[1, -1, N // 2, N // 2]) ** 2
    nc = abs(res[0, -1, N // 2, N // 2]) ** 2
    assert abs(abs(Om - (dx + 1j * gx / 2 - g * nx) * (dc + 1j * gc / 2) / Om) ** 2 * nx / abs(A) ** 2 - 1) < 3e-2
    assert abs(abs(dx + 1j * gx / 2 - g * nx) ** 2 * nx / Om ** 2 / nc - 1) < 3e-2


def windowed_correlation(sol, rs, w1, w2):
    s1 = sol * w1(rs)[:, None]
    s2 = sol * w2(rs)[:, None]
    f1 = np.fft.ifftshift(np.fft.fft(np.fft.fftshift(s1, 0), axis=0), 0)
    f2 = np.fft.ifftshift(np.fft.fft(np.fft.fftshift(s2, 0), axis=0), 0)
    # g1[i, j] = dot(f2[j, :], f1[i, :]) / length(sol)  (dot conjugates its first argument)
    return (f1 @ f2.conj().T) / sol.size


def test_windowed_ft_commutator():
    """test/windowed_ft.jl:22-99: truncated-Wigner vacuum, 10^4 trajectories; the windowed
    FT correlation equals the analytic commutator within rtol 7e-2."""
    L, N = 20.0, 64
    dL = L / N
    hb = 0.6582
    gam, m, d0 = 0.1 / hb, hb ** 2 / 2.5, 0.49 / hb
    B = 10 ** 4
    prob = O.OracleProblem(u0=(np.zeros((B, N), np.complex128),), lengths=(L,),
                           dispersion=lambda k, p: -1j * gam / 2 + hb * k[0] ** 2 / (2 * m) - d0,
                           eta=np.array([math.sqrt(gam / 2 / dL)]))
    rng = np.random.default_rng(1234)
    xi = lambda h: O.complex_normal(rng, (1, B, N))
    ts, res = O.solve(prob, (0.0, 200.0), 4.0, 1, save_start=False, xi_source=xi)
    sol = res[0, 0].T  # (N, B), the reference's (space, trajectory) layout
    rs = -L / 2 + np.arange(N) * (L / N)
    ks = -math.pi / L + np.arange(N) * (2 * math.pi / L)
    for x0 in (-1, 0, 1):
        for w in (3, 4, 5):
            win1 = lambda x, x0=x0, w=w: np.exp(-((x - x0) ** 2) / w ** 2)
            win2 = lambda x, x0=x0, w=w: np.exp(-((x + x0) ** 2) / w ** 2)
            corr = windowed_correlation(sol, rs, win1, win2)
            ph = np.exp(1j * (ks[:, None, None] - ks[None, :, None]) * rs[None, None, :])
            an = (ph * (win1(rs) * np.conj(win2(rs)))[None, None, :]).sum(-1) / (rs[-1] - rs[0]) / 2
            assert np.linalg.norm(corr - an) <= 7e-2 * max(np.linalg.norm(corr), np.linalg.norm(an))


def test_resolve_fixed_timestepping_cases():
    """src/fixed_time_stepping.jl:14-24 on the workloads used here."""
    dt, t0, s = O.resolve_fixed_timestepping(0.01, (0, 0.4), 64)
    assert s == 1 and dt == 0.00625
    dt, t0, s = O.resolve_fixed_timestepping(0.05, (0, 200), 100)
    assert s == 40 and abs(dt - 0.05) < 1e-15
    dt, t0, s = O.resolve_fixed_timestepping(0.1, (0, 100), 256)
    assert s == 4 and dt == 0.09765625


def test_pump_times_follow_the_reference_order():
    """init samples F(t0); step k (end time t_k) samples t_k + dt/2 and t_k + dt."""
    pt = O.pump_times(1.0, 0.5, 3)
    assert np.allclose(pt, [1.0, 1.75, 2.0, 2.25, 2.5, 2.75, 3.0])


def test_matrix_nonlinearity_linear_coupling_closed_form():
    """Matrix family with a constant coupling G = [[d, k], [k, -d]] and a scalar dispersion:
    G and D commute, so the split step is exact, u(t) = exp(-i t G) exp(-i t D) u0, with
    exp(-i t G) = cos(w t) I - i sin(w t) G / w, w = sqrt(d^2 + k^2) (a two-level Rabi
    rotation)."""
    N, L, dt, nsaves = 32, 8.0, 0.07, 15
    dg, rg = O.grids((L, L), (N, N))
    X, Y = O.mesh(dg)
    a0 = np.exp(-((X - 4) ** 2 + (Y - 4) ** 2)) * (1 + 0.3j * X)
    b0 = 0.5 * np.exp(-((X - 3) ** 2 + (Y - 5) ** 2) / 2)
    d, k = 0.4, 1.3
    G = np.array([[d, k], [k, -d]], np.complex128)
    prob = O.OracleProblem(u0=(a0, b0), lengths=(L, L), dispersion=lambda q, p: (q[0] ** 2 + q[1] ** 2) / 2,
                           nonlin_matrix=lambda u: np.broadcast_to(G.reshape(2, 2, *([1] * (u.ndim - 1))),
                                                                   (2, 2) + u.shape[1:]))
    ts, res = O.solve(prob, (0.0, nsaves * dt), dt, nsaves)
    KX, KY = O.mesh(rg)
    K2 = KX ** 2 + KY ** 2
    w = math.hypot(d, k)
    for i, t in enumerate(ts):
        fa = np.fft.ifft2(np.exp(-1j * K2 / 2 * t) * np.fft.fft2(a0))
        fb = np.fft.ifft2(np.exp(-1j * K2 / 2 * t) * np.fft.fft2(b0))
        c, s = math.cos(w * t), math.sin(w * t)
        ea = c * fa - 1j * s / w * (d * fa + k * fb)
        eb = c * fb - 1j * s / w * (k * fa - d * fb)
        assert O.rel_l2(np.stack([res[0, i], res[1, i]]), np.stack([ea, eb])) <= 1e-12


def test_matrix_exponential_matches_scipy():
    """The closed-form 2x2 exponential of the oracle (used for cis(-delta G) of an SMatrix
    nonlinearity) against scipy.linalg.expm on random complex matrices, including nearly
    degenerate ones (the series branch) and exactly diagonal ones."""
    from scipy.linalg import expm
    rng = np.random.default_rng(4)
    A = rng.standard_normal((2, 2, 40)) + 1j * rng.standard_normal((2, 2, 40))
    A[:, :, :10] *= 1e-4
    A[0, 1, 10:15] = A[1, 0, 10:15] = 0
    A[1, 1, 15:20] = A[0, 0, 15:20] + 1e-5
    A[0, 1, 15:20] *= 1e-4
    E = O.expm_2x2_or_1x1(A)
    for q in range(A.shape[-1]):
        want = expm(A[:, :, q])
        assert np.abs(E[:, :, q] - want).max() <= 1e-13 * max(1.0, np.abs(want).max())


def test_diagonal_matrix_nonlinearity_equals_diagonal_family():
    """A 2x2 SMatrix nonlinearity that happens to be diagonal reproduces the per-component
    (SVector) family: cis of a diagonal matrix is the diagonal of the cis values."""
    N, L, dt, nsaves = 32, 10.0, 0.05, 6
    dg, _ = O.grids((L,), (N,))
    (X,) = O.mesh(dg)
    u0 = (np.exp(-(X - 5) ** 2) + 0j, 0.7 * np.exp(-(X - 4) ** 2 / 3) + 0.1j)
    g = np.array([[1.0, 0.4 - 0.05j], [0.3, -0.8]])
    c = np.array([0.2, -0.1 + 0.02j])

    def gmat(u):
        dens = np.abs(u) ** 2
        G = np.zeros((2, 2) + u.shape[1:], np.complex128)
        for j in range(2):
            G[j, j] = g[j, 0] * dens[0] + g[j, 1] * dens[1] + c[j]
        return G

    kw = dict(u0=u0, lengths=(L,), dispersion=lambda q, p: np.stack([q[0] ** 2 / 2, q[0] ** 2 / 3]))
    _, ra = O.solve(O.OracleProblem(nonlin_g=g, nonlin_c=c, **kw), (0.0, nsaves * dt), dt, nsaves)
    _, rb = O.solve(O.OracleProblem(nonlin_matrix=gmat, **kw), (0.0, nsaves * dt), dt, nsaves)
    assert O.rel_l2(ra, rb) <= 1e-13
