"""Pins the C restatement of the stepper (oracle/gpe_ref.c) to the numpy oracle and to the
golden fixtures, on the CPU.  The C oracle is what the large-configuration GPU tests
(2048^2 Kerr over 1000 steps) and the CPU baseline run, so it must agree with the numpy
restatement to FP64 rounding, and its single-precision mode must show the error level of
the reference's ComplexF32 arithmetic."""
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import gpe_oracle as O
from oracle import gpe_oracle_c as OC

ROOT = Path(__file__).resolve().parents[1]


def kerr(N, L, g, width2=1.0, center=None):
    c = L / 2 if center is None else center
    X, Y = O.mesh(O.grids((L, L), (N, N))[0])
    u0 = np.exp(-((X - c) ** 2 + (Y - c) ** 2) / width2).astype(np.complex128)
    return O.OracleProblem(u0=(u0,), lengths=(L, L), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                           nonlin_g=np.array([[g]]))


def polariton(N, B=1, L=256.0, ramp=2.0):
    X, Y = O.mesh(O.grids((L, L), (N, N))[0])
    prof = np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / 50.0 ** 2)

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        one = np.ones_like(k2)
        return np.array([[0.6582 * k2 / (2 / 6) + 0.5 - 0.05j, 5.07 * one], [5.07 * one, -0.005j * one]])

    rng = np.random.default_rng(3)
    shape = ((B,) if B > 1 else ()) + (N, N)
    u = [0.1 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) for _ in range(2)]
    return O.OracleProblem(u0=tuple(u), lengths=(L, L), dispersion=disp,
                           nonlin_g=np.array([[0, 0], [0, 0.003]], np.complex128),
                           pump_profile=np.stack([prof, 0 * prof]).astype(np.complex128),
                           pump_amp=lambda t: np.array([5.0 * min(t / ramp, 1.0), 0.0]))


def test_kerr_matches_numpy_oracle():
    prob = kerr(64, 8.0, -6.0)
    ts, want = O.solve(prob, (0.0, 0.2), 0.01, 5)
    ts2, got = OC.solve(prob, (0.0, 0.2), 0.01, 5)
    assert np.array_equal(ts, ts2)
    for s in range(want.shape[1]):
        assert O.rel_l2(got[:, s], want[:, s]) <= 1e-13


def test_polariton_batch_matches_numpy_oracle():
    prob = polariton(32, B=3)
    ts, want = O.solve(prob, (0.0, 2.0), 0.05, 4)
    _, got = OC.solve(prob, (0.0, 2.0), 0.05, 4)
    assert got.shape == want.shape
    for s in range(want.shape[1]):
        assert O.rel_l2(got[:, s], want[:, s]) <= 1e-13


def test_1d_potential_complex_nonlinearity_matches_numpy_oracle():
    N, L = 128, 20.0
    x = O.direct_grid(L, N)
    u0 = (np.exp(-(x - 10) ** 2) * np.exp(0.5j * x)).astype(np.complex128)
    prob = O.OracleProblem(u0=(u0,), lengths=(L,), dispersion=lambda k, p: k[0] ** 2 / 2 - 0.05j,
                           potential=lambda r, p: 0.01 * (r[0] - 10) ** 2,
                           nonlin_g=np.array([[1.5 - 0.1j]]), nonlin_c=np.array([0.2 + 0.01j]),
                           pump_profile=np.exp(-(x - 5) ** 2)[None].astype(np.complex128),
                           pump_amp=lambda t: np.array([0.3 * math.sin(t) + 0.1j]))
    ts, want = O.solve(prob, (0.0, 3.0), 0.02, 6)
    _, got = OC.solve(prob, (0.0, 3.0), 0.02, 6)
    for s in range(want.shape[1]):
        assert O.rel_l2(got[:, s], want[:, s]) <= 1e-13


def test_golden_plain_case():
    """The reference's plain case (128^2 Kerr, g = -6, 64 saves) against its fixture."""
    G = np.load(ROOT / "tests" / "golden" / "kerr_c0.npz")
    prob = O.OracleProblem(u0=(G["u0"],), lengths=(8.0, 8.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                           nonlin_g=np.array([[-6.0]]))
    ts, res = OC.solve(prob, (0.0, 0.4), 0.01, 64)
    assert np.allclose(ts[G["keep"]], G["ts"], rtol=0, atol=1e-15)
    for i, s in enumerate(G["keep"]):
        assert O.rel_l2(res[0, s], G["saves"][i]) <= 1e-12


def test_golden_polariton():
    G = np.load(ROOT / "tests" / "golden" / "polariton64.npz")
    N, L = 64, 256.0
    X, Y = O.mesh(O.grids((L, L), (N, N))[0])
    prob = polariton(N)
    z = np.zeros((N, N), np.complex128)
    prob.u0 = (z, z.copy())
    ts, res = OC.solve(prob, (0.0, 2.0), 0.05, 4)
    assert np.allclose(ts, G["ts"], rtol=0, atol=1e-15)
    for s in range(res.shape[1]):
        assert O.rel_l2(res[:, s], G["saves"][:, s]) <= 1e-12


def test_stepping_in_chunks_equals_one_run():
    prob = polariton(32)
    a = OC.CIterator(prob, (0.0, 2.0), 0.05, 4)
    a.step(40)
    b = OC.CIterator(prob, (0.0, 2.0), 0.05, 4)
    for n in (7, 13, 20):
        b.step(n)
    assert np.array_equal(a.u, b.u)


def test_fp32_mode_has_the_reference_fp32_error_level():
    """Single-precision FFTs with FP64 table products: the C form (radix-2) and the numpy
    form (scipy's single-precision FFT) both move away from FP64 by about 1e-7 a step on
    this focusing case and agree with each other at that level."""
    prob = kerr(64, 8.0, -2.0)
    _, ref = O.solve(prob, (0.0, 0.5), 0.01, 5)
    _, c32 = OC.solve(prob, (0.0, 0.5), 0.01, 5, fp32=True)
    _, n32 = O.solve_fp32(prob, (0.0, 0.5), 0.01, 5)
    ec, en = O.rel_l2(c32[:, -1], ref[:, -1]), O.rel_l2(n32[:, -1], ref[:, -1])
    assert 1e-7 < ec < 1e-5 and 1e-7 < en < 1e-5
    assert 0.3 < ec / en < 3
    # and the state really is single precision
    assert np.array_equal(c32[:, -1], c32[:, -1].astype(np.complex64).astype(np.complex128))


def test_rejects_what_it_does_not_restate():
    N = 16
    u0 = np.zeros((N, N), np.complex128)
    prob = O.OracleProblem(u0=(u0,), lengths=(1.0, 1.0), dispersion=lambda k, p: k[0] * 0, eta=np.array([0.1]))
    with pytest.raises(NotImplementedError):
        OC.CIterator(prob, (0.0, 1.0), 0.1, 1)  # noise needs the Philox seed
    prob.nonlin_fn = lambda u: u
    with pytest.raises(NotImplementedError):
        OC.CIterator(prob, (0.0, 1.0), 0.1, 1, philox_seed=1)


@pytest.mark.parametrize("M,draw32", [(1, False), (1, True), (2, False)])
def test_philox_noise_matches_numpy_restatement(M, draw32):
    """The C oracle's Philox noise equals the numpy oracle fed with PhiloxNoise (the same
    counter layout, key and Box-Muller transform) on a batched 2D problem with an offset."""
    N, B, seed, traj0 = 16, 3, 977, 5
    X, Y = O.mesh(O.grids((8.0, 8.0), (N, N))[0])
    rng = np.random.default_rng(1)
    u0 = tuple((rng.standard_normal((B, N, N)) + 1j * rng.standard_normal((B, N, N))) * 0.3 for _ in range(M))
    g = np.array([[0.2]]) if M == 1 else np.array([[0.2, 0.1], [0.1, 0.3]])
    prob = O.OracleProblem(u0=u0, lengths=(8.0, 8.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j,
                           nonlin_g=g, eta=np.array([0.7 + 0.1j, 0.4][:M]))
    noise = O.PhiloxNoise(seed, M, (B,), (N, N), fp32=draw32, traj0=traj0)
    _, want = O.solve(prob, (0.0, 0.2), 0.02, 2, xi_source=lambda h: noise(h))
    _, got = OC.CIterator(prob, (0.0, 0.2), 0.02, 2, philox_seed=seed, draw32=draw32, traj0=traj0).solve()
    # FP32 draws are rounded to single precision; a last-place difference between the two
    # libm sin/cos can move that rounding by one FP32 unit on a few draws
    tol = 1e-7 if draw32 else 1e-12
    for s in range(want.shape[1]):
        assert O.rel_l2(got[:, s], want[:, s]) <= tol
