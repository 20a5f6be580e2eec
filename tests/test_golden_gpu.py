"""The CUDA path against the committed golden fixtures (tests/golden/*.npz, outputs of
the FP64 oracle): each problem is built only through the package's reference-shaped API
(closures, Julia index order), run on the GPU and compared to the stored saves at 1e-10
rel L2 in FP64 (double-word and native) -- no oracle run is involved."""
import math
from pathlib import Path

import numpy as np
import pytest

from cases import c_order, jl

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FP64 = ["dw", "native", "bfp"]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def grid(L, N):
    return np.arange(N) * (L / N)


@pytest.mark.parametrize("fp64", FP64)
def test_golden_kerr_plain_case(gpe, lib, fp64):
    """The reference's plain case (128^2 Kerr, g=-6, tspan (0, 0.4), dt 0.01, nsaves 64)."""
    G = np.load(GOLDEN / "kerr_c0.npz")
    N, L = 128, 8.0
    x = grid(L, N)
    X, Y = np.meshgrid(x, x, indexing="ij")
    u0 = np.exp(-(X - 4) ** 2 - (Y - 4) ** 2).astype(np.complex128)
    prob = gpe.GrossPitaevskiiProblem((u0,), (L, L), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                      nonlinearity=lambda u, p: -6.0 * np.abs(u[0]) ** 2)
    ts, (res,) = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.4), dt=0.01, nsaves=64, fp64=fp64)
    assert np.allclose(ts[G["keep"]], G["ts"], rtol=0, atol=1e-15)
    for i, s in enumerate(G["keep"]):
        assert rel(c_order(res[..., s]), G["saves"][i]) <= 1e-10, s


@pytest.mark.parametrize("fp64", FP64)
def test_golden_polariton(gpe, lib, fp64):
    G = np.load(GOLDEN / "polariton64.npz")
    N, L = 64, 256.0

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        return [[0.6582 * k2 / (2 / 6) + 0.5 - 0.05j, 5.07 + 0 * k2], [5.07 + 0 * k2, -0.005j + 0 * k2]]

    z = np.zeros((N, N), np.complex128)
    prob = gpe.GrossPitaevskiiProblem(
        (z, z.copy()), (L, L), dispersion=disp, nonlinearity=lambda u, p: [0 * u[0], 0.003 * np.abs(u[1]) ** 2],
        pump=lambda r, p, t: [5.0 * min(t / 2.0, 1.0) * np.exp(-((r[0] - L / 2) ** 2 + (r[1] - L / 2) ** 2) / 50.0 ** 2),
                              0])
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 2.0), dt=0.05, nsaves=4, fp64=fp64)
    assert np.allclose(ts, G["ts"], rtol=0, atol=1e-14)
    for m in range(2):
        assert rel(c_order(res[m]), G["saves"][m]) <= 1e-10, m


@pytest.mark.parametrize("fp64", FP64)
def test_golden_philox_noise(gpe, lib, fp64):
    """In-kernel Philox draws (seed 2024) reproduce the stored FP64 trajectory."""
    G = np.load(GOLDEN / "philox_noise32.npz")
    N, L, B = 32, 16.0, 2
    u0 = np.ones((N, N, B), np.complex128, order="F")
    prob = gpe.GrossPitaevskiiProblem((u0,), (L, L), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j,
                                      nonlinearity=lambda u, p: 0.05 * np.abs(u[0]) ** 2,
                                      position_noise_func=lambda u, r, p: 0.2 - 0.05j)
    ts, (res,) = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.4), dt=0.02, nsaves=2, rng=int(G["seed"]), fp64=fp64)
    assert rel(c_order(res), G["saves"][0]) <= 1e-10


@pytest.mark.parametrize("fp64", FP64)
def test_golden_matrix_nonlinearity(gpe, lib, fp64):
    G = np.load(GOLDEN / "matrix_nl32.npz")
    L = 12.0

    def gm(u, p):
        d0, d1 = np.abs(u[0]) ** 2, np.abs(u[1]) ** 2
        return [[0.8 * d0 - 0.03j, 0.9 + 0.05 * d1], [0.9 + 0 * d0, 0.5 * d1 + 0.2 * d0 + 0.1 - 0.02j]]

    prob = gpe.GrossPitaevskiiProblem((jl(G["u0a"]), jl(G["u0b"])), (L, L),
                                      dispersion=lambda k, p: [(k[0] ** 2 + k[1] ** 2) / 2, 0.1 + 0 * k[0]],
                                      nonlinearity=gm)
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.4), dt=0.02, nsaves=2, fp64=fp64)
    for m in range(2):
        assert rel(c_order(res[m]), G["saves"][m]) <= 1e-10, m


@pytest.mark.parametrize("fp64", FP64)
def test_golden_bistability_1d(gpe, lib, fp64):
    """The problem of test/bistability_cycle.jl, first 10 time units."""
    G = np.load(GOLDEN / "bistability1d.npz")
    w0, g, d, kz, gam = 1483.0, 0.01, 0.3, 27.0, 0.1
    N, L, Imax, width, tmax = 256, 256.0, 0.6, 50.0, 3300.0
    I = lambda t: max(-Imax * t * (t - tmax) * 4 / tmax ** 2, 0.0)
    prob = gpe.GrossPitaevskiiProblem(
        (np.zeros(N, np.complex128),), (L,),
        dispersion=lambda k, p: -1j * gam / 2 + w0 * (1 + k[0] ** 2 / (2 * kz ** 2)) - (w0 + d),
        nonlinearity=lambda u, p: g * np.abs(u[0]) ** 2,
        pump=lambda r, p, t: math.sqrt(I(t)) * np.exp(-((r[0] - L / 2) ** 2) / width ** 2))
    ts, (res,) = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 10.0), dt=0.05, nsaves=2, fp64=fp64)
    assert np.allclose(ts, G["ts"], rtol=0, atol=1e-13)
    assert rel(c_order(res), G["saves"][0]) <= 1e-10


@pytest.mark.parametrize("fp64", FP64)
def test_golden_kerr_3d(gpe, lib, fp64):
    """3D Kerr with a potential on (32, 16, 16): the x row pass and the y/z column passes."""
    G = np.load(GOLDEN / "kerr3d.npz")
    L, shape = (8.0, 6.0, 5.0), (32, 16, 16)
    X, Y, Z = np.meshgrid(*(grid(l, n) for l, n in zip(L, shape)), indexing="ij")
    u0 = (np.exp(-((X - 4) ** 2 + (Y - 3) ** 2 + (Z - 2.5) ** 2)) * np.exp(1j * X)).astype(np.complex128)
    prob = gpe.GrossPitaevskiiProblem((u0,), L, dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2 + 2 * k[2] ** 2) / 2,
                                      potential=lambda r, p: 0.1 * (r[2] - 2.5) ** 2,
                                      nonlinearity=lambda u, p: -1.5 * np.abs(u[0]) ** 2)
    ts, (res,) = gpe.solve(prob, gpe.StrangSplitting(), (0.0, 0.2), dt=0.01, nsaves=2, fp64=fp64)
    assert res.shape == shape + (3,)
    assert np.allclose(ts, G["ts"], rtol=0, atol=1e-15)
    assert rel(c_order(res[..., -1]), G["last"]) <= 1e-10
