"""Problem builders shared by the parity tests: each returns the same problem in the
package's form (Julia index order) and in the oracle's form (C order)."""
from __future__ import annotations

import math

import numpy as np

from oracle import gpe_oracle as O


def jl(a_c: np.ndarray) -> np.ndarray:
    """C-order oracle array (..., ny, nx) -> Julia-order Fortran array (nx, ny, ...)."""
    return np.asfortranarray(a_c.T)


def c_order(a_jl: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a_jl.T)


def grid_c(lengths, shape_c):
    """Oracle mesh (X, Y, ...) in C order for a spatial C shape."""
    dg, rg = O.grids(lengths, tuple(reversed(shape_c)))
    return O.mesh(dg), O.mesh(rg)


def kerr2d(N=128, L=8.0, g=-6.0, dtype=np.complex128, batch=()):
    """The reference's plain case: u0 = exp(-(x-L/2)^2 - (y-L/2)^2), D = |k|^2/2,
    G = g|u|^2 (x, y in [0, L))."""
    (X, Y), _ = grid_c((L, L), (N, N))
    u0c = np.exp(-(X - L / 2) ** 2 - (Y - L / 2) ** 2).astype(np.complex128)
    if batch:
        rng = np.random.default_rng(3)
        u0c = np.stack([u0c * (1 + 0.1 * rng.standard_normal()) for _ in range(int(np.prod(batch)))]).reshape(batch + u0c.shape)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2
    gpu = dict(u0=(jl(u0c).astype(dtype),), lengths=(L, L), dispersion=disp,
               nonlinearity=lambda u, p: g * np.abs(u[0]) ** 2)
    orc = O.OracleProblem(u0=(u0c,), lengths=(L, L), dispersion=disp, nonlin_g=np.array([[g]]))
    return gpu, orc


POL = dict(hbar=0.6582, m=1 / 6, dc=-0.5, dx=0.0, gc=0.05, gx=0.005, Om=5.07, g=0.003)


def polariton2d(N=128, L=256.0, A=5.0, ramp=200.0, w=50.0, dtype=np.complex128):
    """Two-component exciton-polariton: 2x2 dispersion, G = diag(0, g|u2|^2), pump on
    the photon A(t) exp(-|r - r0|^2 / w^2), A(t) = A min(t / ramp, 1), u0 = 0."""
    p = POL
    (X, Y), _ = grid_c((L, L), (N, N))

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        Dcc = p["hbar"] * k2 / (2 * p["m"]) - p["dc"] - 1j * p["gc"]
        Dxx = -p["dx"] - 1j * p["gx"] + 0 * k2
        Dxc = p["Om"] + 0 * k2
        return [[Dcc, Dxc], [Dxc, Dxx]]

    amp = lambda t: A * min(t / ramp, 1.0)
    prof_c = np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / w ** 2)

    def pump(r, _, t):
        return [amp(t) * np.exp(-((r[0] - L / 2) ** 2 + (r[1] - L / 2) ** 2) / w ** 2), 0]

    z = np.zeros((N, N), np.complex128)
    gpu = dict(u0=(jl(z).astype(dtype), jl(z).astype(dtype)), lengths=(L, L), dispersion=disp,
               nonlinearity=lambda u, _: [0 * u[0], p["g"] * np.abs(u[1]) ** 2], pump=pump)

    def odisp(k, _):
        return np.asarray([[np.asarray(v, np.complex128) * np.ones_like(k[0]) for v in row] for row in disp(k, None)])

    orc = O.OracleProblem(u0=(z, z.copy()), lengths=(L, L), dispersion=odisp,
                          nonlin_g=np.array([[0, 0], [0, p["g"]]], np.complex128),
                          pump_profile=np.stack([prof_c, 0 * prof_c]).astype(np.complex128),
                          pump_amp=lambda t: np.array([amp(t), 0.0]))
    return gpu, orc

