"""Writes the golden fixtures of this directory from the FP64 oracle.

The reference is a Julia package and cannot run where this project is built or tested,
and its own tests store no golden vectors, so these fixtures are outputs of the oracle
(oracle/gpe_oracle.py) on small seeded cases.  They pin the oracle against accidental
change (tests/test_golden.py re-runs it on CPU) and give the GPU tests fixed expected
outputs that need no oracle run (tests/test_golden_gpu.py).

    python tests/golden/make_golden.py     # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import gpe_oracle as O  # noqa: E402


def kerr_c0():
    """The reference's plain case at its own size: 2D Kerr 128^2, L=8, u0 = exp(-(x-4)^2
    - (y-4)^2), D=|k|^2/2, G=-6|u|^2, tspan (0, 0.4), dt 0.01 -> 64 steps of 0.00625,
    nsaves 64 (saves 0, 32 and 64 kept)."""
    N, L = 128, 8.0
    X, Y = O.mesh(O.grids((L, L), (N, N))[0])
    u0 = np.exp(-(X - 4) ** 2 - (Y - 4) ** 2).astype(np.complex128)
    prob = O.OracleProblem(u0=(u0,), lengths=(L, L), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                           nonlin_g=np.array([[-6.0]]))
    ts, res = O.solve(prob, (0.0, 0.4), 0.01, 64)
    keep = np.array([0, 32, 64])
    return dict(u0=u0, ts=ts[keep], saves=res[0, keep], keep=keep)


def polariton64():
    """Two-component polariton at 64^2 (L=256, 2x2 dispersion, G=diag(0, 0.003|u2|^2),
    photon pump 5 exp(-|r - r0|^2/50^2) ramped over t in [0, 2]), u0 = 0, 40 steps of 0.05."""
    N, L = 64, 256.0
    X, Y = O.mesh(O.grids((L, L), (N, N))[0])
    prof = np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / 50.0 ** 2)

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        one = np.ones_like(k2)
        return np.array([[0.6582 * k2 / (2 / 6) + 0.5 - 0.05j, 5.07 * one], [5.07 * one, -0.005j * one]])

    z = np.zeros((N, N), np.complex128)
    prob = O.OracleProblem(u0=(z, z.copy()), lengths=(L, L), dispersion=disp,
                           nonlin_g=np.array([[0, 0], [0, 0.003]], np.complex128),
                           pump_profile=np.stack([prof, 0 * prof]).astype(np.complex128),
                           pump_amp=lambda t: np.array([5.0 * min(t / 2.0, 1.0), 0.0]))
    ts, res = O.solve(prob, (0.0, 2.0), 0.05, 4)
    return dict(ts=ts, saves=res)


def philox_noise32():
    """Scalar damped field with in-kernel Philox noise (seed 2024) on 32^2, 2 trajectories:
    the FP64 draws of the restated generator, 20 steps of 0.02."""
    N, L, B, seed = 32, 16.0, 2, 2024
    u0 = np.ones((B, N, N), np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j
    prob = O.OracleProblem(u0=(u0,), lengths=(L, L), dispersion=disp, nonlin_g=np.array([[0.05]]),
                           eta=np.array([0.2 - 0.05j]))
    ts, res = O.solve(prob, (0.0, 0.4), 0.02, 2, xi_source=O.PhiloxNoise(seed, 1, (B,), (N, N)))
    return dict(ts=ts, saves=res, seed=np.array(seed))


def matrix_nl32():
    """Matrix nonlinearity G = [[0.8|u0|^2 - 0.03i, 0.9 + 0.05|u1|^2], [0.9, 0.5|u1|^2 +
    0.2|u0|^2 + 0.1 - 0.02i]] with D = (|k|^2/2, 0.1) on 32^2, 20 steps of 0.02."""
    N, L = 32, 12.0
    X, Y = O.mesh(O.grids((L, L), (N, N))[0])
    r2 = (X - L / 2) ** 2 + (Y - L / 2) ** 2
    a = (np.exp(-r2 / 2) * (1 + 0.2j * X)).astype(np.complex128)
    b = (0.6 * np.exp(-r2 / 3)).astype(np.complex128)

    def gm(u):
        d0, d1 = np.abs(u[0]) ** 2, np.abs(u[1]) ** 2
        return np.asarray([[0.8 * d0 - 0.03j, 0.9 + 0.05 * d1], [0.9 + 0 * d0, 0.5 * d1 + 0.2 * d0 + 0.1 - 0.02j]],
                          dtype=np.complex128)

    prob = O.OracleProblem(u0=(a, b), lengths=(L, L),
                           dispersion=lambda k, p: np.stack([(k[0] ** 2 + k[1] ** 2) / 2, 0.1 + 0 * k[0]]) + 0j,
                           nonlin_matrix=gm)
    ts, res = O.solve(prob, (0.0, 0.4), 0.02, 2)
    return dict(u0a=a, u0b=b, ts=ts, saves=res)


def bistability1d():
    """The 1D problem of test/bistability_cycle.jl (omega0=1483, g=0.01, delta=0.3, kz=27,
    gamma=0.1, L=256 on 256 points, pump sqrt(I(t)) exp(-(x-L/2)^2/50^2) with I(t) =
    max(-0.6 t (t - 3300) 4/3300^2, 0)), its first 10 time units: 200 steps of 0.05."""
    w0, g, d, kz, gam = 1483.0, 0.01, 0.3, 27.0, 0.1
    N, L, Imax, width, tmax = 256, 256.0, 0.6, 50.0, 3300.0
    I = lambda t: max(-Imax * t * (t - tmax) * 4 / tmax ** 2, 0.0)
    x = O.direct_grid(L, N)
    prof = np.exp(-((x - L / 2) ** 2) / width ** 2)
    prob = O.OracleProblem(u0=(np.zeros(N, np.complex128),), lengths=(L,),
                           dispersion=lambda k, p: -1j * gam / 2 + w0 * (1 + k[0] ** 2 / (2 * kz ** 2)) - (w0 + d),
                           nonlin_g=np.array([[g]]), pump_profile=prof[None].astype(np.complex128),
                           pump_amp=lambda t: np.array([math.sqrt(I(t))]))
    ts, res = O.solve(prob, (0.0, 10.0), 0.05, 2)
    return dict(ts=ts, saves=res)


def kerr3d():
    """3D Kerr on (nx, ny, nz) = (32, 16, 16), L = (8, 6, 5): u0 = exp(-|r - (4, 3, 2.5)|^2)
    exp(i x), D = (kx^2 + ky^2 + 2 kz^2)/2, V = 0.1 (z - 2.5)^2, G = -1.5|u|^2, tspan
    (0, 0.2), dt 0.01, nsaves 2 (the last save kept)."""
    L, shape = (8.0, 6.0, 5.0), (32, 16, 16)
    X, Y, Z = O.mesh(O.grids(L, shape)[0])
    u0 = (np.exp(-((X - 4) ** 2 + (Y - 3) ** 2 + (Z - 2.5) ** 2)) * np.exp(1j * X)).astype(np.complex128)
    prob = O.OracleProblem(u0=(u0,), lengths=L, dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2 + 2 * k[2] ** 2) / 2,
                           potential=lambda r, p: 0.1 * (r[2] - 2.5) ** 2, nonlin_g=np.array([[-1.5]]))
    ts, res = O.solve(prob, (0.0, 0.2), 0.01, 2)
    return dict(ts=ts, last=res[0, -1])


CASES = {"kerr_c0": kerr_c0, "polariton64": polariton64, "philox_noise32": philox_noise32,
         "matrix_nl32": matrix_nl32, "bistability1d": bistability1d, "kerr3d": kerr3d}


def main():
    for name, fn in CASES.items():
        np.savez_compressed(HERE / f"{name}.npz", **fn())
        print("wrote", name)


if __name__ == "__main__":
    main()
