"""Uniform pumps (one value everywhere, folded into the pump coefficients so the passes
load no profile): real and complex constants with a time ramp, on one of two components
and on a single component, two-pass and resident paths, every precision, against the
FP64 oracle."""
import numpy as np
import pytest

from cases import jl
from test_parity_gpu import PREC_IDS, PRECISIONS, TOL, assert_close, fp32_tol, run_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
@pytest.mark.parametrize("M,F", [(1, 1.0), (1, 0.3 - 0.2j), (2, 0.5 + 0.1j)], ids=["m1-real", "m1-complex", "m2-complex"])
@pytest.mark.parametrize("resident", [False, True], ids=["two-pass", "resident"])
def test_uniform_pump(gpe, oracle, lib, dtype, fp64, M, F, resident):
    N, L = 64, 16.0
    rng = np.random.default_rng(21)
    u0c = [(0.5 * (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N)))).astype(np.complex128)
           for _ in range(M)]
    ramp = lambda t: min(t / 0.3, 1.0)
    if M == 1:
        disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j
        nl = lambda u, p: 0.2 * np.abs(u[0]) ** 2
        pump = lambda r, p, t: F * ramp(t) + 0 * r[0]
        odisp, g = (lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j + 0 * k[0]), np.array([[0.2]])
    else:
        disp = lambda k, p: [[(k[0] ** 2 + k[1] ** 2) / 2 - 0.05j, 0.7 + 0 * k[0]], [0.7 + 0 * k[0], -0.01j + 0 * k[0]]]
        nl = lambda u, p: [0 * u[0], 0.3 * np.abs(u[1]) ** 2]
        pump = lambda r, p, t: [F * ramp(t) + 0 * r[0], 0 * r[0]]

        def odisp(k, p):
            v = disp(k, p)
            return np.asarray([[np.asarray(x, np.complex128) + 0 * k[0] for x in row] for row in v])
        g = np.array([[0, 0], [0, 0.3]], np.complex128)
    gkw = dict(u0=tuple(jl(u).astype(dtype) for u in u0c), lengths=(L, L), dispersion=disp, nonlinearity=nl, pump=pump)
    prof = np.ones((M, N, N), np.complex128)
    if M == 2:
        prof[1] = 0
    orc = oracle.OracleProblem(u0=tuple(u0c), lengths=(L, L), dispersion=odisp, nonlin_g=g, pump_profile=F * prof,
                               pump_amp=lambda t: np.array([ramp(t)] + [0.0] * (M - 1)))
    tspan, dt, ns = (0.0, 0.6), 0.01, 3
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, tspan, dt, ns, fp64=fp64, resident=resident)
    tol = TOL[dtype] if dtype == np.complex128 else fp32_tol(oracle, orc, tspan, dt, ns)
    assert_close(oracle, res, ores, tol)
