"""The iterator form (init, then step!) past the span init was given.  The reference
evaluates the pump at any time, so its iterator runs on past tspan; here the sampled
amplitude schedule is extended before such a step, and the field matches both a run
whose span covered every step and the FP64 oracle."""
import numpy as np
import pytest

from cases import c_order

pytestmark = pytest.mark.gpu

N, LB, DT = 64, 16.0, 0.05


def amp(t):
    return min(t / 2.0, 1.0)


def test_step_past_tspan_with_a_time_dependent_pump(gpe, oracle, lib):
    x = np.arange(N) * (LB / N)
    X, Y = np.meshgrid(x, x, indexing="ij")
    u0 = (0.5 * np.exp(-((X - 8) ** 2 + (Y - 8) ** 2) / 4)).astype(np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.05j
    prof = lambda r: np.exp(-((r[0] - 8) ** 2 + (r[1] - 8) ** 2) / 9)
    prob = gpe.GrossPitaevskiiProblem((u0,), (LB, LB), dispersion=disp,
                                      nonlinearity=lambda u, p: 0.3 * np.abs(u[0]) ** 2,
                                      pump=lambda r, p, t: amp(t) * prof(r))
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 1.0), dt=DT, nsaves=1)  # 20 steps sampled
    gpe.step(it, 20)
    gpe.step(it, 30)  # steps 20 .. 49 lie past tspan
    assert it.state().steps == 50
    (a,) = it.get_fields()
    it.close()

    ref = gpe.init(prob, gpe.StrangSplitting(), (0.0, 2.5), dt=DT, nsaves=1)
    gpe.step(ref, 50)
    (b,) = ref.get_fields()
    ref.close()
    assert oracle.rel_l2(a, b) <= 1e-12

    Xc, Yc = oracle.mesh(oracle.grids((LB, LB), (N, N))[0])
    orc = oracle.OracleProblem(u0=(c_order(u0),), lengths=(LB, LB), dispersion=disp, nonlin_g=np.array([[0.3]]),
                               pump_profile=prof((Xc, Yc))[None].astype(np.complex128),
                               pump_amp=lambda t: np.array([amp(t)]))
    _, ores = oracle.solve(orc, (0.0, 2.5), DT, 1)
    assert oracle.rel_l2(c_order(a), ores[0, -1]) <= 1e-10
