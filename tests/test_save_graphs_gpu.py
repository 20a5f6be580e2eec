"""Runs whose saves stream through the save ring launch one CUDA graph per save chunk
(the passes of save_every steps, the last one writing the save into its ring slot).
The passes are those of the direct launches, so the saved trajectory must equal the
direct-launch run (per-launch timing on forces that path) bit for bit: two-component
double-word with a pump ramp, one-component FP32 with Philox noise, a 3D field, and a
setter between two solves (the chunk graphs hold the old arguments and are recaptured)."""
import numpy as np
import pytest

from cases import jl, polariton2d

pytestmark = pytest.mark.gpu


def solve(gpe, lib, prob, tspan, dt, nsaves, direct, **kw):
    it = gpe.init(prob, gpe.StrangSplitting(), tspan, dt=dt, nsaves=nsaves, **kw)
    if direct:
        lib.gpe_set_timing(it.h, 1)
    ts, res = it.solve()
    it.close()
    return ts, [np.array(r) for r in res]


def cases(gpe):
    rng = np.random.default_rng(8)
    gkw, _ = polariton2d(N=128, L=256.0, A=5.0, ramp=2.0)
    yield "polariton-dw", gpe.GrossPitaevskiiProblem(**gkw), (0.0, 3.0), 0.05, 12, {}
    u = jl((1 + 0.3 * (rng.standard_normal((3, 64, 64)) + 1j * rng.standard_normal((3, 64, 64)))).astype(np.complex64))
    p = gpe.GrossPitaevskiiProblem((u,), (32.0, 32.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j,
                                   nonlinearity=lambda u, p: 0.01 * np.abs(u[0]) ** 2, pump=lambda r, p, t: 1.0 + 0 * r[0],
                                   position_noise_func=lambda u, r, p: 0.2)
    yield "noise-f32", p, (0.0, 1.2), 0.02, 10, dict(rng=5, resident=False)
    u3 = jl((0.5 * (rng.standard_normal((16, 32, 32)) + 1j * rng.standard_normal((16, 32, 32)))).astype(np.complex128))
    p3 = gpe.GrossPitaevskiiProblem((u3,), (8.0, 8.0, 4.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2 + k[2] ** 2) / 2,
                                    nonlinearity=lambda u, p: 0.3 * np.abs(u[0]) ** 2)
    yield "3d-dw", p3, (0.0, 0.3), 0.01, 6, {}


@pytest.mark.parametrize("name", ["polariton-dw", "noise-f32", "3d-dw"])
def test_save_chunk_graphs_match_direct_launches(gpe, lib, name):
    (_, prob, tspan, dt, nsaves, kw), = [c for c in cases(gpe) if c[0] == name]
    ts_g, res_g = solve(gpe, lib, prob, tspan, dt, nsaves, False, **kw)
    ts_d, res_d = solve(gpe, lib, prob, tspan, dt, nsaves, True, **kw)
    assert np.array_equal(ts_g, ts_d)
    for a, b in zip(res_g, res_d):
        assert np.isfinite(a).all()
        assert np.array_equal(a, b)


def test_setter_between_graphed_solves(gpe, lib):
    """Two solves on one handle with a new nonlinearity in between: the second must use it."""
    L = gpe._lib
    gkw, _ = polariton2d(N=64, L=256.0, A=5.0, ramp=2.0)
    prob = gpe.GrossPitaevskiiProblem(**gkw)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 1.0), dt=0.05, nsaves=10, resident=False)
    fields0 = it.get_fields()
    it.solve()
    g = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.05, 0.0])  # g[j][l] (re, im): G_1 = 0.05 |u_1|^2
    c = np.zeros(4)
    L.check(lib, it.h, lib.gpe_set_nonlinearity(it.h, L.ptr(g), L.ptr(c)))
    it.set_fields(fields0)
    st = it.state()
    st.steps, st.t = 0, 0.0
    it.set_state(st)
    ts1, res1 = it.solve()
    lib.gpe_set_timing(it.h, 1)
    it.set_fields(fields0)
    it.set_state(st)
    ts2, res2 = it.solve()
    it.close()
    for a, b in zip(res1, res2):
        assert np.array_equal(np.array(a), np.array(b))


@pytest.mark.parametrize("name", ["polariton-dw", "noise-f32", "3d-dw"])
@pytest.mark.parametrize("nsteps", [65, 100, 129])
def test_run_chunk_graphs_match_direct_launches(gpe, lib, name, nsteps):
    """Runs without saves longer than two chunks go through the chunk graph."""
    (_, prob, tspan, dt, nsaves, kw), = [c for c in cases(gpe) if c[0] == name]
    out = []
    for direct in (False, True):
        it = gpe.init(prob, gpe.StrangSplitting(), (0.0, (nsteps + 5) * dt), dt=dt, nsaves=1, **kw)
        if direct:
            lib.gpe_set_timing(it.h, 1)
        it.step(3)
        it.step(nsteps)
        if not direct:
            assert it.last_run_launches() > 0
        out.append([np.array(f) for f in it.get_fields()])
        it.close()
    for a, b in zip(*out):
        assert np.isfinite(a).all()
        assert np.array_equal(a, b)
