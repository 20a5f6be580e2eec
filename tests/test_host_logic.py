"""Host-side logic of the mirror of the reference's surface (no GPU needed): grids,
dt resolution, pump sampling times, closure classification, Philox restatement."""
import math

import numpy as np
import pytest

from oracle import gpe_oracle as O


def test_grids_match_reference_convention(gpe):
    """src/problem.jl:129-139: x_j = j L/N; k = fftfreq(N, 2 pi N / L)."""
    from gpe_gb300 import problem as P
    for L, N in [(8.0, 128), (256.0, 512), (10.0, 64), (3.0, 16)]:
        assert np.array_equal(P.direct_grid_axis(L, N), O.direct_grid(L, N))
        assert np.allclose(P.reciprocal_grid_axis(L, N), np.fft.fftfreq(N, L / N) * 2 * math.pi, rtol=1e-15, atol=1e-13)
        assert np.array_equal(P.reciprocal_grid_axis(L, N), O.reciprocal_grid(L, N))


def test_dt_resolution_and_pump_times_agree_with_oracle(gpe):
    for dt, tspan, ns in [(0.01, (0, 0.4), 64), (0.05, (0, 200), 100), (0.3, (0, 7.7), 13), (4, (0, 200), 1)]:
        a = gpe.resolve_fixed_timestepping(dt, tspan, ns)
        b = O.resolve_fixed_timestepping(dt, tspan, ns)
        assert a[0] == b[0] and a[2] == b[2]
        n = a[2] * ns
        assert np.array_equal(gpe.pump_sample_times(float(tspan[0]), a[0], n), O.pump_times(float(tspan[0]), a[0], n))


def test_nonlinearity_classification(gpe):
    from gpe_gb300.problem import classify_nonlinearity
    g, c = classify_nonlinearity(lambda u, p: -6.0 * np.abs(u[0]) ** 2, 1, None)
    assert np.allclose(g, [[-6.0]]) and np.allclose(c, [0])
    # SVector and SMatrix{1,1} forms of the same closure
    g2, _ = classify_nonlinearity(lambda u, p: [-6.0 * np.abs(u[0]) ** 2], 1, None)
    g3, _ = classify_nonlinearity(lambda u, p: [[-6.0 * np.abs(u[0]) ** 2]], 1, None)
    assert np.allclose(g2, g) and np.allclose(g3, g)
    g, c = classify_nonlinearity(lambda u, p: [0 * u[0], p * np.abs(u[1]) ** 2], 2, 0.003)
    assert np.allclose(g, [[0, 0], [0, 0.003]])
    g, c = classify_nonlinearity(lambda u, p: (0.01 - 0.2j) * (np.abs(u[0]) ** 2 - 1 / 0.5), 1, None)
    assert np.allclose(g, [[0.01 - 0.2j]]) and np.allclose(c, [-(0.01 - 0.2j) * 2])
    with pytest.raises(NotImplementedError):
        classify_nonlinearity(lambda u, p: np.abs(u[0]) ** 4, 1, None)
    # a non-diagonal SMatrix is handed to the matrix family
    from gpe_gb300.problem import MatrixNonlinearity
    with pytest.raises(MatrixNonlinearity):
        classify_nonlinearity(lambda u, p: [[np.abs(u[0]) ** 2, 1.0 + 0 * u[0]], [1.0 + 0 * u[0], np.abs(u[1]) ** 2]], 2, None)


def test_matrix_nonlinearity_classification(gpe):
    """G_ab = sum_l g_abl |u_l|^2 + c_ab recovered from an SMatrix closure; a scalar closure
    is the identity matrix times it; a non-polynomial closure or one component is refused."""
    from gpe_gb300.problem import classify_matrix_nonlinearity
    fn = lambda u, p: [[0.8 * np.abs(u[0]) ** 2 - 0.03j, 0.9 + 0.05 * np.abs(u[1]) ** 2],
                       [0.9 + 0 * u[0], 0.5 * np.abs(u[1]) ** 2 + 0.2 * np.abs(u[0]) ** 2 + 0.1]]
    g, c = classify_matrix_nonlinearity(fn, 2, None)
    assert g.shape == (2, 2, 2) and c.shape == (2, 2)
    assert np.allclose(g[0, 0], [0.8, 0]) and np.allclose(g[0, 1], [0, 0.05])
    assert np.allclose(g[1, 0], [0, 0]) and np.allclose(g[1, 1], [0.2, 0.5])
    assert np.allclose(c, [[-0.03j, 0.9], [0.9, 0.1]])
    g, c = classify_matrix_nonlinearity(lambda u, p: 2.0 * np.abs(u[1]) ** 2, 2, None)
    assert np.allclose(g[0, 0], [0, 2]) and np.allclose(g[1, 1], [0, 2]) and np.allclose(g[0, 1], 0)
    with pytest.raises(NotImplementedError):
        classify_matrix_nonlinearity(lambda u, p: [[np.abs(u[0]) ** 4, 0 * u[0]], [0 * u[0], 0 * u[0]]], 2, None)
    with pytest.raises(NotImplementedError):
        classify_matrix_nonlinearity(lambda u, p: np.abs(u[0]) ** 2, 1, None)


def test_pump_classification(gpe):
    from gpe_gb300.problem import classify_pump, direct_grid_axis
    L, N = 16.0, 32
    axes = (direct_grid_axis(L, N), direct_grid_axis(L, N))
    times = gpe.pump_sample_times(0.0, 0.1, 20)
    amp = lambda t: 2.0 * min(t / 1.0, 1.0) * np.exp(0.3j * t)
    prof = lambda r: np.exp(-((r[0] - 8) ** 2 + (r[1] - 8) ** 2) / 9)
    profiles, amps = classify_pump(lambda r, p, t: [amp(t) * prof(r), 0], axes, None, 2, times)
    assert profiles[1] is None
    X, Y = np.meshgrid(*axes, indexing="ij")
    for i, t in enumerate(times):
        F = amps[0, i] * profiles[0]
        assert np.allclose(F, (amp(t) * prof((X, Y))).ravel(order="F"), rtol=1e-12, atol=1e-14)
    with pytest.raises(NotImplementedError):
        classify_pump(lambda r, p, t: np.exp(-((r[0] - t) ** 2)), axes, None, 1, times)


class _FakeLib:
    """Stands in for libgpe in host-logic tests: records the pump schedules and refuses
    a run whose schedule is too short, as gpe_run does."""

    def __init__(self):
        self.steps, self.amps = 0, {}

    def gpe_create(self, dref, href):
        href._obj.value = 1
        return 0

    def gpe_set_field(self, h, m, p):
        return 0

    def gpe_set_dispersion(self, h, p, kind):
        return 0

    def gpe_set_pump(self, h, m, prof, cplx, a, n):
        import ctypes
        v = np.frombuffer((ctypes.c_double * (2 * n)).from_address(a), np.float64)
        self.amps[m] = v[0::2] + 1j * v[1::2]
        return 0

    def gpe_get_state(self, h, st):
        st._obj.steps = self.steps
        return 0

    def gpe_run(self, h, nsteps, save_every, out, ts):
        if any(len(a) > 1 and len(a) < 2 * (self.steps + nsteps) + 1 for a in self.amps.values()):
            return -1
        self.steps += nsteps
        return 0

    def gpe_run_ex(self, h, nsteps, save_every, xi, out, stride, ts):
        import ctypes
        if any(len(a) > 1 and len(a) < 2 * (self.steps + nsteps) + 1 for a in self.amps.values()):
            return -1
        ns = nsteps // save_every
        t = np.frombuffer((ctypes.c_double * ns).from_address(ts), np.float64)
        t[:] = 0.1 * (self.steps + save_every * np.arange(1, ns + 1))  # the handle's time: t0 + steps * dt
        self.steps += nsteps
        return 0

    def gpe_last_error(self, h):
        return b"pump schedule too short"

    def gpe_destroy(self, h):
        return 0


def test_iterator_extends_the_pump_schedule(gpe, monkeypatch):
    """The reference's iterator samples the pump at any time, so step! may run past
    tspan; the schedule on the device is extended, with the reference's sampling times."""
    fake = _FakeLib()
    monkeypatch.setattr(gpe._lib, "load", lambda path=None: fake)
    N, Lb, dt = 16, 8.0, 0.1
    amp = lambda t: min(t / 2.0, 1.0) * np.exp(0.2j * t)
    prob = gpe.GrossPitaevskiiProblem((np.zeros((N, N), np.complex128),), (Lb, Lb),
                                      dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                      pump=lambda r, p, t: amp(t) * np.exp(-((r[0] - 4) ** 2 + (r[1] - 4) ** 2)))
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 1.0), dt=dt, nsaves=2)
    assert len(fake.amps[0]) == 2 * 10 + 1
    gpe.step(it, 10)
    assert len(fake.amps[0]) == 21
    it.step(5)
    assert len(fake.amps[0]) >= 2 * 15 + 1
    times = gpe.pump_sample_times(0.0, it.dt, (len(fake.amps[0]) - 1) // 2)
    a = fake.amps[0]
    assert np.allclose(a / a[-1], np.array([amp(t) for t in times]) / amp(times[-1]), rtol=1e-12, atol=1e-15)
    it.close()


def test_noise_classification(gpe):
    from gpe_gb300.problem import classify_noise, direct_grid_axis
    axes = (direct_grid_axis(10.0, 16),)
    eta, prof = classify_noise(lambda u, r, p: 0.5, axes, None, 1, (16,))
    assert np.allclose(eta, [0.5]) and prof is None
    eta, prof = classify_noise(lambda u, r, p: [0.5, 0.25j], axes, None, 2, (16,))
    assert np.allclose(eta, [0.5, 0.25j]) and prof is None
    eta, prof = classify_noise(lambda u, r, p: 0.5 * np.exp(-r[0] ** 2), axes, None, 1, (16,))
    assert prof is not None and np.allclose(eta[0] * prof[0], 0.5 * np.exp(-axes[0] ** 2))
    with pytest.raises(NotImplementedError):
        classify_noise(lambda u, r, p: 0.1 * np.abs(u[0]), axes, None, 1, (16,))


def test_table_sampling_kinds(gpe):
    from gpe_gb300 import _lib as L
    from gpe_gb300.problem import sample_table, reciprocal_grid_axis
    ax = (reciprocal_grid_axis(8.0, 16), reciprocal_grid_axis(4.0, 32))
    v, k = sample_table(lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2, ax, None, 1)
    assert k == L.GPE_TABLE_SCALAR and v.shape == (1, 512)
    KX, KY = np.meshgrid(*ax, indexing="ij")
    assert np.array_equal(v[0], ((KX ** 2 + KY ** 2) / 2).ravel(order="F"))
    v, k = sample_table(lambda k, p: [[k[0], 1.0], [1.0, -0.1j]], ax, None, 2)
    assert k == L.GPE_TABLE_MATRIX and v.shape == (4, 512) and np.all(v[1] == 1.0)
    v, k = sample_table(lambda k, p: [k[0], k[1]], ax, None, 2)
    assert k == L.GPE_TABLE_DIAG
    v, k = sample_table(lambda k, p: [[(k[0] ** 2 + k[1] ** 2) / 2]], ax, None, 1)
    assert k == L.GPE_TABLE_SCALAR


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors (Random123 kat_vectors)."""
    kats = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
            ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
            ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
             (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kats:
        got = O.philox4x32_10(*[np.array([c], np.uint64) for c in ctr], *key)
        assert tuple(int(g[0]) for g in got) == want


def test_philox_noise_statistics():
    xi = O.PhiloxNoise(42, 2, (4,), (64, 64))(3)
    assert xi.shape == (2, 4, 64, 64)
    assert abs(np.mean(np.abs(xi) ** 2) - 1) < 0.02
    assert abs(np.mean(xi)) < 0.02
    assert abs(np.mean(xi.real ** 2) - 0.5) < 0.02 and abs(np.mean(xi.real * xi.imag)) < 0.02
    # independent streams per half step and per component
    assert np.abs(np.mean(xi[0] * np.conj(xi[1]))) < 0.02
    assert not np.allclose(O.PhiloxNoise(42, 1, (), (16,))(0), O.PhiloxNoise(42, 1, (), (16,))(1))


def test_autotune_picks_fastest_and_caches(gpe, tmp_path, monkeypatch):
    """The ensemble autotuner (host logic only: the ensemble is faked) times every
    (path, tiling, chunk) candidate, keeps the fastest, and answers from its cache next time."""
    import importlib
    A = importlib.import_module("gpe_gb300.autotune")
    T = importlib.import_module("gpe_gb300.twa")
    monkeypatch.setenv("GPE_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    cost = {(True, 0): 5.0, (False, 0): 3.0, (False, 1): 2.0}
    made = []

    class FakeIt:
        def __init__(self, resident, variant):
            self.cfg = (resident, variant)

        def close(self):
            pass

    class FakeEnsemble:
        def __init__(self, its):
            self.cfg = its[0].cfg
            self.ms = 0.0

        def run(self, nsteps, chunk):
            self.ms = cost[self.cfg] * nsteps + 100.0 / chunk

        def last_run_ms(self):
            return self.ms

        def close(self):
            pass

    monkeypatch.setattr(T, "Ensemble", FakeEnsemble)

    def make(resident, variant):
        made.append((resident, variant))
        return FakeIt(resident, variant)

    res, var, chunk, timings = A.tune(make, "k1", chunks=(10, 50, 200), trial_steps=200, variants=(0, 1))
    assert (res, var, chunk) == (False, 1, 200)
    assert len(timings) == 9 and len(made) == 9
    made.clear()
    assert A.tune(make, "k1", variants=(0, 1))[:3] == (False, 1, 200)
    assert not made  # answered from the cache


def test_autotune_leaves_out_a_resident_kernel_that_does_not_fit(gpe, tmp_path, monkeypatch):
    """Grids too large for the resident plane kernel are tuned over the two-pass tilings
    only, and a cached answer never claims the resident kernel for them."""
    import importlib
    A = importlib.import_module("gpe_gb300.autotune")
    T = importlib.import_module("gpe_gb300.twa")
    monkeypatch.setenv("GPE_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    assert A.resident_fits(128, 1, 8) and A.resident_fits(64, 2, 16)
    assert not A.resident_fits(256, 1, 8) and not A.resident_fits(128, 2, 16) and not A.resident_fits(8, 1, 8)
    made = []

    class FakeIt:
        def __init__(self, resident, variant):
            self.cfg = (resident, variant)

        def close(self):
            pass

    class FakeEnsemble:
        def __init__(self, its):
            self.cfg = its[0].cfg

        def run(self, nsteps, chunk):
            self.ms = (1.0 if self.cfg[0] else 2.0) * nsteps  # a "resident" run that would win

        def last_run_ms(self):
            return self.ms

        def close(self):
            pass

    monkeypatch.setattr(T, "Ensemble", FakeEnsemble)

    def make(resident, variant):
        made.append((resident, variant))
        return FakeIt(resident, variant)

    res, var, chunk, _ = A.tune(make, "k256", chunks=(50,), trial_steps=200, variants=(0,), resident_ok=False)
    assert res is False and all(not r for r, _ in made)
    # a cache entry from a tuner that did try it is not trusted for a grid that cannot fit
    A.tune(make, "kfits", chunks=(50,), trial_steps=200, variants=(0,))
    assert A.tune(make, "kfits", chunks=(50,), variants=(0,), resident_ok=False)[0] is False


def test_per_point_closures_match_array_closures(gpe):
    """Closures written for one point (math functions, branches on a coordinate), as
    grid_map! calls them (src/misc.jl:1-10), sample to the same tables and pumps as their
    array forms."""
    from gpe_gb300.problem import classify_pump, direct_grid_axis, reciprocal_grid_axis, sample_table
    L, N = 16.0, 32
    ax = (direct_grid_axis(L, N), direct_grid_axis(L, N))
    kax = (reciprocal_grid_axis(L, N), reciprocal_grid_axis(L, N))
    a, ka = sample_table(lambda k, p: 0.5 * (k[0] ** 2 + k[1] ** 2), kax, None, 1)
    b, kb = sample_table(lambda k, p: 0.5 * math.fsum(x * x for x in k), kax, None, 1)
    assert ka == kb and np.array_equal(a, b)
    a, _ = sample_table(lambda r, p: np.where(r[0] < 4, 1.0, 0.0), ax, None, 1)
    b, _ = sample_table(lambda r, p: 1.0 if r[0] < 4 else 0.0, ax, None, 1)
    assert np.array_equal(a, b)
    a, ka = sample_table(lambda k, p: [[k[0] ** 2, 1.0 + 0 * k[0]], [1.0 + 0 * k[0], math.sin(1.0) * k[1]]], kax, None, 2)
    b, kb = sample_table(lambda k, p: [[k[0] ** 2, 1.0], [1.0, math.sin(1.0) * float(k[1])]], kax, None, 2)
    assert ka == kb == gpe._lib.GPE_TABLE_MATRIX and np.array_equal(a, b)
    times = gpe.pump_sample_times(0.0, 0.1, 20)
    pa, aa = classify_pump(lambda r, p, t: [min(t, 1.0) * np.exp(-((r[0] - 8) ** 2 + (r[1] - 8) ** 2) / 9), 0],
                           ax, None, 2, times)
    pb, ab = classify_pump(lambda r, p, t: [min(t, 1.0) * math.exp(-((r[0] - 8) ** 2 + (r[1] - 8) ** 2) / 9), 0.0],
                           ax, None, 2, times)
    assert pb[1] is None
    assert np.allclose(aa[0][:, None] * pa[0][None], ab[0][:, None] * pb[0][None], rtol=1e-14, atol=1e-16)
    # closures that reduce over the point's coordinates (norm(r), the natural form of code
    # ported from Julia) run on the coordinate arrays without an error but reduce over the
    # whole grid there: they must still sample point by point
    a, ka = sample_table(lambda r, p: 0.5 * (r[0] ** 2 + r[1] ** 2), ax, None, 1)
    b, kb = sample_table(lambda r, p: 0.5 * np.linalg.norm(r) ** 2, ax, None, 1)
    assert ka == kb and np.allclose(a, b, rtol=1e-13, atol=0) and np.ptp(b.real) > 0
    pa, aa = classify_pump(lambda r, p, t: min(t, 1.0) * np.exp(-((r[0] - 8) ** 2 + (r[1] - 8) ** 2) / 9),
                           ax, None, 1, times)
    pb, ab = classify_pump(lambda r, p, t: min(t, 1.0) * np.exp(-np.linalg.norm(np.asarray(r) - 8.0) ** 2 / 9),
                           ax, None, 1, times)
    assert pb[0] is not None
    assert np.allclose(aa[0][:, None] * pa[0][None], ab[0][:, None] * pb[0][None], rtol=1e-13, atol=1e-16)
    for shape in ((16,), (16, 8, 4)):
        axes = tuple(direct_grid_axis(3.0 + a, n) for a, n in enumerate(shape))
        a, _ = sample_table(lambda r, p: np.exp(-sum((x - 1.0) ** 2 for x in r)) * (r[-1] + 1), axes, None, 1)
        b, _ = sample_table(lambda r, p: math.exp(-math.fsum((x - 1.0) ** 2 for x in r)) * (r[-1] + 1), axes, None, 1)
        assert np.allclose(a, b, rtol=1e-15, atol=0), shape


def test_solve_after_step_continues_from_the_handle(gpe, monkeypatch):
    """solve_ after step continues the handle's clock: its saves and times follow the k
    steps already taken, and the pump schedule is extended to cover them.  (The
    reference's solve! restarts t at tspan[1] while keeping the advanced field; the
    difference is documented with the iterator form of the C ABI.)"""
    fake = _FakeLib()
    monkeypatch.setattr(gpe._lib, "load", lambda path=None: fake)
    N, Lb, dt = 16, 8.0, 0.1
    prob = gpe.GrossPitaevskiiProblem((np.zeros((N, N), np.complex128),), (Lb, Lb),
                                      dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                      pump=lambda r, p, t: min(t, 1.0) * np.exp(-((r[0] - 4) ** 2 + (r[1] - 4) ** 2)))
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 1.0), dt=dt, nsaves=2)
    gpe.step(it, 3)
    ts, _ = gpe.solve_(it)
    assert fake.steps == 13
    assert np.allclose(ts, [0.0, 0.8, 1.3])  # u0's slot keeps t0; the saves follow the 3 steps taken
    assert len(fake.amps[0]) >= 2 * 13 + 1
    it.close()
