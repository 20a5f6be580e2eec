"""The C ABI's argument checks: every misuse returns its GPE_ERR_* code with a message
(gpe_last_error), nothing crosses the ABI as an exception, and a handle that refused a
call keeps working: after a volley of bad calls it still steps to the same bits as a
fresh handle."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 64


def desc(L, **over):
    d = L.GpeDesc()
    d.abi_version = L.GPE_ABI_VERSION
    d.ndim = 2
    d.n[0], d.n[1], d.n[2] = N, N, 1
    d.lengths[0], d.lengths[1], d.lengths[2] = 10.0, 10.0, 1.0
    d.batch = 1
    d.ncomp = 1
    d.dtype = L.GPE_C128
    d.dt = 0.01
    d.t0 = 0.0
    d.device = 0
    d.flags = L.GPE_FLAG_NO_RESIDENT
    for k, v in over.items():
        if k == "n":
            d.n[0], d.n[1], d.n[2] = v
        else:
            setattr(d, k, v)
    return d


def create(lib, L, **over):
    h = ctypes.c_void_p()
    rc = lib.gpe_create(ctypes.byref(desc(L, **over)), ctypes.byref(h))
    return rc, h


def configure(lib, L, h):
    k = 2 * np.pi * np.fft.fftfreq(N, 10.0 / N)
    KX, KY = np.meshgrid(k, k, indexing="xy")  # [y][x], x fastest
    D = np.ascontiguousarray(((KX ** 2 + KY ** 2) / 2 + 0j).ravel())
    assert lib.gpe_set_dispersion(h, D.ctypes.data, 1) == L.GPE_OK
    g = np.array([0.5, 0.0])
    assert lib.gpe_set_nonlinearity(h, g.ctypes.data, None) == L.GPE_OK
    x = np.arange(N) * (10.0 / N)
    X, Y = np.meshgrid(x, x, indexing="xy")
    u = np.ascontiguousarray(np.exp(-((X - 5) ** 2 + (Y - 5) ** 2)).astype(np.complex128).ravel())
    assert lib.gpe_set_field(h, 0, u.ctypes.data) == L.GPE_OK
    return u


def field(lib, h):
    out = np.empty(N * N, np.complex128)
    lib.gpe_get_field(h, 0, out.ctypes.data)
    return out


def test_create_rejects_bad_descriptors(gpe, lib):
    L = gpe._lib
    bad = [dict(abi_version=999), dict(ndim=0), dict(ndim=4), dict(n=(100, N, 1)), dict(n=(8, N, 1)),
           dict(n=(N, 2 ** 13, 1)), dict(batch=0), dict(ncomp=3), dict(dtype=7), dict(dt=0.0), dict(dt=float("nan")),
           dict(lengths=(ctypes.c_double * 3)(-1.0, 10.0, 1.0))]
    for over in bad:
        rc, h = create(lib, L, **over)
        assert rc in (L.GPE_ERR_INVALID, L.GPE_ERR_UNSUPPORTED), (over, rc)
        assert not h.value, over
        assert lib.gpe_last_error(None), over


def test_bad_calls_leave_the_handle_working(gpe, lib):
    L = gpe._lib
    rc, h = create(lib, L)
    assert rc == L.GPE_OK
    u = configure(lib, L, h)
    nanf = u.copy()
    nanf[7] = np.nan
    z = np.zeros(N * N * 2)
    calls = [
        (lib.gpe_set_field(h, 1, u.ctypes.data), L.GPE_ERR_INVALID),           # no component 1
        (lib.gpe_set_field(h, 0, None), L.GPE_ERR_INVALID),
        (lib.gpe_set_field(h, 0, nanf.ctypes.data), L.GPE_ERR_NONFINITE),      # refused, state kept
        (lib.gpe_set_dispersion(h, z.ctypes.data, 9), L.GPE_ERR_INVALID),      # no table kind 9
        (lib.gpe_set_nonlinearity(h, np.array([np.inf, 0.0]).ctypes.data, None), L.GPE_ERR_NONFINITE),
        (lib.gpe_set_pump(h, 0, np.ones(N * N).ctypes.data, 0, None, 0), L.GPE_ERR_INVALID),  # no amplitudes
        (lib.gpe_set_variant(h, 5), L.GPE_ERR_INVALID),
        (lib.gpe_set_variant(h, 1), L.GPE_ERR_UNSUPPORTED),                     # FP32 one-component only
        (lib.gpe_run(h, -1, 0, None, None), L.GPE_ERR_INVALID),
        (lib.gpe_run(h, 10, 3, z.ctypes.data, None), L.GPE_ERR_INVALID),       # 10 not a multiple of 3
        (lib.gpe_run(h, 10, 5, None, None), L.GPE_ERR_INVALID),                # saves need a buffer
        (lib.gpe_run_replay(h, 4, 0, None, None, None), L.GPE_ERR_INVALID),    # no replay draws
        (lib.gpe_set_graph(h, -3), L.GPE_ERR_INVALID),
        (lib.gpe_norm(h, None), L.GPE_ERR_INVALID),
        (lib.gpe_spectral_moments(h, 0, None, None), L.GPE_ERR_INVALID),
        (lib.gpe_spectral_moments(h, 2, z.ctypes.data, None), L.GPE_ERR_INVALID),
    ]
    for i, (rc, want) in enumerate(calls):
        assert rc == want, (i, rc, want, lib.gpe_last_error(h))
        assert lib.gpe_last_error(h), i
    # the handle still steps exactly like a fresh one
    assert lib.gpe_run(h, 8, 0, None, None) == L.GPE_OK
    got = field(lib, h)
    lib.gpe_destroy(h)
    rc, h2 = create(lib, L)
    configure(lib, L, h2)
    assert lib.gpe_run(h2, 8, 0, None, None) == L.GPE_OK
    want = field(lib, h2)
    lib.gpe_destroy(h2)
    assert np.array_equal(got, want)


def test_refused_setters_keep_the_old_settings(gpe, lib):
    """A refused pump or noise call leaves the previous pump / noise in place: the run
    afterwards equals the run of a handle that never saw the bad call."""
    L = gpe._lib
    amp = np.zeros(2 * 41)
    amp[0::2] = 0.7
    eta = np.array([0.05, 0.0])
    outs = []
    for bad in (False, True):
        rc, h = create(lib, L)
        configure(lib, L, h)
        assert lib.gpe_set_pump(h, 0, np.ones(N * N).ctypes.data, 0, amp.ctypes.data, 41) == L.GPE_OK
        assert lib.gpe_set_noise(h, L.GPE_NOISE_PHILOX, 9, eta.ctypes.data, None) == L.GPE_OK
        if bad:
            nan_amp = amp.copy()
            nan_amp[4] = np.nan
            assert lib.gpe_set_pump(h, 0, np.ones(N * N).ctypes.data, 0, nan_amp.ctypes.data, 41) == L.GPE_ERR_NONFINITE
            assert lib.gpe_set_pump(h, 0, np.ones(N * N).ctypes.data, 0, None, 0) == L.GPE_ERR_INVALID
            assert lib.gpe_set_noise(h, L.GPE_NOISE_PHILOX, 3, None, None) == L.GPE_ERR_INVALID
            assert lib.gpe_set_noise(h, L.GPE_NOISE_PHILOX, 3, np.array([np.inf, 0]).ctypes.data,
                                     None) == L.GPE_ERR_NONFINITE
        assert lib.gpe_run(h, 20, 0, None, None) == L.GPE_OK
        outs.append(field(lib, h))
        lib.gpe_destroy(h)
    assert np.array_equal(outs[0], outs[1])


def test_pump_amplitudes_must_cover_the_run(gpe, lib):
    L = gpe._lib
    rc, h = create(lib, L)
    configure(lib, L, h)
    amp = np.zeros(2 * 9)  # a(t) at 9 sampling times: enough for 4 steps
    amp[0::2] = 1.0
    assert lib.gpe_set_pump(h, 0, np.ones(N * N).ctypes.data, 0, amp.ctypes.data, 9) == L.GPE_OK
    assert lib.gpe_run(h, 4, 0, None, None) == L.GPE_OK
    assert lib.gpe_run(h, 1, 0, None, None) == L.GPE_ERR_INVALID  # step 5 has no amplitude
    lib.gpe_destroy(h)


def test_energy_refuses_the_matrix_family(gpe, lib):
    L = gpe._lib
    rc, h = create(lib, L, ncomp=2)
    assert rc == L.GPE_OK
    g = np.zeros(16)
    g[0] = 0.3
    assert lib.gpe_set_matrix_nonlinearity(h, g.ctypes.data, None) == L.GPE_OK
    out = np.zeros(4)
    assert lib.gpe_energy(h, out.ctypes.data) == L.GPE_ERR_UNSUPPORTED
    lib.gpe_destroy(h)
