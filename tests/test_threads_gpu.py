"""Distinct handles driven from several host threads at once (ctypes releases the GIL
around each library call): every handle's result equals its run alone, bit for bit.
The handles differ in precision, components, dimension and noise, so their kernels,
launch shapes and shared-memory limits interleave on the device."""
import threading

import numpy as np
import pytest

from cases import jl

pytestmark = pytest.mark.gpu


def problems(gpe):
    rng = np.random.default_rng(4)

    def field(shape, dtype, scale=0.5):
        return (scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))).astype(dtype)

    out = []
    # two-component FP64 (double-word), 128^2 x 2, 2x2 dispersion, pump
    u = [jl(field((2, 128, 128), np.complex128)) for _ in range(2)]
    out.append((gpe.GrossPitaevskiiProblem(
        tuple(u), (64.0, 64.0),
        dispersion=lambda k, p: [[(k[0] ** 2 + k[1] ** 2) / 2 - 0.05j, 0.8 + 0 * k[0]], [0.8 + 0 * k[0], -0.01j + 0 * k[0]]],
        nonlinearity=lambda u, p: [0 * u[0], 0.3 * np.abs(u[1]) ** 2],
        pump=lambda r, p, t: [0.2 * np.exp(-((r[0] - 32) ** 2 + (r[1] - 32) ** 2) / 30.0), 0]), dict(fp64="dw")))
    # one-component FP32, 256^2 x 4, Philox noise
    out.append((gpe.GrossPitaevskiiProblem(
        (jl(field((4, 256, 256), np.complex64)),), (64.0, 64.0),
        dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.1j, nonlinearity=lambda u, p: 0.05 * np.abs(u[0]) ** 2,
        position_noise_func=lambda u, r, p: 0.1), dict(rng=77)))
    # 1D native FP64, 1024 points x 8
    out.append((gpe.GrossPitaevskiiProblem(
        (jl(field((8, 1024), np.complex128)),), (100.0,),
        dispersion=lambda k, p: k[0] ** 2 / 2, nonlinearity=lambda u, p: -0.5 * np.abs(u[0]) ** 2),
        dict(fp64="native")))
    # 3D FP32, 32 x 32 x 64
    out.append((gpe.GrossPitaevskiiProblem(
        (jl(field((32, 32, 64), np.complex64)),), (10.0, 10.0, 20.0),
        dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2 + k[2] ** 2) / 2, nonlinearity=lambda u, p: 0.2 * np.abs(u[0]) ** 2),
        dict()))
    return out


def run_one(gpe, prob, kw, steps, out, i):
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, steps * 0.01), dt=0.01, nsaves=1, **kw)
    for _ in range(steps // 5):
        it.step(5)
    out[i] = [np.array(f) for f in it.get_fields()]
    it.close()


def test_handles_in_parallel_threads(gpe, lib):
    probs = problems(gpe)
    steps = 40
    alone = [None] * len(probs)
    for i, (p, kw) in enumerate(probs):
        run_one(gpe, p, kw, steps, alone, i)
    together = [None] * len(probs)
    errors = []

    def worker(i):
        try:
            run_one(gpe, probs[i][0], probs[i][1], steps, together, i)
        except Exception as e:  # surfaced below
            errors.append(e)

    for rep in range(2):
        threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(probs))]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        assert not errors, errors
        for i in range(len(probs)):
            for a, b in zip(alone[i], together[i]):
                assert np.array_equal(a, b), (rep, i)
