"""TMA-staged column passes (cp.async.bulk.tensor into shared memory, the next tile in
flight while the current one is transformed) against the plain per-thread loads: the
same arithmetic on the same data, so the fields must agree bit for bit, in every
precision, for one and two components, square and rectangular grids, short lines (one
box per tile) and batches.  Also the bounded device wait: a wait that nothing completes
returns GPE_ERR_TIMEOUT and leaves the context usable."""
import numpy as np
import pytest

from cases import jl

pytestmark = pytest.mark.gpu


def run(gpe, shape, M, B, dtype, fp64, tma, steps=6, seed=0):
    rng = np.random.default_rng(seed)
    L = (20.0, 24.0)
    u0 = []
    for m in range(M):
        f = (rng.standard_normal((B,) + shape) + 1j * rng.standard_normal((B,) + shape)) * (0.8 - 0.2 * m)
        u0.append(jl(f if B > 1 else f[0]).astype(dtype))
    if M == 1:
        disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.05j
        nl = lambda u, p: 0.4 * np.abs(u[0]) ** 2
    else:
        disp = lambda k, p: [[(k[0] ** 2 + k[1] ** 2) / 2 - 0.05j, 0.7 + 0 * k[0]], [0.7 + 0 * k[0], -0.01j + 0 * k[0]]]
        nl = lambda u, p: [0 * u[0], 0.3 * np.abs(u[1]) ** 2]
    prob = gpe.GrossPitaevskiiProblem(tuple(u0), L, dispersion=disp, nonlinearity=nl)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, steps * 0.01), dt=0.01, nsaves=1, fp64=fp64, resident=False,
                  tma=tma)
    it.step(steps)
    out = [np.array(f) for f in it.get_fields()]
    it.close()
    return out


CASES = [
    # (shape C order (y, x), M, B, dtype, fp64)
    ((512, 512), 2, 2, np.complex128, "dw"),
    ((512, 512), 2, 2, np.complex64, "dw"),
    ((512, 512), 2, 1, np.complex128, "native"),
    ((256, 256), 1, 3, np.complex64, "dw"),
    ((512, 256), 1, 2, np.complex128, "dw"),
    ((128, 64), 2, 3, np.complex128, "dw"),
    ((16, 64), 2, 2, np.complex64, "dw"),
    ((32, 128), 1, 2, np.complex128, "native"),
]


@pytest.mark.parametrize("shape,M,B,dtype,fp64", CASES, ids=[f"{c[0][0]}x{c[0][1]}-m{c[1]}-b{c[2]}-"
                                                              f"{np.dtype(c[3]).name}-{c[4]}" for c in CASES])
def test_tma_columns_bit_identical(gpe, lib, shape, M, B, dtype, fp64):
    a = run(gpe, shape, M, B, dtype, fp64, tma=True)
    b = run(gpe, shape, M, B, dtype, fp64, tma=False)
    for x, y in zip(a, b):
        assert np.isfinite(x).all()
        assert np.array_equal(x, y)


@pytest.mark.parametrize("shape,M,B,dtype", [((512, 512), 2, 64, np.complex128), ((512, 512), 2, 64, np.complex64),
                                               ((256, 256), 1, 341, np.complex64)], ids=["m2-dw", "m2-f32", "m1-f32"])
def test_tma_many_tiles_per_cta(gpe, lib, shape, M, B, dtype):
    """Batches whose every CTA streams tens of tiles, each refilling the staging buffer
    that its threads just read (the fence between those reads and the next copy is what
    keeps the results exact); the default rule (tma=None) stages the one-component case."""
    for rep in range(2):
        a = run(gpe, shape, M, B, dtype, "dw", tma=True, steps=12, seed=rep)
        b = run(gpe, shape, M, B, dtype, "dw", tma=False, steps=12, seed=rep)
        c = run(gpe, shape, M, B, dtype, "dw", tma=None, steps=12, seed=rep)
        for x, y, z in zip(a, b, c):
            assert np.array_equal(x, y)
            assert np.array_equal(x, z)


def test_bounded_wait_times_out_and_context_survives(gpe, lib):
    L = gpe._lib
    assert lib.gpe_selftest_wait(0, 1, 10 ** 9) == L.GPE_OK
    assert lib.gpe_selftest_wait(0, 0, 2 * 10 ** 6) == L.GPE_ERR_TIMEOUT
    # a limit above the library's own 1 s bound is refused before anything is launched
    assert lib.gpe_selftest_wait(0, 0, 10 ** 9 + 1) == L.GPE_ERR_INVALID
    assert lib.gpe_selftest_wait(0, 0, 2 ** 62) == L.GPE_ERR_INVALID
    # the context still runs a solve afterwards
    a = run(gpe, (64, 64), 2, 1, np.complex128, "dw", tma=True, steps=2)
    assert all(np.isfinite(x).all() for x in a)
