"""The code paths that the default FP64 mode picks by problem and size, checked against
the paths they stand in for:

* the pipelined row pass (one-component FP64 lines in large batches: two line groups of a
  block half a cycle apart) against the one-block-one-program row pass, bit for bit: every
  copy of a batch that takes it equals a single-copy run that does not;
* the compile-time specialised half step of the common families (Kerr, the polariton)
  against the generic one, which the same problem takes once a potential table is present
  (a zero potential: its table is exp(0) = 1, so the arithmetic is the same up to the
  phase polynomial's tier and the pump terms' merging, a few units of FP64 rounding);
* the k-space table applied in Q62 fixed point between the column transforms against FP64
  floating point transforms with the FP64 table, and both against the oracle."""
import numpy as np
import pytest

from cases import c_order, polariton2d

pytestmark = pytest.mark.gpu


def kerr(gpe, N, B=1, potential=None, g=1.0):
    x = np.arange(N) * (32.0 / N)
    X, Y = np.meshgrid(x, x, indexing="ij")
    u0 = (np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0) * (1 + 0.2j * np.sin(X))).astype(np.complex128)
    if B > 1:
        u0 = np.repeat(u0[:, :, None], B, axis=2)
    return gpe.GrossPitaevskiiProblem((np.asfortranarray(u0),), (32.0, 32.0),
                                      dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                      nonlinearity=lambda u, p: g * np.abs(u[0]) ** 2, potential=potential)


def run(gpe, prob, nsteps, dt, fp64="bfp"):
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, nsteps * dt), dt=dt, nsaves=1, fp64=fp64)
    try:
        it.step(nsteps)
        return it.get_fields()
    finally:
        it.close()


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(a), np.linalg.norm(b)))


def test_pipelined_row_pass_equals_single_copy_run(gpe, oracle, lib):
    """512^2 Kerr, 16 copies (8192 lines: the pipelined row pass) against one copy (512
    lines: the plain row pass), 30 steps: every copy bit for bit; the single run against
    the oracle at 1e-10."""
    N, B, dt, nsteps = 512, 16, 0.005, 30
    one = run(gpe, kerr(gpe, N), nsteps, dt)[0]
    many = run(gpe, kerr(gpe, N, B), nsteps, dt)[0]
    for b in range(B):
        assert np.array_equal(many[:, :, b], one), b
    X, Y = oracle.mesh(oracle.grids((32.0, 32.0), (N, N))[0])
    u0c = (np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0) * (1 + 0.2j * np.sin(X))).astype(np.complex128)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(32.0, 32.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                               nonlin_g=np.array([[1.0]]))
    _, ores = oracle.solve(orc, (0.0, nsteps * dt), dt, 1)
    assert oracle.rel_l2(c_order(one), ores[0, -1]) <= 1e-10


@pytest.mark.parametrize("fp64", ["bfp", "native"])
def test_lean_half_step_matches_generic_kerr(gpe, lib, fp64):
    """Kerr 256^2 (G = 4|u|^2: phases up to 0.01, the 2^-10 and 2^-6 tiers both in use),
    200 steps: the specialised half step against the generic one within 1e-13."""
    N, dt, nsteps = 256, 0.005, 200
    lean = run(gpe, kerr(gpe, N, g=4.0), nsteps, dt, fp64)[0]
    gen = run(gpe, kerr(gpe, N, g=4.0, potential=lambda r, p: 0 * r[0]), nsteps, dt, fp64)[0]
    e = rel(lean, gen)
    print(f"Kerr lean vs generic ({fp64}): {e:.2e}")
    assert e <= 1e-13


@pytest.mark.parametrize("fp64", ["bfp", "native"])
def test_lean_half_step_matches_generic_polariton(gpe, lib, fp64):
    """Polariton 128^2 from u = 0 under the pump ramp, 300 steps: the specialised half step
    against the generic one within 1e-12 on both components.  The photon, driven from zero,
    differs most (1e-13 on GB300): the specialised step adds its two pump terms as one, the
    generic one around the potential's unit factor."""
    gkw, _ = polariton2d(N=128, L=256.0, A=5.0, ramp=20.0)
    nsteps, dt = 300, 0.05
    lean = run(gpe, gpe.GrossPitaevskiiProblem(**gkw), nsteps, dt, fp64)
    gkw2 = dict(gkw)
    gkw2["potential"] = lambda r, p: [0 * r[0], 0 * r[0]]
    gen = run(gpe, gpe.GrossPitaevskiiProblem(**gkw2), nsteps, dt, fp64)
    for m in range(2):
        e = rel(lean[m], gen[m])
        print(f"polariton comp {m} lean vs generic ({fp64}): {e:.2e}")
        assert e <= 1e-12


def test_fixed_point_table_matches_fp64_table(gpe, oracle, lib):
    """Polariton 256^2, 200 steps: the default mode (Q62 k-space table between fixed point
    transforms) against FP64 floating point transforms with the FP64 table within 1e-12,
    and both against the oracle at 1e-10."""
    gkw, orc = polariton2d(N=256, L=256.0, A=5.0, ramp=20.0)
    nsteps, dt = 200, 0.05
    fx = run(gpe, gpe.GrossPitaevskiiProblem(**gkw), nsteps, dt, "bfp")
    fl = run(gpe, gpe.GrossPitaevskiiProblem(**gkw), nsteps, dt, "native")
    _, ores = oracle.solve(orc, (0.0, nsteps * dt), dt, 1)
    for m in range(2):
        assert rel(fx[m], fl[m]) <= 1e-12
        assert oracle.rel_l2(c_order(fx[m]), ores[m, -1]) <= 1e-10
        assert oracle.rel_l2(c_order(fl[m]), ores[m, -1]) <= 1e-10
