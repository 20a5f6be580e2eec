"""The precision sweep at its full configuration: 2D Kerr on 2048^2, L = 32,
u0 = exp(-|r - r0|^2 / 2^2) with r0 = (16, 16), D = |k|^2/2, G = g|u|^2 for g = +1 (smooth)
and g = -2 (a packet driven past the 2D collapse threshold, which amplifies every rounding
difference), dt = 0.005, 1000 steps, 20 saves.  Every save of the GPU path is compared with
the FP64 oracle (the C restatement, pinned to the numpy oracle by tests/test_oracle_c.py):

* ComplexF64 fields in the default native FP64 arithmetic, and with the line transforms in
  block floating point ("bfp"): rel L2 <= 1e-10 at every save;
* the opt-in double-word mode (unit roundoff 2^-48, 32x FP64's): rel L2 <= 1e-10 at every
  save of the smooth case; on the collapsing case it reaches 5e-10 at the collapse (native
  FP64: 5e-11), so there it is held to 1e-9 and does not meet the 1e-10 bar -- runs that
  need the bar on such problems use the default native FP64;
* ComplexF32 fields: rel L2 <= 1e-5 at every save where the reference's own ComplexF32
  arithmetic (single-precision FFTs, FP64 table products rounded to single precision; the
  C oracle's fp32 mode) stays within 1e-5 of FP64, and within 2x that reference FP32 error
  where the reference's FP32 arithmetic itself does not reach 1e-5.

Norm and energy drifts are printed for every mode; for g = +1 the FP64 norm is conserved
to rounding (the split step is unitary for real D and G)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, LBOX, DT, NSTEPS, NSAVES = 2048, 32.0, 0.005, 1000, 20
PER = NSTEPS // NSAVES
_cache = {}


def oracle_saves(g: float, fp32: bool):
    """(NSAVES, ny, nx) complex128 saves of the C oracle, FP64 or the reference's FP32."""
    key = (g, fp32)
    if key not in _cache:
        from oracle import gpe_oracle as O
        from oracle import gpe_oracle_c as OC
        X, Y = O.mesh(O.grids((LBOX, LBOX), (N, N))[0])
        u0 = np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0).astype(np.complex128)
        prob = O.OracleProblem(u0=(u0,), lengths=(LBOX, LBOX), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                               nonlin_g=np.array([[g]]))
        it = OC.CIterator(prob, (0.0, NSTEPS * DT), DT, NSAVES, fp32=fp32)
        _cache[key] = it.step(NSTEPS, PER)[0]
    return _cache[key]


def gpu_run(gpe, g: float, dtype, fp64: str):
    """Saves (as FP64 arrays [y][x]), norms and energies of the GPU path, save by save."""
    x = np.arange(N) * (LBOX / N)
    X, Y = np.meshgrid(x, x, indexing="ij")  # the reference's order: x first
    u0 = np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0).astype(dtype)
    prob = gpe.GrossPitaevskiiProblem((u0,), (LBOX, LBOX), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                      nonlinearity=lambda u, p: g * np.abs(u[0]) ** 2)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, NSTEPS * DT), dt=DT, nsaves=NSAVES, fp64=fp64)
    try:
        n0, e0 = it.norm()[0], it.energy().sum()
        out = []
        for s in range(NSAVES):
            it.step(PER)
            u = np.ascontiguousarray(it.get_fields()[0].T).astype(np.complex128)
            out.append((u, it.norm()[0] / n0 - 1, (it.energy().sum() - e0) / abs(e0)))
        return out
    finally:
        it.close()


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(a), np.linalg.norm(b)))


@pytest.mark.parametrize("g", [1.0, -2.0], ids=["g+1", "g-2"])
@pytest.mark.parametrize("fp64", ["native", "bfp", "dw"], ids=["f64", "f64-bfp", "f64-dw"])
def test_c3_fp64_every_save(gpe, lib, g, fp64):
    ref = oracle_saves(g, False)
    runs = gpu_run(gpe, g, np.complex128, fp64)
    errs = [rel_l2(u, ref[s]) for s, (u, _, _) in enumerate(runs)]
    print(f"C3 g={g:+.0f} {fp64}: rel L2 per save {['%.2e' % e for e in errs]}; "
          f"norm drift {runs[-1][1]:.2e}, energy drift {runs[-1][2]:.2e}")
    assert max(errs) <= (1e-9 if fp64 == "dw" and g < 0 else 1e-10), errs
    if g > 0:
        assert max(abs(r[1]) for r in runs) <= 1e-11


@pytest.mark.parametrize("g", [1.0, -2.0], ids=["g+1", "g-2"])
def test_c3_fp32_every_save(gpe, lib, g):
    ref = oracle_saves(g, False)
    ref32 = oracle_saves(g, True)
    runs = gpu_run(gpe, g, np.complex64, "native")
    errs = [rel_l2(u, ref[s]) for s, (u, _, _) in enumerate(runs)]
    errs_ref32 = [rel_l2(ref32[s], ref[s]) for s in range(NSAVES)]
    print(f"C3 g={g:+.0f} f32: rel L2 per save {['%.2e' % e for e in errs]}; reference FP32 arithmetic "
          f"{['%.2e' % e for e in errs_ref32]}; norm drift {runs[-1][1]:.2e}, energy drift {runs[-1][2]:.2e}")
    for s in range(NSAVES):
        bound = 1e-5 if errs_ref32[s] <= 1e-5 else 2.0 * errs_ref32[s]
        assert errs[s] <= bound, (s, errs[s], errs_ref32[s])
