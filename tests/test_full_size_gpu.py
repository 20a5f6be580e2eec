"""Full-size and edge-size checks: the benchmark configurations themselves (512^2
two-component polariton with 64 copies, 1024^2 and 2048^2 scalar Kerr), the longest
supported lines (4096 points along x and along y), and properties that hold at any size
(copies of one field stay bit-identical, a unitary step conserves the norm)."""
import numpy as np
import pytest

from cases import c_order, jl, polariton2d
from test_parity_gpu import PREC_IDS, PRECISIONS, TOL, assert_close, fp32_tol, run_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,fp64", PRECISIONS, ids=PREC_IDS)
@pytest.mark.parametrize("shape_c", [(16, 4096), (4096, 16)], ids=["x4096", "y4096"])
def test_longest_lines(gpe, oracle, lib, dtype, fp64, shape_c):
    """4096-point lines, the longest a pass supports, along x (row pass) and y (column pass)."""
    ny, nx = shape_c
    L = (64.0, 64.0 * ny / nx)
    X, Y = oracle.mesh(oracle.grids(L, (nx, ny))[0])
    u0c = (np.exp(-((X - L[0] / 2) ** 2 + (Y - L[1] / 2) ** 2) / 8) * (1 + 0.3j * np.sin(X))).astype(np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2
    gkw = dict(u0=(jl(u0c).astype(dtype),), lengths=L, dispersion=disp,
               nonlinearity=lambda u, p: 0.7 * np.abs(u[0]) ** 2)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=L, dispersion=disp, nonlin_g=np.array([[0.7]]))
    tspan, dt, ns = (0.0, 0.05), 0.005, 2
    ts, res, ots, ores = run_both(gpe, oracle, gkw, orc, tspan, dt, ns, fp64=fp64)
    tol = TOL[dtype] if dtype == np.complex128 else fp32_tol(oracle, orc, tspan, dt, ns)
    assert_close(oracle, res, ores, tol)


@pytest.mark.parametrize("fp64", ["dw", "native", "bfp"])
def test_polariton_bench_config_full_batch(gpe, oracle, lib, fp64):
    """The throughput workload as benchmarked (512^2, two components, 64 copies): every
    copy equals the single-copy run bit for bit, and that run matches the oracle."""
    N, B, nsteps = 512, 64, 20
    gkw, orc = polariton2d(N=N, L=256.0, A=5.0, ramp=200.0)
    one = gpe.init(gpe.GrossPitaevskiiProblem(**gkw), gpe.StrangSplitting(), (0.0, nsteps * 0.05), dt=0.05,
                   nsaves=1, fp64=fp64, variant=0)  # the batch's tiling (one field alone would take the fine one)
    one.step(nsteps)
    f1 = one.get_fields()
    one.close()
    bkw = dict(gkw)
    bkw["u0"] = tuple(np.asfortranarray(np.repeat(u[:, :, None], B, axis=2)) for u in gkw["u0"])
    many = gpe.init(gpe.GrossPitaevskiiProblem(**bkw), gpe.StrangSplitting(), (0.0, nsteps * 0.05), dt=0.05,
                    nsaves=1, fp64=fp64)
    many.step(nsteps)
    fb = many.get_fields()
    many.close()
    for m in range(2):
        for b in range(B):
            assert np.array_equal(fb[m][:, :, b], f1[m]), (m, b)
    ots, ores = oracle.solve(orc, (0.0, nsteps * 0.05), 0.05, 1)
    for m in range(2):
        assert oracle.rel_l2(c_order(f1[m]), ores[m, -1]) <= 1e-10


def kerr_gaussian(gpe, N, dtype, g=1.0):
    x = np.arange(N) * (32.0 / N)
    X, Y = np.meshgrid(x, x, indexing="ij")
    u0 = np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0).astype(dtype)
    return gpe.GrossPitaevskiiProblem((np.asfortranarray(u0),), (32.0, 32.0),
                                      dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                      nonlinearity=lambda u, p: g * np.abs(u[0]) ** 2)


@pytest.mark.parametrize("fp64", ["dw", "native", "bfp"])
def test_kerr1024_target_point_matches_oracle(gpe, oracle, lib, fp64):
    """The scalar Kerr 1024^2 FP64 point of the performance target, 10 steps."""
    N, dt, nsteps = 1024, 0.005, 10
    prob = kerr_gaussian(gpe, N, np.complex128)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, nsteps * dt), dt=dt, nsaves=1, fp64=fp64)
    it.step(nsteps)
    got = c_order(it.get_fields()[0])
    it.close()
    X, Y = oracle.mesh(oracle.grids((32.0, 32.0), (N, N))[0])
    u0c = np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0).astype(np.complex128)
    orc = oracle.OracleProblem(u0=(u0c,), lengths=(32.0, 32.0), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                               nonlin_g=np.array([[1.0]]))
    ots, ores = oracle.solve(orc, (0.0, nsteps * dt), dt, 1)
    assert oracle.rel_l2(got, ores[0, -1]) <= 1e-10


@pytest.mark.parametrize("dtype,fp64,tol", [(np.complex128, "dw", 1e-12), (np.complex128, "native", 1e-12),
                                            (np.complex128, "bfp", 1e-12), (np.complex64, "dw", 5e-5)], ids=PREC_IDS)
def test_kerr2048_norm_is_conserved(gpe, lib, dtype, fp64, tol):
    """Real D and G make every split step unitary: the norm of the 2048^2 field is
    conserved to rounding over 100 steps (the precision-sweep grid)."""
    it = gpe.init(kerr_gaussian(gpe, 2048, dtype, g=-2.0), gpe.StrangSplitting(), (0.0, 0.5), dt=0.005, nsaves=1,
                  fp64=fp64)
    n0 = it.norm()[0]
    it.step(100)
    n1 = it.norm()[0]
    it.close()
    assert abs(n1 / n0 - 1) <= tol


@pytest.mark.parametrize("fp64", ["dw", "native", "bfp"])
def test_polariton_full_length_run(gpe, oracle, lib, fp64):
    """The polariton configuration over its full length (tspan (0, 200), dt 0.05: 4000
    steps, 100 saves, the pump ramp over the whole span) on a 128^2 grid: the error
    stays at rounding level over every save, no drift."""
    gkw, orc = polariton2d(N=128, L=256.0, A=5.0, ramp=200.0)
    ts, res = gpe.solve(gpe.GrossPitaevskiiProblem(**gkw), gpe.StrangSplitting(), (0.0, 200.0), dt=0.05,
                        nsaves=100, fp64=fp64)
    ots, ores = oracle.solve(orc, (0.0, 200.0), 0.05, 100)
    assert np.array_equal(ts, ots)
    assert_close(oracle, res, ores, 1e-10)


_C1 = {}


def _c1_oracle(oracle, fp32: bool):
    """Saves of the C oracle on the polariton configuration at its own size (512^2,
    tspan (0, 200), dt 0.05: 4000 steps, 100 saves), FP64 or the reference's FP32."""
    if fp32 not in _C1:
        from oracle import gpe_oracle_c as OC
        _, orc = polariton2d(N=512, L=256.0, A=5.0, ramp=200.0)
        _C1[fp32] = OC.solve(orc, (0.0, 200.0), 0.05, 100, fp32=fp32)
    return _C1[fp32]


@pytest.mark.parametrize("dtype,fp64", [(np.complex128, "native"), (np.complex128, "bfp"), (np.complex64, "native")],
                         ids=["f64", "f64-bfp", "f32"])
def test_polariton_c1_full_size_every_save(gpe, oracle, lib, dtype, fp64):
    """The polariton configuration exactly as specified (512^2, two components, 2x2
    dispersion, pump ramp over t in [0, 200], 4000 steps, 100 saves) against the C oracle
    at every save: ComplexF64 <= 1e-10; ComplexF32 <= 1e-5 where the reference's own
    ComplexF32 arithmetic (the C oracle's fp32 mode) stays within 1e-5, else within 2x it."""
    gkw, _ = polariton2d(N=512, L=256.0, A=5.0, ramp=200.0, dtype=dtype)
    ts, res = gpe.solve(gpe.GrossPitaevskiiProblem(**gkw), gpe.StrangSplitting(), (0.0, 200.0), dt=0.05,
                        nsaves=100, fp64=fp64)
    ots, ores = _c1_oracle(oracle, False)
    assert np.array_equal(ts, ots)
    got = np.stack([c_order(r) for r in res], 0).astype(np.complex128)  # (M, nsaves+1, y, x)
    errs = [oracle.rel_l2(got[:, s], ores[:, s]) for s in range(1, 101)]
    if dtype == np.complex128:
        print(f"C1 f64: worst save {max(errs):.2e}")
        assert max(errs) <= 1e-10, max(errs)
        return
    _, r32 = _c1_oracle(oracle, True)
    ref32 = [oracle.rel_l2(r32[:, s], ores[:, s]) for s in range(1, 101)]
    print(f"C1 f32: worst save {max(errs):.2e}, reference FP32 arithmetic worst {max(ref32):.2e}")
    for s in range(100):
        bound = 1e-5 if ref32[s] <= 1e-5 else 2.0 * ref32[s]
        assert errs[s] <= bound, (s, errs[s], ref32[s])
