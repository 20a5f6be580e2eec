"""The plain cuFFT split step that bench.py times beside the fused passes (PlainSplitStep)
computes the reference's step: against the FP64 oracle on a pumped two-component
polariton with a nonlinear phase that matters, at 1e-10 rel L2 in FP64 (on the CPU
through torch's own FFT, and on the GPU through cuFFT)."""
import numpy as np
import pytest


def _case(oracle, N, B, steps, seed=3):
    import bench
    prm = dict(bench.POL, ramp=2.0, A=5.0)
    L, dt = 256.0, bench.DT
    rng = np.random.default_rng(seed)
    x = np.arange(N) * (L / N)
    Y, X = np.meshgrid(x, x, indexing="ij")
    env = np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / 60.0 ** 2)
    u0 = np.stack([np.stack([env * (3 + 2 * rng.standard_normal((N, N))) * np.exp(1j * rng.uniform(0, 6.3, (N, N)))
                             for _ in range(B)]) for _ in range(2)]).astype(np.complex128)
    dg, _ = oracle.grids((L, L), (N, N))
    Xo, Yo = oracle.mesh(dg)
    prof = np.exp(-((Xo - L / 2) ** 2 + (Yo - L / 2) ** 2) / prm["w"] ** 2)

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        one = np.ones_like(k2)
        return np.array([[prm["hbar"] * k2 / (2 * prm["m"]) - prm["dc"] - 1j * prm["gc"], prm["Om"] * one],
                         [prm["Om"] * one, (-prm["dx"] - 1j * prm["gx"]) * one]])

    prob = oracle.OracleProblem(u0=(u0[0], u0[1]), lengths=(L, L), dispersion=disp,
                                nonlin_g=np.array([[0, 0], [0, prm["g"]]], np.complex128),
                                pump_profile=np.stack([prof, 0 * prof]).astype(np.complex128),
                                pump_amp=lambda t: np.array([prm["A"] * min(t / prm["ramp"], 1.0), 0.0]))
    _, res = oracle.solve(prob, (0.0, steps * dt), dt, 1)
    return bench, prm, u0, res[:, -1]


def _check(oracle, dtype, tol, device, N):
    B, steps = 2, 40
    bench, prm, u0, ref = _case(oracle, N, B, steps)
    ps = bench.PlainSplitStep(N, 256.0, B, dtype, device, u0=u0.astype(dtype), prm=prm)
    ps.step(steps)
    got = ps.u.cpu().numpy().astype(np.complex128)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err <= tol, err
    # the transforms alone are an identity up to rounding
    ps.u = ps.u.new_tensor(u0.astype(dtype))
    ps.fft_only(2)
    back = ps.u.cpu().numpy().astype(np.complex128)
    assert np.linalg.norm(back - u0) / np.linalg.norm(u0) <= (1e-14 if dtype == np.complex128 else 1e-6)


CASES = [(np.complex128, 1e-10), (np.complex64, 1e-4)]


@pytest.mark.parametrize("dtype,tol", CASES, ids=["f64", "f32"])
def test_plain_split_step_matches_oracle_cpu(oracle, dtype, tol):
    _check(oracle, dtype, tol, "cpu", 32)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,tol", CASES, ids=["f64", "f32"])
def test_plain_split_step_matches_oracle_gpu(oracle, dtype, tol):
    _check(oracle, dtype, tol, "cuda:0", 64)


@pytest.mark.gpu
def test_fused_matches_plain_split_step(gpe, lib):
    """The fused double-word passes and the plain FP64 cuFFT form agree at the benchmark
    size (one pumped 512^2 field, 60 steps from u = 0)."""
    import bench
    err = bench.plain_vs_fused_rel_l2(gpe, 0, steps=60)
    assert err <= 1e-10, err
