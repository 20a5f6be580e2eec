"""Seeded random problems against the FP64 oracle: random grid shapes (1D, 2D, 3D), batch
sizes, one or two components, dispersion / potential table kinds (scalar, diagonal,
matrix), complex nonlinearity coefficients, separable pumps with time-dependent
amplitudes, replayed noise, and every precision.  Each case is built twice from the same
random coefficients: through the package's closures and in the oracle's coefficient form."""
import math

import numpy as np
import pytest

from cases import jl
from test_parity_gpu import TOL, assert_close, fp32_tol

pytestmark = pytest.mark.gpu


def rc(rng, scale=1.0):
    return complex(scale * rng.standard_normal(), scale * rng.standard_normal())


def make_case(seed):
    rng = np.random.default_rng(seed)
    ndim = int(rng.choice([1, 2, 2, 3]))
    if ndim == 1:
        shape = (int(rng.choice([64, 128, 256])),)
    elif ndim == 2:
        shape = (int(rng.choice([16, 32, 64])), int(rng.choice([16, 32, 64, 128])))
    else:
        shape = tuple(int(rng.choice([16, 32])) for _ in range(3))
    shape_c = tuple(reversed(shape))        # oracle / C order (..., y, x)
    lengths = tuple(float(rng.uniform(4, 12)) for _ in range(ndim))
    M = int(rng.choice([1, 2]))
    B = int(rng.choice([1, 2, 3]))
    dkind = str(rng.choice(["scalar", "diag", "matrix"] if M == 2 else ["scalar"]))
    vkind = str(rng.choice(["none", "scalar", "diag"] if M == 2 else ["none", "scalar"]))
    if vkind == "diag" and dkind == "matrix":
        vkind = "scalar"
    # dispersion D = a |k|^2/2 + b (- i gamma), per component or 2x2 with coupling w
    a = [float(rng.uniform(0.5, 1.5)) for _ in range(M)]
    b = [complex(rng.uniform(-0.5, 0.5), -rng.uniform(0, 0.1)) for _ in range(M)]
    w = float(rng.uniform(0.2, 1.0))
    vamp = [float(rng.uniform(0.01, 0.2)) for _ in range(M)]
    g = np.array([[complex(rng.uniform(-1, 1), -rng.uniform(0, 0.05)) for _ in range(M)] for _ in range(M)])
    c = np.array([complex(rng.uniform(-0.3, 0.3), 0.0) for _ in range(M)])
    pump = bool(rng.random() < 0.6)
    pamp = [rc(rng, 0.3) for _ in range(M)]
    pw = float(rng.uniform(1.0, 3.0))
    noise = bool(rng.random() < 0.5)
    eta = [complex(rng.uniform(0.02, 0.1), 0.0) for _ in range(M)]
    dt = float(rng.choice([0.005, 0.01, 0.02]))
    nsaves = int(rng.choice([2, 3]))
    steps = int(rng.choice([2, 4]))

    grids = [np.arange(n) * (L / n) for n, L in zip(shape, lengths)]
    mesh_c = np.meshgrid(*reversed(grids), indexing="ij")      # C order, x last
    X = list(reversed(mesh_c))                                  # X[0] = x
    r2 = sum((Xi - L / 2) ** 2 for Xi, L in zip(X, lengths))
    u0c = []
    for m in range(M):
        base = np.exp(-r2 / (2 + m)) * (1 + 0.3j * np.cos(X[0]))
        per = [base * (1 + 0.1 * rng.standard_normal()) for _ in range(B)]
        u0c.append(np.stack(per).astype(np.complex128) if B > 1 else per[0].astype(np.complex128))
    return dict(ndim=ndim, shape=shape, shape_c=shape_c, lengths=lengths, M=M, B=B, dkind=dkind, vkind=vkind,
                a=a, b=b, w=w, vamp=vamp, g=g, c=c, pump=pump, pamp=pamp, pw=pw, noise=noise, eta=eta, dt=dt,
                nsaves=nsaves, steps=steps, u0c=u0c, seed=seed)


def k2(k):
    return sum(kk ** 2 for kk in k)


def dispersion_gpu(cs):
    a, b, w, M, kind = cs["a"], cs["b"], cs["w"], cs["M"], cs["dkind"]
    if kind == "scalar":
        return lambda k, p: a[0] * k2(k) / 2 + b[0]
    if kind == "diag":
        return lambda k, p: [a[m] * k2(k) / 2 + b[m] for m in range(M)]
    return lambda k, p: [[a[0] * k2(k) / 2 + b[0], w + 0 * k[0]], [w + 0 * k[0], a[1] * k2(k) / 2 + b[1]]]


def dispersion_oracle(cs):
    f = dispersion_gpu(cs)
    kind = cs["dkind"]

    def d(k, p):
        v = f(k, p)
        if kind == "scalar":
            return np.asarray(v, np.complex128) + 0 * k[0]
        if kind == "diag":
            return np.stack([np.asarray(x, np.complex128) + 0 * k[0] for x in v])
        return np.asarray([[np.asarray(x, np.complex128) + 0 * k[0] for x in row] for row in v])
    return d


def potential(cs, oracle_form):
    if cs["vkind"] == "none":
        return None
    L, M, vamp = cs["lengths"], cs["M"], cs["vamp"]

    def base(r, m):
        return vamp[m] * sum((ri - Li / 2) ** 2 for ri, Li in zip(r, L)) / max(L) ** 2
    if cs["vkind"] == "scalar":
        return (lambda r, p: base(r, 0) + 0j) if oracle_form else (lambda r, p: base(r, 0))
    if oracle_form:
        return lambda r, p: np.stack([base(r, m) + 0j for m in range(M)])
    return lambda r, p: [base(r, m) for m in range(M)]


def run_case(gpe, oracle, seed, dtype, fp64):
    cs = make_case(seed)
    M, B, L = cs["M"], cs["B"], cs["lengths"]
    g, c = cs["g"], cs["c"]
    # package side
    u0 = tuple(jl(u).astype(dtype) for u in cs["u0c"])
    kw = dict(dispersion=dispersion_gpu(cs), potential=potential(cs, False),
              nonlinearity=lambda u, p: [sum(g[j, l] * np.abs(u[l]) ** 2 for l in range(M)) + c[j] for j in range(M)])
    amp = lambda t: 1.0 + 0.5 * math.sin(3.0 * t)
    prof_fn = lambda r: np.exp(-sum((ri - Li / 2) ** 2 for ri, Li in zip(r, L)) / cs["pw"] ** 2)
    if cs["pump"]:
        kw["pump"] = lambda r, p, t: [cs["pamp"][m] * amp(t) * prof_fn(r) for m in range(M)]
    if cs["noise"]:
        kw["position_noise_func"] = lambda u, r, p: [cs["eta"][m] for m in range(M)]
    if M == 1:
        for key in ("pump", "position_noise_func"):
            if key in kw:
                f = kw[key]
                kw[key] = (lambda f: (lambda *args: f(*args)[0]))(f)
        nl = kw["nonlinearity"]
        kw["nonlinearity"] = lambda u, p, nl=nl: nl(u, p)[0]
    prob = gpe.GrossPitaevskiiProblem(u0, L, **kw)
    # oracle side
    X_c = oracle.mesh(oracle.grids(L, cs["shape"])[0])
    okw = dict(dispersion=dispersion_oracle(cs), potential=potential(cs, True), nonlin_g=g, nonlin_c=c)
    if cs["pump"]:
        pr = prof_fn(X_c)
        okw["pump_profile"] = np.stack([cs["pamp"][m] * pr for m in range(M)]).astype(np.complex128)
        okw["pump_amp"] = lambda t: np.array([amp(t)] * M)
    xi = None
    if cs["noise"]:
        okw["eta"] = np.array(cs["eta"])
        rn = oracle.ReplayNoise(seed, (M,) + ((B,) if B > 1 else ()) + cs["shape_c"])
        xi = (lambda h: rn(h).astype(np.complex64).astype(np.complex128)) if dtype == np.complex64 else rn
    orc = oracle.OracleProblem(u0=tuple(cs["u0c"]), lengths=L, **okw)
    tspan = (0.0, cs["nsaves"] * cs["steps"] * cs["dt"])
    solve_kw = dict(dt=cs["dt"], nsaves=cs["nsaves"], fp64=fp64)
    if xi is not None:
        solve_kw["noise_replay"] = lambda h: np.ascontiguousarray(xi(h))
    ts, res = gpe.solve(prob, gpe.StrangSplitting(), tspan, **solve_kw)
    ots, ores = oracle.solve(orc, tspan, cs["dt"], cs["nsaves"], xi_source=xi)
    assert np.array_equal(ts, ots)
    if dtype == np.complex128:
        assert_close(oracle, res, ores, TOL[dtype])
    else:
        assert_close(oracle, res, ores, fp32_tol(oracle, orc, tspan, cs["dt"], cs["nsaves"], xi=xi), per_save=False)


@pytest.mark.parametrize("seed", list(range(24)))
@pytest.mark.parametrize("dtype,fp64", [(np.complex128, "dw"), (np.complex128, "native"), (np.complex128, "bfp"),
                                        (np.complex64, "dw")], ids=["c128-dw", "c128-native", "c128-bfp", "c64"])
def test_random_problem(gpe, oracle, lib, seed, dtype, fp64):
    run_case(gpe, oracle, seed, dtype, fp64)
