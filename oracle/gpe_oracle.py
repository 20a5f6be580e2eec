"""FP64 CPU oracle for the StrangSplitting time stepper of GeneralizedGrossPitaevskii.jl.

TEST INFRASTRUCTURE ONLY.  This module is the oracle that the GPU path is compared
against; only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it.  The product path never calls it.

It restates, in vectorised numpy FP64, the reference algorithm (paths relative to the
reference project):

* grids ...................... src/problem.jl:129-139
* dt resolution .............. src/fixed_time_stepping.jl:14-24
* host save loop ............. src/fixed_time_stepping.jl:26-54
* init / step order .......... src/strang_splitting.jl:32-90
* per-point update ........... src/kernels.jl:37-54
* tables, pump, noise, FFT ... src/misc.jl:12-64

The reference is Julia and no ``julia`` binary exists where this project is built, so
the reference itself cannot be executed to produce golden outputs, and no reference test
stores golden vectors.  Parity of this oracle is therefore pinned to the reference's own
known-answer tests (test/free_propagation.jl, test/kerr_propagation.jl closure-shape
invariance, test/bistability_cycle.jl, test/exciton_polariton_test.jl,
test/windowed_ft.jl), restated in ``tests/test_oracle_known_answers.py``; bit-level parity
with FFTW / StaticArrays arithmetic is unpinned (the FP64 FFT here is numpy's pocketfft).

Supported closure families (the coefficient form the GPU backend accepts):

* dispersion / potential: any callable ``f(coords, param)`` returning a scalar, an
  ``(M,)`` vector (diagonal) or an ``(M, M)`` matrix per point; it is sampled on the grid
  in FP64 and exponentiated (``cis(-dt*D)``, ``cis(-dt/2*V)``), see src/misc.jl:12-20.
* nonlinearity: ``G_j(u) = sum_l g[j, l] |u_l|^2 + c[j]`` (complex ``g``, ``c``), or an
  arbitrary vectorised callable ``G(fields) -> (M, ...)`` returning the diagonal, or
  (``nonlin_matrix``) a callable returning a 2x2 matrix per point, whose ``cis`` is a
  matrix exponential (src/kernels.jl:23-25).
* pump: ``F_m(r, t) = a_m(t) * p_m(r)`` given as the profile array and an amplitude
  callable, or an arbitrary vectorised callable ``F(t) -> (M, *spatial)``.
* position noise: ``eta_m`` constants (optionally times a real profile) with complex
  Gaussian xi, E|xi|^2 = 1.  ``xi_source(h)`` supplies xi for half step ``h`` so that the
  same draws can be replayed into the GPU path.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

TWO_PI = 2.0 * math.pi


# --------------------------------------------------------------------------- grids
def direct_grid(L: float, N: int) -> np.ndarray:
    """x_j = 0 + j * (L/N), j = 0..N-1 (src/problem.jl:129, StepRangeLen(0, L/N, N))."""
    step = float(L) / N
    return np.arange(N, dtype=np.float64) * step


def reciprocal_grid(L: float, N: int) -> np.ndarray:
    """fftfreq(N, 2pi*N/L) (src/problem.jl:135).

    AbstractFFTs.Frequencies multiplies the signed integer frequency by fs/n, with
    fs = (2pi * N) / L evaluated left to right as written in the reference.
    """
    fs = (TWO_PI * N) / float(L)
    mult = fs / N
    j = np.arange(N)
    nneg = (N - 1) // 2 + 1
    signed = np.where(j < nneg, j, j - N).astype(np.float64)
    return signed * mult


def grids(lengths: Sequence[float], shape: Sequence[int]):
    """Per-axis direct and reciprocal grids, axis 0 = x (the fastest Julia dimension)."""
    dg = [direct_grid(L, N) for L, N in zip(lengths, shape)]
    rg = [reciprocal_grid(L, N) for L, N in zip(lengths, shape)]
    return dg, rg


def mesh(axes: Sequence[np.ndarray]):
    """Coordinate arrays in C order (..., y, x): axis 0 of the reference is the LAST numpy
    axis here, because a Julia column-major array (x fastest) is a C array [..., y, x]."""
    rev = list(reversed(axes))
    mg = np.meshgrid(*rev, indexing="ij")
    return tuple(reversed(mg))  # (X, Y, ...) each with shape (..., ny, nx)


# --------------------------------------------------------------------------- time steps
def resolve_fixed_timestepping(dt: float, tspan, nsaves: int):
    """src/fixed_time_stepping.jl:14-24: dT = (t1 - t0)/nsaves, s = ceil(dT/dt),
    dt_eff = dT / s.  Returns (dt_eff, t0, steps_per_save)."""
    t0, t1 = tspan
    dT = float(t1 - t0) / nsaves
    steps_per_save = int(math.ceil(dT / float(dt)))
    return dT / steps_per_save, float(t0), steps_per_save


def step_end_times(t0: float, dt: float, nsteps: int) -> np.ndarray:
    """t accumulated by repeated ``t += dt`` before each step!
    (src/fixed_time_stepping.jl:44)."""
    ts = np.empty(nsteps, dtype=np.float64)
    t = float(t0)
    for k in range(nsteps):
        t = t + dt
        ts[k] = t
    return ts


def pump_times(t0: float, dt: float, nsteps: int) -> np.ndarray:
    """Times at which the pump is sampled, in the order the reference samples them.

    ``init`` evaluates F(t0) into the ``next`` buffer (src/strang_splitting.jl:58).
    Each half step copies next -> now and evaluates next at its time argument
    (src/misc.jl:39-42).  ``step!(iter, t, dt)`` receives the END time t of the step
    (src/fixed_time_stepping.jl:44-45) and calls the half steps at t + dt/2 and t + dt
    (src/strang_splitting.jl:86-90).  So entry 0 is t0, entry 2k+1 is t_k + dt/2 and entry
    2k+2 is t_k + dt, where t_k is step k's end time; half step h uses
    now = F(times[h]), next = F(times[h+1]).
    """
    te = step_end_times(t0, dt, nsteps)
    out = np.empty(2 * nsteps + 1, dtype=np.float64)
    out[0] = t0
    out[1::2] = te + dt / 2
    out[2::2] = te + dt
    return out


# --------------------------------------------------------------------------- tables
def cis_table(values: np.ndarray, kind: str, delta: float) -> np.ndarray:
    """cis(-delta * f) for scalar / diagonal / matrix samples (src/misc.jl:12-20,
    src/kernels.jl:23-25).  ``values`` has shape spatial (scalar), (M,)+spatial (diag) or
    (M, M)+spatial (matrix).  Matrix case: exp(-i*delta*A) per point."""
    if kind in ("scalar", "diag"):
        return np.exp(-1j * delta * values.astype(np.complex128))
    if kind == "matrix":
        return expm_2x2_or_1x1(-1j * delta * values.astype(np.complex128))
    raise ValueError(kind)


def expm_2x2_or_1x1(A: np.ndarray) -> np.ndarray:
    """Matrix exponential of a field of small matrices, A with shape (M, M, *spatial).

    The reference calls LinearAlgebra/StaticArrays ``cis`` on an SMatrix
    (src/kernels.jl:23 via src/misc.jl:15); that arithmetic lives in a third-party
    package, so this restates the mathematics instead:
    exp(A) = e^{tr/2} [cosh(s) I + sinh(s)/s (A - tr/2 I)], s^2 = ((a-d)/2)^2 + b c,
    with a series for sinh(s)/s near s = 0.
    """
    M = A.shape[0]
    if M == 1:
        return np.exp(A)
    if M != 2:
        raise NotImplementedError("matrices larger than 2x2")
    a, b, c, d = A[0, 0], A[0, 1], A[1, 0], A[1, 1]
    half_tr = 0.5 * (a + d)
    s = np.sqrt((0.5 * (a - d)) ** 2 + b * c)
    ch = np.cosh(s)
    small = np.abs(s) < 1e-3
    s_safe = np.where(small, 1.0, s)
    sh = np.where(small, 1.0 + s * s / 6.0 + (s * s) ** 2 / 120.0, np.sinh(s_safe) / s_safe)
    e = np.exp(half_tr)
    out = np.empty_like(A)
    out[0, 0] = e * (ch + sh * (a - half_tr))
    out[1, 1] = e * (ch + sh * (d - half_tr))
    out[0, 1] = e * sh * b
    out[1, 0] = e * sh * c
    return out


def classify(values: np.ndarray, M: int, nspatial: int) -> str:
    """Scalar / diagonal / matrix by the shape the closure returned (the three closure
    shapes of docs/src/multicomponent_systems.md)."""
    extra = values.ndim - nspatial
    if extra == 0:
        return "scalar"
    if extra == 1:
        return "diag"
    if extra == 2:
        return "matrix"
    raise ValueError("bad closure output shape")


def sample_on_grid(f: Callable, axes, param, M: int):
    """grid_map! of a user closure (src/misc.jl:1-10), vectorised: ``f`` receives the
    tuple of coordinate arrays (x, y, ...) shaped like the spatial field."""
    coords = mesh(axes)
    vals = np.asarray(f(coords, param))
    spatial = coords[0].shape
    if vals.shape == ():
        vals = np.broadcast_to(vals, spatial)
    kind = classify(vals, M, len(spatial))
    if kind != "scalar" and vals.shape[-len(spatial):] != spatial:
        vals = np.broadcast_to(vals, vals.shape[: vals.ndim - len(spatial)] + spatial)
    if kind == "scalar" and vals.shape != spatial:
        vals = np.broadcast_to(vals, spatial)
    return np.array(vals, dtype=np.complex128), kind


# --------------------------------------------------------------------------- problem
@dataclass
class OracleProblem:
    """The data of GrossPitaevskiiProblem (src/problem.jl:97-123) in coefficient form.

    u0: tuple of M complex arrays in C order (*batch, *spatial[::-1]); lengths per axis
    with axis 0 = x.  ``ktable`` / ``vtable`` are the raw closure samples D(k) / V(r)
    (exponentiated by ``init``).  nonlinearity is (g, c) or a callable.
    """

    u0: tuple
    lengths: tuple
    dispersion: Optional[Callable] = None
    potential: Optional[Callable] = None
    nonlin_g: Optional[np.ndarray] = None  # (M, M) complex
    nonlin_c: Optional[np.ndarray] = None  # (M,) complex
    nonlin_fn: Optional[Callable] = None   # fields (M, ...) -> diag G (M, ...)
    nonlin_matrix: Optional[Callable] = None  # fields (2, ...) -> matrix G (2, 2, ...)
    pump_profile: Optional[np.ndarray] = None   # (M, *spatial) complex
    pump_amp: Optional[Callable] = None         # t -> (M,) complex
    pump_fn: Optional[Callable] = None          # t -> (M, *spatial) complex
    eta: Optional[np.ndarray] = None            # (M,) complex noise amplitude
    eta_profile: Optional[np.ndarray] = None    # (M, *spatial) real
    param: object = None

    @property
    def M(self):
        return len(self.u0)

    @property
    def ndim(self):
        return len(self.lengths)

    @property
    def spatial_shape_c(self):
        """Spatial shape in C order (..., ny, nx)."""
        return self.u0[0].shape[-self.ndim:]


class OracleIterator:
    """StrangSplittingIterator restated (src/strang_splitting.jl:9-67)."""

    def __init__(self, prob: OracleProblem, tspan, dt: float, nsaves: int,
                 save_start: bool = True, xi_source: Optional[Callable] = None,
                 fft_workers: Optional[int] = None):
        self.prob = prob
        self.fft_workers = fft_workers
        self.dt, self.t0, self.steps_per_save = resolve_fixed_timestepping(dt, tspan, nsaves)
        self.nsaves = nsaves
        self.save_start = save_start
        self.xi_source = xi_source
        nd = prob.ndim
        self.u = np.stack([np.array(x, dtype=np.complex128) for x in prob.u0])  # (M, *batch, *sp)
        sp_c = prob.spatial_shape_c
        n_xfirst = tuple(reversed(sp_c))
        self.dg, self.rg = grids(prob.lengths, n_xfirst)
        M = prob.M
        # exp tables (src/strang_splitting.jl:53-54, src/misc.jl:12-20)
        if prob.dispersion is not None:
            D, kind = sample_on_grid(prob.dispersion, self.rg, prob.param, M)
            self.ekind = kind
            self.exp_D = cis_table(D, kind, self.dt)
        else:
            self.ekind, self.exp_D = None, None
        if prob.potential is not None:
            V, kind = sample_on_grid(prob.potential, self.dg, prob.param, M)
            self.vkind = kind
            self.exp_V = cis_table(V, kind, self.dt / 2)
        else:
            self.vkind, self.exp_V = None, None
        self.fft_axes = tuple(range(-nd, 0))
        self.P = int(np.prod(sp_c))
        # pump buffers: next <- F(t0) at init (src/strang_splitting.jl:56-58)
        self.pump_next = self._pump(self.t0)
        self.pump_now = None
        self.half = 0  # absolute half-step counter (for replayed noise)

    # -- pump: F(t) as an (M, *spatial) array or None
    def _pump(self, t):
        p = self.prob
        if p.pump_fn is not None:
            return np.asarray(p.pump_fn(t), dtype=np.complex128)
        if p.pump_profile is not None:
            a = np.asarray(p.pump_amp(t), dtype=np.complex128)
            prof = np.asarray(p.pump_profile, dtype=np.complex128)
            return a.reshape((-1,) + (1,) * (prof.ndim - 1)) * prof
        return None

    def _diag_G(self, u):
        """G(u): per component (M, ...) for the diagonal families, (M, M, ...) for the
        matrix family (an SMatrix-valued nonlinearity, src/kernels.jl:23-25)."""
        p = self.prob
        if p.nonlin_matrix is not None:
            return np.asarray(p.nonlin_matrix(u), dtype=np.complex128)
        if p.nonlin_fn is not None:
            return np.asarray(p.nonlin_fn(u), dtype=np.complex128)
        if p.nonlin_g is None and p.nonlin_c is None:
            return None
        M = p.M
        g = np.zeros((M, M), np.complex128) if p.nonlin_g is None else np.asarray(p.nonlin_g, np.complex128)
        c = np.zeros(M, np.complex128) if p.nonlin_c is None else np.asarray(p.nonlin_c, np.complex128)
        dens = (u.real ** 2 + u.imag ** 2)
        G = np.empty_like(u)
        for j in range(M):
            acc = np.zeros(u.shape[1:], np.complex128)
            for l in range(M):
                if g[j, l] != 0:
                    acc = acc + g[j, l] * dens[l]
            G[j] = acc + c[j]
        return G

    def _bcast(self, table, lead: int, u_ndim: int):
        """Insert the batch axes into a spatial table with ``lead`` leading axes so it
        broadcasts against a field of ndim ``u_ndim`` (src/kernels.jl:27, _getindex)."""
        nb = (u_ndim - 1) - (table.ndim - lead)
        return table.reshape(table.shape[:lead] + (1,) * nb + table.shape[lead:])

    def _apply(self, table, kind, v, G=None, dt_half=None):
        """_mul(cis(-dt G), table) applied to the M-vector v (src/kernels.jl:44,48):
        scalar and diagonal tables act elementwise, a matrix table as a mat-vec."""
        E = None
        if G is not None and G.ndim == v.ndim + 1:
            # matrix family: E = cis(-dt G) as a 2x2 exponential, times the table (scalar or
            # matrix, src/kernels.jl:44), then a mat-vec
            E = expm_2x2_or_1x1(-1j * dt_half * G)
            if table is not None:
                if kind == "diag":
                    raise NotImplementedError("matrix G with a diagonal table is not supported")
                T = self._bcast(table, 2 if kind == "matrix" else 0, v.ndim)
                if kind == "matrix":
                    E = np.stack([np.stack([E[i, 0] * T[0, j] + E[i, 1] * T[1, j] for j in range(2)])
                                  for i in range(2)])
                else:
                    E = E * T
            return np.stack([E[i, 0] * v[0] + E[i, 1] * v[1] for i in range(2)])
        if G is not None:
            E = np.exp(-1j * dt_half * G)
        if table is not None:
            if kind == "matrix":
                if E is not None:
                    raise NotImplementedError("diagonal G with a matrix table is undefined in the reference")
                T = self._bcast(table, 2, v.ndim)
                out = np.zeros_like(v)
                for i in range(v.shape[0]):
                    for j in range(v.shape[0]):
                        out[i] = out[i] + T[i, j] * v[j]
                return out
            T = self._bcast(table, 0 if kind == "scalar" else 1, v.ndim)
            if kind == "scalar":
                T = T[None]
            E = T if E is None else E * T
        return v if E is None else E * v

    # -- src/kernels.jl:37-54 for the real-space half step
    def _potential_pump_step(self, t, dt_half):
        p = self.prob
        # sample_noise! (src/misc.jl:44-51): fresh xi for every half step
        noise = None
        if p.eta is not None:
            xi = self.xi_source(self.half)  # (M, *batch, *spatial)
            eta = np.asarray(p.eta, np.complex128).reshape((-1,) + (1,) * (xi.ndim - 1))
            if p.eta_profile is not None:
                eta = eta * self._bcast(np.asarray(p.eta_profile, np.float64), 1, xi.ndim)
            noise = (-1j * math.sqrt(dt_half)) * (eta * xi)
        # evaluate_pump! (src/misc.jl:39-42)
        self.pump_now = self.pump_next
        self.pump_next = self._pump(t)
        u = self.u
        G = self._diag_G(u)   # on u BEFORE the pump is added (src/kernels.jl:40,44)
        v = u
        if self.pump_now is not None:
            v = v + (dt_half / 2) * self._bcast(self.pump_now, 1, u.ndim)
        v = self._apply(self.exp_V, self.vkind, v, G, dt_half)
        if self.pump_next is not None:
            v = v + (dt_half / 2) * self._bcast(self.pump_next, 1, u.ndim)
        if noise is not None:
            v = v + noise
        self.u = v
        self.half += 1

    def _diffusion_step(self):
        """src/strang_splitting.jl:69-76: unnormalised FFT, table, 1/P-normalised inverse
        over the spatial axes only (src/misc.jl:53-64)."""
        if self.exp_D is None:
            return
        if self.fft_workers:
            import scipy.fft as sfft
            ft = sfft.fftn(self.u, axes=self.fft_axes, workers=self.fft_workers)
            ft = self._apply(self.exp_D, self.ekind, ft)
            self.u = sfft.ifftn(ft, axes=self.fft_axes, workers=self.fft_workers)
            return
        ft = np.fft.fftn(self.u, axes=self.fft_axes)
        ft = self._apply(self.exp_D, self.ekind, ft)
        self.u = np.fft.ifftn(ft, axes=self.fft_axes)

    def step(self, t, dt):
        """step! (src/strang_splitting.jl:86-90); t is the END time of the step."""
        self._potential_pump_step(t + dt / 2, dt / 2)
        self._diffusion_step()
        self._potential_pump_step(t + dt, dt / 2)

    def solve(self):
        """solve! (src/fixed_time_stepping.jl:26-54).  Returns (ts, result) with result of
        shape (M, nsaves+save_start, *batch, *spatial)."""
        nres = self.nsaves + int(self.save_start)
        res = np.empty((self.prob.M, nres) + self.u.shape[1:], np.complex128)
        ts = np.empty(self.nsaves + 1, np.float64)
        ts[0] = self.t0
        if self.save_start:
            res[:, 0] = self.u
        t = self.t0
        dt = self.dt
        off = int(self.save_start)
        for n in range(self.nsaves):
            for _ in range(self.steps_per_save):
                t = t + dt
                self.step(t, dt)
            res[:, n + off] = self.u
            ts[n + 1] = t
        return (ts if self.save_start else ts[1:]), res


def solve(prob: OracleProblem, tspan, dt: float, nsaves: int, save_start: bool = True,
          xi_source: Optional[Callable] = None):
    """``solve(prob, StrangSplitting(), tspan; dt, nsaves, save_start)``
    (src/fixed_time_stepping.jl:79-81)."""
    return OracleIterator(prob, tspan, dt, nsaves, save_start, xi_source).solve()


# --------------------------------------------------------------------------- noise
def complex_normal(rng: np.random.Generator, shape) -> np.ndarray:
    """Complex Gaussian with E|xi|^2 = 1 (re, im ~ N(0, 1/2)), the distribution of Julia's
    ``randn!`` on a ComplexF64 array (src/misc.jl:44-45)."""
    z = rng.standard_normal(shape + (2,))
    return (z[..., 0] + 1j * z[..., 1]) * math.sqrt(0.5)


class ReplayNoise:
    """Deterministic xi per half step: a PCG64 stream seeded by (seed, half step), so the
    same draws can be handed to the GPU path in replay mode."""

    def __init__(self, seed: int, shape):
        self.seed = seed
        self.shape = tuple(shape)

    def __call__(self, h: int) -> np.ndarray:
        rng = np.random.Generator(np.random.PCG64([self.seed, h]))
        return complex_normal(rng, self.shape)


# --------------------------------------------------------------------------- diagnostics
def norm(u: np.ndarray, lengths, ndim: int) -> np.ndarray:
    """sum |u|^2 dV over the spatial axes (per leading index)."""
    sp = u.shape[-ndim:]
    dV = float(np.prod([L / n for L, n in zip(lengths, reversed(sp))]))
    return (np.abs(u) ** 2).sum(axis=tuple(range(-ndim, 0))) * dV


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b|| / max(||a||, ||b||): the tolerance form of Julia's isapprox on arrays."""
    na, nb = np.linalg.norm(a), np.linalg.norm(b)
    den = max(na, nb)
    if den == 0:
        return 0.0
    return float(np.linalg.norm(a - b) / den)


# --------------------------------------------------------------------------- Philox noise
_MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0: int, k1: int):
    """Philox4x32-10 (Salmon et al., SC'11) on uint64 arrays holding 32-bit words; the
    CPU restatement of the counter-based generator of the GPU noise path."""
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    W0, W1 = 0x9E3779B9, 0xBB67AE85
    c0, c1, c2, c3 = (np.asarray(v, np.uint64) & _MASK32 for v in (c0, c1, c2, c3))
    for r in range(10):
        if r:
            k0 = (k0 + W0) & 0xFFFFFFFF
            k1 = (k1 + W1) & 0xFFFFFFFF
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK32
        c0, c1, c2, c3 = hi1 ^ c1 ^ np.uint64(k0), lo1, hi0 ^ c3 ^ np.uint64(k1), lo0
    return c0, c1, c2, c3


def box_muller_f64(w0, w1):
    """sqrt(-ln u1) (cos 2 pi u2 + i sin 2 pi u2), u1 = (w0 + 1/2) 2^-32, u2 = w1 2^-32."""
    u1 = (w0.astype(np.float64) + 0.5) * 2.0 ** -32
    u2 = w1.astype(np.float64) * 2.0 ** -32
    mag = np.sqrt(-np.log(u1))
    th = 2.0 * math.pi * u2
    return mag * np.cos(th) + 1j * mag * np.sin(th)


def box_muller_f32(w0, w1):
    """FP32 variant on the top 24 bits of each word, evaluated exactly; the GPU's FP32
    path uses hardware log / sin / cos approximations (absolute error near 2^-21), so it
    matches this to that accuracy, not bit for bit."""
    u1 = ((w0 >> np.uint64(8)).astype(np.float32) + np.float32(0.5)) * np.float32(2.0 ** -24)
    u2 = (w1 >> np.uint64(8)).astype(np.float32) * np.float32(2.0 ** -24)
    mag = np.sqrt(-np.log(u1.astype(np.float64)))
    th = 2.0 * math.pi * u2.astype(np.float64)
    return (mag * np.cos(th) + 1j * mag * np.sin(th)).astype(np.complex64)


class PhiloxNoise:
    """xi for half step h as drawn by the GPU noise path: counter (point, traj0 + trajectory,
    h mod 2^32, h >> 32), key (seed mod 2^32, seed >> 32).  Two components: point p draws
    its own block, components 0 and 1 use word pairs (0,1) and (2,3).  One component: the
    points x and x + nx/2 of a row share the block of the lower one, which takes words
    (0,1) and the upper one (2,3).  Returns (M, *batch, *spatial) in C order."""

    def __init__(self, seed: int, M: int, batch_shape, spatial_shape_c, fp32: bool = False, traj0: int = 0):
        self.seed = int(seed)
        self.traj0 = int(traj0)  # global index of the first trajectory (counter word 1)
        self.M = M
        self.batch_shape = tuple(batch_shape)
        self.spatial = tuple(spatial_shape_c)
        self.fp32 = fp32

    def __call__(self, h: int) -> np.ndarray:
        P = int(np.prod(self.spatial))
        B = int(np.prod(self.batch_shape)) if self.batch_shape else 1
        p = np.tile(np.arange(P, dtype=np.uint64), B)
        b = np.repeat(np.arange(B, dtype=np.uint64) + np.uint64(self.traj0), P)
        upper = None
        if self.M == 1:
            half = np.uint64(self.spatial[-1] // 2)
            upper = (p % np.uint64(self.spatial[-1])) >= half
            p = np.where(upper, p - half, p)
        hl = np.full(P * B, h & 0xFFFFFFFF, np.uint64)
        hh = np.full(P * B, (h >> 32) & 0xFFFFFFFF, np.uint64)
        w = philox4x32_10(p, b, hl, hh, self.seed & 0xFFFFFFFF, (self.seed >> 32) & 0xFFFFFFFF)
        bm = box_muller_f32 if self.fp32 else box_muller_f64
        if self.M == 1:
            xs = [np.where(upper, bm(w[2], w[3]), bm(w[0], w[1]))]
        else:
            xs = [bm(w[0], w[1]), bm(w[2], w[3])]
        return np.stack(xs).astype(np.complex128).reshape((self.M,) + self.batch_shape + self.spatial)


class Fp32Iterator(OracleIterator):
    """The reference's arithmetic for ComplexF32 fields: FFTs in single precision,
    FP64 tables (dt is FP64, src/misc.jl:16) multiplied into the FP32 field with the
    product rounded back to FP32 when stored (src/kernels.jl:51-53).  Used to bound
    what an FP32 implementation can reach on a given problem."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        self.u = self.u.astype(np.complex64)

    def _diffusion_step(self):
        import scipy.fft as sfft
        if self.exp_D is None:
            return
        ft = sfft.fftn(self.u.astype(np.complex64), axes=self.fft_axes)
        ft = self._apply(self.exp_D, self.ekind, ft.astype(np.complex128)).astype(np.complex64)
        self.u = sfft.ifftn(ft, axes=self.fft_axes).astype(np.complex64)

    def _potential_pump_step(self, t, dt_half):
        self.u = self.u.astype(np.complex128)
        super()._potential_pump_step(t, dt_half)
        self.u = self.u.astype(np.complex64)


def solve_fp32(prob: OracleProblem, tspan, dt: float, nsaves: int, save_start: bool = True,
               xi_source: Optional[Callable] = None):
    it = Fp32Iterator(prob, tspan, dt, nsaves, save_start, xi_source)
    it.u = it.u.astype(np.complex64)
    return it.solve()


# --------------------------------------------------------------------------- energy
def energy(it: "OracleIterator", u: Optional[np.ndarray] = None) -> np.ndarray:
    """[kinetic, interaction, potential] of the state u (M, *batch, *spatial), FP64, summed
    over the batch: kinetic = Re sum_k u~^H D u~ dV / P, interaction = sum_j [(1/2) sum_l
    Re g_jl |u_l|^2 + Re c_j] |u_j|^2 dV, potential = Re sum_r u^H V u dV."""
    p = it.prob
    u = it.u if u is None else u
    nd = p.ndim
    sp = u.shape[-nd:]
    dV = float(np.prod([L / n for L, n in zip(p.lengths, reversed(sp))]))
    P = int(np.prod(sp))
    out = np.zeros(3)
    M = u.shape[0]

    def quad(T, kind, v):
        if kind == "scalar":
            return sum(np.real(np.conj(v[m]) * T * v[m]).sum() for m in range(M))
        if kind == "diag":
            return sum(np.real(np.conj(v[m]) * T[m] * v[m]).sum() for m in range(M))
        return sum(np.real(np.conj(v[i]) * T[i, j] * v[j]).sum() for i in range(M) for j in range(M))

    if p.dispersion is not None:
        D, kind = sample_on_grid(p.dispersion, it.rg, p.param, M)
        ft = np.fft.fftn(u, axes=tuple(range(-nd, 0)))
        out[0] = quad(D, kind, ft) * dV / P
    g = np.zeros((M, M)) if p.nonlin_g is None else np.real(np.asarray(p.nonlin_g))
    c = np.zeros(M) if p.nonlin_c is None else np.real(np.asarray(p.nonlin_c))
    d = np.abs(u) ** 2
    out[1] = sum(((0.5 * sum(g[j, l] * d[l] for l in range(M)) + c[j]) * d[j]).sum() for j in range(M)) * dV
    if p.potential is not None:
        V, kind = sample_on_grid(p.potential, it.dg, p.param, M)
        out[2] = quad(V, kind, u) * dV
    return out
