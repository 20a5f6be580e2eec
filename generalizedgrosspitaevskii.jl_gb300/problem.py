"""``GrossPitaevskiiProblem`` and its grids, mirrored from src/problem.jl.

Arrays follow the reference's index order: a field has shape ``(n1, ..., nd, batch...)``
with x first, stored column-major (Fortran order), so its memory is exactly what the
C ABI expects ([batch][z][y][x]).  User closures keep the reference's signatures and
meaning but are called vectorised: ``dispersion(k, param)`` receives the tuple of
coordinate arrays over the whole grid instead of one point, and may return

* an array of the grid's shape (a scalar per point),
* a length-M sequence of such arrays (an ``SVector``: diagonal coupling), or
* an M x M nested sequence (an ``SMatrix``: full coupling).

The closures that are not turned into tables (nonlinearity, pump, position noise) are
classified into the coefficient families the GPU backend runs (see ``classify_*``);
a closure outside those families raises ``NotImplementedError``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from . import _lib as L


def _complex_dtype(a: np.ndarray):
    """``complex.(u0)`` (src/problem.jl:114): Float32 -> ComplexF32, else ComplexF64."""
    if a.dtype in (np.float32, np.complex64):
        return np.complex64
    return np.complex128


class GrossPitaevskiiProblem:
    """src/problem.jl:97-123.  ``u0`` is a tuple of M arrays of shape
    ``(n1, ..., nd, batch...)``; ``lengths`` has one entry per spatial axis."""

    def __init__(self, u0, lengths, *, dispersion=None, potential=None, nonlinearity=None, pump=None,
                 position_noise_func=None, momentum_noise_func=None, noise_prototype=None, param=None):
        if isinstance(u0, np.ndarray):
            raise TypeError("u0 must be a tuple of arrays (one per component)")
        u0 = tuple(np.asarray(x) for x in u0)
        lengths = tuple(lengths)
        # src/problem.jl:112-113
        if not all(x.ndim >= len(lengths) for x in u0):
            raise ValueError("every component needs at least as many dims as lengths")
        if not all(x.shape == u0[0].shape for x in u0):
            raise ValueError("all components must have the same shape")
        cdt = _complex_dtype(u0[0])
        self.u0 = tuple(np.asfortranarray(x.astype(cdt, copy=False)) for x in u0)
        self.lengths = tuple(float(v) for v in lengths)  # promote(lengths...)
        self.dispersion = dispersion
        self.potential = potential
        self.nonlinearity = nonlinearity
        self.pump = pump
        self.position_noise_func = position_noise_func
        self.momentum_noise_func = momentum_noise_func
        self.noise_prototype = noise_prototype
        self.param = param

    @property
    def N(self) -> int:
        return len(self.lengths)

    @property
    def M(self) -> int:
        return len(self.u0)

    @property
    def spatial_shape(self):
        return self.u0[0].shape[: self.N]

    @property
    def batch_shape(self):
        return self.u0[0].shape[self.N:]

    def __repr__(self):
        return f"{self.N}D GrossPitaevskiiProblem"


# ---------------------------------------------------------------- grids (src/problem.jl:129-139)
def direct_grid_axis(L: float, N: int) -> np.ndarray:
    """StepRangeLen(0, L/N, N): x_j = j * (L/N)."""
    return np.arange(N, dtype=np.float64) * (float(L) / N)


def reciprocal_grid_axis(L: float, N: int) -> np.ndarray:
    """fftfreq(N, 2 pi N / L): signed integer frequency times ((2 pi N)/L)/N."""
    mult = ((2.0 * math.pi * N) / float(L)) / N
    j = np.arange(N)
    nneg = (N - 1) // 2 + 1
    return np.where(j < nneg, j, j - N).astype(np.float64) * mult


def direct_grid(prob: GrossPitaevskiiProblem):
    return tuple(direct_grid_axis(L, n) for L, n in zip(prob.lengths, prob.spatial_shape))


def reciprocal_grid(prob: GrossPitaevskiiProblem):
    return tuple(reciprocal_grid_axis(L, n) for L, n in zip(prob.lengths, prob.spatial_shape))


def mesh(axes):
    """Coordinate arrays of the grid in the reference's index order (x first)."""
    return tuple(np.meshgrid(*axes, indexing="ij"))


# ---------------------------------------------------------------- closure sampling

def as_array(val, shape) -> np.ndarray:
    """Closure output -> complex array: nested lists/tuples (SVector / SMatrix written
    as sequences) are broadcast entry by entry to the grid ``shape``."""
    if isinstance(val, (list, tuple)):
        return np.stack([as_array(v, shape) for v in val])
    a = np.asarray(val, dtype=np.complex128)
    if a.ndim == 0:
        return np.broadcast_to(a, shape)
    return a

def _value_at(vals: np.ndarray, gshape, idx):
    """The entries of a whole-grid closure result at the grid multi-index idx."""
    nd = len(gshape)
    if vals.ndim >= nd and vals.shape[vals.ndim - nd:] == gshape:
        return vals[(Ellipsis,) + tuple(idx)]
    return np.broadcast_to(vals, vals.shape[:max(vals.ndim - nd, 0)] + gshape)[(Ellipsis,) + tuple(idx)]


def _agrees_per_point(f: Callable, coords, vals, args) -> bool:
    """Whether the whole-grid result of f equals f called on single points (a corner, the
    centre and one seeded random point).  A closure written for one point can run on the
    coordinate arrays without an error and still compute something else there: a
    reduction such as np.linalg.norm(r) then spans the whole grid instead of one point."""
    gshape = coords[0].shape
    if int(np.prod(gshape)) <= 1:
        return True
    rng = np.random.default_rng(20240607)
    picks = [tuple(0 for _ in gshape), tuple(n // 2 for n in gshape), tuple(int(rng.integers(n)) for n in gshape)]
    try:
        arr = as_array(vals, gshape)
    except (TypeError, ValueError):
        return False
    for idx in picks:
        pt = tuple(float(c[idx]) for c in coords)
        try:
            one = as_array(f(pt, *args), ())
        except Exception:
            return True  # the closure only works on arrays: nothing to compare against
        try:
            got = _value_at(arr, gshape, idx)
            ok = np.shape(got) == np.shape(one) and np.allclose(got, one, rtol=1e-10, atol=1e-300)
        except (TypeError, ValueError):
            ok = False
        if not ok:
            return False
    return True


def eval_on_grid(f: Callable, coords, *args):
    """A closure over the grid: called once with the coordinate arrays when it takes
    them (numpy arithmetic) and gives there what it gives point by point, else once per
    point with a tuple of floats, as grid_map! calls it (src/misc.jl:1-10) -- closures
    written for one point (math functions, branches on a coordinate, reductions over the
    point's coordinates such as norm(r)) then work unchanged.  Returns an array of shape
    (entries..., *grid)."""
    try:
        vals = f(coords, *args)
    except (TypeError, ValueError):
        vals = None
    if vals is not None and _agrees_per_point(f, coords, vals, args):
        return vals
    gshape = coords[0].shape
    flat = [np.ravel(c) for c in coords]
    vals = np.stack([as_array(f(tuple(float(c[i]) for c in flat), *args), ()) for i in range(flat[0].size)], -1)
    return vals.reshape(vals.shape[:-1] + gshape)


def sample_table(f: Callable, axes, param, M: int):
    """Evaluate a dispersion/potential closure over the grid (src/misc.jl:1-20's
    grid_map!).  Returns (values, kind): values has shape (entries, P) complex128 in
    C-ABI point order (x fastest) and kind is one of the GPE_TABLE_* constants."""
    coords = mesh(axes)
    gshape = coords[0].shape
    vals = as_array(eval_on_grid(f, coords, param), gshape)
    nd = len(gshape)
    extra = vals.ndim - nd if vals.shape[-nd:] == gshape else vals.ndim
    if vals.ndim == 0 or extra == 0 and vals.shape != gshape:
        vals = np.broadcast_to(vals, gshape)
        extra = 0
    if extra == 0:
        kind, lead = L.GPE_TABLE_SCALAR, ()
    elif extra == 1:
        kind, lead = L.GPE_TABLE_DIAG, vals.shape[:1]
    elif extra == 2:
        kind, lead = L.GPE_TABLE_MATRIX, vals.shape[:2]
    else:
        raise ValueError("closure returned an array of unexpected rank")
    vals = np.broadcast_to(vals, lead + gshape)
    ne = int(np.prod(lead)) if lead else 1
    if kind == L.GPE_TABLE_DIAG and lead != (M,):
        raise ValueError(f"vector closure must have {M} entries")
    if kind == L.GPE_TABLE_MATRIX and lead != (M, M):
        raise ValueError(f"matrix closure must be {M}x{M}")
    # Julia-order grid (nx, ny) -> point index x + nx*y: Fortran flattening of each entry
    out = np.empty((ne, int(np.prod(gshape))), np.complex128)
    flat = vals.reshape((ne,) + gshape)
    for e in range(ne):
        out[e] = flat[e].ravel(order="F")
    if M == 1 and kind != L.GPE_TABLE_SCALAR:
        kind = L.GPE_TABLE_SCALAR  # SVector{1} / SMatrix{1,1}: the same numbers
    return out, kind


class MatrixNonlinearity(NotImplementedError):
    """Raised by the diagonal fit when the closure returns a non-diagonal SMatrix; the
    caller then fits the matrix family (``classify_matrix_nonlinearity``)."""


def _as_components(G, M, shape):
    G = as_array(G, shape)
    if G.shape == shape or G.ndim == 0:
        return np.broadcast_to(G, (M,) + shape)  # scalar G acts on every component alike
    if G.ndim == len(shape) + 2 and G.shape[:2] == (M, M):
        # an SMatrix: accepted when it is diagonal (an SMatrix{1,1} always is)
        off = G.copy()
        for j in range(M):
            off[j, j] = 0
        if np.any(off != 0):
            raise MatrixNonlinearity("the nonlinearity returns a non-diagonal matrix")
        G = np.stack([G[j, j] for j in range(M)])
    return np.broadcast_to(G, (M,) + shape)


def classify_nonlinearity(fn: Callable, M: int, param, rng=None):
    """Fit G_j(u) = sum_l g[j,l] |u_l|^2 + c[j] to a nonlinearity closure and verify the
    fit on random fields.  Returns (g (M,M) complex, c (M,) complex)."""
    K = 8
    zeros = tuple(np.zeros(K, np.complex128) for _ in range(M))
    c = _as_components(fn(zeros, param), M, (K,))[:, 0].copy()
    g = np.zeros((M, M), np.complex128)
    for l in range(M):
        u = tuple((np.ones(K, np.complex128) if m == l else np.zeros(K, np.complex128)) for m in range(M))
        g[:, l] = _as_components(fn(u, param), M, (K,))[:, 0] - c
    rng = rng or np.random.default_rng(12345)
    for scale in (0.3, 1.7, 11.0):
        u = tuple(scale * (rng.standard_normal(K) + 1j * rng.standard_normal(K)) for _ in range(M))
        G = _as_components(fn(u, param), M, (K,))
        dens = np.stack([np.abs(x) ** 2 for x in u])
        fit = c[:, None] + g @ dens
        err = np.abs(G - fit).max()
        if err > 1e-9 * max(1.0, np.abs(G).max()):
            raise NotImplementedError(
                "nonlinearity is not of the form G_j = sum_l g_jl |u_l|^2 + c_j supported by the GPU backend")
    return g, c


def classify_matrix_nonlinearity(fn: Callable, M: int, param, rng=None):
    """Fit the matrix family G_ab(u) = sum_l g[a,b,l] |u_l|^2 + c[a,b] to a closure that
    returns a 2x2 SMatrix per point (src/kernels.jl:23-25,44 applies cis(-delta G) as a
    matrix exponential) and verify the fit on random fields.  Returns (g (2,2,2) complex,
    c (2,2) complex), C order, as gpe_set_matrix_nonlinearity takes them."""
    if M != 2:
        raise NotImplementedError("the matrix nonlinearity family needs two components")
    K = 8
    shape = (K,)

    def mat(u):
        G = as_array(fn(u, param), shape)
        if G.ndim == 0 or G.shape == shape:
            G = np.broadcast_to(G, shape)[None, None] * np.eye(2)[:, :, None]
        if G.shape[:2] != (2, 2):
            raise NotImplementedError(f"nonlinearity of shape {G.shape} is neither per component nor a 2x2 matrix")
        return np.broadcast_to(G, (2, 2) + shape).astype(np.complex128)

    zeros = tuple(np.zeros(K, np.complex128) for _ in range(2))
    c = mat(zeros)[:, :, 0].copy()
    g = np.zeros((2, 2, 2), np.complex128)
    for l in range(2):
        u = tuple((np.ones(K, np.complex128) if m == l else np.zeros(K, np.complex128)) for m in range(2))
        g[:, :, l] = mat(u)[:, :, 0] - c
    rng = rng or np.random.default_rng(12345)
    for scale in (0.3, 1.7, 11.0):
        u = tuple(scale * (rng.standard_normal(K) + 1j * rng.standard_normal(K)) for _ in range(2))
        G = mat(u)
        dens = np.stack([np.abs(x) ** 2 for x in u])
        fit = c[:, :, None] + np.einsum("abl,lk->abk", g, dens)
        if np.abs(G - fit).max() > 1e-9 * max(1.0, np.abs(G).max()):
            raise NotImplementedError(
                "matrix nonlinearity is not of the form G_ab = sum_l g_abl |u_l|^2 + c_ab supported by the GPU backend")
    return g, c


@dataclass
class SeparablePump:
    """F_m(r, t) = amplitude(t, param)[m] * profile(r, param)[m]."""
    profile: Callable
    amplitude: Callable


def _pump_values(fn, coords, param, t, M, gshape):
    F = as_array(eval_on_grid(fn, coords, param, t), gshape)
    if F.ndim == 0 or F.shape == gshape:
        F = np.broadcast_to(F, gshape)[None]
        if M != 1:
            raise ValueError("a scalar pump needs a single component")
    elif F.shape[:1] == (1,) and F.ndim == len(gshape) + 2:
        F = F[0]  # SMatrix{1,1}
    return np.broadcast_to(F, (M,) + gshape)


def classify_pump(pump, axes, param, M: int, times: np.ndarray):
    """Split a pump into profiles p_m(r) (shape (M, P), C-ABI order) and amplitudes
    a_m(t) at ``times`` (shape (M, len(times)) complex).  Components without pump get a
    None profile.  A closure ``pump(r, param, t)`` must be separable per component."""
    coords = mesh(axes)
    gshape = coords[0].shape
    if isinstance(pump, SeparablePump):
        pr = as_array(pump.profile(coords, param), gshape)
        prof = np.broadcast_to(pr, (M,) + gshape) if pr.shape != gshape else np.broadcast_to(pr, (M,) + gshape)
        amps = np.stack([np.broadcast_to(as_array(pump.amplitude(t, param), ()), (M,)) for t in times], 1)
        profiles = [prof[m].ravel(order="F").copy() if np.any(prof[m] != 0) else None for m in range(M)]
        return profiles, amps
    # probe a few of the sampling times and pick the strongest as the reference
    idx = np.unique(np.linspace(0, len(times) - 1, min(len(times), 9)).astype(int))
    probes = [(_pump_values(pump, coords, param, float(times[i]), M, gshape), float(times[i])) for i in idx]
    profiles, amps = [], np.zeros((M, len(times)), np.complex128)
    for m in range(M):
        best = max(probes, key=lambda ft: np.abs(ft[0][m]).max())
        Fref, tref = best
        p = Fref[m]
        if not np.any(p != 0):
            profiles.append(None)
            continue
        star = np.unravel_index(np.argmax(np.abs(p)), p.shape)
        pstar = p[star]
        pt = tuple(np.asarray([c[star]]) for c in coords)
        for i, t in enumerate(times):
            v = as_array(eval_on_grid(pump, pt, param, float(t)), (1,)).reshape(-1)
            val = v[m] if v.size >= M and M > 1 else v[0]
            amps[m, i] = val / pstar
        # verify separability on the probes
        for F, t in probes:
            a = as_array(eval_on_grid(pump, pt, param, t), (1,)).reshape(-1)
            a = (a[m] if a.size >= M and M > 1 else a[0]) / pstar
            if np.abs(F[m] - a * p).max() > 1e-10 * max(1.0, np.abs(F[m]).max()):
                raise NotImplementedError("pump is not separable as a(t) * p(r); the GPU backend needs that form")
        profiles.append(p.ravel(order="F").copy())
    return profiles, amps


def classify_noise(fn: Callable, axes, param, M: int, shape_sp, rng=None):
    """eta_m(r) from position_noise_func(u, r, param); it must not depend on u.
    Returns (eta (M,) complex, profile (M, P) real or None)."""
    coords = mesh(axes)
    gshape = coords[0].shape
    z = tuple(np.zeros(gshape, np.complex128) for _ in range(M))
    e0 = as_array(fn(z, coords, param), gshape)
    rng = rng or np.random.default_rng(7)
    ur = tuple(rng.standard_normal(gshape) + 1j * rng.standard_normal(gshape) for _ in range(M))
    e1 = as_array(fn(ur, coords, param), gshape)
    if e0.shape != e1.shape or np.abs(e0 - e1).max() > 1e-12 * max(1.0, np.abs(e0).max()):
        raise NotImplementedError("field-dependent noise amplitudes are not supported by the GPU backend")
    if e0.ndim == 0 or e0.shape == gshape:
        e0 = np.broadcast_to(e0, gshape)[None].repeat(M, 0) if M > 1 else np.broadcast_to(e0, gshape)[None]
    else:
        e0 = np.broadcast_to(e0.reshape(e0.shape[:1] + e0.shape[1:]), (M,) + gshape)
    eta = np.zeros(M, np.complex128)
    prof = np.ones((M, int(np.prod(gshape))), np.float64)
    varying = False
    for m in range(M):
        f = e0[m]
        star = np.unravel_index(np.argmax(np.abs(f)), f.shape)
        eta[m] = f[star]
        if eta[m] == 0:
            prof[m] = 0
            continue
        r = (f / eta[m])
        if np.abs(r.imag).max() > 1e-12:
            raise NotImplementedError("noise profile must be a complex constant times a real function")
        if np.abs(r.real - 1).max() > 0:
            varying = True
        prof[m] = r.real.ravel(order="F")
    return eta, (prof if varying else None)
