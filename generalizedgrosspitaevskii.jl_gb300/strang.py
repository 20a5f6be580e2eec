"""``StrangSplitting``, ``init`` / ``solve`` / ``step``: the reference's solver surface
(src/strang_splitting.jl, src/fixed_time_stepping.jl) on top of libgpe.

``solve(prob, StrangSplitting(), tspan; dt, nsaves, save_start, rng)`` returns
``(ts, result)`` exactly as src/fixed_time_stepping.jl:53 does: ``ts`` has
``nsaves + save_start`` times and ``result`` is a tuple of M arrays of shape
``(n1, ..., nd, batch..., nsaves + save_start)`` (Fortran order, time last).
"""
from __future__ import annotations

import ctypes
import math
from typing import Callable, Optional

import numpy as np

from . import _lib as L
from .problem import (GrossPitaevskiiProblem, MatrixNonlinearity, SeparablePump, classify_matrix_nonlinearity,
                      classify_noise, classify_nonlinearity,
                      classify_pump, direct_grid, reciprocal_grid, sample_table)


class StrangSplitting:
    """src/strang_splitting.jl:7: the only algorithm of the reference."""

    def __repr__(self):
        return "StrangSplitting()"


def resolve_fixed_timestepping(dt: float, tspan, nsaves: int):
    """src/fixed_time_stepping.jl:14-24 -> (dt_eff, ts, steps_per_save); ts[0] = t0."""
    t0, t1 = tspan
    ts = np.zeros(nsaves + 1, np.float64)
    ts[0] = float(t0)
    dT = float(t1 - t0) / nsaves
    steps_per_save = int(math.ceil(dT / float(dt)))
    return dT / steps_per_save, ts, steps_per_save


def pump_sample_times(t0: float, dt: float, nsteps: int) -> np.ndarray:
    """Times at which the reference samples the pump: t0 at init
    (src/strang_splitting.jl:58), then t_k + dt/2 and t_k + dt for every step k, with
    t_k the step's end time accumulated by t += dt (src/fixed_time_stepping.jl:44,
    src/strang_splitting.jl:86-90)."""
    out = np.empty(2 * nsteps + 1, np.float64)
    out[0] = t0
    t = float(t0)
    for k in range(nsteps):
        t = t + dt
        out[2 * k + 1] = t + dt / 2
        out[2 * k + 2] = t + dt
    return out


def _seed_from(rng) -> int:
    if rng is None:
        return int(np.random.default_rng().integers(0, 2 ** 63))
    if isinstance(rng, (int, np.integer)):
        return int(rng) & 0xFFFFFFFFFFFFFFFF
    if isinstance(rng, np.random.Generator):
        return int(rng.integers(0, 2 ** 63))
    raise TypeError("rng must be None, an int seed or a numpy Generator")


class StrangSplittingIterator:
    """src/strang_splitting.jl:9-67 with the device state owned by a libgpe handle."""

    def __init__(self, prob: GrossPitaevskiiProblem, tspan, *, dt, nsaves, save_start=True, rng=None,
                 noise_replay: Optional[Callable] = None, total_steps: Optional[int] = None,
                 device: int = -1, fp64: str = "bfp", resident: bool = True, variant: Optional[int] = None,
                 tma: Optional[bool] = None):
        self.lib = L.load()
        self.variant = variant
        self.prob = prob
        self.nsaves = int(nsaves)
        self.save_start = bool(save_start)
        self.dt, self.ts, self.steps_per_save = resolve_fixed_timestepping(dt, tspan, nsaves)
        self.t0 = float(tspan[0])
        self.total_steps = total_steps if total_steps is not None else self.nsaves * self.steps_per_save
        self.noise_replay = noise_replay
        self.dtype = np.complex128 if prob.u0[0].dtype == np.complex128 else np.complex64
        N, M = prob.N, prob.M
        sp = prob.spatial_shape
        batch = int(np.prod(prob.batch_shape)) if prob.batch_shape else 1
        self.P = int(np.prod(sp))
        self.B = batch
        d = L.GpeDesc()
        d.abi_version = L.GPE_ABI_VERSION
        d.ndim = N
        for a in range(3):
            d.n[a] = sp[a] if a < N else 1
            d.lengths[a] = prob.lengths[a] if a < N else 1.0
        d.batch = batch
        d.ncomp = M
        d.dtype = L.GPE_C128 if self.dtype == np.complex128 else L.GPE_C64
        d.dt = self.dt
        d.t0 = self.t0
        d.device = device
        if fp64 not in ("bfp", "native", "dw"):
            raise ValueError("fp64 must be 'bfp' (FP64 with block floating point line transforms on the integer "
                             "pipes, the default), 'native' (FP64 floating point throughout) or 'dw' (double-word "
                             "on the FP32 pipes)")
        self.fp64 = fp64 if self.dtype == np.complex128 else None
        mode_flag = {"bfp": L.GPE_FLAG_FFT_BFP, "native": L.GPE_FLAG_FP64_NATIVE, "dw": L.GPE_FLAG_FP64_DW}
        d.flags = (mode_flag.get(self.fp64, 0)
                   | (0 if resident else L.GPE_FLAG_NO_RESIDENT)
                   | (0 if tma is None else L.GPE_FLAG_TMA if tma else L.GPE_FLAG_NO_TMA))
        h = ctypes.c_void_p()
        rc = self.lib.gpe_create(ctypes.byref(d), ctypes.byref(h))
        L.check(self.lib, None, rc)
        self.h = h
        try:
            self._configure(rng)
        except Exception:
            self.close()
            raise

    # -- set-up: the work of init (src/strang_splitting.jl:32-67) done on the host
    def _configure(self, rng):
        prob, lib, h = self.prob, self.lib, self.h
        M = prob.M
        if self.variant is not None:
            L.check(lib, h, lib.gpe_set_variant(h, int(self.variant)))
        for m in range(M):
            L.check(lib, h, lib.gpe_set_field(h, m, L.ptr(prob.u0[m])))
        dg, rg = direct_grid(prob), reciprocal_grid(prob)
        if prob.dispersion is not None:
            D, kind = sample_table(prob.dispersion, rg, prob.param, M)
            L.check(lib, h, lib.gpe_set_dispersion(h, L.ptr(np.ascontiguousarray(D)), kind))
        if prob.nonlinearity is not None:
            try:
                g, c = classify_nonlinearity(prob.nonlinearity, M, prob.param)
            except MatrixNonlinearity:
                g, c = classify_matrix_nonlinearity(prob.nonlinearity, M, prob.param)
                L.check(lib, h, lib.gpe_set_matrix_nonlinearity(h, L.ptr(np.ascontiguousarray(g)),
                                                                L.ptr(np.ascontiguousarray(c))))
            else:
                L.check(lib, h, lib.gpe_set_nonlinearity(h, L.ptr(np.ascontiguousarray(g)),
                                                         L.ptr(np.ascontiguousarray(c))))
        if prob.potential is not None:
            V, kind = sample_table(prob.potential, dg, prob.param, M)
            L.check(lib, h, lib.gpe_set_potential(h, L.ptr(np.ascontiguousarray(V)), kind))
        if prob.pump is not None:
            self._upload_pumps(dg)
        if prob.position_noise_func is not None:
            eta, prof = classify_noise(prob.position_noise_func, dg, prob.param, M, prob.spatial_shape)
            mode = L.GPE_NOISE_REPLAY if self.noise_replay is not None else L.GPE_NOISE_PHILOX
            seed = 0 if self.noise_replay is not None else _seed_from(rng)
            e = np.ascontiguousarray(eta)
            pr = None if prof is None else np.ascontiguousarray(prof)
            L.check(lib, h, lib.gpe_set_noise(h, mode, seed, L.ptr(e), L.ptr(pr)))

    def _upload_pumps(self, dg=None):
        """Pump profiles and the amplitudes at the reference's sampling times of steps
        0 .. total_steps - 1 (the device schedule is indexed by the absolute step)."""
        prob, lib, h = self.prob, self.lib, self.h
        dg = direct_grid(prob) if dg is None else dg
        times = pump_sample_times(self.t0, self.dt, self.total_steps)
        profiles, amps = classify_pump(prob.pump, dg, prob.param, prob.M, times)
        for m in range(prob.M):
            if profiles[m] is None:
                continue
            a = np.ascontiguousarray(amps[m])
            n_amp = len(a)
            if np.all(a == a[0]):
                a, n_amp = a[:1].copy(), 1
            prof = profiles[m]
            cplx = int(np.any(prof.imag != 0))
            pbuf = np.ascontiguousarray(prof if cplx else prof.real)
            L.check(lib, h, lib.gpe_set_pump(h, m, L.ptr(pbuf), cplx, L.ptr(a), n_amp))

    def _cover_pump_schedule(self, nsteps: int):
        """The reference's iterator evaluates the pump at any time, so stepping past tspan
        is allowed there: extend the sampled schedule (at least doubling it) when the next
        nsteps steps would run past it."""
        if self.prob.pump is None:
            return
        need = int(self.state().steps) + int(nsteps)
        if need <= self.total_steps:
            return
        self.total_steps = max(need, 2 * self.total_steps)
        self._upload_pumps()

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gpe_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping
    def _replay_xi(self, nsteps: int) -> Optional[np.ndarray]:
        """The replayed draws of the next nsteps steps, [half][m][batch][p], or None."""
        if self.noise_replay is None:
            return None
        h0 = 2 * self.state().steps
        return np.concatenate([np.ascontiguousarray(self.noise_replay(h0 + j), dtype=self.dtype).reshape(-1)
                               for j in range(2 * nsteps)])

    def _run(self, nsteps: int, save_every: int, out: Optional[np.ndarray], ts: Optional[np.ndarray]):
        lib, h = self.lib, self.h
        self._cover_pump_schedule(nsteps)
        xi = self._replay_xi(nsteps)
        if xi is not None:
            L.check(lib, h, lib.gpe_run_replay(h, nsteps, save_every, L.ptr(xi), L.ptr(out), L.ptr(ts)))
        else:
            L.check(lib, h, lib.gpe_run(h, nsteps, save_every, L.ptr(out), L.ptr(ts)))

    def step(self, nsteps: int = 1):
        """Advance nsteps full Strang steps (step!, src/strang_splitting.jl:86-90)."""
        self._run(int(nsteps), 0, None, None)

    def set_noise_offset(self, traj0: int):
        """Draw the Philox noise of trajectories traj0 .. traj0 + batch - 1 of a larger
        ensemble with the same seed (gpe_set_noise_offset)."""
        L.check(self.lib, self.h, self.lib.gpe_set_noise_offset(self.h, int(traj0)))

    def state(self) -> L.GpeState:
        st = L.GpeState()
        L.check(self.lib, self.h, self.lib.gpe_get_state(self.h, ctypes.byref(st)))
        return st

    def set_state(self, st: L.GpeState):
        L.check(self.lib, self.h, self.lib.gpe_set_state(self.h, ctypes.byref(st)))

    def get_fields(self):
        """Current fields as a tuple of Julia-order arrays."""
        out = []
        for m in range(self.prob.M):
            buf = np.empty(self.B * self.P, self.dtype)
            L.check(self.lib, self.h, self.lib.gpe_get_field(self.h, m, L.ptr(buf)))
            out.append(self._as_julia(buf))
        return tuple(out)

    def set_fields(self, fields):
        for m, f in enumerate(fields):
            a = np.asfortranarray(np.asarray(f, self.dtype))
            L.check(self.lib, self.h, self.lib.gpe_set_field(self.h, m, L.ptr(a)))

    def norm(self) -> np.ndarray:
        out = np.zeros(4, np.float64)
        L.check(self.lib, self.h, self.lib.gpe_norm(self.h, L.ptr(out)))
        return out[: self.prob.M].copy()

    def energy(self) -> np.ndarray:
        """[kinetic, interaction, potential] energies of the current state (gpe_energy)."""
        out = np.zeros(4, np.float64)
        L.check(self.lib, self.h, self.lib.gpe_energy(self.h, L.ptr(out)))
        return out[:3].copy()

    def last_run_ms(self) -> float:
        return float(self.lib.gpe_last_run_ms(self.h))

    def last_run_launches(self) -> int:
        return int(self.lib.gpe_last_run_launches(self.h))

    def _as_julia(self, flat: np.ndarray, extra=()):
        prob = self.prob
        cshape = tuple(extra) + tuple(reversed(prob.batch_shape)) + tuple(reversed(prob.spatial_shape))
        return flat.reshape(cshape).T

    def solve(self):
        """solve! (src/fixed_time_stepping.jl:26-54) -> (ts, result).  The saves land in
        place in the result (component stride nsaves + save_start, gpe_run_ex), with u0 in
        slot 0 when save_start."""
        M, ns, off = self.prob.M, self.nsaves, int(self.save_start)
        plane = self.B * self.P
        full = np.empty((M, ns + off, plane), self.dtype)
        if off:
            for m in range(M):
                full[m, 0] = np.asarray(self.prob.u0[m]).ravel(order="F")
        ts = np.empty(ns, np.float64)
        nsteps = ns * self.steps_per_save
        self._cover_pump_schedule(nsteps)
        xi = self._replay_xi(nsteps)
        out = full[0, off:] if ns > 0 else full
        L.check(self.lib, self.h, self.lib.gpe_run_ex(self.h, nsteps, self.steps_per_save, L.ptr(xi), L.ptr(out),
                                                      ns + off, L.ptr(ts)))
        res = [self._as_julia(full[m], extra=(ns + off,)) for m in range(M)]
        self.ts[1:] = ts
        times = self.ts if self.save_start else self.ts[1:]
        return times.copy(), tuple(res)


def init(prob: GrossPitaevskiiProblem, alg: StrangSplitting, tspan, *, dt, nsaves, show_progress=False,
         progress=None, save_start=True, workgroup_size=(), rng=None, noise_replay=None, fp64="bfp", device=-1,
         resident=True, variant=None, tma=None):
    """init(prob, StrangSplitting(), tspan; dt, nsaves, ...) (src/strang_splitting.jl:32-67).
    show_progress / progress / workgroup_size are accepted for signature parity and
    have no effect: the backend picks its own launch shapes.  Extra keywords: ``rng``
    (Philox seed or numpy Generator), ``noise_replay`` (callable h -> xi for replayed
    noise), ``fp64`` (ComplexF64 fields: "bfp", the default, FP64 pointwise steps with the
    line transforms in block floating point on the integer pipes (64-bit integers under
    one exponent a line, rescaled every stage; measured closer to an FP64 oracle than FP64
    floating-point transforms); "native", FP64 floating point throughout, the reference's
    Float64 arithmetic; "dw", the opt-in fast mode in double-word arithmetic on the FP32
    pipes, unit roundoff 2^-48; ignored for ComplexF32), ``device`` (CUDA ordinal),
    ``resident`` (False forces the two-pass HBM path for small square 2D grids),
    ``variant`` (line tiling of the two-pass passes, see gpe_set_variant; None lets the
    library choose by field size), ``tma`` (TMA staging of 2D column tiles: True wherever
    it fits, False never, None by the library's measured rule)."""
    if not isinstance(alg, StrangSplitting):
        raise TypeError("the only algorithm is StrangSplitting()")
    return StrangSplittingIterator(prob, tspan, dt=dt, nsaves=nsaves, save_start=save_start, rng=rng,
                                   noise_replay=noise_replay, fp64=fp64, device=device, resident=resident,
                                   variant=variant, tma=tma)


def step(it: StrangSplittingIterator, nsteps: int = 1) -> StrangSplittingIterator:
    """CommonSolve.step!(iterator) (src/strang_splitting.jl:86-90): advance nsteps steps."""
    it.step(nsteps)
    return it


def solve_(it: StrangSplittingIterator):
    """CommonSolve.solve!(iterator) (src/fixed_time_stepping.jl:26-54) -> (ts, result)."""
    return it.solve()


def solve(prob: GrossPitaevskiiProblem, alg: StrangSplitting, tspan, **kwargs):
    """solve(prob, StrangSplitting(), tspan; dt, nsaves, ...) (src/fixed_time_stepping.jl:79-81)."""
    it = init(prob, alg, tspan, **kwargs)
    try:
        return it.solve()
    finally:
        it.close()
