"""ctypes wrapper of oracle/gpe_ref.c, the C (OpenMP) restatement of the reference's
StrangSplitting stepper.

TEST INFRASTRUCTURE ONLY, like oracle/gpe_oracle.py: only ``tests/``,
``__graft_entry__.smoke()`` and bench.py's CPU legs load it; the product never does.

The tables, grids, pump sampling times and dt resolution come from
``gpe_oracle.OracleIterator`` (the numpy restatement); the C code does the stepping:
pump rotation and half steps (src/strang_splitting.jl:78-90, src/kernels.jl:37-54) and the
transforms (src/misc.jl:53-64), in FP64 or in the reference's ComplexF32 arithmetic
(single-precision FFTs, FP64 table / G / pump products rounded to single precision when
stored).  It is pinned to the numpy oracle by tests/test_oracle_c.py and runs the large
configurations (2048^2 Kerr over 1000 steps) in seconds on the host cores.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

from . import gpe_oracle as O

HERE = Path(__file__).resolve().parent
SRC = HERE / "gpe_ref.c"
LIB = HERE / "libgpe_ref.so"
CFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


class Desc(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("n", ctypes.c_int64 * 2), ("M", ctypes.c_int32), ("B", ctypes.c_int64),
                ("fp32", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("ktab", ctypes.c_void_p), ("kkind", ctypes.c_int32),
                ("vtab", ctypes.c_void_p), ("vkind", ctypes.c_int32),
                ("g", ctypes.c_void_p), ("c", ctypes.c_void_p),
                ("pprof", ctypes.c_void_p * 2), ("pamp", ctypes.c_void_p * 2), ("namp", ctypes.c_int64),
                ("dt", ctypes.c_double), ("noise", ctypes.c_int32), ("draw32", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("traj0", ctypes.c_int64), ("eta", ctypes.c_void_p)]


def build(force: bool = False) -> Path:
    """Compile libgpe_ref.so next to its source (gcc, OpenMP)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True, capture_output=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        lib.oref_run.restype = ctypes.c_int
        lib.oref_run.argtypes = [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.c_void_p]
        _lib = lib
    return _lib


_KIND = {"scalar": 1, "diag": 2, "matrix": 3}


class CIterator:
    """The stepper of ``O.OracleIterator`` with the stepping done in C.  ``u`` is the
    state (M, *batch, *spatial) complex128 in C order, as in the numpy oracle."""

    def __init__(self, prob: O.OracleProblem, tspan, dt: float, nsaves: int, save_start: bool = True,
                 fp32: bool = False, threads: int = 0, philox_seed=None, draw32: bool = False, traj0: int = 0):
        """philox_seed: position noise (prob.eta, constant amplitudes) drawn in C by
        Philox4x32-10 as the GPU path draws it (draw32: its FP32 draws, the top 24 bits of
        each word, evaluated in FP64); traj0: global index of the first trajectory."""
        if prob.nonlin_fn is not None or prob.nonlin_matrix is not None or prob.pump_fn is not None:
            raise NotImplementedError("the C oracle covers the coefficient families")
        if prob.eta is not None and (philox_seed is None or prob.eta_profile is not None):
            raise NotImplementedError("the C oracle draws noise by Philox only, with constant amplitudes")
        it = O.OracleIterator(prob, tspan, dt, nsaves, save_start)
        if prob.ndim not in (1, 2) or prob.M not in (1, 2):
            raise NotImplementedError("the C oracle covers 1D and 2D grids with one or two components")
        if it.vkind == "matrix":
            raise NotImplementedError("matrix potentials are not restated in C")
        self.prob, self.dt, self.t0, self.steps_per_save = prob, it.dt, it.t0, it.steps_per_save
        self.nsaves, self.save_start, self.fp32 = nsaves, save_start, fp32
        self.u = np.ascontiguousarray(it.u, np.complex128)
        if fp32:
            self.u = self.u.astype(np.complex64).astype(np.complex128)
        sp = prob.spatial_shape_c
        self.P = int(np.prod(sp))
        self.B = int(np.prod(self.u.shape[1:-prob.ndim])) if self.u.ndim > 1 + prob.ndim else 1
        self.step_count = 0
        self._keep = []
        d = Desc()
        d.ndim = prob.ndim
        for a, n in enumerate(reversed(sp)):
            d.n[a] = n
        d.M, d.B, d.fp32, d.threads, d.dt = prob.M, self.B, int(fp32), int(threads), it.dt
        if it.exp_D is not None:
            d.ktab, d.kkind = self._ptr(it.exp_D), _KIND[it.ekind]
        if it.exp_V is not None:
            d.vtab, d.vkind = self._ptr(it.exp_V), _KIND[it.vkind]
        if prob.nonlin_g is not None or prob.nonlin_c is not None:
            M = prob.M
            g = np.zeros((M, M), np.complex128) if prob.nonlin_g is None else np.asarray(prob.nonlin_g, np.complex128)
            d.g = self._ptr(g)
            if prob.nonlin_c is not None:
                d.c = self._ptr(np.asarray(prob.nonlin_c, np.complex128))
        if prob.eta is not None:
            d.noise, d.draw32, d.seed, d.traj0 = 1, int(draw32), int(philox_seed) & (2 ** 64 - 1), int(traj0)
            d.eta = self._ptr(np.asarray(prob.eta, np.complex128))
        self.desc = d
        self._pump_steps = 0
        self._set_pump(nsaves * it.steps_per_save)

    def _ptr(self, a) -> int:
        a = np.ascontiguousarray(a, np.complex128)
        self._keep.append(a)
        return a.ctypes.data

    def _set_pump(self, nsteps: int):
        """Amplitudes a_j at the reference's sampling times of steps 0 .. nsteps - 1."""
        p = self.prob
        if p.pump_profile is None or nsteps <= self._pump_steps:
            return
        times = O.pump_times(self.t0, self.dt, nsteps)
        amps = np.stack([np.asarray(p.pump_amp(t), np.complex128).reshape(-1) for t in times], 1)  # (M, T)
        prof = np.asarray(p.pump_profile, np.complex128)
        for j in range(p.M):
            if np.any(prof[j] != 0):
                self.desc.pprof[j] = self._ptr(prof[j])
                self.desc.pamp[j] = self._ptr(amps[j] if amps.shape[0] > j else amps[0])
        self.desc.namp = len(times)
        self._pump_steps = nsteps

    def step(self, nsteps: int = 1, save_every: int = 0):
        """Advance nsteps full steps; with save_every > 0 returns the saves
        (M, nsteps // save_every, *batch, *spatial)."""
        self._set_pump(self.step_count + nsteps)
        ns = nsteps // save_every if save_every else 0
        saves = np.empty((self.prob.M, ns) + self.u.shape[1:], np.complex128) if ns else None
        rc = load().oref_run(ctypes.byref(self.desc), self.u.ctypes.data, self.step_count, nsteps, save_every,
                             saves.ctypes.data if ns else None)
        if rc != 0:
            raise RuntimeError(f"oref_run failed ({rc})")
        self.step_count += nsteps
        return saves

    def solve(self):
        """solve! (src/fixed_time_stepping.jl:26-54) -> (ts, result (M, nsaves+save_start,
        *batch, *spatial)), the layout of ``O.solve``."""
        off = int(self.save_start)
        res = np.empty((self.prob.M, self.nsaves + off) + self.u.shape[1:], np.complex128)
        if off:
            res[:, 0] = self.u
        saves = self.step(self.nsaves * self.steps_per_save, self.steps_per_save)
        if self.nsaves:
            res[:, off:] = saves
        ts = np.empty(self.nsaves + 1)
        ts[0] = self.t0
        t = self.t0
        for n in range(self.nsaves):
            for _ in range(self.steps_per_save):
                t = t + self.dt
            ts[n + 1] = t
        return (ts if self.save_start else ts[1:]), res


def solve(prob: O.OracleProblem, tspan, dt: float, nsaves: int, save_start: bool = True, fp32: bool = False,
          threads: int = 0):
    """``O.solve`` with the stepping in C (fp32: the reference's ComplexF32 arithmetic)."""
    return CIterator(prob, tspan, dt, nsaves, save_start, fp32, threads).solve()
