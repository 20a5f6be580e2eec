"""Truncated-Wigner ensembles over grids of different sizes, advanced by one CUDA graph.

The reference batches stochastic trajectories along the trailing dims of u0, all on one
grid (docs/src/stochastic_simulations.md:36-48, examples/truncated_wigner.jl:86-100).
Here each grid size is one group (one libgpe handle whose batch holds that group's
trajectories) and ``Ensemble`` advances every group together with a single captured CUDA
graph (``gpe_ensemble_run``): square grids that fit in one CTA's shared memory run as one
resident launch per chunk of steps, larger grids as their two-pass chain, each group on
its own stream inside the graph.  ``autotune`` picks, per group, the path and the chunk
length.
"""
from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L
from .problem import GrossPitaevskiiProblem
from .strang import StrangSplitting, StrangSplittingIterator


@dataclass
class DampedDrivenParams:
    """i du = [|k|^2/2 - i gamma/2 + g |u|^2 + i F] u dt + sqrt(gamma / (2 dV)) dW:
    the damped-driven scalar field of the truncated-Wigner example
    (examples/truncated_wigner.jl:32-42,96), with the decay in the dispersion."""
    L: float = 64.0
    gamma: float = 0.2
    g: float = 0.01
    F: float = 1.0
    dt: float = 0.02


def wigner_initial(N: int, traj0: int, ntraj: int, prm: DampedDrivenParams, seed: int, dtype=np.complex64):
    """Trajectories traj0 .. traj0 + ntraj - 1 of an ensemble on an N x N grid, each starting
    from the coherent state 1 plus Wigner vacuum noise xi / sqrt(2 dV)
    (examples/truncated_wigner.jl:89).  Trajectory b draws its xi from its own generator
    (seed, b), so any slice of the ensemble is the same whichever process builds it."""
    dV = (prm.L / N) ** 2
    u0 = np.empty((N, N, ntraj), dtype, order="F")
    for j in range(ntraj):
        rng = np.random.default_rng([seed, traj0 + j])
        xi = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * math.sqrt(0.5)
        u0[:, :, j] = 1.0 + xi / math.sqrt(2 * dV)
    return u0


def wigner_problem(N: int, ntraj: int, prm: DampedDrivenParams, seed: int, dtype=np.complex64, traj0: int = 0):
    """One group: trajectories traj0 .. traj0 + ntraj - 1 of the damped-driven ensemble on
    an N x N grid (wigner_initial)."""
    dV = (prm.L / N) ** 2
    u0 = wigner_initial(N, traj0, ntraj, prm, seed, dtype)
    eta = math.sqrt(prm.gamma / (2 * dV))
    return GrossPitaevskiiProblem(
        (np.asfortranarray(u0),), (prm.L, prm.L),
        dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.5j * prm.gamma,
        nonlinearity=lambda u, p: prm.g * np.abs(u[0]) ** 2,
        pump=lambda r, p, t: prm.F + 0 * r[0],
        position_noise_func=lambda u, r, p: eta)


class Ensemble:
    """Groups advanced together by one CUDA graph (``gpe_ensemble_run``)."""

    def __init__(self, iterators: Sequence[StrangSplittingIterator]):
        self.its = list(iterators)
        self.lib = L.load()
        arr = (ctypes.c_void_p * len(self.its))(*[it.h.value for it in self.its])
        e = ctypes.c_void_p()
        rc = self.lib.gpe_ensemble_create(arr, len(self.its), ctypes.byref(e))
        if rc != L.GPE_OK:
            raise L.GPEError(rc, self.lib.gpe_ensemble_last_error(None).decode())
        self.e = e

    def run(self, nsteps: int, steps_per_graph: int):
        rc = self.lib.gpe_ensemble_run(self.e, int(nsteps), int(steps_per_graph))
        if rc != L.GPE_OK:
            raise L.GPEError(rc, self.lib.gpe_ensemble_last_error(self.e).decode())

    def last_run_ms(self) -> float:
        return float(self.lib.gpe_ensemble_last_run_ms(self.e))

    def last_run_launches(self) -> int:
        return int(self.lib.gpe_ensemble_last_run_launches(self.e))

    def close(self):
        if getattr(self, "e", None) is not None and self.e.value:
            self.lib.gpe_ensemble_destroy(self.e)
            self.e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_group(N: int, ntraj: int, prm: DampedDrivenParams, nsteps: int, seed: int, dtype=np.complex64,
               resident: bool = True, noise_seed: Optional[int] = None, variant: int = 0,
               tma: Optional[bool] = None, traj0: int = 0, device: int = -1) -> StrangSplittingIterator:
    """A handle advancing trajectories traj0 .. traj0 + ntraj - 1 of the ensemble (initial
    state and Philox noise both indexed by the global trajectory number)."""
    prob = wigner_problem(N, ntraj, prm, seed, dtype, traj0)
    it = StrangSplittingIterator(prob, (0.0, nsteps * prm.dt), dt=prm.dt, nsaves=1,
                                 rng=seed + 1 if noise_seed is None else noise_seed,
                                 resident=resident, variant=variant, tma=tma, device=device)
    if traj0:
        it.set_noise_offset(traj0)
    return it


def shard_range(ntraj: int, rank: int, world: int):
    """Contiguous slice of an ensemble of ntraj trajectories owned by rank: (first, count),
    the first ntraj % world ranks taking one trajectory more."""
    if not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(ntraj), int(world))
    return rank * base + min(rank, extra), base + (1 if rank < extra else 0)


def run_shard(N: int, ntraj: int, prm: DampedDrivenParams, nsteps: int, seed: int, rank: int, world: int,
              dtype=np.complex64, noise_seed: Optional[int] = None, device: int = -1, group=None):
    """One rank's part of an ensemble sharded over processes (one GPU each): it advances its
    contiguous slice of trajectories (shard_range) with no exchange during the run, then
    all-reduces the per-site density moments.  Because initial states and noise are indexed
    by the global trajectory number, the union of the shards is the single-GPU ensemble.
    Returns (mean, variance) of |u|^2 per site over all ntraj trajectories, and the slice."""
    first, count = shard_range(ntraj, rank, world)
    it = make_group(N, count, prm, nsteps, seed, dtype, noise_seed=noise_seed, traj0=first, device=device)
    try:
        it.step(nsteps)
        fields = it.get_fields()[0]
    finally:
        it.close()
    mean, var = allreduce_moments(fields, group=group)
    return mean, var, (first, count)


def density_moments(it: StrangSplittingIterator):
    """Per-site ensemble mean and variance of |u|^2 over the group's trajectories (FP64)."""
    u = it.get_fields()[0]  # (N, N, ntraj)
    n = np.abs(u.astype(np.complex128)) ** 2
    return n.mean(axis=-1), n.var(axis=-1)


def plain_per_trajectory_rate(N: int, prm: DampedDrivenParams, ntraj: int, nsteps: int, seed: int = 0,
                              dtype=np.complex64) -> float:
    """traj-steps/s of the plain per-trajectory form: one trajectory per handle on the
    two-pass path, trajectories run one after another (the form the batched resident
    ensemble is measured against)."""
    total_ms = 0.0
    for j in range(ntraj):
        it = make_group(N, 1, prm, nsteps + 2, seed + 7 * j, dtype, resident=False)
        it.step(2)  # warm-up
        it.step(nsteps)
        total_ms += it.last_run_ms()
        it.close()
    return ntraj * nsteps / (total_ms * 1e-3)


def spectral_moments(it: StrangSplittingIterator, comp: int = 0, second: bool = True):
    """GPU trajectory statistics of n_b(k) = |FFT(u)_b(k)|^2 / P^2 (k in FFT order):
    returns (mean over trajectories, and the matrix (1/B) sum_b n_b(k) n_b(k') or None)."""
    lib = it.lib
    P = it.P
    mean = np.zeros(P)
    sec = np.zeros((P, P)) if second else None
    L.check(lib, it.h, lib.gpe_spectral_moments(it.h, comp, L.ptr(mean), L.ptr(sec)))
    return mean, sec


def momentum_statistics(it: StrangSplittingIterator, commutator: float, comp: int = 0):
    """n(k) and g2(k, k') of a 1D ensemble as the reference's truncated-Wigner example
    computes them (examples/truncated_wigner.jl:110-165): with psi(k) = fftshift(fft(u))/N,
    n(k) = <|psi(k)|^2> - c/2 and G2(k,k') = <|psi(k)|^2 |psi(k')|^2 - (1 + delta_kk') c/2
    (|psi(k)|^2 + |psi(k')|^2 - c/2)>, g2 = G2 / (n(k) n(k')), c = the commutator (1/L).
    Returns (n, G2, g2) in fftshifted k order."""
    if it.prob.N != 1:
        raise ValueError("momentum_statistics follows the 1D example; use spectral_moments for other grids")
    mean, sec = spectral_moments(it, comp, True)
    mean = np.fft.fftshift(mean)
    sec = np.fft.fftshift(sec)
    c = commutator
    nk = mean - c / 2
    delta = np.eye(len(mean))
    G2 = sec - (1 + delta) * c / 2 * (mean[:, None] + mean[None, :] - c / 2)
    return nk, G2, G2 / np.outer(nk, nk)


def local_moments(fields: np.ndarray, batch_axis: int = -1):
    """Per-site moments of n = |u|^2 over the local trajectories, in FP64: (count, mean,
    M2) with M2 = sum (n - mean)^2, each formed in two passes (mean first), so the spread
    keeps its digits when it is small next to the mean density."""
    n = np.abs(np.asarray(fields).astype(np.complex128)) ** 2
    n = np.moveaxis(n, batch_axis, 0)
    mean = n.mean(axis=0)
    return n.shape[0], mean, ((n - mean) ** 2).sum(axis=0)


def merge_moments(parts):
    """Chan, Golub and LeVeque's pairwise update ("Updating formulae and a pairwise
    algorithm for computing sample variances", 1979) over (count, mean, M2) triples, in
    the order given: n = na + nb, d = mean_b - mean_a, mean = mean_a + d nb / n,
    M2 = M2_a + M2_b + d^2 na nb / n."""
    na, ma, qa = parts[0]
    for nb, mb, qb in parts[1:]:
        if nb == 0:
            continue
        n = na + nb
        d = mb - ma
        ma = ma + d * (nb / n)
        qa = qa + qb + d * d * (na * nb / n)
        na = n
    return na, ma, qa


def allreduce_moments(fields: np.ndarray, group=None, batch_axis: int = -1):
    """Ensemble mean and variance (population, ddof 0) of |u|^2 per site when the
    trajectories are sharded over ranks (one process per GPU, each advancing its own
    trajectories with no exchange during the run).  The one collective is an all-gather
    of every rank's (count, mean, M2) in FP64 over torch.distributed (NCCL or gloo); each
    rank merges them in rank order with Chan's pairwise formula, so every rank gets the
    same bits.  Without an initialised process group it uses the local trajectories only."""
    cnt, mean, m2 = local_moments(fields, batch_axis)
    try:
        import torch
        import torch.distributed as dist
        active = dist.is_available() and dist.is_initialized()
    except ImportError:
        active = False
    if active:
        buf = torch.from_numpy(np.concatenate([[float(cnt)], mean.ravel(), m2.ravel()]))
        if dist.get_backend(group) == "nccl":  # NCCL moves device tensors only
            buf = buf.to(torch.device("cuda", torch.cuda.current_device()))
        parts = [torch.empty_like(buf) for _ in range(dist.get_world_size(group))]
        dist.all_gather(parts, buf, group=group)
        triples = []
        for v in parts:
            v = v.cpu().numpy()
            triples.append((v[0], v[1:1 + mean.size].reshape(mean.shape), v[1 + mean.size:].reshape(mean.shape)))
        cnt, mean, m2 = merge_moments(triples)
    return mean, m2 / cnt
