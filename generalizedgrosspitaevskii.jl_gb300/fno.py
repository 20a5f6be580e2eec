"""Fourier-neural-operator surrogate of the StrangSplitting solver.

The network maps the two-component field at time t (Re/Im of both components) plus the
pump amplitude to the field at t + window, window = ``steps_per_window`` solver steps:

    v0 = lift(a)                                     pointwise 5 -> width
    v_{l+1} = act(W_l v_l + b_l + S_l v_l)            l = 0..3, act = GELU except last
    S_l v = Re iDFT_trunc( R_l(k) . DFT_trunc(v) )   modes x modes retained modes
    out = u + proj(v4)                               pointwise width -> 4, residual

Every linear map (and its gradient) is a BF16 tensor-core GEMM (gpe_fno_gemm: tcgen05.mma
with FP32 accumulation in tensor memory); DFTs along x and y are GEMMs against fixed DFT bases restricted to the
retained modes; the per-mode mixing R_l(k) is a real (2 width) x (2 width) matrix per
mode (a real-linear map of the complex channel vector), applied as one batched GEMM over
modes.  Layout changes between the GEMMs are permutation kernels; GELU, bias, loss and
Adam are elementwise kernels.  torch tensors only hold device memory.

The training data come from the solver itself (``generate_pairs``) and the solver is the
fallback of the surrogate and measures its error (``hybrid_rollout``).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import _lib as L


class GemmDesc(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("C", ctypes.c_void_p),
                ("M", ctypes.c_int64), ("N", ctypes.c_int64), ("K", ctypes.c_int64),
                ("a_r", ctypes.c_int64), ("a_c", ctypes.c_int64), ("a_z", ctypes.c_int64),
                ("b_r", ctypes.c_int64), ("b_c", ctypes.c_int64), ("b_z", ctypes.c_int64),
                ("c_r", ctypes.c_int64), ("c_c", ctypes.c_int64), ("c_z", ctypes.c_int64),
                ("batch", ctypes.c_int64), ("alpha", ctypes.c_float), ("beta", ctypes.c_float)]


class PermDesc(ctypes.Structure):
    _fields_ = [("nd", ctypes.c_int32), ("perm", ctypes.c_int32 * 6), ("d", ctypes.c_int64 * 6)]


FNO_SIGNATURES = {
    "gpe_fno_gemm": (ctypes.c_int, [ctypes.POINTER(GemmDesc), ctypes.c_void_p]),
    "gpe_fno_take_status": (ctypes.c_int, []),
    "gpe_fno_permute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(PermDesc), ctypes.c_void_p]),
    "gpe_fno_bias_act": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]),
    "gpe_fno_gelu_bwd": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "gpe_fno_bias_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_int64, ctypes.c_void_p]),
    "gpe_fno_axpy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_int64, ctypes.c_int64,
                                    ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]),
    "gpe_fno_mse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int64, ctypes.c_void_p]),
    "gpe_fno_sum_slices": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                          ctypes.c_void_p]),
    "gpe_fno_adam": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_int64, ctypes.c_void_p]),
}


def _lib():
    lib = L.load()
    if not getattr(lib, "_fno_declared", False):
        for name, (res, args) in FNO_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._fno_declared = True
    return lib


def _ptr(t) -> int:
    return t.data_ptr()


def _stream():
    """torch's current CUDA stream, so the kernels order with torch's copies and can be
    captured into a CUDA graph."""
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _chk(rc):
    if rc != 0:
        raise L.GPEError(rc, "FNO kernel launch failed")


def gemm(A, B, C, M, N, K, a, b, c, batch=1, alpha=1.0, beta=0.0):
    """C = alpha A B + beta C with (row, col, batch) strides a, b, c (element units)."""
    d = GemmDesc(_ptr(A), _ptr(B), _ptr(C), M, N, K, a[0], a[1], a[2] if len(a) > 2 else 0,
                 b[0], b[1], b[2] if len(b) > 2 else 0, c[0], c[1], c[2] if len(c) > 2 else 0, batch, alpha, beta)
    _chk(_lib().gpe_fno_gemm(ctypes.byref(d), _stream()))


def take_status() -> int:
    """GPE_ERR_TIMEOUT if a GEMM's bounded wait ran out since the last call, else 0."""
    return int(_lib().gpe_fno_take_status())


def permute(src, dst, dims, perm):
    d = PermDesc()
    d.nd = len(dims)
    for i, (x, p) in enumerate(zip(dims, perm)):
        d.d[i] = x
        d.perm[i] = p
    _chk(_lib().gpe_fno_permute(_ptr(src), _ptr(dst), ctypes.byref(d), _stream()))


def inverse_perm(perm):
    inv = [0] * len(perm)
    for a, p in enumerate(perm):
        inv[p] = a
    return inv


@dataclass
class FNOConfig:
    N: int = 128          # grid side
    width: int = 32       # channels
    modes: int = 16       # retained modes per axis (half positive, half negative)
    layers: int = 4
    cin: int = 5          # Re/Im of two components + pump amplitude
    cout: int = 4         # Re/Im of two components


def mode_indices(N: int, modes: int) -> np.ndarray:
    h = modes // 2
    return np.concatenate([np.arange(h), np.arange(N - h, N)])


def dft_bases(cfg: FNOConfig):
    """Fixed real bases of the truncated transforms (FP64 -> FP32):
    Bx (N x 2m): real input -> (Re, Im) over retained kx;
    By (2N x 2m): (Re(y), Im(y)) -> (Re, Im) over retained ky;
    Iy (2m x 2N) and Ix (2m x N) the inverses (scaled 1/N per axis, Ix keeps the real part)."""
    N, m = cfg.N, cfg.modes
    k = mode_indices(N, m)
    x = np.arange(N)
    th = 2 * math.pi * np.outer(x, k) / N  # (N, m)
    c, s = np.cos(th), np.sin(th)
    Bx = np.concatenate([c, -s], axis=1)
    By = np.zeros((2 * N, 2 * m))
    By[:N, :m], By[N:, :m], By[:N, m:], By[N:, m:] = c, s, -s, c
    Iy = np.zeros((2 * m, 2 * N))
    Iy[:m, :N], Iy[m:, :N], Iy[:m, N:], Iy[m:, N:] = c.T / N, -s.T / N, s.T / N, c.T / N
    Ix = np.concatenate([c.T, -s.T], axis=0) / N
    return {k_: v.astype(np.float32) for k_, v in dict(Bx=Bx, By=By, Iy=Iy, Ix=Ix).items()}


def init_params(cfg: FNOConfig, seed: int = 0) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    C, m2 = cfg.width, cfg.modes * cfg.modes
    p = {"lift_w": rng.standard_normal((C, cfg.cin)) / math.sqrt(cfg.cin), "lift_b": np.zeros(C),
         "proj_w": rng.standard_normal((cfg.cout, C)) * (0.1 / math.sqrt(C)), "proj_b": np.zeros(cfg.cout)}
    for l in range(cfg.layers):
        p[f"w{l}"] = rng.standard_normal((C, C)) / math.sqrt(C)
        p[f"b{l}"] = np.zeros(C)
        p[f"r{l}"] = rng.standard_normal((m2, 2 * C, 2 * C)) * (1.0 / (2 * C))
    return {k: v.astype(np.float32) for k, v in p.items()}


class FNO:
    """Device-resident FNO: parameters, Adam moments, and the forward / backward passes."""

    def __init__(self, cfg: FNOConfig, params: Optional[Dict[str, np.ndarray]] = None, device="cuda", seed: int = 0):
        import torch
        self.torch = torch
        self.cfg = cfg
        self.dev = device
        params = params if params is not None else init_params(cfg, seed)
        self.p = {k: torch.tensor(v, device=device).contiguous() for k, v in params.items()}
        self.g = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.t = 0
        self.bases = {k: torch.tensor(v, device=device).contiguous() for k, v in dft_bases(cfg).items()}
        self.cache = None

    def _empty(self, *shape):
        return self.torch.empty(*shape, device=self.dev, dtype=self.torch.float32)

    # -- pointwise channel map: out[b][o][p] (+)= sum_i W[o][i] x[b][i][p]
    def _pointwise(self, W, x, out, B, cin, cout, P, beta=0.0):
        gemm(x, W, out, P, cout, cin, (1, P, cin * P), (1, cin, 0), (1, P, cout * P), batch=B, beta=beta)

    def _pointwise_wgrad(self, dy, x, dW, B, cin, cout, P):
        """dW[o][i] = sum_{b,p} dy[b][o][p] x[b][i][p]: split over (b, chunk of p)."""
        chunks = 32
        pc = P // chunks
        part = self._empty(B * chunks, cout, cin)
        # batch z = (b, chunk): A(o, k) = dy[b][o][chunk*pc + k], B(k, i) = x[b][i][chunk*pc + k]
        for b in range(B):
            gemm(dy[b], x[b], part[b * chunks:], cout, cin, pc, (P, 1, pc), (1, P, pc), (cin, 1, cout * cin),
                 batch=chunks)
        _chk(_lib().gpe_fno_sum_slices(_ptr(part), _ptr(dW), cout * cin, B * chunks, _stream()))

    # -- spectral path S v
    def _spectral(self, l, v, B, save):
        cfg, C, N, m = self.cfg, self.cfg.width, self.cfg.N, self.cfg.modes
        m2, BC = m * m, B * C
        bs = self.bases
        Vx = self._empty(BC * N, 2 * m)
        gemm(v, bs["Bx"], Vx, BC * N, 2 * m, N, (N, 1), (2 * m, 1), (2 * m, 1))
        Vt = self._empty(BC * m, 2 * N)
        permute(Vx, Vt, (BC, N, 2, m), (0, 3, 2, 1))
        G = self._empty(BC * m, 2 * m)
        gemm(Vt, bs["By"], G, BC * m, 2 * m, 2 * N, (2 * N, 1), (2 * m, 1), (2 * m, 1))
        Gm = self._empty(m2, B, 2 * C)
        permute(G, Gm, (B, C, m, 2, m), (4, 2, 0, 3, 1))
        Hm = self._empty(m2, B, 2 * C)
        gemm(Gm, self.p[f"r{l}"], Hm, B, 2 * C, 2 * C, (2 * C, 1, B * 2 * C), (2 * C, 1, 4 * C * C),
             (2 * C, 1, B * 2 * C), batch=m2)
        H = self._empty(BC * m, 2 * m)
        permute(Hm, H, (m, m, B, 2, C), inverse_perm((4, 2, 0, 3, 1)))
        Ht = self._empty(BC * m, 2 * N)
        gemm(H, bs["Iy"], Ht, BC * m, 2 * N, 2 * m, (2 * m, 1), (2 * N, 1), (2 * N, 1))
        Hx = self._empty(BC * N, 2 * m)
        permute(Ht, Hx, (BC, m, 2, N), (0, 3, 2, 1))
        S = self._empty(B, C, N * N)
        gemm(Hx, bs["Ix"], S, BC * N, N, 2 * m, (2 * m, 1), (N, 1), (N, 1))
        if save is not None:
            save["Gm"] = Gm
        return S

    def _spectral_bwd(self, l, dS, B, Gm):
        cfg, C, N, m = self.cfg, self.cfg.width, self.cfg.N, self.cfg.modes
        m2, BC = m * m, B * C
        bs = self.bases
        dHx = self._empty(BC * N, 2 * m)
        gemm(dS, bs["Ix"], dHx, BC * N, 2 * m, N, (N, 1), (1, N), (2 * m, 1))  # dS Ix^T
        dHt = self._empty(BC * m, 2 * N)
        permute(dHx, dHt, (BC, N, 2, m), (0, 3, 2, 1))
        dH = self._empty(BC * m, 2 * m)
        gemm(dHt, bs["Iy"], dH, BC * m, 2 * m, 2 * N, (2 * N, 1), (1, 2 * N), (2 * m, 1))  # dHt Iy^T
        dHm = self._empty(m2, B, 2 * C)
        permute(dH, dHm, (B, C, m, 2, m), (4, 2, 0, 3, 1))
        R = self.p[f"r{l}"]
        # dR[z] = Gm[z]^T dHm[z]
        gemm(Gm, dHm, self.g[f"r{l}"], 2 * C, 2 * C, B, (1, 2 * C, B * 2 * C), (2 * C, 1, B * 2 * C),
             (2 * C, 1, 4 * C * C), batch=m2)
        dGm = self._empty(m2, B, 2 * C)
        gemm(dHm, R, dGm, B, 2 * C, 2 * C, (2 * C, 1, B * 2 * C), (1, 2 * C, 4 * C * C), (2 * C, 1, B * 2 * C),
             batch=m2)  # dHm R^T
        dG = self._empty(BC * m, 2 * m)
        permute(dGm, dG, (m, m, B, 2, C), inverse_perm((4, 2, 0, 3, 1)))
        dVt = self._empty(BC * m, 2 * N)
        gemm(dG, bs["By"], dVt, BC * m, 2 * N, 2 * m, (2 * m, 1), (1, 2 * m), (2 * N, 1))  # dG By^T
        dVx = self._empty(BC * N, 2 * m)
        permute(dVt, dVx, (BC, m, 2, N), (0, 3, 2, 1))
        dv = self._empty(B, C, N * N)
        gemm(dVx, bs["Bx"], dv, BC * N, N, 2 * m, (2 * m, 1), (1, 2 * m), (N, 1))  # dVx Bx^T
        return dv

    def forward(self, a, train: bool = False):
        """a: (B, cin, N*N) float32 device tensor; returns (B, cout, N*N)."""
        cfg, C, P = self.cfg, self.cfg.width, self.cfg.N ** 2
        B = a.shape[0]
        lib = _lib()
        cache = {"a": a, "layers": []}
        v = self._empty(B, C, P)
        self._pointwise(self.p["lift_w"], a, v, B, cfg.cin, C, P)
        _chk(lib.gpe_fno_bias_act(_ptr(v), _ptr(self.p["lift_b"]), None, B, C, P, 0, _stream()))
        for l in range(cfg.layers):
            save = {} if train else None
            S = self._spectral(l, v, B, save)
            self._pointwise(self.p[f"w{l}"], v, S, B, C, C, P, beta=1.0)
            act = int(l < cfg.layers - 1)
            pre = self._empty(B, C, P) if (train and act) else None
            _chk(lib.gpe_fno_bias_act(_ptr(S), _ptr(self.p[f"b{l}"]), _ptr(pre) if pre is not None else None,
                                      B, C, P, act, _stream()))
            if train:
                save.update(v=v, pre=pre)
                cache["layers"].append(save)
            v = S
        out = self._empty(B, cfg.cout, P)
        self._pointwise(self.p["proj_w"], v, out, B, C, cfg.cout, P)
        _chk(lib.gpe_fno_bias_act(_ptr(out), _ptr(self.p["proj_b"]), None, B, cfg.cout, P, 0, _stream()))
        # residual: the output is the input field (channels 0..cout-1 of a) plus the change
        _chk(lib.gpe_fno_axpy(_ptr(out), _ptr(a), 1.0, cfg.cout * P, B, cfg.cout * P, cfg.cin * P, _stream()))
        cache["v_last"] = v
        if train:
            self.cache = cache
        return out

    def graphed(self, B: int):
        """The inference forward pass for batch B captured once into a CUDA graph.  Returns
        run(x) -> out; out is a static buffer that the next run overwrites."""
        import torch
        graphs = self.__dict__.setdefault("_graphs", {})
        if B not in graphs:
            xs = torch.zeros((B, self.cfg.cin, self.cfg.N ** 2), device=self.dev)
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self.forward(xs)  # allocations happen outside the capture
            torch.cuda.current_stream().wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                out = self.forward(xs)
            graphs[B] = (g, xs, out)
        g, xs, out = graphs[B]

        def run(x):
            xs.copy_(x)
            g.replay()
            return out
        return run

    def backward(self, dout):
        """Gradients of the last training forward with respect to every parameter
        (into self.g) given dL/dout."""
        cfg, C, P = self.cfg, self.cfg.width, self.cfg.N ** 2
        cache = self.cache
        B = dout.shape[0]
        lib = _lib()
        _chk(lib.gpe_fno_bias_grad(_ptr(dout), _ptr(self.g["proj_b"]), B, cfg.cout, P, _stream()))
        self._pointwise_wgrad(dout, cache["v_last"], self.g["proj_w"], B, C, cfg.cout, P)
        dv = self._empty(B, C, P)
        # dv = proj_w^T dout
        gemm(dout, self.p["proj_w"], dv, P, C, cfg.cout, (1, P, cfg.cout * P), (C, 1, 0), (1, P, C * P), batch=B)
        for l in reversed(range(cfg.layers)):
            sv = cache["layers"][l]
            if sv["pre"] is not None:
                _chk(lib.gpe_fno_gelu_bwd(_ptr(dv), _ptr(sv["pre"]), B * C * P, _stream()))
            _chk(lib.gpe_fno_bias_grad(_ptr(dv), _ptr(self.g[f"b{l}"]), B, C, P, _stream()))
            self._pointwise_wgrad(dv, sv["v"], self.g[f"w{l}"], B, C, C, P)
            dvin = self._spectral_bwd(l, dv, B, sv["Gm"])
            # pointwise path: dvin += W^T dv
            gemm(dv, self.p[f"w{l}"], dvin, P, C, C, (1, P, C * P), (C, 1, 0), (1, P, C * P), batch=B, beta=1.0)
            dv = dvin
        _chk(lib.gpe_fno_bias_grad(_ptr(dv), _ptr(self.g["lift_b"]), B, C, P, _stream()))
        self._pointwise_wgrad(dv, cache["a"], self.g["lift_w"], B, cfg.cin, C, P)
        self.cache = None

    def loss_and_grad(self, pred, target):
        """MSE loss (host float) and its gradient (device tensor)."""
        torch = self.torch
        n = pred.numel()
        grad = torch.empty_like(pred)
        acc = torch.zeros(1, dtype=torch.float64, device=self.dev)
        _chk(_lib().gpe_fno_mse(_ptr(pred), _ptr(target), _ptr(grad), _ptr(acc), n, _stream()))
        return float(acc.item()) / n, grad

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        for k in self.p:
            _chk(_lib().gpe_fno_adam(_ptr(self.p[k]), _ptr(self.g[k]), _ptr(self.m[k]), _ptr(self.v[k]),
                                     self.p[k].numel(), lr, b1, b2, eps, self.t, _stream()))

    def params_numpy(self):
        return {k: v.detach().cpu().numpy() for k, v in self.p.items()}


# ---------------------------------------------------------------- data, training, rollout
POLARITON = dict(hbar=0.6582, m=1 / 6, dc=-0.5, dx=0.0, gc=0.05, gx=0.005, Om=5.07, g=0.003, w=50.0)


def polariton_problem(N: int, L: float, A: float, dtype=np.complex64, u0=None):
    """The two-component exciton-polariton problem of the throughput benchmark, with a
    constant pump amplitude A (Gaussian photon pump of width 50 centred in the box)."""
    from .problem import GrossPitaevskiiProblem
    p = POLARITON

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        return [[p["hbar"] * k2 / (2 * p["m"]) - p["dc"] - 1j * p["gc"], p["Om"]], [p["Om"], -p["dx"] - 1j * p["gx"]]]

    z = np.zeros((N, N), dtype) if u0 is None else None
    fields = (z, z.copy()) if u0 is None else tuple(np.asfortranarray(x.astype(dtype)) for x in u0)
    return GrossPitaevskiiProblem(
        fields, (L, L), dispersion=disp,
        nonlinearity=lambda u, _: [0 * u[0], p["g"] * np.abs(u[1]) ** 2],
        pump=lambda r, _, t: [A * np.exp(-((r[0] - L / 2) ** 2 + (r[1] - L / 2) ** 2) / p["w"] ** 2), 0])


def fields_to_channels(u1, u2, A, scale, amp_scale=6.0):
    """(N, N) complex fields -> (5, N*N) float32 channels [Re u1, Im u1, Re u2, Im u2, A]
    in row-major (y, x) point order, fields divided by scale."""
    ch = [u1.real, u1.imag, u2.real, u2.imag]
    out = np.empty((5, u1.size), np.float32)
    for i, c in enumerate(ch):
        out[i] = (np.ascontiguousarray(c.T) / scale).ravel()
    out[4] = A / amp_scale
    return out


def generate_pairs(n_traj: int, windows: int, steps_per_window: int = 20, N: int = 128, L: float = 256.0,
                   dt: float = 0.05, amp_range=(0.0, 6.0), seed: int = 0):
    """Training pairs from the solver itself: n_traj trajectories from u0 = 0 with constant
    pump amplitudes drawn uniformly from amp_range, each advanced windows x
    steps_per_window steps with a save every window.  Returns (amps, saves) with saves of
    shape (n_traj, windows + 1, 2, N, N) complex64 (time 0 included)."""
    from .strang import StrangSplitting, init
    rng = np.random.default_rng(seed)
    amps = rng.uniform(*amp_range, size=n_traj)
    saves = np.empty((n_traj, windows + 1, 2, N, N), np.complex64)
    for j, A in enumerate(amps):
        prob = polariton_problem(N, L, float(A))
        ts, res = (lambda it: (it.solve(), it.close())[0])(
            init(prob, StrangSplitting(), (0.0, windows * steps_per_window * dt), dt=dt, nsaves=windows))
        saves[j, :, 0] = np.moveaxis(res[0], -1, 0)
        saves[j, :, 1] = np.moveaxis(res[1], -1, 0)
    return amps, saves


def pairs_to_tensors(amps, saves, scale: float, device="cuda"):
    """Inputs (n, 5, N*N) and targets (n, 4, N*N) as device float32 tensors."""
    import torch
    n_traj, W1 = saves.shape[:2]
    N = saves.shape[-1]
    X = np.empty((n_traj * (W1 - 1), 5, N * N), np.float32)
    Y = np.empty((n_traj * (W1 - 1), 4, N * N), np.float32)
    k = 0
    for j in range(n_traj):
        for w in range(W1 - 1):
            X[k] = fields_to_channels(saves[j, w, 0], saves[j, w, 1], amps[j], scale)
            Y[k] = fields_to_channels(saves[j, w + 1, 0], saves[j, w + 1, 1], amps[j], scale)[:4]
            k += 1
    return torch.tensor(X, device=device), torch.tensor(Y, device=device)


def train(model: "FNO", X, Y, epochs: int, batch: int = 16, lr: float = 1e-3, seed: int = 0, log=None):
    """Adam on the MSE loss; returns the per-epoch mean losses."""
    import torch
    n = X.shape[0]
    gen = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen)
        tot, cnt = 0.0, 0
        lr_ep = lr * 0.5 * (1 + math.cos(math.pi * ep / max(1, epochs)))
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch].to(X.device)
            xb = X.index_select(0, idx).contiguous()
            yb = Y.index_select(0, idx).contiguous()
            pred = model.forward(xb, train=True)
            loss, grad = model.loss_and_grad(pred, yb)
            model.backward(grad)
            model.adam_step(lr=lr_ep)
            tot += loss
            cnt += 1
        losses.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {losses[-1]:.3e}")
    return losses


def channels_to_fields(ch: np.ndarray, scale: float, N: int):
    """(>=4, N*N) channels -> (u1, u2) complex (N, N) fields in the reference's (x, y) order."""
    u1 = (ch[0] + 1j * ch[1]).reshape(N, N).T * scale
    u2 = (ch[2] + 1j * ch[3]).reshape(N, N).T * scale
    return u1.astype(np.complex64), u2.astype(np.complex64)


def hybrid_rollout(model: "FNO", A: float, windows: int, scale: float, check_every: int = 10, tol: float = 1e-2,
                   N: int = 128, L: float = 256.0, dt: float = 0.05, steps_per_window: int = 20):
    """Advance the polariton from u0 = 0 by `windows` windows with the surrogate.  Every
    check_every-th window is judged: the plain solver advances the same state one window
    and the surrogate's prediction is accepted only if its rel L2 distance to the solver's
    is <= tol.  Otherwise (fallback), and when the state left the training range or is no
    longer finite (restart), the plain solver redoes the windows since the last accepted
    state, so the result is never further from the plain solver than the accepted
    surrogate windows make it.  Returns (u1, u2, stats)
    with stats = {checks, fallbacks, restarts, max_check_err, ms}."""
    import time
    import torch
    from .strang import StrangSplitting, init
    prob = polariton_problem(N, L, float(A))
    it = init(prob, StrangSplitting(), (0.0, (windows + 1) * steps_per_window * dt), dt=dt, nsaves=windows + 1)
    it.lib.gpe_set_graph(it.h, steps_per_window)
    state = torch.tensor(fields_to_channels(np.zeros((N, N)), np.zeros((N, N)), A, scale), device="cuda")[None]
    good, good_w = state.clone(), 0
    checks = fallbacks = restarts = 0
    max_err = 0.0

    def solver_windows(st, w0, n):
        u1, u2 = channels_to_fields(st[0].cpu().numpy(), scale, N)
        it.set_fields((u1, u2))
        s = it.state()
        s.steps, s.t = w0 * steps_per_window, w0 * steps_per_window * dt
        it.set_state(s)
        it.step(n * steps_per_window)
        v1, v2 = it.get_fields()
        return fields_to_channels(v1, v2, A, scale)

    fwd = model.graphed(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for w in range(windows):
        pred = fwd(state)
        if (w + 1) % check_every == 0:
            checks += 1
            # a state that left the range of the training data (|channel| <= 1) or is no
            # longer finite has diverged: the solver redoes the windows since the last
            # accepted state
            amax = float(state[0, :4].abs().max())
            if not math.isfinite(amax) or amax > 4.0:
                restarts += 1
                ref = solver_windows(good, good_w, w + 1 - good_w)
                state = torch.tensor(ref, device="cuda")[None]
                good, good_w = state.clone(), w + 1
                continue
            ref = solver_windows(state, w, 1)
            got = pred[0, :4].cpu().numpy()
            err = float(np.linalg.norm(got - ref[:4]) / max(np.linalg.norm(ref[:4]), 1e-30))
            if not math.isfinite(err):
                err = float("inf")
            max_err = max(max_err, err)
            if err > tol:
                # the surrogate is off here, so the windows since the last accepted state
                # are not trusted either: the solver redoes them
                fallbacks += 1
                ref = solver_windows(good, good_w, w + 1 - good_w)
                state = torch.tensor(ref, device="cuda")[None]
            else:
                nxt = torch.empty_like(state)
                nxt[:, :4] = pred
                nxt[:, 4] = state[:, 4]
                state = nxt
            good, good_w = state.clone(), w + 1
            continue
        nxt = torch.empty_like(state)
        nxt[:, :4] = pred
        nxt[:, 4] = state[:, 4]
        state = nxt
    amax = float(state[0, :4].abs().max())
    if not math.isfinite(amax) or amax > 4.0:
        restarts += 1
        state = torch.tensor(solver_windows(good, good_w, windows - good_w), device="cuda")[None]
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    it.close()
    u1, u2 = channels_to_fields(state[0].cpu().numpy(), scale, N)
    return u1, u2, {"checks": checks, "fallbacks": fallbacks, "restarts": restarts, "max_check_err": max_err,
                    "ms": ms}


def surrogate_window_ms(model: "FNO", batch: int, reps: int = 20) -> float:
    """Mean time of one surrogate window (one graph-replayed forward pass) for `batch`
    fields at once."""
    import time
    import torch
    x = torch.zeros((batch, model.cfg.cin, model.cfg.N ** 2), device="cuda")
    fwd = model.graphed(batch)
    fwd(x)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        fwd(x)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) * 1e3 / reps


def plain_rollout(A: float, windows: int, N: int = 128, L: float = 256.0, dt: float = 0.05,
                  steps_per_window: int = 20):
    """The plain solver over the same span (graph mode, one graph per window); returns
    (u1, u2, ms)."""
    from .strang import StrangSplitting, init
    prob = polariton_problem(N, L, float(A))
    it = init(prob, StrangSplitting(), (0.0, windows * steps_per_window * dt), dt=dt, nsaves=windows)
    it.lib.gpe_set_graph(it.h, steps_per_window)
    it.step(steps_per_window)  # capture the graph outside the timed region
    st = it.state()
    it.set_fields(tuple(np.zeros((N, N), np.complex64) for _ in range(2)))
    st.steps, st.t = 0, 0.0
    it.set_state(st)
    import time
    t0 = time.perf_counter()
    it.step(windows * steps_per_window)
    ms = (time.perf_counter() - t0) * 1e3
    u1, u2 = it.get_fields()
    it.close()
    return u1, u2, ms


def plain_window_ms(batch: int, reps: int = 10, N: int = 128, L: float = 256.0, dt: float = 0.05,
                    steps_per_window: int = 20, A: float = 3.0) -> float:
    """Mean time of one plain-solver window (steps_per_window steps, graph mode) for
    `batch` independent fields at once."""
    import time
    from .strang import StrangSplitting, init
    z = np.zeros((N, N, batch), np.complex64) if batch > 1 else np.zeros((N, N), np.complex64)
    prob = polariton_problem(N, L, A, u0=(z, z))
    it = init(prob, StrangSplitting(), (0.0, (reps + 2) * steps_per_window * dt), dt=dt, nsaves=1)
    it.lib.gpe_set_graph(it.h, steps_per_window)
    it.step(steps_per_window)
    t0 = time.perf_counter()
    it.step(reps * steps_per_window)
    ms = (time.perf_counter() - t0) * 1e3 / reps
    it.close()
    return ms
