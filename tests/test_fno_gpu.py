"""The FNO surrogate's kernels: the BF16 tensor-core GEMM against numpy, and the
network's forward pass and every parameter gradient against a CPU oracle (torch autograd
in FP32 with the same BF16 rounding of GEMM operands)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fno_mod(gpe):
    return __import__("gpe_gb300.fno", fromlist=["FNO"])


def bf16(x):
    """Round to bfloat16 (round to nearest even) and back to float32, in numpy."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("M,N,K,ta,tb,batch,beta", [(200, 70, 96, False, False, 1, 0.0), (64, 128, 40, True, False, 3, 0.0),
                                                     (33, 17, 300, False, True, 2, 1.0), (129, 65, 16, True, True, 1, 1.0),
                                                     (4096, 32, 32, True, False, 2, 0.0), (1000, 64, 64, False, True, 1, 1.0),
                                                     (256, 200, 1024, False, False, 1, 0.0), (128, 32, 8, True, True, 1, 0.0),
                                                     (512, 64, 64, False, False, 1, 0.0), (512, 64, 64, True, True, 2, 0.0)])
@pytest.mark.parametrize("shift", [0, 1], ids=["aligned", "shifted"])
def test_gemm_matches_numpy(gpe, lib, M, N, K, ta, tb, batch, beta, shift):
    """Every stride pattern in both staging forms: 16-byte aligned operands whose K index
    is contiguous are staged with float4 loads, the rest and operands shifted by one
    element (not 16-byte aligned) element by element."""
    torch = pytest.importorskip("torch")
    F = fno_mod(gpe)
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((batch, K, M) if ta else (batch, M, K)).astype(np.float32)
    B = rng.standard_normal((batch, N, K) if tb else (batch, K, N)).astype(np.float32)
    C0 = rng.standard_normal((batch, M, N)).astype(np.float32)

    def dev(x):
        buf = torch.zeros(x.size + shift, device="cuda")
        buf[shift:] = torch.tensor(x.ravel(), device="cuda")
        return buf[shift:]  # the operand starts `shift` elements into its buffer

    At, Bt = dev(A), dev(B)
    Ct = torch.tensor(C0, device="cuda")
    a = (1, M, K * M) if ta else (K, 1, M * K)
    b = (1, K, N * K) if tb else (N, 1, K * N)
    F.gemm(At, Bt, Ct, M, N, K, a, b, (N, 1, M * N), batch=batch, alpha=1.5, beta=beta)
    Aop = np.swapaxes(A, 1, 2) if ta else A
    Bop = np.swapaxes(B, 1, 2) if tb else B
    want = 1.5 * np.matmul(bf16(Aop).astype(np.float64), bf16(Bop).astype(np.float64)) + beta * C0
    got = Ct.cpu().numpy()
    assert F.take_status() == 0  # no bounded wait of the tcgen05 kernel ran out
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max() + 1e-5


def reference_forward(torch, P, a, cfg, bases):
    """The same network in torch (CPU, FP32), GEMM operands rounded to BF16."""
    bf = lambda x: x.to(torch.bfloat16).to(torch.float32)
    B, C, N, m = a.shape[0], cfg.width, cfg.N, cfg.modes
    v = torch.einsum("oi,bip->bop", bf(P["lift_w"]), bf(a)) + P["lift_b"][None, :, None]
    for l in range(cfg.layers):
        Vx = bf(v.reshape(B * C * N, N)) @ bf(bases["Bx"])
        Vt = Vx.reshape(B * C, N, 2, m).permute(0, 3, 2, 1).reshape(B * C * m, 2 * N)
        G = bf(Vt) @ bf(bases["By"])
        Gm = G.reshape(B, C, m, 2, m).permute(4, 2, 0, 3, 1).reshape(m * m, B, 2 * C)
        Hm = torch.bmm(bf(Gm), bf(P[f"r{l}"]))
        H = Hm.reshape(m, m, B, 2, C).permute(2, 4, 1, 3, 0).reshape(B * C * m, 2 * m)
        Ht = bf(H) @ bf(bases["Iy"])
        Hx = Ht.reshape(B * C, m, 2, N).permute(0, 3, 2, 1).reshape(B * C * N, 2 * m)
        S = (bf(Hx) @ bf(bases["Ix"])).reshape(B, C, N * N)
        S = S + torch.einsum("oi,bip->bop", bf(P[f"w{l}"]), bf(v)) + P[f"b{l}"][None, :, None]
        v = torch.nn.functional.gelu(S) if l < cfg.layers - 1 else S
    return torch.einsum("oc,bcp->bop", bf(P["proj_w"]), bf(v)) + P["proj_b"][None, :, None] + a[:, :cfg.cout]


def test_fno_forward_and_gradients_match_cpu_autograd(gpe, lib):
    torch = pytest.importorskip("torch")
    F = fno_mod(gpe)
    cfg = F.FNOConfig(N=32, width=8, modes=8, layers=3)
    params = F.init_params(cfg, seed=3)
    for k in params:  # non-zero biases so their gradients are exercised
        if k.endswith("_b") or k.startswith("b"):
            params[k] = (0.1 * np.random.default_rng(len(k)).standard_normal(params[k].shape)).astype(np.float32)
    rng = np.random.default_rng(0)
    B, P = 2, cfg.N ** 2
    a = rng.standard_normal((B, cfg.cin, P)).astype(np.float32)
    y = rng.standard_normal((B, cfg.cout, P)).astype(np.float32)
    model = F.FNO(cfg, params)
    pred = model.forward(torch.tensor(a, device="cuda"), train=True)
    loss, grad = model.loss_and_grad(pred, torch.tensor(y, device="cuda"))
    model.backward(grad)
    # CPU oracle
    Pc = {k: torch.tensor(v, requires_grad=True) for k, v in params.items()}
    bases = {k: torch.tensor(v) for k, v in F.dft_bases(cfg).items()}
    out = reference_forward(torch, Pc, torch.tensor(a), cfg, bases)
    ref_loss = ((out - torch.tensor(y)) ** 2).mean()
    ref_loss.backward()
    got = pred.cpu().numpy()
    want = out.detach().numpy()
    assert np.linalg.norm(got - want) <= 2e-3 * np.linalg.norm(want)
    assert abs(loss - ref_loss.item()) <= 2e-3 * ref_loss.item()
    for k in params:
        g_gpu = model.g[k].cpu().numpy()
        g_ref = Pc[k].grad.numpy()
        err = np.linalg.norm(g_gpu - g_ref) / max(np.linalg.norm(g_ref), 1e-30)
        assert err <= 2e-2, (k, err)
