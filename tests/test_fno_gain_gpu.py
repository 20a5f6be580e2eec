"""What the trained surrogate gains, and what it does not, on a small budget: trained on
solver windows (polariton 128^2, 20 steps of dt 0.05 per window), its one-window error on
held-out trajectories falls well below the untrained network's and below persistence
(u(t + 20 dt) ~ u(t)); the hybrid rollout (surrogate windows, a solver check every 10,
solver redo on a failed check) stays within 1e-2 of the plain solver.  The cost ratio of
the hybrid to the plain rollout is reported, not asserted: on GB300 the fused solver
advances a window for less than one surrogate evaluation costs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_trained_surrogate_gain(gpe, lib):
    torch = pytest.importorskip("torch")
    F = __import__("gpe_gb300.fno", fromlist=["FNO"])
    amps, saves = F.generate_pairs(12, 60, seed=3)
    scale = float(np.abs(saves).max())
    X, Y = F.pairs_to_tensors(amps, saves, scale)
    va, vs = F.generate_pairs(2, 40, seed=99)
    VX, VY = F.pairs_to_tensors(va, vs, scale)

    def heldout_err(model):
        with torch.no_grad():
            pred = torch.cat([model.forward(VX[i:i + 16].contiguous()) for i in range(0, VX.shape[0], 16)])
        return float(torch.linalg.norm(pred - VY) / torch.linalg.norm(VY))

    model = F.FNO(F.FNOConfig(), seed=0)
    err_untrained = heldout_err(model)
    err_persist = float(torch.linalg.norm(VX[:, :4] - VY) / torch.linalg.norm(VY))
    losses = F.train(model, X, Y, epochs=4, batch=16, lr=2e-3)
    err_trained = heldout_err(model)
    print(f"held-out one-window rel L2: untrained {err_untrained:.3f}, persistence {err_persist:.3f}, "
          f"trained {err_trained:.3f}; losses {['%.2e' % v for v in losses]}")
    assert losses[-1] < losses[0]
    assert err_trained < 0.5 * err_untrained
    assert err_trained < err_persist

    A, windows = 3.0, 40
    h1, h2, st = F.hybrid_rollout(model, A, windows, scale)
    p1, p2, ms_plain = F.plain_rollout(A, windows)
    err = rel(np.concatenate([h1.ravel(), h2.ravel()]), np.concatenate([p1.ravel(), p2.ravel()]))
    print(f"hybrid vs plain after {windows} windows: rel L2 {err:.2e}, checks {st['checks']}, "
          f"fallbacks {st['fallbacks']}, restarts {st['restarts']}, hybrid {st['ms']:.1f} ms, "
          f"plain {ms_plain:.1f} ms (gain x{ms_plain / st['ms']:.2f})")
    assert err <= 1e-2
