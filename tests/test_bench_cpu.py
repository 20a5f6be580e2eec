"""bench.py's line contract and helpers, on the CPU: the reference arm prints one JSON
line with every key the measurement contract names; the algorithmic-byte model and
roofline object, and the closed-form 2x2 exponential of the plain comparator."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_warmup_below_three_is_refused():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "2"],
                       capture_output=True, text=True, timeout=120, cwd=ROOT)
    assert r.returncode != 0 and "warmup" in r.stderr


def test_algorithmic_bytes_and_roofline_fields():
    import bench
    ab = bench.algorithmic_bytes(np.complex128, 64)
    assert ab["row"] == 64 + 8 / 64 and ab["col"] == 64 + 64 / 64
    ab = bench.algorithmic_bytes(np.complex64, 128)
    assert ab["row"] == 32 + 4 / 128 and ab["col"] == 32 + 32 / 128
    # the roofline object is built from the run's own event timings; DRAM traffic is not
    # measured in the run, so it is null rather than read from a file
    m = {"kms": np.array([2.0, 1.0, 0.0]), "kn": np.array([10, 10, 0])}
    r = bench.roofline_of(m, np.complex128, "native", 64)
    assert r["traffic"] is None and r["kernel"] == "row pass" and r["bound"] == "hbm"
    want = ab_row = bench.algorithmic_bytes(np.complex128, 64)["row"] * 512 * 512 * 64 / 0.2e-3 / 1e9
    assert abs(r["achieved"] - want) <= 1e-9 * want and abs(r["frac"] - want / r["peak"]) <= 1e-12
    assert "profiles/" not in r["binding_limit"] and ab_row > 0


def test_closed_form_2x2_exponential():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    import bench
    rng = np.random.default_rng(2)
    A = rng.standard_normal((2, 2, 50)) + 1j * rng.standard_normal((2, 2, 50))
    A[:, :, :5] *= 1e-5  # near-degenerate: the series branch
    A[0, 1, 5:10] = 0.0  # triangular
    E = bench.expm2_np([[A[i, j] for j in range(2)] for i in range(2)])
    for n in range(A.shape[2]):
        want = scipy_linalg.expm(A[:, :, n])
        got = np.array([[E[i][j][n] for j in range(2)] for i in range(2)])
        assert np.abs(got - want).max() <= 1e-13 * max(1.0, np.abs(want).max()), n


def test_reference_arm_under_torchrun_prints_one_line():
    """Two ranks launched as the multi-GPU bench is: rank 0 alone runs the reference arm
    and prints; the other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29517", str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
