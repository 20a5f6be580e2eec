"""The C ABI driven from plain C (no Python on the path), the way a Julia ccall shim
drives it: tests/c_abi/kerr_c0.c runs the reference's plain case (128^2 Kerr, g=-6,
64 saves) through gpe_create / gpe_set_field / gpe_set_dispersion /
gpe_set_nonlinearity / gpe_run and writes the last save, compared here with the golden
fixture at 1e-10."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("mode", ["dw", "native", "bfp"])
def test_plain_case_from_c(gpe, lib, tmp_path, mode):
    libdir = Path(lib._name).resolve().parent
    exe = tmp_path / "kerr_c0"
    subprocess.run(["gcc", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "c_abi" / "kerr_c0.c"),
                    f"-L{libdir}", "-lgpe", f"-Wl,-rpath,{libdir}", "-lm", "-o", str(exe)], check=True)
    out = tmp_path / "out.bin"
    args = [str(exe), str(out)] + ([] if mode == "bfp" else [mode])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.float64)
    N = 128
    u = (raw[0:2 * N * N:2] + 1j * raw[1:2 * N * N:2]).reshape(N, N)
    t = raw[2 * N * N]
    G = np.load(ROOT / "tests" / "golden" / "kerr_c0.npz")
    assert abs(t - G["ts"][-1]) <= 1e-15
    want = G["saves"][-1]
    assert np.linalg.norm(u - want) / np.linalg.norm(want) <= 1e-10
