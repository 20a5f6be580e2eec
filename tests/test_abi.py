"""The C ABI: libgpe.so loads, exports every function include/gpe.h declares, the
ctypes structs match the C layout, and argument validation happens before any CUDA
call (so it is testable without a GPU)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = []
    for h in HEADERS:
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(gpe_[a-z0-9_]+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib, gpe):
    names = declared_functions()
    assert len(names) >= 20
    L = __import__("gpe_gb300._lib", fromlist=["SIGNATURES"])
    F = __import__("gpe_gb300.fno", fromlist=["FNO_SIGNATURES"])
    sigs = dict(L.SIGNATURES, **F.FNO_SIGNATURES)
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"
        assert n in sigs, f"{n} has no ctypes signature"


def test_struct_layout_matches_c(gpe, tmp_path):
    L = __import__("gpe_gb300._lib", fromlist=["GpeDesc"])
    src = tmp_path / "layout.c"
    src.write_text(f'''#include <stdio.h>
#include <stddef.h>
#include "{ROOT / 'include' / 'gpe.h'}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gpe_desc), offsetof(gpe_desc, n),
         offsetof(gpe_desc, lengths), offsetof(gpe_desc, batch), offsetof(gpe_desc, ncomp),
         offsetof(gpe_desc, dt), offsetof(gpe_desc, t0), offsetof(gpe_desc, device),
         sizeof(gpe_state), offsetof(gpe_state, noise_mode));
  return 0;
}}''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-O0", "-o", str(exe), str(src)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    D, S = L.GpeDesc, L.GpeState
    want = [ctypes.sizeof(D), D.n.offset, D.lengths.offset, D.batch.offset, D.ncomp.offset, D.dt.offset,
            D.t0.offset, D.device.offset, ctypes.sizeof(S), S.noise_mode.offset]
    assert got == want


def test_fno_struct_layouts_match_c(gpe, tmp_path):
    F = __import__("gpe_gb300.fno", fromlist=["GemmDesc"])
    src = tmp_path / "fno_layout.c"
    src.write_text(f'''#include <stdio.h>
#include <stddef.h>
#include "{ROOT / 'include' / 'gpe_fno.h'}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(gpe_gemm_desc), offsetof(gpe_gemm_desc, c_z),
         offsetof(gpe_gemm_desc, alpha), sizeof(gpe_permute_desc), offsetof(gpe_permute_desc, d),
         offsetof(gpe_gemm_desc, batch));
  return 0;
}}''')
    exe = tmp_path / "fno_layout"
    subprocess.run(["gcc", "-O0", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    G, Pm = F.GemmDesc, F.PermDesc
    assert got == [ctypes.sizeof(G), G.c_z.offset, G.alpha.offset, ctypes.sizeof(Pm), Pm.d.offset, G.batch.offset]


def _desc(L, **kw):
    d = L.GpeDesc()
    d.abi_version = L.GPE_ABI_VERSION
    d.ndim = 2
    d.n[0], d.n[1], d.n[2] = 64, 64, 1
    d.lengths[0], d.lengths[1], d.lengths[2] = 1.0, 1.0, 1.0
    d.batch = 1
    d.ncomp = 1
    d.dtype = L.GPE_C128
    d.dt = 0.01
    d.t0 = 0.0
    d.device = -1
    for k, v in kw.items():
        if k == "n":
            for i, x in enumerate(v):
                d.n[i] = x
        else:
            setattr(d, k, v)
    return d


@pytest.mark.parametrize("kw,code", [
    (dict(abi_version=99), -1),
    (dict(ndim=0), -1),
    (dict(ndim=4), -1),
    (dict(ncomp=3), -2),
    (dict(dtype=7), -1),
    (dict(batch=0), -1),
    (dict(dt=-1.0), -1),
    (dict(dt=float("nan")), -1),
    (dict(n=(100, 64, 1)), -2),
    (dict(n=(8, 64, 1)), -2),
    (dict(n=(64, 8192, 1)), -2),
    (dict(dtype=1, flags=32), -1),     # block floating point transforms: FP64 fields only
    (dict(flags=32 | 16), -1),         # ... and not with the double-word mode
])
def test_create_rejects_bad_descriptors(lib, gpe, kw, code):
    L = __import__("gpe_gb300._lib", fromlist=["GpeDesc"])
    h = ctypes.c_void_p()
    rc = lib.gpe_create(ctypes.byref(_desc(L, **kw)), ctypes.byref(h))
    assert rc == code
    assert not h.value
    assert lib.gpe_last_error(None)


def test_wait_probe_refuses_limits_beyond_one_second(lib, gpe):
    """gpe_selftest_wait checks its limit before it touches the device, so a caller cannot
    make the probe spin for longer than the library's own wait bound."""
    L = gpe._lib
    assert lib.gpe_selftest_wait(0, 0, 10 ** 9 + 1) == L.GPE_ERR_INVALID
    assert lib.gpe_selftest_wait(0, 0, -1) == L.GPE_ERR_INVALID
    assert lib.gpe_selftest_wait(0, 1, 2 ** 63 - 1) == L.GPE_ERR_INVALID


def test_null_arguments(lib, gpe):
    assert lib.gpe_create(None, None) == -1
    assert lib.gpe_destroy(None) == 0
    assert lib.gpe_run(None, 1, 0, None, None) == -1
    assert lib.gpe_version().startswith(b"libgpe")


def test_no_cpu_fallback(gpe, tmp_path):
    """Loading a missing library raises instead of falling back to the CPU."""
    L = __import__("gpe_gb300._lib", fromlist=["load"])
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        L.load(tmp_path / "missing.so")


def test_c_driver_compiles_and_links(lib, gpe, tmp_path):
    """The plain-C driver of the reference's plain case (tests/c_abi/kerr_c0.c) builds
    against include/gpe.h and links against libgpe.so: the ABI is usable without Python."""
    libdir = Path(lib._name).resolve().parent
    exe = tmp_path / "kerr_c0"
    subprocess.run(["gcc", "-O2", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_abi" / "kerr_c0.c"), f"-L{libdir}", "-lgpe", "-lm", "-o", str(exe)],
                   check=True)
    assert exe.exists()
