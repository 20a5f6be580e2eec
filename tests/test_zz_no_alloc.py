"""gpe_norms_noalloc: the entry point for callers that cannot allocate device memory
(their device memory belongs to another allocator, or cudaMalloc's implicit device
synchronisation is not acceptable where they run).  It must give the same norms as
the handle-based gpe_norm, call after call, while allocating nothing itself.

This file is collected last so that a run stopping at the first failure has already
run every other test; it also passes when run alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from cases import kerr2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,fp64", [(np.complex128, "dw"), (np.complex128, "native"), (np.complex64, "dw")],
                         ids=["c128-dw", "c128-native", "c64"])
def test_noalloc_norms_match_gpe_norm(gpe, lib, dtype, fp64):
    torch = pytest.importorskip("torch")
    L = __import__("gpe_gb300._lib", fromlist=["GPE_C128"])
    B = 3
    gpu_kw, _ = kerr2d(64, 8.0, -2.0, dtype, batch=(B,))
    x = gpu_kw["u0"][0]
    gpu_kw["u0"] = (x, (0.5 * x).astype(dtype))
    gpu_kw["nonlinearity"] = lambda u, p: [-2.0 * np.abs(u[0]) ** 2, 0.5 * np.abs(u[1]) ** 2]
    gpu_kw["dispersion"] = lambda k, p: [(k[0] ** 2 + k[1] ** 2) / 2, (k[0] ** 2 + k[1] ** 2) / 3]
    prob = gpe.GrossPitaevskiiProblem(**gpu_kw)
    it = gpe.init(prob, gpe.StrangSplitting(), (0.0, 0.1), dt=0.01, nsaves=1, fp64=fp64)
    P, dV = 64 * 64, (8.0 / 64) ** 2
    tdt = torch.float64 if dtype == np.complex128 else torch.float32
    cdt = L.GPE_C128 if dtype == np.complex128 else L.GPE_C64
    bufs = [torch.empty(2 * B * P, dtype=tdt, device="cuda") for _ in range(2)]
    ptrs = (ctypes.c_void_p * 2)(*[b.data_ptr() for b in bufs])
    tol = 1e-12 if dtype == np.complex128 else 1e-6
    try:
        for call in range(2):  # two calls in a row, the state advancing in between
            it.step(3)
            ref = it.norm()
            for m in range(2):
                L.check(lib, it.h, lib.gpe_get_field_dev(it.h, m, ctypes.c_void_p(bufs[m].data_ptr())))
            torch.cuda.synchronize()
            out = np.full(2 * B, np.nan)
            rc = lib.gpe_norms_noalloc(ptrs, 2, P, B, cdt, dV, out.ctypes.data)
            assert rc == 0, lib.gpe_noalloc_last_error()
            per = out.reshape(2, B)
            assert np.all(np.isfinite(per))
            for m in range(2):
                assert abs(per[m].sum() - ref[m]) <= tol * abs(ref[m]), (call, m, per[m].sum(), ref[m])
            # each trajectory's norm against the host copy of the state
            host = it.get_fields()
            for m in range(2):
                hv = np.asarray(host[m]).reshape(P, B, order="F")
                want = (np.abs(hv) ** 2).sum(0) * dV
                assert np.allclose(per[m], want, rtol=tol, atol=0)
    finally:
        it.close()


def test_noalloc_rejects_sizes_beyond_the_scratch(gpe, lib):
    L = __import__("gpe_gb300._lib", fromlist=["GPE_C128"])
    ptrs = (ctypes.c_void_p * 2)(1, 1)
    out = np.zeros(4)
    rc = lib.gpe_norms_noalloc(ptrs, 2, 16, 8192, L.GPE_C128, 1.0, out.ctypes.data)
    assert rc == L.GPE_ERR_INVALID
    assert b"GPE_NOALLOC_MAX_NORMS" in lib.gpe_noalloc_last_error()
    assert lib.gpe_norms_noalloc(ptrs, 3, 16, 1, L.GPE_C128, 1.0, out.ctypes.data) == L.GPE_ERR_INVALID
