"""The golden fixtures of tests/golden/ (outputs of the FP64 oracle on small seeded
cases, written by tests/golden/make_golden.py) still come out of the oracle: guards the
oracle against accidental change.  CPU only."""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _maker():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["kerr_c0", "polariton64", "philox_noise32", "matrix_nl32", "bistability1d", "kerr3d"])
def test_oracle_reproduces_golden(name):
    mk = _maker()
    want = np.load(GOLDEN / f"{name}.npz")
    got = mk.CASES[name]()
    assert set(got) == set(want.files)
    for k in want.files:
        a, b = np.asarray(got[k]), want[k]
        assert a.shape == b.shape, k
        if np.iscomplexobj(b) or b.dtype.kind == "f":
            scale = max(np.abs(b).max(), 1e-300)
            assert np.abs(a - b).max() <= 1e-13 * scale, k
        else:
            assert np.array_equal(a, b), k
