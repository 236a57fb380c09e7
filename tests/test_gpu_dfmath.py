"""The fit's double-float functions (pairs of floats on the FP32 pipes, which replace FP64
division, square root, exp and log on the fit's serial paths) against numpy's FP64, over the
ranges the fit uses, with the relative tolerances their use needs (the FP64 fit's parity with the
oracle is 1e-7 in e and 1e-9 in maxL)."""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib
from radiolensfit2_gb300.abi import dptr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def _run(lib, op, x, y=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    yy = np.ascontiguousarray(y, dtype=np.float64) if y is not None else None
    assert lib.rlf_debug_df_math(op, x.size, dptr(x), dptr(yy) if yy is not None else None, dptr(out)) == 0
    return out


def rel(a, b, floor=0.0):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


def test_df_math(lib):
    rng = np.random.default_rng(5)
    n = 1 << 16
    e = rng.uniform(-40.0, 40.0, n)
    v = np.exp(rng.uniform(-80.0, 80.0, n))
    w = np.exp(rng.uniform(-700.0, 700.0, n))
    a, b = rng.uniform(-1e3, 1e3, n), rng.uniform(1e-3, 1e3, n) * rng.choice([-1.0, 1.0], n)
    s = np.exp(rng.uniform(-60.0, 60.0, n))
    q = np.exp(rng.uniform(-20.0, 20.0, n))
    d = rng.standard_normal(n) * np.exp(rng.uniform(-40.0, 40.0, n))
    # largest relative errors (logs: of max(|log|, 1)) and their bounds: the measured ones with
    # margin, all far below the FP64 fit's parity tolerances
    errs = {
        "exp": (rel(_run(lib, 0, e), np.exp(e)), 5e-13),
        "log": (rel(_run(lib, 1, v), np.log(v), floor=1.0), 2e-12),
        "log_double": (rel(_run(lib, 2, w), np.log(w), floor=1.0), 2e-12),
        "div": (rel(_run(lib, 3, a, b), a / b), 1e-13),
        "sqrt": (rel(_run(lib, 4, s), np.sqrt(s)), 1e-13),
        "profile": (rel(_run(lib, 5, q), (1.0 + q) ** -1.5), 5e-13),
        "split": (rel(_run(lib, 6, d), d), 2e-14),
    }
    print({k: f"{v[0]:.2e}" for k, v in errs.items()})
    for k, (err, bound) in errs.items():
        assert err < bound, (k, err)


def test_df_math_edges(lib):
    out = _run(lib, 4, [0.0, -1.0])
    assert out[0] == 0.0 and np.isnan(out[1])
    out = _run(lib, 1, [0.0, -1.0, np.inf])
    assert out[0] == -np.inf and np.isnan(out[1]) and out[2] == np.inf
    out = _run(lib, 0, [np.nan, -100.0, 100.0])
    assert np.isnan(out[0]) and out[1] == 0.0 and out[2] == np.inf
    assert _run(lib, 6, [0.0, -0.0, 1.0, -2.5]).tolist() == [0.0, 0.0, 1.0, -2.5]
