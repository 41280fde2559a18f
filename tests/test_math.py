"""include/er_math.h: accuracy against float64 numpy on the host."""
import numpy as np
import pytest

import oracle_lib as OL


def ulp_err(got, want):
    want32 = want.astype(np.float32)
    sp = np.spacing(np.abs(want32).astype(np.float32))
    return np.abs(got.astype(np.float64) - want) / sp


def run(oracle, fn, x, y=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x) if y is None else np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(x)
    oracle.math_eval(fn, len(x), OL.ptr(x), OL.ptr(y), OL.ptr(out))
    return out


@pytest.mark.parametrize("fn,lo,hi,ref,tol", [
    (0, 1e-30, 1e30, np.log, 2.0),
    (1, -87.0, 88.0, np.exp, 2.0),
    (2, -7.0, 7.0, np.sin, 2.0),
    (3, -7.0, 7.0, np.cos, 2.0),
])
def test_unary_accuracy(oracle, fn, lo, hi, ref, tol):
    rng = np.random.default_rng(fn)
    if fn == 0:
        x = np.exp(rng.uniform(np.log(lo), np.log(hi), 200000)).astype(np.float32)
    else:
        x = rng.uniform(lo, hi, 200000).astype(np.float32)
    got = run(oracle, fn, x)
    want = ref(x.astype(np.float64))
    if fn in (2, 3):
        # relative to 1 near zeros of sin/cos (absolute error bound)
        err = np.abs(got.astype(np.float64) - want) / np.spacing(np.float32(1.0))
        assert err.max() < 4.0
    else:
        assert ulp_err(got, want).max() <= tol


def test_log_special(oracle):
    x = np.array([0.0, -0.0, -1.0, np.inf, np.nan, 1.0, 1e-45, 3.4e38], np.float32)
    got = run(oracle, 0, x)
    assert got[0] == -np.inf and got[1] == -np.inf and np.isnan(got[2]) and got[3] == np.inf and np.isnan(got[4])
    assert got[5] == 0.0 and np.isfinite(got[6]) and np.isfinite(got[7])


def test_pow_accuracy(oracle):
    rng = np.random.default_rng(9)
    x = rng.uniform(0.0, 1.0, 100000).astype(np.float32)
    y = np.exp(rng.uniform(np.log(0.5), np.log(1e6), 100000)).astype(np.float32)
    got = run(oracle, 5, x, y)
    want = np.power(x.astype(np.float64), y.astype(np.float64))
    mask = want > 1e-37
    assert ulp_err(got[mask], want[mask]).max() <= 4.0
    # integer exponents of negative bases, zeros
    g = run(oracle, 5, np.array([-2.0, -2.0, 0.0, 0.0, 1.0, 5.0], np.float32), np.array([2.0, 3.0, 2.0, 0.0, 1e6, 0.0], np.float32))
    assert list(g) == [4.0, -8.0, 0.0, 1.0, 1.0, 1.0]


def test_acos_atan2(oracle):
    rng = np.random.default_rng(10)
    x = rng.uniform(-1, 1, 50000).astype(np.float32)
    assert ulp_err(run(oracle, 6, x), np.arccos(x.astype(np.float64))).max() <= 3.0
    a = rng.normal(size=50000).astype(np.float32)
    b = rng.normal(size=50000).astype(np.float32)
    assert ulp_err(run(oracle, 7, a, b), np.arctan2(a.astype(np.float64), b.astype(np.float64))).max() <= 3.0
