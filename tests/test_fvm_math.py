"""fv_math.h: the apps' sin/cos/exp/tanh, evaluated alike on host and device.

Each float result must be the correctly rounded value of the function
(computed here in float64 by numpy and rounded once) except, rarely, by one
ulp near a rounding tie; and within one ulp of float32 libm values.
"""
import numpy as np
import pytest

from oracle.oracle import fvm_eval

FUNCS = {"sin": np.sin, "cos": np.cos, "exp": np.exp, "tanh": np.tanh}


def _args(fn, n=200_000, seed=0):
    rng = np.random.default_rng(seed)
    if fn in ("sin", "cos"):
        # source phases reach ISPW * T ~ 2 pi * 1000
        return np.concatenate([rng.uniform(-7000, 7000, n), rng.uniform(-4, 4, n)]).astype(np.float32)
    if fn == "exp":
        return rng.uniform(-103, 88, n).astype(np.float32)
    return np.concatenate([rng.uniform(-12, 12, n), rng.uniform(-1e-3, 1e-3, n)]).astype(np.float32)


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


@pytest.mark.parametrize("fn", list(FUNCS))
def test_correctly_rounded(fn):
    x = _args(fn)
    got = fvm_eval(fn, x)
    ref = FUNCS[fn](x.astype(np.float64)).astype(np.float32)
    u = _ulps(got, ref)
    assert u.max() <= 1
    assert np.count_nonzero(u) <= 1e-5 * x.size


@pytest.mark.parametrize("fn", list(FUNCS))
def test_special_values(fn):
    x = np.array([0.0, -0.0, 1e-30, -1e-30, 20.0, -20.0], np.float32)
    got = fvm_eval(fn, x)
    ref = FUNCS[fn](x.astype(np.float64)).astype(np.float32)
    assert np.all(_ulps(got, ref) <= 1)
    if fn == "exp":
        big = fvm_eval("exp", np.array([100.0, -200.0, -1e30], np.float32))
        assert np.isinf(big[0]) and big[1] == 0 and big[2] == 0
