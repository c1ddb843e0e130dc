"""The FP64 path's own exp, log, pow and reciprocal (table-driven and Newton
methods that trade the last ulp for fewer FP64 instructions) against numpy's
libm over the ranges the day step feeds them, plus the hardware approximation
the reciprocal starts from."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ULP = 2.0 ** -52


def _rel(a, b):
    return np.abs(a - b) / np.abs(b)


def test_exp_log_pow_within_a_few_ulp():
    from watergap2_gb300.gpu import math_eval
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-700, 700, 20000), rng.uniform(-1, 1, 20000), [0.0, 1e-300, -1e-300]])
    assert _rel(math_eval("exp", x), np.exp(x)).max() < 4 * ULP
    lx = np.concatenate([10.0 ** rng.uniform(-300, 300, 20000), rng.uniform(0.5, 2.0, 20000), [1.0]])
    got = math_eval("log", lx)
    ref = np.log(lx)
    # a few ulp of max(|log x|, 1): just below x = 1 the sum m ln2 + log F cancels,
    # and an absolute error is what pow = exp(y log x) passes on
    assert np.all(np.abs(got - ref) <= 4 * ULP * np.maximum(np.abs(ref), 1.0))
    assert got[lx == 1.0].max() == 0.0
    px = 10.0 ** rng.uniform(-8, 6, 20000)
    py = rng.uniform(0.1, 5.0, 20000)
    ref = px ** py
    bound = (4 + np.abs(py * np.log(px)) * 2) * ULP      # the error of y log x, amplified by exp
    assert np.all(_rel(math_eval("pow", px, py), ref) < bound)
    assert np.array_equal(math_eval("pow", np.array([0.0, 1.0]), np.array([0.66, 2.5])), [0.0, 1.0])


def test_reciprocal_from_the_hardware_approximation():
    from watergap2_gb300.gpu import math_eval
    rng = np.random.default_rng(2)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 50000), rng.uniform(1.0, 2.0, 50000),
                        -rng.uniform(1e-3, 1e3, 1000), [1.0, 2.0, 0.5, 237.3, 2.501]])
    ref = 1.0 / x
    approx = math_eval("rcp_approx", x)
    assert _rel(approx, ref).max() < 2.0 ** -20          # the start the Newton step needs
    assert _rel(math_eval("rcp", x), ref).max() < 2 * ULP
