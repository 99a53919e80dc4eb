"""Accuracy of the exp/expm1/tanh/log/pow/atan restatements shared (as a method) by the oracle and
the FP64 GPU path, against the platform libm, in units in the last place."""
import math

import numpy as np
import pytest

from oracle import oracle


def ulp_err(got, want):
    if want == 0.0:
        return abs(got) / 5e-324
    return abs(got - want) / math.ulp(want)


@pytest.fixture(scope="module")
def lib():
    return oracle.load()


@pytest.mark.parametrize("fn,ref,lo,hi,tol", [
    ("exp", math.exp, -700.0, 700.0, 4),
    ("exp", math.exp, -2.0, 2.0, 3),
    ("expm1", math.expm1, -0.5, 0.5, 3),
    ("expm1", math.expm1, -30.0, 30.0, 6),
    ("tanh", math.tanh, -25.0, 25.0, 4),
    ("tanh", math.tanh, -1e-3, 1e-3, 3),
    ("log", math.log, 1e-300, 1e300, 3),
    ("log", math.log, 0.5, 2.0, 3),
    ("atan", math.atan, -60.0, 60.0, 3),
    ("atan", math.atan, -1.0, 1.0, 3),
    ("atan", math.atan, 1e-12, 1e12, 3),
])
def test_accuracy(lib, fn, ref, lo, hi, tol):
    rng = np.random.default_rng(1)
    if lo > 0:
        xs = np.exp(rng.uniform(math.log(lo), math.log(hi), 20000))
    else:
        xs = rng.uniform(lo, hi, 20000)
    f = getattr(lib, "oracle_tm_" + fn)
    worst = max(ulp_err(f(float(x)), ref(float(x))) for x in xs)
    assert worst <= tol, f"{fn}: {worst:.2f} ulp"


def test_pow_accuracy(lib):
    rng = np.random.default_rng(2)
    # exp(y log x) carries the rounding of y log x into the result: bound 2 + 1.5 |y log x| ulp
    for x, y in zip(rng.uniform(0.05, 20.0, 5000), rng.choice([2.5, 1.4, 1.0 / 3.5, 1.5], 5000)):
        x, y = float(x), float(y)
        err = ulp_err(lib.oracle_tm_pow(x, y), x ** y)
        assert err <= 2 + 1.5 * abs(y * math.log(x)), f"pow({x}, {y}): {err:.2f} ulp"


def test_special_values(lib):
    assert lib.oracle_tm_exp(0.0) == 1.0
    assert lib.oracle_tm_tanh(0.0) == 0.0 and math.copysign(1, lib.oracle_tm_tanh(-0.0)) < 0
    assert lib.oracle_tm_tanh(40.0) == 1.0 and lib.oracle_tm_tanh(-40.0) == -1.0
    assert lib.oracle_tm_log(1.0) == 0.0
    assert math.isnan(lib.oracle_tm_tanh(float("nan")))
    assert lib.oracle_tm_atan(0.0) == 0.0 and math.copysign(1, lib.oracle_tm_atan(-0.0)) < 0
    assert lib.oracle_tm_atan(float("inf")) == math.pi / 2 and lib.oracle_tm_atan(-float("inf")) == -math.pi / 2
    assert abs(lib.oracle_tm_atan(1.0) - math.pi / 4) <= math.ulp(math.pi / 4)
