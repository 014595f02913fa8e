"""Accuracy of the shared float math library (rmath.h) against float64."""
import numpy as np
import pytest

import oracle


def ulp_err(got, ref):
    ref32 = ref.astype(np.float32)
    sp = np.maximum(np.spacing(np.abs(ref32)).astype(np.float64), 1.4e-45)
    return np.nanmax(np.abs(got.astype(np.float64) - ref) / sp)


CASES = [
    (0, lambda r: r.uniform(-100, 88, 400000), None, np.exp, 2),
    (1, lambda r: np.exp(r.uniform(-80, 80, 400000)), None, np.log, 2),
    (2, lambda r: r.uniform(-50, 50, 400000), None, np.sin, 3),
    (3, lambda r: r.uniform(-50, 50, 400000), None, np.cos, 3),
    (5, lambda r: r.uniform(-1, 1, 400000), None, np.arcsin, 4),
    (6, lambda r: r.uniform(-1, 1, 400000), None, np.arccos, 4),
    (7, lambda r: r.uniform(-12, 12, 400000), None, np.tanh, 4),
    (8, lambda r: r.uniform(-3, 3, 400000), None, np.expm1, 5),
]


@pytest.mark.parametrize("fn,gen,_b,ref,tol", CASES)
def test_unary_ulp(fn, gen, _b, ref, tol):
    x = gen(np.random.default_rng(fn)).astype(np.float32)
    assert ulp_err(oracle.math(fn, x), ref(x.astype(np.float64))) <= tol


def test_atan2_ulp_and_special_cases():
    r = np.random.default_rng(9)
    y = r.standard_normal(400000).astype(np.float32)
    x = r.standard_normal(400000).astype(np.float32)
    assert ulp_err(oracle.math(4, y, x), np.arctan2(y.astype(np.float64), x.astype(np.float64))) <= 3
    ys = np.array([0, 0, -0., 1, np.inf, -np.inf, 1, -1, np.nan], np.float32)
    xs = np.array([-0., 0, -1, 0, np.inf, -np.inf, -np.inf, np.inf, 1], np.float32)
    got = oracle.math(4, ys, xs)
    exp = np.arctan2(ys, xs)
    assert np.allclose(got, exp, equal_nan=True, atol=1e-7)
    assert np.array_equal(np.signbit(got[:8]), np.signbit(exp[:8]))


def test_edge_values():
    assert oracle.math(0, np.array([-104.0], np.float32))[0] == 0.0
    assert np.isinf(oracle.math(0, np.array([89.0], np.float32))[0])
    assert np.isnan(oracle.math(1, np.array([-1.0], np.float32))[0])
    assert oracle.math(1, np.array([0.0], np.float32))[0] == -np.inf
    assert np.isnan(oracle.math(6, np.array([1.0000001], np.float32))[0])
    assert oracle.math(6, np.array([1.0], np.float32))[0] == 0.0
    assert oracle.math(7, np.array([20.0, -20.0], np.float32)).tolist() == [1.0, -1.0]
