"""Edge cases of the device path against the oracle: the smallest problems
(n = 1, 2, 3, 7 with m larger than n - 1, so that every block conditions on
all earlier rows), one input dimension, the largest input dimension the
block kernels take (d = 64), and rows that are all the same point (every
maximin step a tie, every block singular but for the nugget).  The ordering
and the neighbour sets are compared exactly; the likelihood, score, Fisher
information and beta to the float64 form's oracle tolerances
(test_parity_with_oracle_larger), and the split forms to the float64 form's
bounds of test_split_matches_float64 (or, where they fall back to float64,
bit for bit)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ordered(oracle, X, lam, m):
    """Device ordering and neighbour sets, checked against the oracle's."""
    from pyscaledvecchia_gb300.ordering import _nn_groups, find_ordered_nn, maximin_order
    Xs = X / lam
    order = maximin_order(Xs)
    np.testing.assert_array_equal(order, oracle.maximin_order(Xs))
    nn = find_ordered_nn(Xs[order], m)
    np.testing.assert_array_equal(nn, oracle.ordered_nn(Xs[order], m))
    return order, _nn_groups(nn, m)


def _check_loglik(oracle, theta, Xo, yo, Zo, groups, nu, tol=1e-10):
    import pyscaledvecchia_gb300 as sv
    got = sv.vecchia_profile_loglik(theta, Xo, yo, Zo, groups, nu)
    ref = oracle.vecchia_loglik(theta, Xo, yo, Zo, groups, nu)
    assert abs(got[0] - ref[0]) <= tol * max(abs(ref[0]), 1.0), (got[0], ref[0])
    np.testing.assert_allclose(got[1], ref[1], rtol=1e-8, atol=1e-8 * max(np.abs(ref[1]).max(), 1.0))
    np.testing.assert_allclose(got[2], ref[2], rtol=1e-8, atol=1e-8 * max(np.abs(ref[2]).max(), 1.0))
    if Zo is not None:
        np.testing.assert_allclose(got[3], ref[3], rtol=1e-8, atol=1e-10)
    for form in ("split", "split_df"):
        s = sv.vecchia_profile_loglik(theta, Xo, yo, Zo, groups, nu, precision=form)
        assert abs(s[0] - got[0]) <= 5e-6 * max(abs(got[0]), 1.0), (form, s[0], got[0])
        assert np.abs(s[1] - got[1]).max() <= 1e-3 * max(np.abs(got[1]).max(), 1e-12)
        assert np.abs(s[2] - got[2]).max() <= 1e-3 * max(np.abs(got[2]).max(), 1e-12)
    return got


@pytest.mark.parametrize("n", [1, 2, 3, 7])
@pytest.mark.parametrize("d", [1, 3])
def test_smallest_problems(oracle, n, d):
    rng = np.random.default_rng(10 * n + d)
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    lam = np.exp(rng.uniform(math.log(0.2), math.log(2.0), d))
    theta = np.concatenate([[math.log(1.4)], np.log(lam), [math.log(1e-2)]])
    order, groups = _ordered(oracle, X, lam, 5)
    assert sum(len(g[0]) for g in groups) == n
    _check_loglik(oracle, theta, X[order], y[order], np.ones((n, 1)), groups, 2.5)
    _check_loglik(oracle, theta, X[order], y[order], None, groups, 1.5)


def test_one_input_dimension(oracle):
    rng = np.random.default_rng(5)
    n, m = 4000, 20
    X = rng.random((n, 1))
    y = np.sin(6 * X[:, 0]) + 0.1 * rng.standard_normal(n)
    lam = np.array([0.3])
    theta = np.array([math.log(0.8), math.log(0.3), math.log(1e-3)])
    order, groups = _ordered(oracle, X, lam, m)
    _check_loglik(oracle, theta, X[order], y[order], np.ones((n, 1)), groups, 2.5)


def test_largest_input_dimension(oracle):
    """d = 64: P = 66 parameters, so the split forms' right-hand sides exceed
    32 columns and the whole evaluation runs the float64 kernels (the same
    bits)."""
    import pyscaledvecchia_gb300 as sv
    rng = np.random.default_rng(64)
    n, d, m = 600, 64, 10
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    lam = np.exp(rng.uniform(math.log(1.0), math.log(8.0), d))
    theta = np.concatenate([[math.log(1.1)], np.log(lam), [math.log(1e-2)]])
    order, groups = _ordered(oracle, X, lam, m)
    got = _check_loglik(oracle, theta, X[order], y[order], np.ones((n, 1)), groups, 0.5)
    s = sv.vecchia_profile_loglik(theta, X[order], y[order], np.ones((n, 1)), groups, 0.5,
                                  precision="split")
    assert s[0] == got[0]
    np.testing.assert_array_equal(s[2], got[2])


def test_all_rows_the_same_point(oracle):
    """Every maximin step is a tie (the reference keeps the first index at
    the largest distance) and every block's covariance is s2 (J + tau I)."""
    rng = np.random.default_rng(9)
    n, d, m = 60, 2, 6
    X = np.tile(rng.random((1, d)), (n, 1))
    y = rng.standard_normal(n)
    lam = np.array([0.5, 0.25])
    theta = np.array([math.log(2.0), math.log(0.5), math.log(0.25), math.log(0.1)])
    order, groups = _ordered(oracle, X, lam, m)
    _check_loglik(oracle, theta, X[order], y[order], np.ones((n, 1)), groups, 2.5)
