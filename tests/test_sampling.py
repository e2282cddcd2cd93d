"""Unconditional Vecchia draws (pyscaledvecchia_gb300/sampling.py) against
dense covariances.

y = U^-T eps has covariance (U U^T)^-1.  Drawing with eps = the identity
(one column per point) gives Y = U^-T, so Y Y^T is that covariance exactly,
without Monte Carlo error:
  * with every point conditioning on all earlier ones (m = n - 1) the
    Vecchia factor is exact and Y Y^T equals the dense covariance
    sigma^2 (M_nu(|x_i - x_j| / lambda) + tau I) of the model;
  * with m < n - 1 it equals (U U^T)^-1 for the factor U built on the CPU
    from dense block Cholesky factors (column i of U is a_i = L_i^-T e_K of
    block (neighbours of i, i), likelihood.py:27-29 of the reference).
A Monte Carlo draw at the benchmark's block shape checks the sample variance.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matern25(r):
    c = math.sqrt(5.0) * r
    return (1.0 + c + c * c / 3.0) * np.exp(-c)


def _dense_cov(X, theta):
    d = X.shape[1]
    s2, lam, tau = math.exp(theta[0]), np.exp(theta[1:1 + d]), math.exp(theta[-1])
    U = X / lam
    r = np.sqrt(((U[:, None, :] - U[None, :, :]) ** 2).sum(-1))
    return s2 * (_matern25(r) + tau * np.eye(X.shape[0]))


def _factor_cpu(Xo, nn, theta):
    n = Xo.shape[0]
    S = _dense_cov(Xo, theta)
    Umat = np.zeros((n, n))
    for i in range(n):
        nb = [j for j in nn[i, 1:] if j >= 0]
        blk = nb + [i]
        L = np.linalg.cholesky(S[np.ix_(blk, blk)])
        e = np.zeros(len(blk))
        e[-1] = 1.0
        a = np.linalg.solve(L.T, e)
        Umat[blk, i] = a
    return Umat


def _inputs(n, d, m, seed):
    from pyscaledvecchia_gb300.ordering import find_ordered_nn, maximin_order
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    lam = np.exp(rng.uniform(math.log(0.2), math.log(2.0), d))
    theta = np.concatenate([[math.log(1.7)], np.log(lam), [math.log(1e-3)]])
    order = maximin_order(X / lam)
    Xo = X[order]
    return Xo, find_ordered_nn(Xo / lam, m), theta


def test_exact_conditioning_gives_the_dense_covariance():
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample
    n, d = 60, 3
    Xo, nn, theta = _inputs(n, d, n - 1, seed=5)
    Y = vecchia_prior_sample(Xo, nn, theta, 2.5, np.eye(n))
    C = Y @ Y.T
    S = _dense_cov(Xo, theta)
    np.testing.assert_allclose(C, S, rtol=1e-8, atol=1e-10 * np.abs(S).max())


@pytest.mark.parametrize("m", [3, 10])
def test_vecchia_covariance_of_the_factor(m):
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample
    n, d = 80, 4
    Xo, nn, theta = _inputs(n, d, m, seed=7 + m)
    Y = vecchia_prior_sample(Xo, nn, theta, 2.5, np.eye(n))
    U = _factor_cpu(Xo, nn, theta)
    C_ref = np.linalg.inv(U @ U.T)
    np.testing.assert_allclose(Y @ Y.T, C_ref, rtol=1e-8, atol=1e-10 * np.abs(C_ref).max())
    # the draw itself: U^T y = eps
    eps = np.random.default_rng(1).standard_normal(n)
    y = vecchia_prior_sample(Xo, nn, theta, 2.5, eps)
    np.testing.assert_allclose(U.T @ y, eps, rtol=1e-9, atol=1e-9)


def test_sample_variance_at_the_benchmark_block_shape():
    """20,000 draws of 2,000 points, d = 10, m = 30: every point's sample
    variance lies within 5 standard errors of its variance under the Vecchia
    factor, the diagonal of (U U^T)^-1."""
    import torch

    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample_device
    n, d, m, nsim = 2000, 10, 30, 20000
    Xo, nn, theta = _inputs(n, d, m, seed=3)
    U = _factor_cpu(Xo, nn, theta)
    target = np.diag(np.linalg.inv(U @ U.T))
    eps = torch.randn((n, nsim), dtype=torch.float64, device="cuda",
                      generator=torch.Generator(device="cuda").manual_seed(0))
    Y = vecchia_prior_sample_device(torch, _lib.to_dev(torch, Xo, np.float64),
                                    _lib.to_dev(torch, nn, np.int64), theta, 2.5, eps)
    v = (Y * Y).mean(dim=1).cpu().numpy()
    se = target * math.sqrt(2.0 / nsim)
    assert np.all(np.abs(v - target) < 5.0 * se), float(np.max(np.abs(v - target) / se))
