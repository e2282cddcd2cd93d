"""CPU restatement of the reference's fit and marginal prediction.

TEST INFRASTRUCTURE ONLY: used by tests/ to check the device path and by ``bench.py``
for its CPU baseline of the fit + predict workload.  The product package
(pyscaledvecchia_gb300) never imports, loads or calls anything here.

Restates (jdtuck/pyscaledvecchia, src/scaled_vecchia/...):
  * ScaledVecchiaGP.fit        gp.py:138-239 (standardisation, subsample,
                               initial theta, clipping :126-135, fixed-nugget
                               freeze, reorder hook, variance correction)
  * _fisher_scoring            optimize.py:11-73 (ridged Fisher step, step cap,
                               backtracking line search, reorders at 2, 4, 8..)
  * predict / _predict_scaled  gp.py:242-304
  * _estimate_b                gp.py:410-425
on top of the oracle's C kernels (maximin, ordered kNN, the closed-form-nu
likelihood and the marginal prediction blocks of oracle/sv_oracle.c), for
closed-form smoothness nu in {0.5, 1.5, 2.5}.  Pinned against the fitted
parameters, log-likelihood and variance factor that the reference itself
produced (tests/golden/gp.npz; tests/test_oracle_golden.py).
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle


class LinAlgFail(Exception):
    pass


def _design(trend, X):
    """gp.py:93-100."""
    if trend == "zero":
        return np.zeros((X.shape[0], 0))
    if trend == "constant":
        return np.ones((X.shape[0], 1))
    if trend == "linear":
        return np.column_stack([np.ones(X.shape[0]), X])
    raise ValueError("trend must be 'zero', 'constant' or 'linear'")


def fisher_scoring(theta0, objective, max_iter=40, tol=1e-4, reorder_hook=None, max_step=3.0):
    """optimize.py:11-73."""
    theta = np.array(theta0, dtype=float)
    ll, g, M, beta = objective(theta)
    next_reorder = 2
    for k in range(1, max_iter + 1):
        if reorder_hook is not None and k == next_reorder:
            next_reorder *= 2
            if reorder_hook(theta, k):
                ll, g, M, beta = objective(theta)
        step = None
        ridge = 0.0
        diag = np.maximum(np.diag(M), 1e-8)
        for _ in range(12):
            try:
                cand = np.linalg.solve(M + ridge * np.diag(diag), g)
            except np.linalg.LinAlgError:
                ridge = max(1e-6, ridge * 10.0)
                continue
            if np.dot(cand, g) > 0 and np.all(np.isfinite(cand)):
                step = cand
                break
            ridge = max(1e-6, ridge * 10.0)
        if step is None:
            step = g / max(np.linalg.norm(g), 1e-12)
        nrm = np.linalg.norm(step)
        if nrm > max_step:
            step *= max_step / nrm
        alpha, ok = 1.0, False
        for _ in range(20):
            try:
                cand_ll, cand_g, cand_M, cand_beta = objective(theta + alpha * step)
            except np.linalg.LinAlgError:
                alpha *= 0.5
                continue
            if np.isfinite(cand_ll) and cand_ll > ll:
                theta = theta + alpha * step
                ll, g, M, beta = cand_ll, cand_g, cand_M, cand_beta
                ok = True
                break
            alpha *= 0.5
        if not ok:
            break
        if abs(np.dot(alpha * step, g)) < tol:
            break
    return theta, ll, beta


class OracleGP:
    """The fitted state of gp.py's ScaledVecchiaGP for closed-form nu."""

    def __init__(self, m_est=30, m_pred=140, n_est=5000, nu=2.5, trend="constant", nugget=None,
                 var_penalty=1.0, var_correction=True, lambda_max=1e3, max_iter=40, tol=1e-4,
                 random_state=0):
        if nu not in (0.5, 1.5, 2.5):
            raise ValueError("the oracle fit takes closed-form nu only")
        self.m_est, self.m_pred, self.n_est, self.nu = m_est, m_pred, n_est, nu
        self.trend, self.nugget, self.var_penalty = trend, nugget, var_penalty
        self.var_correction, self.lambda_max = var_correction, lambda_max
        self.max_iter, self.tol, self.random_state = max_iter, tol, random_state

    def _clip(self, theta, d):
        """gp.py:126-135 (fixed nu)."""
        hi = math.log(self.lambda_max) if np.isfinite(self.lambda_max) else np.inf
        theta[1:1 + d] = np.clip(theta[1:1 + d], math.log(1e-8), hi)
        theta[-1] = np.clip(theta[-1], math.log(1e-12), math.log(1e3))
        return theta

    def fit(self, X, y):
        """gp.py:138-239."""
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=float)
        y = np.asarray(y, dtype=float).ravel()
        n, d = X.shape
        self.d_ = d
        self._lo = X.min(0)
        self._span = np.where(X.max(0) - X.min(0) > 0, X.max(0) - X.min(0), 1.0)
        self._ymu = y.mean()
        self._ysd = y.std() if y.std() > 0 else 1.0
        self.X_ = (X - self._lo) / self._span
        self.y_ = (y - self._ymu) / self._ysd
        rng = np.random.default_rng(self.random_state)
        if self.n_est is not None and n > self.n_est:
            sub = rng.choice(n, self.n_est, replace=False)
        else:
            sub = np.arange(n)
        Xe, ye = self.X_[sub], self.y_[sub]
        Ze = _design(self.trend, Xe)
        m = min(self.m_est, len(sub) - 1)
        theta = np.empty(d + 2)
        theta[0] = math.log(max(ye.var(), 1e-8))
        theta[1:1 + d] = math.log(0.2 * math.sqrt(d))
        fixed = self.nugget is not None
        theta[-1] = math.log(self.nugget if fixed else 0.1)
        theta = self._clip(theta, d)
        state = {}

        def rebuild(th):
            Xs = Xe / np.exp(th[1:1 + d])
            order = oracle.maximin_order(Xs)
            nn = oracle.ordered_nn(Xs[order], m)
            state["groups"] = oracle.nn_groups(nn, m)
            state["Xo"], state["yo"], state["Zo"] = Xe[order], ye[order], Ze[order]

        rebuild(theta)
        last = {"r": np.exp(theta[1:1 + d]).copy()}
        log_var_target = math.log(max(ye.var(), 1e-8))

        def objective(th):
            th = self._clip(np.array(th, dtype=float), d)
            if fixed:
                th[-1] = math.log(self.nugget)
            ll, g, M, beta = oracle.vecchia_loglik(th, state["Xo"], state["yo"], state["Zo"],
                                                   state["groups"], self.nu,
                                                   var_penalty=self.var_penalty,
                                                   log_var_target=log_var_target)
            if fixed:
                g = g.copy()
                g[-1] = 0.0
                M = M.copy()
                M[-1, :] = 0.0
                M[:, -1] = 0.0
                M[-1, -1] = 1.0
            return ll, g, M, beta

        def reorder_hook(th, k):
            r = np.exp(self._clip(np.array(th), d)[1:1 + d])
            if np.max(np.abs(np.log(r / last["r"]))) < 1e-3:
                return False
            rebuild(th)
            last["r"] = r.copy()
            return True

        theta, ll, beta = fisher_scoring(theta, objective, max_iter=self.max_iter, tol=self.tol,
                                         reorder_hook=reorder_hook)
        theta = self._clip(np.array(theta), d)
        if fixed:
            theta[-1] = math.log(self.nugget)
        self.theta_, self.beta_, self.loglik_ = theta, beta, ll
        self.b_ = 1.0
        if self.var_correction and n >= 200:
            self.b_ = self._estimate_b(rng)
        return self

    def _predict_scaled(self, Xs_std, X_tr, resid, m):
        """gp.py:242-277 (noise-free target)."""
        mean, var, _ = oracle.predict_marginal(X_tr, resid, Xs_std, self.theta_, self.nu,
                                               min(m, X_tr.shape[0]))
        return mean, var

    def _estimate_b(self, rng):
        """gp.py:410-425."""
        n = self.X_.shape[0]
        n_in = min(2000, n // 5)
        idx = rng.permutation(n)
        te, tr = idx[:n_in], idx[n_in:]
        Z_tr = _design(self.trend, self.X_[tr])
        resid = self.y_[tr] - (Z_tr @ self.beta_ if self.beta_.size else 0.0)
        mu, va = self._predict_scaled(self.X_[te], self.X_[tr], resid, min(self.m_pred, len(tr)))
        if self.beta_.size:
            mu = mu + _design(self.trend, self.X_[te]) @ self.beta_
        va = np.maximum(va, 1e-300)
        return max(float(np.mean((self.y_[te] - mu) ** 2 / va)), 1e-8)

    def predict(self, Xstar, return_std=False, m=None):
        """gp.py:279-304."""
        Xstar = np.ascontiguousarray(np.atleast_2d(Xstar), dtype=float)
        Xs = (Xstar - self._lo) / self._span
        m = self.m_pred if m is None else m
        Z_tr = _design(self.trend, self.X_)
        resid = self.y_ - (Z_tr @ self.beta_ if self.beta_.size else 0.0)
        mu, va = self._predict_scaled(Xs, self.X_, resid, m)
        if self.beta_.size:
            mu = mu + _design(self.trend, Xs) @ self.beta_
        mean = self._ymu + self._ysd * mu
        if not return_std:
            return mean
        return mean, np.sqrt((self._ysd ** 2) * self.b_ * va)
