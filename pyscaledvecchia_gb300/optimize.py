"""Fisher scoring with a backtracking line search (Guinness 2021), as used by
the reference to maximise the Vecchia log-likelihood (optimize.py:11-73).

The step rules have to be the reference's own for the fitted parameters to
agree: a Fisher direction ridged (x10 from 1e-6, up to 12 tries) until it
ascends, else the normalised gradient; the step capped at ``max_step`` in
norm; up to 20 halvings of alpha, a LinAlgError counting as a failed try;
stop when no step ascends or |alpha step . g| < tol; reorder at
k = 2, 4, 8, 16, ...  Each objective call is one GPU likelihood evaluation.
"""
from __future__ import annotations

import numpy as np

__all__ = ["_fisher_scoring"]


def _scoring_direction(M, g):
    diag = np.maximum(np.diag(M), 1e-8)
    ridge = 0.0
    for _ in range(12):
        try:
            cand = np.linalg.solve(M + ridge * np.diag(diag), g)
        except np.linalg.LinAlgError:
            ridge = max(1e-6, 10.0 * ridge)
            continue
        if np.dot(cand, g) > 0 and np.all(np.isfinite(cand)):
            return cand
        ridge = max(1e-6, 10.0 * ridge)
    return g / max(np.linalg.norm(g), 1e-12)


def _fisher_scoring(theta0, objective, max_iter=40, tol=1e-4, verbose=False,
                    reorder_hook=None, max_step=3.0):
    """Maximise ``objective(theta) -> (loglik, grad, fisher, beta)``.

    ``reorder_hook(theta, k)`` is called at k = 2, 4, 8, ...; when it returns
    True the objective changed and is re-evaluated at the current theta.
    Returns (theta, loglik, beta).
    """
    theta = np.array(theta0, dtype=float)
    ll, g, M, beta = objective(theta)
    reorder_at = 2
    for k in range(1, max_iter + 1):
        if reorder_hook is not None and k == reorder_at:
            reorder_at *= 2
            if reorder_hook(theta, k):
                ll, g, M, beta = objective(theta)

        step = _scoring_direction(M, g)
        nrm = np.linalg.norm(step)
        if nrm > max_step:
            step *= max_step / nrm

        alpha, accepted = 1.0, False
        for _ in range(20):
            try:
                c_ll, c_g, c_M, c_beta = objective(theta + alpha * step)
            except np.linalg.LinAlgError:
                alpha *= 0.5
                continue
            if np.isfinite(c_ll) and c_ll > ll:
                theta = theta + alpha * step
                ll, g, M, beta = c_ll, c_g, c_M, c_beta
                accepted = True
                break
            alpha *= 0.5
        if verbose:
            print(f"    [FS {k:2d}] loglik = {ll:14.4f}   "
                  f"|step.grad| = {abs(np.dot(alpha * step, g)):.3e}")
        if not accepted:
            break
        if abs(np.dot(alpha * step, g)) < tol:
            break
    return theta, ll, beta
