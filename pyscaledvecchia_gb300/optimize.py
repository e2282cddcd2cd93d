"""Fisher scoring with a backtracking line search (Guinness 2021), as used by
the reference to maximise the Vecchia log-likelihood (optimize.py:11-73).

The step rules have to be the reference's own for the fitted parameters to
agree: a Fisher direction ridged (x10 from 1e-6, up to 12 tries) until it
ascends, else the normalised gradient; the step capped at ``max_step`` in
norm; up to 20 halvings of alpha, a LinAlgError counting as a failed try;
stop when no step ascends or |alpha step . g| < tol; reorder at
k = 2, 4, 8, 16, ...

The iteration is written once, as a generator that asks its driver for
objective values (``("eval", theta)``) and reorders (``("reorder", theta,
k)``).  ``_fisher_scoring`` drives it with a direct objective call (one GPU
likelihood evaluation each); the batched driver (batched.py) advances many
problems' generators together and answers all their evaluation requests
with one batched launch.
"""
from __future__ import annotations

import numpy as np

__all__ = ["_fisher_scoring", "fisher_scoring_steps"]


class EvalFailed:
    """Sent to a generator in place of an objective value when the
    evaluation raised numpy.linalg.LinAlgError."""


EVAL_FAILED = EvalFailed()


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


def fisher_scoring_steps(theta0, max_iter=40, tol=1e-4, verbose=False, reorder=True,
                         max_step=3.0):
    """Generator form of the Fisher-scoring iteration.

    Yields ("eval", theta) and expects (ll, grad, fisher, beta) back, or
    EVAL_FAILED when the objective raised LinAlgError (only tolerated in the
    line search, as in the reference); yields ("reorder", theta, k) and
    expects a bool.  Returns (theta, ll, beta).
    """
    theta = np.array(theta0, dtype=float)
    res = yield ("eval", theta.copy())
    if res is EVAL_FAILED:
        raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
    ll, g, M, beta = res
    reorder_at = 2
    for k in range(1, max_iter + 1):
        if reorder and k == reorder_at:
            reorder_at *= 2
            changed = yield ("reorder", theta.copy(), k)
            if changed:
                res = yield ("eval", theta.copy())
                if res is EVAL_FAILED:
                    raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
                ll, g, M, beta = res

        step = _scoring_direction(M, g)
        nrm = np.linalg.norm(step)
        if nrm > max_step:
            step *= max_step / nrm

        alpha, accepted = 1.0, False
        for _ in range(20):
            res = yield ("eval", theta + alpha * step)
            if res is EVAL_FAILED:
                alpha *= 0.5
                continue
            c_ll, c_g, c_M, c_beta = res
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


def _fisher_scoring(theta0, objective, max_iter=40, tol=1e-4, verbose=False,
                    reorder_hook=None, max_step=3.0):
    """Maximise ``objective(theta) -> (loglik, grad, fisher, beta)``.

    ``reorder_hook(theta, k)`` is called at k = 2, 4, 8, ...; when it returns
    True the objective changed and is re-evaluated at the current theta.
    Returns (theta, loglik, beta).
    """
    gen = fisher_scoring_steps(theta0, max_iter=max_iter, tol=tol, verbose=verbose,
                               reorder=reorder_hook is not None, max_step=max_step)
    msg = next(gen)
    while True:
        if msg[0] == "eval":
            try:
                reply = objective(msg[1])
            except np.linalg.LinAlgError:
                reply = EVAL_FAILED
        else:
            reply = bool(reorder_hook(msg[1], msg[2]))
        try:
            msg = gen.send(reply)
        except StopIteration as stop:
            return stop.value
