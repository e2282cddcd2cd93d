"""Deterministic toy objectives for pinning the Fisher-scoring iteration.

Used by make_golden.py (run against the reference's optimize._fisher_scoring)
and by tests/test_optimize.py (run against this package's), so both see the
same arithmetic.  Each objective records every theta it is asked about, and
the reorder hook records its calls, so the whole trace can be compared.
"""
from __future__ import annotations

import numpy as np


class Toy:
    """f(th) = -sum_i w_i (exp(th_i - c_i) - (th_i - c_i)) - 1/2 th' A th,
    concave; grad and a Fisher-like matrix (the negative Hessian, optionally
    made indefinite) are returned with beta = [sum th].  ``fail_above``
    raises LinAlgError when th[0] exceeds it (a failed line-search try)."""

    def __init__(self, P, seed, indefinite=False, fail_above=None, shift_on_reorder=0.0):
        rng = np.random.default_rng(seed)
        self.c = rng.uniform(-1.0, 1.0, P)
        self.w = rng.uniform(0.5, 2.0, P)
        B = rng.standard_normal((P, P)) * 0.2
        self.A = B @ B.T
        self.indefinite = indefinite
        self.fail_above = fail_above
        self.shift = shift_on_reorder
        self.trace = []
        self.reorders = []

    def objective(self, th):
        th = np.asarray(th, dtype=float)
        self.trace.append(th.copy())
        if self.fail_above is not None and th[0] > self.fail_above:
            raise np.linalg.LinAlgError("toy failure")
        u = th - self.c
        e = np.exp(u)
        ll = float(-np.sum(self.w * (e - u)) - 0.5 * th @ self.A @ th)
        g = -self.w * (e - 1.0) - self.A @ th
        M = np.diag(self.w * e) + self.A
        if self.indefinite:
            M = M.copy()
            M[0, 1] = M[1, 0] = 3.0 * np.sqrt(M[0, 0] * M[1, 1])
        return ll, g, M, np.array([th.sum()])

    def reorder_hook(self, th, k):
        self.reorders.append((k, np.asarray(th, dtype=float).copy()))
        if self.shift and k == 2:
            self.c = self.c + self.shift
            return True
        return False


CASES = {
    # name: (P, seed, indefinite, fail_above, shift, theta0 scale, max_step)
    "smooth": (6, 11, False, None, 0.0, 2.0, 3.0),
    "indefinite": (5, 12, True, None, 0.0, 1.5, 3.0),
    "failing": (4, 13, False, 0.9, 0.0, 1.0, 3.0),
    "reorder": (7, 14, False, None, 0.25, 2.5, 3.0),
    "short_step": (5, 15, False, None, 0.1, 4.0, 0.5),
}


def make(name):
    P, seed, indef, fail, shift, scale, max_step = CASES[name]
    toy = Toy(P, seed, indefinite=indef, fail_above=fail, shift_on_reorder=shift)
    theta0 = np.random.default_rng(seed + 100).uniform(-scale, scale, P)
    if fail is not None:
        theta0[0] = min(theta0[0], fail - 0.5)
    return toy, theta0, max_step
