"""Generate the golden input/output vectors under tests/golden/ by running the
reference implementation (jdtuck/pyscaledvecchia, Python + Numba) in this
container.

Numba is not installed here, so the reference is imported with a no-op
``numba`` stand-in (``njit`` = identity decorator, ``prange`` = ``range``).
That executes the reference's own loops as plain Python with IEEE-sequential
double arithmetic (Numba's ``fastmath`` reassociation is the only semantic
difference).  The reference source is read in place and never copied.

Usage (only where the reference checkout is available):

    python tests/golden/make_golden.py [--ref /path/to/pyscaledvecchia]

Every case is seeded; the fixtures are small ``.npz`` files committed beside
this script.  Nothing at test time reads the reference.
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_SHIM = '''
def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    def deco(f):
        return f
    return deco
prange = range
'''


def import_reference(ref_root):
    sys.dont_write_bytecode = True
    shim_dir = tempfile.mkdtemp(prefix="numba_shim_")
    os.makedirs(os.path.join(shim_dir, "numba"))
    with open(os.path.join(shim_dir, "numba", "__init__.py"), "w") as fh:
        fh.write(_SHIM)
    sys.path.insert(0, shim_dir)
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import scaled_vecchia  # noqa: F401
    from scaled_vecchia import _covariance, _matern_general, gp, likelihood, ordering
    return dict(cov=_covariance, gen=_matern_general, gp=gp, lik=likelihood, ordr=ordering)


def nn_to_groups(ordr, nn, m):
    return ordr._nn_groups(nn, m)


def gen_ordering(R, out):
    ordr = R["ordr"]
    cases = {}
    specs = [("a", 200, 4, 0), ("b", 50, 2, 0), ("c", 120, 3, 2), ("d", 500, 10, 5),
             ("e", 1500, 3, 6), ("f", 64, 1, 7)]
    for name, n, d, seed in specs:
        X = np.random.default_rng(seed).random((n, d))
        o = ordr.maximin_order(X)
        cases[f"mm_{name}_X"] = X
        cases[f"mm_{name}_order"] = o
    # ties: integer lattice (many exactly equal distances) -> exercises tie-breaking
    g = np.arange(7, dtype=float)
    Xg = np.array([[a, b] for a in g for b in g])
    cases["mm_grid_X"] = Xg
    cases["mm_grid_order"] = ordr.maximin_order(Xg)
    # duplicates
    Xd = np.random.default_rng(9).random((40, 3))
    Xd = np.vstack([Xd, Xd[:10]])
    cases["mm_dup_X"] = Xd
    cases["mm_dup_order"] = ordr.maximin_order(Xd)
    # explicit first point
    Xf = np.random.default_rng(10).random((80, 3))
    cases["mm_first_X"] = Xf
    cases["mm_first_order"] = ordr.maximin_order(Xf, first=17)

    # ordered kNN on maximin-ordered inputs
    nn_specs = [("a", 120, 3, 8, 0, 2), ("b", 60, 2, 6, 40, 4), ("c", 500, 10, 30, 0, 11),
                ("d", 2000, 4, 12, 0, 12), ("e", 300, 5, 40, 100, 13)]
    for name, n, d, m, start, seed in nn_specs:
        X = np.random.default_rng(seed).random((n, d))
        Xo = X[ordr.maximin_order(X)]
        nn = ordr.find_ordered_nn(Xo, m, start=start)
        cases[f"nn_{name}_X"] = Xo
        cases[f"nn_{name}_nn"] = nn
        cases[f"nn_{name}_meta"] = np.array([m, start])
    np.savez_compressed(os.path.join(out, "ordering.npz"), **cases)


def _problem(R, n, d, seed, theta, m, scale_only=True):
    ordr = R["ordr"]
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    lam = np.exp(theta[1:1 + d])
    order = ordr.maximin_order(X / lam)
    nn = ordr.find_ordered_nn((X / lam)[order], m)
    return X[order], y[order], nn


def gen_likelihood(R, out):
    lik, ordr = R["lik"], R["ordr"]
    cases = {}
    L = math.log
    specs = [
        # name, n, d, seed, theta, m, nu, estimate_nu, trend, need_grad, var_penalty, log_var_target
        ("toy_const", 60, 3, 1, [L(1.7), L(0.35), L(0.9), L(3.0), L(0.05)], 10, 2.5, False, "const", True, 0.0, 0.0),
        ("toy_none", 60, 3, 1, [L(1.7), L(0.35), L(0.9), L(3.0), L(0.05)], 10, 2.5, False, "zero", True, 0.0, 0.0),
        ("toy_nograd", 60, 3, 1, [L(1.7), L(0.35), L(0.9), L(3.0), L(0.05)], 10, 2.5, False, "const", False, 0.0, 0.0),
        ("toy_full", 60, 3, 1, [L(1.7), L(0.35), L(0.9), L(3.0), L(0.05)], 59, 2.5, False, "zero", True, 0.0, 0.0),
        ("nu05", 80, 2, 3, [L(0.8), L(0.3), L(0.6), L(0.01)], 12, 0.5, False, "const", True, 0.0, 0.0),
        ("nu15", 80, 4, 4, [L(2.2), L(0.3), L(0.6), L(1.2), L(0.2), L(0.02)], 15, 1.5, False, "linear", True, 0.0, 0.0),
        ("nu25_pen", 70, 3, 5, [L(3.0), L(0.5), L(0.4), L(0.7), L(0.05)], 8, 2.5, False, "const", True, 1.0, L(1.1)),
        ("nu08", 60, 3, 6, [L(1.3), L(0.4), L(0.5), L(0.8), L(0.03)], 10, 0.8, False, "const", True, 0.0, 0.0),
        ("nu175", 50, 2, 7, [L(1.0), L(0.3), L(0.5), L(0.02)], 9, 1.75, False, "zero", True, 0.0, 0.0),
        ("estnu", 60, 3, 1, [L(1.7), L(0.35), L(0.9), L(0.5), L(1.8), L(0.05)], 10, None, True, "const", True, 0.0, 0.0),
        ("estnu_full", 50, 2, 2, [L(1.2), L(0.4), L(0.3), L(1.75), L(0.02)], 49, None, True, "zero", True, 0.0, 0.0),
        ("c2like", 400, 10, 8, [L(2.0)] + [L(v) for v in (0.1, 0.2, 0.5, 1.0, 2.0, 5.0, 10.0, 20.0, 40.0, 0.3)] + [L(1e-3)], 30, 2.5, False, "const", True, 0.0, 0.0),
        ("nug1e8", 200, 3, 9, [L(1.0), L(0.5), L(0.8), L(1.5), L(1e-8)], 20, 2.5, False, "const", True, 0.0, 0.0),
    ]
    for (name, n, d, seed, theta, m, nu, est, trend, need_grad, vp, lvt) in specs:
        theta = np.array(theta, dtype=float)
        Xo, yo, nn = _problem(R, n, d, seed, theta, m)
        if trend == "zero":
            Zo = None
        elif trend == "const":
            Zo = np.ones((n, 1))
        else:
            Zo = np.column_stack([np.ones(n), Xo])
        groups = ordr._nn_groups(nn, m)
        t0 = time.time()
        ll, g, M, beta = lik.vecchia_profile_loglik(theta, Xo, yo, Zo, groups, nu,
                                                     estimate_nu=est, need_grad=need_grad,
                                                     var_penalty=vp, log_var_target=lvt)
        print(f"  lik {name}: {time.time() - t0:.1f}s ll={ll:.12g}")
        pre = f"{name}_"
        cases[pre + "X"] = Xo
        cases[pre + "y"] = yo
        cases[pre + "Z"] = Zo if Zo is not None else np.zeros((n, 0))
        cases[pre + "nn"] = nn
        cases[pre + "theta"] = theta
        cases[pre + "meta"] = np.array([m, -1.0 if nu is None else nu, float(est), float(need_grad), vp, lvt])
        cases[pre + "ll"] = np.array(ll)
        cases[pre + "grad"] = g if g is not None else np.zeros(0)
        cases[pre + "fish"] = M if M is not None else np.zeros((0, 0))
        cases[pre + "beta"] = beta
    np.savez_compressed(os.path.join(out, "likelihood.npz"), **cases)


def gen_blocks(R, out):
    cov, gen = R["cov"], R["gen"]
    cases = {}
    rng = np.random.default_rng(21)
    B, K, d = 5, 9, 3
    Xb = rng.random((B, K, d))
    ranges = np.array([0.3, 0.7, 1.9])
    mask = (rng.random((B, K)) > 0.3).astype(float)
    cases["Xb"] = Xb
    cases["ranges"] = ranges
    cases["mask"] = mask
    for nu in (0.5, 1.5, 2.5, 0.8, 1.75):
        S, dS = cov._block_cov(Xb, ranges, 1.3, 0.07, nu, derivs=True, nug_mask=mask)
        cases[f"S_{nu}"] = S
        cases[f"dS_{nu}"] = dS
    S, dS = gen._block_cov_general(Xb, ranges, 1.3, 0.07, 1.2, derivs=True, estimate_nu=True)
    cases["S_est1.2"] = S
    cases["dS_est1.2"] = dS
    r = np.concatenate([[0.0, 1e-9, 1e-7, 5e-7], np.linspace(1e-6, 5.0, 300), [7.5, 12.0, 30.0, 100.0]])
    cases["r"] = r
    for nu in (0.3, 0.5, 0.8, 1.5, 1.75, 2.5, 3.3, 6.1, 9.7):
        cases[f"Mg_{nu}"] = gen._matern_corr_general(r, nu)
        cases[f"gg_{nu}"] = gen._matern_g_general(r, nu)
    for nu in (0.5, 1.5, 2.5):
        cases[f"Mc_{nu}"] = cov._matern_corr(r, nu)
        cases[f"gc_{nu}"] = cov._matern_g(r, nu)
    np.savez_compressed(os.path.join(out, "blocks.npz"), **cases)


def _sine_data(n, d=2, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = np.sin(3 * X[:, 0]) + 0.1 * X[:, 1]
    return X, y


def gen_gp(R, out):
    GP = R["gp"].ScaledVecchiaGP
    cases = {}
    specs = [
        ("sine", dict(m_est=10, m_pred=20, n_est=150, random_state=0), 150, 2, 2, 20),
        ("linear", dict(m_est=8, m_pred=15, n_est=100, trend="linear", random_state=0), 100, 2, 13, 10),
        ("fixnug", dict(m_est=10, m_pred=20, n_est=120, nugget=1e-8, random_state=0), 120, 2, 6, 12),
        ("sub", dict(m_est=10, m_pred=25, n_est=150, random_state=3), 400, 3, 31, 30),
        ("nu175", dict(m_est=10, m_pred=20, n_est=150, nu=1.75, random_state=0), 150, 2, 20, 10),
    ]
    for name, kw, n, d, seed, nte in specs:
        X, y = _sine_data(n, d=d, seed=seed)
        t0 = time.time()
        gp = GP(**kw).fit(X, y)
        Xte = np.random.default_rng(seed + 100).random((nte, d))
        mu, sd = gp.predict(Xte, return_std=True)
        joint = gp.predict_joint(Xte, m=kw["m_pred"], n_sim=6, exact_var=True, random_state=5)
        print(f"  gp {name}: {time.time() - t0:.1f}s ll={gp.loglik_:.10g}")
        pre = f"{name}_"
        cases[pre + "X"] = X
        cases[pre + "y"] = y
        cases[pre + "Xte"] = Xte
        cases[pre + "theta"] = gp.theta_
        cases[pre + "beta"] = gp.beta_
        cases[pre + "b"] = np.array(gp.b_)
        cases[pre + "loglik"] = np.array(gp.loglik_)
        cases[pre + "mu"] = mu
        cases[pre + "sd"] = sd
        cases[pre + "jmean"] = joint["mean"]
        cases[pre + "jvar"] = joint["var"]
        cases[pre + "jsamples"] = joint["samples"]
        # the fitted nugget often sits on its 1e-12 clip, where predictive
        # variances are rounding-dominated; also record a well-conditioned
        # parameter point (nugget 1e-3, b = 1) on the same fitted object
        gp.theta_ = gp.theta_.copy()
        gp.theta_[-1] = math.log(1e-3)
        gp.b_ = 1.0
        mu2, sd2 = gp.predict(Xte, return_std=True)
        joint2 = gp.predict_joint(Xte, m=kw["m_pred"], n_sim=6, exact_var=True, random_state=7)
        cases[pre + "wc_theta"] = gp.theta_
        cases[pre + "wc_mu"] = mu2
        cases[pre + "wc_sd"] = sd2
        cases[pre + "wc_jmean"] = joint2["mean"]
        cases[pre + "wc_jvar"] = joint2["var"]
        cases[pre + "wc_jsamples"] = joint2["samples"]
    np.savez_compressed(os.path.join(out, "gp.npz"), **cases)


def gen_optimize(R, out):
    """Traces of the reference's Fisher scoring (optimize.py:11-73) on the
    toy objectives of toy_objectives.py: every evaluated theta, every reorder
    call and the result."""
    sys.path.insert(0, HERE)
    import toy_objectives as T
    from scaled_vecchia import optimize
    cases = {}
    for name in T.CASES:
        toy, theta0, max_step = T.make(name)
        th, ll, beta = optimize._fisher_scoring(theta0, toy.objective, max_iter=25, tol=1e-6,
                                                reorder_hook=toy.reorder_hook, max_step=max_step)
        cases[f"{name}_theta0"] = theta0
        cases[f"{name}_trace"] = np.array(toy.trace)
        cases[f"{name}_reorder_k"] = np.array([k for k, _ in toy.reorders], dtype=np.int64)
        cases[f"{name}_reorder_th"] = np.array([t for _, t in toy.reorders]).reshape(len(toy.reorders), -1)
        cases[f"{name}_theta"] = th
        cases[f"{name}_ll"] = np.array(ll)
        cases[f"{name}_beta"] = beta
    np.savez_compressed(os.path.join(out, "optimize.npz"), **cases)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    R = import_reference(a.ref)
    which = a.only.split(",") if a.only else ["ordering", "blocks", "likelihood", "gp", "optimize"]
    for w in which:
        t0 = time.time()
        {"ordering": gen_ordering, "blocks": gen_blocks,
         "likelihood": gen_likelihood, "gp": gen_gp, "optimize": gen_optimize}[w](R, HERE)
        print(f"{w}: {time.time() - t0:.1f}s")


if __name__ == "__main__":
    main()
