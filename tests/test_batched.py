"""Batched evaluation of many likelihoods (sv_vecchia_loglik_batched) and the
batched fitter.

A batch runs each problem's arithmetic unchanged (likelihood.py:66-175), so
every problem's ll, score, Fisher matrix and beta must equal, bit for bit,
what the one-problem entry point gives for it, whatever else shares the
launch: other d, q, m (blocks above 32 included), estimated or general nu,
variance penalties, split precision.  Skipped problems keep their previous
outputs, a captured graph replays with new parameters, and the batched
fitter in float64 reproduces ScaledVecchiaGP.fit model by model.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mk(seed, n, d, m, q, nu=2.5, estimate_nu=False, var_penalty=0.0, tau=0.05):
    from pyscaledvecchia_gb300 import find_ordered_nn, maximin_order
    from pyscaledvecchia_gb300.batched import BatchProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = np.sin(4 * X).sum(1) + 0.1 * rng.standard_normal(n)
    lam = np.exp(rng.uniform(math.log(0.1), math.log(2.0), d))
    Xs = X / lam
    order = maximin_order(Xs)
    nn = find_ordered_nn(Xs[order], m)
    groups = _nn_groups(nn, m)
    Z = None
    if q == 1:
        Z = np.ones((n, 1))
    elif q > 1:
        Z = np.column_stack([np.ones(n), X[:, :q - 1]])
    th = [math.log(1.2)] + list(np.log(lam) + rng.uniform(-0.2, 0.2, d))
    if estimate_nu:
        th.append(math.log(1.7))
    th.append(math.log(tau))
    pr = BatchProblem(X[order], y[order], None if Z is None else Z[order], groups, nu=nu,
                      estimate_nu=estimate_nu, var_penalty=var_penalty,
                      log_var_target=math.log(0.7))
    return pr, np.array(th)


def _mixed_batch():
    specs = [
        dict(seed=1, n=300, d=3, m=10, q=1),
        dict(seed=2, n=450, d=7, m=30, q=1, tau=1e-8),
        dict(seed=3, n=220, d=4, m=40, q=2),                # blocks with k + 1 > 32
        dict(seed=4, n=180, d=2, m=12, q=0, nu=0.8),        # Bessel form
        dict(seed=5, n=260, d=5, m=15, q=1, estimate_nu=True),
        dict(seed=6, n=350, d=12, m=20, q=1, nu=1.5, var_penalty=2.0),
        dict(seed=7, n=90, d=3, m=30, q=3, nu=0.5),
    ]
    return [_mk(**s) for s in specs]


def _single(pr, th, precision="float64", need_grad=True, team_lanes=0):
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    dp = DeviceProblem(pr.Xo, pr.yo, pr.Zo, pr.groups)
    return dp.evaluate(th, pr.nu, estimate_nu=pr.estimate_nu, need_grad=need_grad,
                       var_penalty=pr.var_penalty, log_var_target=pr.log_var_target,
                       precision=precision, team_lanes=team_lanes)


def _assert_same(res, ref):
    st, ll, g, M, beta = res
    assert st == 0
    assert ll == ref[0]
    if ref[1] is None:
        assert g is None
    else:
        np.testing.assert_array_equal(g, ref[1])
        np.testing.assert_array_equal(M, ref[2])
    np.testing.assert_array_equal(beta, ref[3])


@pytest.mark.parametrize("need_grad", [True, False])
def test_batched_float64_equals_single(need_grad):
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    items = _mixed_batch()
    BL = BatchedLikelihood([p for p, _ in items], need_grad=need_grad)
    res = BL.evaluate([t for _, t in items])
    for (pr, th), r in zip(items, res):
        _assert_same(r, _single(pr, th, need_grad=need_grad))


def test_batched_split_equals_single():
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    # every problem of the mixed batch: closed forms, a fixed general nu and
    # an estimated nu (float32 tables), blocks beyond 32 points (float64)
    items = _mixed_batch()
    # bit for bit at the same team width (the autotuner may pick another
    # width per problem on its own)
    for lanes in (8, 16):
        BL = BatchedLikelihood([p for p, _ in items], precisions=("split",), team_lanes=lanes)
        res = BL.evaluate([t for _, t in items])
        for (pr, th), r in zip(items, res):
            _assert_same(r, _single(pr, th, precision="split", team_lanes=lanes))


def test_skipped_problems_keep_outputs_and_graph_replay():
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    items = _mixed_batch()
    BL = BatchedLikelihood([p for p, _ in items], precisions=("float64", "split"))
    th0 = [t for _, t in items]
    first = BL.evaluate(th0)
    BL.capture("float64")
    th1 = [t + 0.05 for t in th0]
    active = np.array([i % 2 == 0 for i in range(len(items))])
    res = BL.evaluate(th1, active=active, precision="float64")
    out, info = BL.fetch()
    for i, (pr, _) in enumerate(items):
        if active[i]:
            _assert_same(res[i], _single(pr, th1[i]))
        else:
            assert res[i] is None
            kept = BL.unpack(out, info, i)
            assert kept[1] == first[i][1]
            np.testing.assert_array_equal(kept[2], first[i][2])
    # replay again with all problems on
    res2 = BL.evaluate(th0, active=np.ones(len(items), bool), precision="float64")
    for i in range(len(items)):
        assert res2[i][1] == first[i][1]


def test_batched_cholesky_failure_is_per_problem():
    """A problem whose blocks cannot be factorised reports SV_ECHOL in its
    own status words only."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    items = _mixed_batch()[:3]
    pr, th = items[1]
    Xd = pr.Xo.copy()
    Xd[7, 0] = np.nan  # no jitter level factorises a block holding this row
    from pyscaledvecchia_gb300.batched import BatchProblem
    items[1] = (BatchProblem(Xd, pr.yo, pr.Zo, pr.groups, nu=pr.nu), th)
    BL = BatchedLikelihood([p for p, _ in items])
    res = BL.evaluate([t for _, t in items])
    ref_status = []
    for pr_, th_ in items:
        try:
            _single(pr_, th_)
            ref_status.append(0)
        except np.linalg.LinAlgError:
            ref_status.append(2)
    assert [r[0] for r in res] == ref_status
    for i in (0, 2):
        _assert_same(res[i], _single(*items[i]))


def _fit_data(seed, n, d):
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = np.sin(3 * X[:, 0]) + X[:, 1] ** 2 + 0.05 * rng.standard_normal(n)
    return X, y


def test_fit_batched_float64_matches_individual_fits():
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    from pyscaledvecchia_gb300.fit_batched import fit_batched
    cfg = [(21, 300, 2, 20, None), (22, 420, 3, 10, 1e-8), (23, 250, 4, 30, None)]
    data = [_fit_data(s, n, d) for s, n, d, _, _ in cfg]
    solo = [ScaledVecchiaGP(m_est=m, nugget=nug, n_est=None, var_correction=True).fit(X, y)
            for (_, _, _, m, nug), (X, y) in zip(cfg, data)]
    batch = [ScaledVecchiaGP(m_est=m, nugget=nug, n_est=None, var_correction=True)
             for (_, _, _, m, nug) in cfg]
    fit_batched(batch, [X for X, _ in data], [y for _, y in data], precision="float64", graphs=True)
    for a, b in zip(solo, batch):
        np.testing.assert_array_equal(b.theta_, a.theta_)
        assert b.loglik_ == a.loglik_
        np.testing.assert_array_equal(b.beta_, a.beta_)
        assert b.b_ == a.b_


def test_fit_batched_split_ends_at_a_float64_optimum():
    """Split iterations + float64 polish: the reported loglik is the float64
    objective at the final theta and ordering, and that point is a float64
    stationary point (the polish's own stopping rule holds there).  The
    final ordering can differ from a float64-only fit's (reorders happen at
    the iterates, which differ slightly), so the two optima are compared
    only loosely."""
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    from pyscaledvecchia_gb300.fit_batched import fit_batched
    from pyscaledvecchia_gb300.optimize import _scoring_direction
    cfg = [(31, 500, 3, 20, None), (32, 400, 5, 10, 1e-8), (33, 600, 4, 30, None)]
    data = [_fit_data(s, n, d) for s, n, d, _, _ in cfg]
    f64 = [ScaledVecchiaGP(m_est=m, nugget=nug, n_est=None, var_correction=False) for *_, m, nug in cfg]
    spl = [ScaledVecchiaGP(m_est=m, nugget=nug, n_est=None, var_correction=False) for *_, m, nug in cfg]
    Xs, ys = [X for X, _ in data], [y for _, y in data]
    fit_batched(f64, Xs, ys, precision="float64")
    st = {}
    fit_batched(spl, Xs, ys, precision="split", stats=st)
    BL = st["batch"]
    th = [g._objective_theta(t, g.d_, False) for g, t in zip(spl, st["thetas"])]
    res = BL.evaluate(th, active=np.ones(len(spl), bool), precision="float64")
    for g, a, r in zip(spl, f64, res):
        assert g.fit_stats_["split"] >= 1 and g.fit_stats_["float64"] >= 1
        assert r[1] == g.loglik_
        grad, fish = g._freeze_nugget(r[2], r[3])
        step = _scoring_direction(fish, grad)
        nrm = np.linalg.norm(step)
        if nrm > 3.0:
            step *= 3.0 / nrm
        # at most 5 float64 iterations after the split phase: near a float64
        # stationary point (Newton decrement below 0.05)
        assert abs(step @ grad) < 5e-2
        assert abs(g.loglik_ - a.loglik_) <= 2e-2 * max(1.0, abs(a.loglik_))
