"""The Matern table of a fixed general smoothness (nu outside {0.5, 1.5,
2.5}) against the per-entry Bessel routine (a batched evaluation built with
matern_tables=False) and the oracle (scipy.special.kv,
_matern_general.py:87-116 of the reference); batched evaluations with tables
equal the one-problem evaluation bit for bit.

The table interpolates e^c M(c) and e^c g(c), c = sqrt(2 nu) r, by 16-term
Chebyshev series on half-octave intervals; its error is at the level of
float64 rounding, so the likelihood, score and Fisher information agree
with the Bessel routine to about 1e-13 relative."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(seed, n, d, m, nu):
    from pyscaledvecchia_gb300.ordering import _nn_groups, find_ordered_nn, maximin_order
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = np.sin(3 * X[:, 0]) + X[:, 1] ** 2 + 0.1 * rng.standard_normal(n)
    lam = np.exp(rng.uniform(math.log(0.05), math.log(2.0), d))
    theta = np.concatenate([[math.log(1.3)], np.log(lam), [math.log(2e-3)]])
    order = maximin_order(X / lam)
    nn = find_ordered_nn((X / lam)[order], m)
    return X[order], y[order], np.ones((n, 1)), _nn_groups(nn, m), theta


@pytest.mark.parametrize("nu", [0.3, 0.8, 1.75, 3.2])
def test_table_matches_the_bessel_routine(nu):
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    Xo, yo, Zo, groups, theta = _problem(3, 4000, 4, 25, nu)
    ll_t, g_t, F_t, b_t = DeviceProblem(Xo, yo, Zo, groups).evaluate(theta, nu)
    BT = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=nu)])
    st, ll_2, g_2, F_2, b_2 = BT.evaluate([theta])[0]
    assert st == 0 and ll_2 == ll_t
    np.testing.assert_array_equal(g_2, g_t)
    np.testing.assert_array_equal(F_2, F_t)
    BL = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=nu)], matern_tables=False)
    st, ll_b, g_b, F_b, b_b = BL.evaluate([theta])[0]
    assert st == 0
    assert abs(ll_t - ll_b) <= 1e-12 * abs(ll_b), (ll_t, ll_b)
    np.testing.assert_allclose(g_t, g_b, rtol=1e-10, atol=1e-11 * np.abs(g_b).max())
    np.testing.assert_allclose(F_t, F_b, rtol=1e-10, atol=1e-11 * np.abs(F_b).max())
    np.testing.assert_allclose(b_t, b_b, rtol=1e-11, atol=1e-13)


def test_table_against_the_oracle():
    """scipy's kv through the oracle at nu = 0.8 (the benchmark's general
    smoothness), a small problem."""
    from oracle import oracle
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    nu = 0.8
    Xo, yo, Zo, groups, theta = _problem(4, 600, 3, 15, nu)
    ll, g, F, b = DeviceProblem(Xo, yo, Zo, groups).evaluate(theta, nu)
    ll_o, g_o, F_o, b_o = oracle.vecchia_loglik_np(theta, Xo, yo, Zo, groups, nu)[:4]
    assert abs(ll - ll_o) <= 1e-10 * abs(ll_o), (ll, ll_o)
    np.testing.assert_allclose(g, g_o, rtol=1e-8, atol=1e-8 * np.abs(g_o).max())
    np.testing.assert_allclose(F, F_o, rtol=1e-8, atol=1e-8 * np.abs(F_o).max())


def test_split_table_against_the_oracle():
    """The split form with the float32 table at nu = 0.8 against the oracle
    (scipy's kv), with test_split_against_oracle's bounds: ll within 1e-7
    relative, each score entry within 1e-3 of its standard deviation
    sqrt(F_ii), Fisher within 1e-5 of its largest entry, beta within 1e-4."""
    from oracle import oracle
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    nu = 0.8
    Xo, yo, Zo, groups, theta = _problem(4, 600, 3, 15, nu)
    prob = DeviceProblem(Xo, yo, Zo, groups)
    ll, g, F, b = prob.evaluate(theta, nu, precision="split")
    ll_o, g_o, F_o, b_o = oracle.vecchia_loglik_np(theta, Xo, yo, Zo, groups, nu)[:4]
    assert ll != prob.evaluate(theta, nu)[0]  # the split form ran
    assert abs(ll - ll_o) <= 1e-7 * abs(ll_o), (ll, ll_o)
    sd = np.sqrt(np.diag(F_o))
    assert np.all(np.abs(g - g_o) <= 1e-3 * sd), np.abs(g - g_o) / sd
    assert np.abs(F - F_o).max() <= 1e-5 * np.abs(F_o).max()
    np.testing.assert_allclose(b, b_o, rtol=1e-4, atol=1e-8)


def test_no_table_above_nu_10():
    """Above nu = 10 the 16-term series lose float64 accuracy, so the
    evaluation keeps the per-entry Bessel routine: bit for bit the batched
    evaluation built without tables."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    nu = 12.5
    Xo, yo, Zo, groups, theta = _problem(5, 2000, 3, 15, nu)
    ll, g, F, b = DeviceProblem(Xo, yo, Zo, groups).evaluate(theta, nu)
    BL = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=nu)], matern_tables=False)
    st, ll_b, g_b, F_b, b_b = BL.evaluate([theta])[0]
    assert st == 0 and ll == ll_b
    np.testing.assert_array_equal(g, g_b)
    np.testing.assert_array_equal(F, F_b)


def _est_theta(theta, nu):
    """theta of an estimated-nu evaluation: log nu inserted before log tau."""
    return np.concatenate([theta[:-1], [math.log(nu)], theta[-1:]])


@pytest.mark.parametrize("nu", [0.45, 1.3, 3.7])
def test_estimated_nu_tables(nu):
    """An estimated nu interpolates M and g at nu, and M at nu +- h for the
    central difference dM/dnu (_matern_general.py:170-176), from three tables
    built for the evaluation's nu: against the per-entry Bessel routine (a
    batched evaluation built with matern_tables=False) ll within 1e-12, the
    score and Fisher information within 1e-9 of their largest entries (the
    difference of two tabulated values over 2h = 2e-3 carries their 1e-15
    rounding times 500), and the batched evaluation with tables equals the
    one-problem one bit for bit."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    Xo, yo, Zo, groups, theta = _problem(6, 3000, 4, 20, nu)
    th = _est_theta(theta, nu)
    ll_t, g_t, F_t, b_t = DeviceProblem(Xo, yo, Zo, groups).evaluate(th, None, estimate_nu=True)
    BT = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=None, estimate_nu=True)])
    st, ll_2, g_2, F_2, b_2 = BT.evaluate([th])[0]
    assert st == 0 and ll_2 == ll_t
    np.testing.assert_array_equal(g_2, g_t)
    np.testing.assert_array_equal(F_2, F_t)
    BL = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=None, estimate_nu=True)],
                           matern_tables=False)
    st, ll_b, g_b, F_b, b_b = BL.evaluate([th])[0]
    assert st == 0
    assert ll_t != ll_b or np.any(g_t != g_b)  # the tables were used
    assert abs(ll_t - ll_b) <= 1e-12 * abs(ll_b), (ll_t, ll_b)
    np.testing.assert_allclose(g_t, g_b, rtol=0, atol=1e-9 * np.abs(g_b).max())
    np.testing.assert_allclose(F_t, F_b, rtol=0, atol=1e-9 * np.abs(F_b).max())
    np.testing.assert_allclose(b_t, b_b, rtol=1e-11, atol=1e-13)


def test_estimated_nu_beyond_the_tables():
    """An estimated nu whose nu + h exceeds 10 keeps the per-entry Bessel
    routine: bit for bit the evaluation without tables."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    nu = 10.0
    Xo, yo, Zo, groups, theta = _problem(7, 1500, 3, 15, nu)
    th = _est_theta(theta, nu)
    a = DeviceProblem(Xo, yo, Zo, groups).evaluate(th, None, estimate_nu=True)
    BL = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=None, estimate_nu=True)],
                           matern_tables=False)
    st, ll, g, F, b = BL.evaluate([th])[0]
    assert st == 0 and ll == a[0]
    np.testing.assert_array_equal(g, a[1])
    np.testing.assert_array_equal(F, a[2])


def test_estimated_nu_tables_against_the_oracle():
    """The estimated-nu evaluation with tables against the oracle (scipy's kv
    per entry, the reference's central difference)."""
    from oracle import oracle
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    nu = 1.3
    Xo, yo, Zo, groups, theta = _problem(8, 500, 3, 12, nu)
    th = _est_theta(theta, nu)
    ll, g, F, b = DeviceProblem(Xo, yo, Zo, groups).evaluate(th, None, estimate_nu=True)
    ll_o, g_o, F_o, b_o = oracle.vecchia_loglik_np(th, Xo, yo, Zo, groups, None,
                                                    estimate_nu=True)[:4]
    assert abs(ll - ll_o) <= 1e-10 * abs(ll_o), (ll, ll_o)
    np.testing.assert_allclose(g, g_o, rtol=1e-7, atol=1e-7 * np.abs(g_o).max())
    np.testing.assert_allclose(F, F_o, rtol=1e-7, atol=1e-7 * np.abs(F_o).max())


def test_prediction_with_the_table(monkeypatch):
    """Prediction blocks (sv_predict_blocks) of a general nu interpolate M
    from the table of sv_matern_table, as the likelihood does: the marginal
    mean and sd and the joint mean agree with the per-entry Bessel routine
    to 1e-10, and so do unconditional draws (sampling.vecchia_prior_sample)."""
    from pyscaledvecchia_gb300 import sampling
    from pyscaledvecchia_gb300.gp import ScaledVecchiaGP
    from pyscaledvecchia_gb300.ordering import find_ordered_nn, maximin_order
    rng = np.random.default_rng(12)
    X = rng.random((1500, 3))
    y = np.sin(4 * X[:, 0]) + X[:, 1] + 0.05 * rng.standard_normal(1500)
    Xq = rng.random((400, 3))
    gp = ScaledVecchiaGP(nu=0.8, m_est=15, m_pred=60, var_correction=False).fit(X, y)
    assert gp._matern_table() is not None
    mu_t, sd_t = gp.predict(Xq, return_std=True)
    jm_t = gp.predict_joint(Xq)["mean"]
    gp._matern_table = lambda: None  # K_nu per entry
    mu_b, sd_b = gp.predict(Xq, return_std=True)
    jm_b = gp.predict_joint(Xq)["mean"]
    assert np.any(mu_t != mu_b)  # the table was used
    np.testing.assert_allclose(mu_t, mu_b, rtol=1e-10, atol=1e-10 * np.abs(mu_b).max())
    np.testing.assert_allclose(sd_t, sd_b, rtol=1e-10)
    np.testing.assert_allclose(jm_t, jm_b, rtol=1e-10, atol=1e-10 * np.abs(jm_b).max())
    th = np.array([0.2, math.log(0.3), math.log(0.6), math.log(0.4), math.log(1e-3)])
    order = maximin_order(X / np.exp(th[1:4]))
    Xo = X[order]
    nn = find_ordered_nn(Xo / np.exp(th[1:4]), 12)
    eps = rng.standard_normal(1500)
    y_t = sampling.vecchia_prior_sample(Xo, nn, th, 0.8, eps)
    monkeypatch.setattr(sampling, "matern_table_nu", lambda nu: False)
    y_b = sampling.vecchia_prior_sample(Xo, nn, th, 0.8, eps)
    assert np.any(y_t != y_b)
    np.testing.assert_allclose(y_t, y_b, rtol=1e-10, atol=1e-10 * np.abs(y_b).max())


def test_table_entry_point_checks():
    """sv_matern_table takes a nu with a table only (no closed form, at most
    10) and a buffer of sv_matern_table_doubles(); sv_predict_blocks takes a
    table only for a general nu with one."""
    import torch

    from pyscaledvecchia_gb300 import _lib
    lib, _ = _lib.device_ready()
    nd = int(lib.sv_matern_table_doubles())
    t = torch.empty(nd, dtype=torch.float64, device="cuda")
    st = _lib.stream_handle(torch)
    assert lib.sv_matern_table(0.8, _lib.ptr(t), nd, st) == _lib.SV_OK
    assert lib.sv_matern_table(2.5, _lib.ptr(t), nd, st) == _lib.SV_EINVAL
    assert lib.sv_matern_table(12.0, _lib.ptr(t), nd, st) == _lib.SV_EINVAL
    assert lib.sv_matern_table(0.8, _lib.ptr(t), nd - 1, st) == _lib.SV_EINVAL
    D = _lib.PredDesc()
    D.nall, D.nobs, D.nblk, D.d, D.k, D.ldnbr = 4, 4, 1, 2, 1, 1
    D.general, D.nu, D.matern_table = 0, 2.5, t.data_ptr()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    th = torch.zeros(4, dtype=torch.float64, device="cuda")
    tgt = torch.zeros(1, dtype=torch.int32, device="cuda")
    nbr = torch.zeros(1, dtype=torch.int32, device="cuda")
    info = _lib.new_info(torch)
    rc = lib.sv_predict_blocks(D, _lib.ptr(th), _lib.ptr(x), _lib.ptr(tgt), _lib.ptr(nbr), None,
                               None, None, None, None, _lib.ptr(info), st)
    assert rc == _lib.SV_EINVAL
    torch.cuda.synchronize()
