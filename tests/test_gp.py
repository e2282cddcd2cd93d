"""End-to-end ScaledVecchiaGP on the GPU.

The properties of the reference's tests/test_gp.py (errors, accuracy on a
smooth function, std/var consistency, fixed nugget, positive parameters,
joint vs marginal mean, sample shapes, summary, trends, general and
estimated nu) and parity with the reference's fitted parameters and
predictions on identical data (tests/golden/gp.npz).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def GP(**kw):
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    return ScaledVecchiaGP(**kw)


def _wave(n, d=2, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    return X, np.sin(3 * X[:, 0]) + 0.1 * X[:, 1]


def test_shape_mismatch_raises():
    with pytest.raises(ValueError):
        GP().fit(np.random.rand(12, 2), np.random.rand(11))


def test_predict_before_fit_raises():
    with pytest.raises(RuntimeError):
        GP().predict(np.zeros((2, 2)))


def test_recovers_smooth_function():
    X, y = _wave(300, seed=0)
    gp = GP(m_est=15, m_pred=30, nu=2.5, n_est=300, random_state=0).fit(X, y)
    Xt, yt = _wave(200, seed=1)
    mu, sd = gp.predict(Xt, return_std=True)
    assert np.sqrt(np.mean((mu - yt) ** 2)) < 0.25
    assert np.all(sd >= 0)


def test_std_and_var_agree():
    X, y = _wave(150, seed=2)
    gp = GP(m_est=10, m_pred=20, n_est=150, random_state=0).fit(X, y)
    Xt = np.random.default_rng(3).random((20, 2))
    m1, sd = gp.predict(Xt, return_std=True)
    m2, var = gp.predict(Xt, return_var=True)
    np.testing.assert_allclose(m1, m2)
    np.testing.assert_allclose(sd ** 2, var, rtol=1e-10)
    np.testing.assert_allclose(gp.predict(Xt), m1)


def test_fixed_nugget_and_positive_parameters():
    X, y = _wave(120, seed=6)
    gp = GP(m_est=10, m_pred=20, n_est=120, nugget=1e-8, random_state=0).fit(X, y)
    assert gp.nugget_ == pytest.approx(1e-8, rel=1e-6)
    assert np.all(gp.ranges_ > 0) and np.all(gp.relevance_ > 0) and gp.variance_ > 0


def test_joint_mean_close_to_marginal_mean():
    X, y = _wave(200, seed=8)
    gp = GP(m_est=15, m_pred=30, n_est=200, random_state=0).fit(X, y)
    Xt = np.random.default_rng(9).random((25, 2))
    joint = gp.predict_joint(Xt, m=30, exact_var=True)
    np.testing.assert_allclose(gp.predict(Xt), joint["mean"], atol=0.05)
    assert np.all(joint["var"] >= 0)


def test_sample_joint_shape():
    X, y = _wave(150, seed=10)
    gp = GP(m_est=10, m_pred=20, n_est=150, random_state=0).fit(X, y)
    s = gp.sample_joint(np.random.default_rng(11).random((12, 2)), n_sim=25, m=20)
    assert s.shape == (25, 12) and np.all(np.isfinite(s))


@pytest.mark.parametrize("trend", ["zero", "constant", "linear"])
def test_trends(trend):
    X, y = _wave(100, seed=13)
    gp = GP(m_est=8, m_pred=15, n_est=100, trend=trend, random_state=0).fit(X, y)
    assert gp.predict(X[:5]).shape == (5,)
    assert "loglik" in gp.summary()


def test_bad_trend_raises():
    with pytest.raises(ValueError):
        GP(trend="cubic").fit(np.random.rand(20, 2), np.random.rand(20))


def test_fixed_general_nu():
    X, y = _wave(150, seed=20)
    gp = GP(m_est=10, m_pred=20, n_est=150, nu=1.75, random_state=0).fit(X, y)
    assert gp.nu_ == pytest.approx(1.75)
    mu = gp.predict(X[:5])
    assert np.all(np.isfinite(mu)) and gp._estimate_nu is False


def test_estimated_nu_on_matern_draw():
    from scipy.spatial.distance import cdist
    from pyscaledvecchia_gb300._matern_general import _matern_corr_general
    rng = np.random.default_rng(0)
    n = 500
    X = rng.random((n, 2))
    lam = np.array([0.25, 0.4])
    K = 1.5 * (_matern_corr_general(cdist(X / lam, X / lam), 1.75) + 0.02 * np.eye(n))
    y = np.linalg.cholesky(K + 1e-10 * np.eye(n)) @ rng.standard_normal(n)
    gp = GP(m_est=25, m_pred=50, nu=None, n_est=500, trend="zero", var_correction=False,
            random_state=0).fit(X, y)
    assert gp._estimate_nu is True
    assert 0.5 < gp.nu_ < 5.0
    assert gp.nugget_ == pytest.approx(0.02, rel=0.5)
    assert gp.relevance_[0] > gp.relevance_[1]
    # the split form with nu estimated (float32 tables of D, g and dM/dnu at
    # each iterate) fits the same model: nu, the nugget and the loglik within
    # the split form's reach of the float64 fit
    gs = GP(m_est=25, m_pred=50, nu=None, n_est=500, trend="zero", var_correction=False,
            random_state=0, precision="split").fit(X, y)
    assert gs._estimate_nu is True
    assert gs.nu_ == pytest.approx(gp.nu_, rel=1e-2)
    assert gs.nugget_ == pytest.approx(gp.nugget_, rel=1e-2)
    assert abs(gs.loglik_ - gp.loglik_) <= 1e-4 * abs(gp.loglik_)


# ---------------------------------------------------------------------------
# parity with the reference on identical data
# ---------------------------------------------------------------------------
GP_CASES = {
    "sine": dict(m_est=10, m_pred=20, n_est=150, random_state=0),
    "linear": dict(m_est=8, m_pred=15, n_est=100, trend="linear", random_state=0),
    "fixnug": dict(m_est=10, m_pred=20, n_est=120, nugget=1e-8, random_state=0),
    "sub": dict(m_est=10, m_pred=25, n_est=150, random_state=3),
    "nu175": dict(m_est=10, m_pred=20, n_est=150, nu=1.75, random_state=0),
}


@pytest.mark.parametrize("name", sorted(GP_CASES))
def test_fit_parity_with_reference(golden_gp, name):
    """Same Fisher-scoring path: parameters and log-likelihood agree.

    When the estimated nugget runs onto its 1e-12 clip the blocks are nearly
    singular and the reference's own fit is chaotic at the rounding level:
    perturbing y by 1e-15 relative moves its final loglik by ~6e-4 (sine)
    and 1e-13 by ~2e-3 (sub), and theta by ~3e-5 relative.  The Bessel case
    (nu = 1.75) is more sensitive still: eight perturbations of y between
    1e-15 and 1e-14 relative moved the reference's loglik by up to 9.5e-3
    (spread 1.55e-2), theta by up to 1.2e-4 and beta by up to 2.7e-4
    relative.  Those cases get bands of about twice that size; the
    fixed-nugget case is well posed and is held to 1e-8."""
    g = golden_gp
    gp = GP(**GP_CASES[name]).fit(g[name + "_X"], g[name + "_y"])
    ll_ref = float(g[name + "_loglik"])
    clipped = g[name + "_theta"][-1] < np.log(1e-11)
    if clipped:
        ll_tol, th_tol = (2e-2, 5e-4) if name == "nu175" else (5e-3, 3e-4)
    else:
        ll_tol, th_tol = 1e-8 * abs(ll_ref), 1e-6
    assert abs(gp.loglik_ - ll_ref) <= ll_tol, (gp.loglik_, ll_ref)
    np.testing.assert_allclose(gp.theta_, g[name + "_theta"], rtol=th_tol, atol=th_tol)
    np.testing.assert_allclose(gp.beta_, g[name + "_beta"], rtol=th_tol, atol=th_tol)
    # variance correction b of _estimate_b (gp.py:410-425): estimated when
    # n >= 200 (the "sub" case), else 1; in the clipped cases it inherits the
    # fit's sensitivity (the oracle's restatement lands 2e-4 away as well)
    b_ref = float(g[name + "_b"])
    b_tol = 2e-3 if clipped else 1e-8
    assert abs(gp.b_ - b_ref) <= b_tol * b_ref, (gp.b_, b_ref)


@pytest.mark.parametrize("name", ["sine", "linear", "fixnug", "sub", "nu175"])
def test_prediction_parity_with_reference(golden_gp, name):
    """Predictions at a well-conditioned parameter point set on the fitted
    object (nugget 1e-3, b = 1): marginal mean/sd and the joint mean, exact
    variance and samples (same NumPy draws)."""
    g = golden_gp
    gp = GP(**GP_CASES[name]).fit(g[name + "_X"], g[name + "_y"])
    gp.theta_ = g[name + "_wc_theta"].copy()
    gp.beta_ = g[name + "_beta"].copy()
    gp.b_ = 1.0
    Xt = g[name + "_Xte"]
    mu, sd = gp.predict(Xt, return_std=True)
    np.testing.assert_allclose(mu, g[name + "_wc_mu"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(sd, g[name + "_wc_sd"], rtol=1e-7, atol=1e-12)
    m = GP_CASES[name]["m_pred"]
    joint = gp.predict_joint(Xt, m=m, n_sim=6, exact_var=True, random_state=7)
    np.testing.assert_allclose(joint["mean"], g[name + "_wc_jmean"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(joint["var"], g[name + "_wc_jvar"], rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(joint["samples"], g[name + "_wc_jsamples"], rtol=1e-7, atol=1e-9)
    assert math.isfinite(float(np.sum(joint["samples"])))
