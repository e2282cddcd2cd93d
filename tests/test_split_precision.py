"""Split-precision likelihood against the float64 form and the oracle.

Two split forms share the float32 parts (distances, Matern assembly through
an accurate correlation deficit, dSigma.a, the Fisher / score Gram products)
and the float64 records and reductions:
  "split"    : float64 LDL^T, triangular solves, log-determinant and GLS
               sums (the contracted split form);
  "split_df" : the same steps in double-float (float32 pairs, ~46 bits).
Blocks whose smallest pivot ratio d_k / Sigma_kk is below 1e-4 are
re-evaluated in float64, so the float32 assembly error stays bounded on
ill-conditioned problems.  Stated error bounds relative to the float64 form
on the same inputs (measured maxima on these cases are 1e-8 .. 2e-6):
ll within 5e-6 relative, score within 1e-3 of its largest entry, Fisher
within 1e-3 of its largest entry; beta within 2e-4 relative (the GLS
coefficients inherit the float32 assembly error of a = L^-T e_K).  Against
the oracle (the CPU float64 restatement of the reference) at n = 20,000,
d = 10, m = 30 the "split" form is held to the bounds written in
test_split_against_oracle."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(n, d, m, tau, seed, lam_range=(0.05, 50.0)):
    """Ordered inputs: X in maximin order, the ordered neighbour table, y a
    Vecchia draw, Z = 1, theta."""
    from pyscaledvecchia_gb300.ordering import find_ordered_nn, maximin_order
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    lam = np.exp(rng.uniform(math.log(lam_range[0]), math.log(lam_range[1]), d))
    theta = np.concatenate([[math.log(2.0)], np.log(lam), [math.log(tau)]])
    order = maximin_order(X / lam)
    nn = find_ordered_nn((X / lam)[order], m)
    Xo = X[order]
    y = vecchia_prior_sample(Xo, nn, theta, 2.5, rng.standard_normal(n))
    return Xo, y, np.ones((n, 1)), nn, theta


def _setup(n, d, m, tau, seed, lam_range=(0.05, 50.0)):
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups
    Xo, y, Z, nn, theta = _inputs(n, d, m, tau, seed, lam_range)
    return DeviceProblem(Xo, y, Z, _nn_groups(nn, m)), theta


SPLIT_FORMS = ("split", "split_df")


@pytest.mark.parametrize("form", SPLIT_FORMS)
@pytest.mark.parametrize("n,d,m,tau,lanes", [(20000, 10, 30, 1e-3, 8), (8000, 3, 20, 1e-8, 8),
                                             (6000, 5, 30, 1e-6, 16), (5000, 4, 10, 1e-4, 4),
                                             (4000, 6, 25, 1e-3, 32)])
def test_split_matches_float64(n, d, m, tau, lanes, form):
    prob, theta = _setup(n, d, m, tau, seed=n + d)
    ll0, g0, F0, b0 = prob.evaluate(theta, 2.5)
    ll1, g1, F1, b1 = prob.evaluate(theta, 2.5, precision=form, team_lanes=lanes)
    assert abs(ll1 - ll0) <= 5e-6 * abs(ll0), (ll1, ll0)
    assert np.abs(g1 - g0).max() <= 1e-3 * np.abs(g0).max()
    assert np.abs(F1 - F0).max() <= 1e-3 * np.abs(F0).max()
    np.testing.assert_allclose(b1, b0, rtol=2e-4, atol=1e-6)


@pytest.mark.parametrize("form", SPLIT_FORMS)
@pytest.mark.parametrize("nu", [0.5, 1.5])
def test_split_other_closed_forms(nu, form):
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups, find_ordered_nn, maximin_order
    rng = np.random.default_rng(3)
    n, d, m = 3000, 4, 20
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    theta = np.array([0.3, -1.0, -0.5, 0.2, 1.0, math.log(1e-2)])
    order = maximin_order(X / np.exp(theta[1:1 + d]))
    nn = find_ordered_nn((X / np.exp(theta[1:1 + d]))[order], m)
    prob = DeviceProblem(X[order], y[order], None, _nn_groups(nn, m))
    a = prob.evaluate(theta, nu)
    b = prob.evaluate(theta, nu, precision=form)
    assert abs(a[0] - b[0]) <= 5e-6 * abs(a[0])
    assert np.abs(a[1] - b[1]).max() <= 1e-3 * np.abs(a[1]).max()


@pytest.mark.parametrize("form", SPLIT_FORMS)
@pytest.mark.parametrize("what", ["y", "s2"])
def test_split_out_of_float32_range_goes_to_float64(what, form):
    """Data above 1e30 in magnitude, or a scale outside [1e-30, 1e30], leave
    float32's exponent range: those blocks are evaluated by the float64 pass,
    so the result is the float64 form's."""
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups, find_ordered_nn, maximin_order
    rng = np.random.default_rng(11)
    n, d, m = 2000, 3, 15
    X = rng.random((n, d))
    theta = np.array([0.0, -1.0, -0.5, 0.2, math.log(1e-3)])
    y = rng.standard_normal(n)
    if what == "y":
        y = y * 1e31
    else:
        theta[0] = math.log(1e31)
    order = maximin_order(X / np.exp(theta[1:1 + d]))
    nn = find_ordered_nn((X / np.exp(theta[1:1 + d]))[order], m)
    prob = DeviceProblem(X[order], y[order], np.ones((n, 1)), _nn_groups(nn, m))
    a = prob.evaluate(theta, 2.5)
    b = prob.evaluate(theta, 2.5, precision=form)
    assert np.isfinite(b[0])
    assert abs(a[0] - b[0]) <= 1e-12 * abs(a[0])
    np.testing.assert_allclose(b[1], a[1], rtol=1e-10, atol=1e-10 * np.abs(a[1]).max())
    np.testing.assert_allclose(b[2], a[2], rtol=1e-10, atol=1e-10 * np.abs(a[2]).max())


@pytest.mark.parametrize("lanes", [8, 16])
def test_split_against_oracle(oracle, lanes):
    """The split form (float32 assembly, float64 factorisation) against the
    oracle on the benchmark's block shape: n = 20,000, d = 10, m = 30,
    nu = 2.5, tau = 1e-3, lambda log-uniform in [0.05, 50], y a Vecchia draw.
    Bounds (measured: ll 6.3e-9, score 2.3e-5 sd, Fisher 3.8e-7, beta
    1.1e-5): ll within 1e-7 relative; every score entry within 1e-3 of its
    standard deviation sqrt(F_ii) (the score is a sum of zero-mean terms, so
    a relative error says nothing); Fisher within 1e-5 of its largest entry;
    beta within 1e-4 relative."""
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups
    n, d, m = 20000, 10, 30
    Xo, yo, Zo, nn, theta = _inputs(n, d, m, 1e-3, seed=20010)
    groups = _nn_groups(nn, m)
    prob = DeviceProblem(Xo, yo, Zo, groups)
    ll0, g0, F0, b0 = oracle.vecchia_loglik(theta, Xo, yo, Zo, groups, 2.5)
    ll1, g1, F1, b1 = prob.evaluate(theta, 2.5, precision="split", team_lanes=lanes)
    sd = np.sqrt(np.diag(F0))
    e_ll = abs(ll1 - ll0) / abs(ll0)
    e_g = float(np.max(np.abs(g1 - g0) / sd))
    e_F = float(np.abs(F1 - F0).max() / np.abs(F0).max())
    e_b = float(np.max(np.abs(b1 - b0) / np.abs(b0)))
    print(f"split vs oracle (lanes {lanes}): ll {e_ll:.2e} score/sd {e_g:.2e} fisher {e_F:.2e} beta {e_b:.2e}")
    assert e_ll <= 1e-7, e_ll
    assert e_g <= 1e-3, e_g
    assert e_F <= 1e-5, e_F
    assert e_b <= 1e-4, e_b


@pytest.mark.parametrize("form", SPLIT_FORMS)
def test_split_general_nu(form):
    """A fixed general nu runs the split forms through the float32 Matern
    table (nu = 0.8: the float64 form's bounds of test_split_matches_float64);
    within 1e-3 of an integer (nu = 2.0) there is no table and a one-problem
    call runs the float64 kernels (the float64 form's result bit for bit).  In
    a batch, the split kernels send the nu = 2.0 problem's blocks to the
    float64 pass (all counted as redone) while the nu = 0.8 and nu = 2.5
    problems beside it stay in the split form, each equal bit for bit to its
    one-problem evaluation."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups
    Xo, y, Z, nn, theta = _inputs(3000, 4, 20, 1e-3, seed=77)
    groups = _nn_groups(nn, 20)
    prob = DeviceProblem(Xo, y, Z, groups)
    one = {}
    for nu in (0.8, 2.0, 2.5):
        a = prob.evaluate(theta, nu)
        b = prob.evaluate(theta, nu, precision=form, team_lanes=16)
        one[nu] = b
        if nu == 2.0:
            assert b[0] == a[0]
            for u, v in zip(a[1:], b[1:]):
                np.testing.assert_array_equal(u, v)
            continue
        assert b[0] != a[0]  # the split form ran
        assert int(prob.last_info[3]) < Xo.shape[0] // 10
        assert abs(b[0] - a[0]) <= 5e-6 * abs(a[0]), (nu, b[0], a[0])
        assert np.abs(b[1] - a[1]).max() <= 1e-3 * np.abs(a[1]).max()
        assert np.abs(b[2] - a[2]).max() <= 1e-3 * np.abs(a[2]).max()
        np.testing.assert_allclose(b[3], a[3], rtol=2e-4, atol=1e-6)
    nus = (2.0, 0.8, 2.5)
    BL = BatchedLikelihood([BatchProblem(Xo, y, Z, groups, nu=nu) for nu in nus],
                           precisions=(form,), team_lanes=16)
    res = BL.evaluate([theta] * 3)
    a20 = prob.evaluate(theta, 2.0)
    st, ll, g, F, b = res[0]
    assert st == 0
    assert abs(ll - a20[0]) <= 1e-12 * abs(a20[0]), (ll, a20[0])
    np.testing.assert_allclose(g, a20[1], rtol=1e-10, atol=1e-10 * np.abs(a20[1]).max())
    np.testing.assert_allclose(F, a20[2], rtol=1e-10, atol=1e-10 * np.abs(a20[2]).max())
    # every block has at most 21 points, so every block runs the split kernels
    assert int(BL.last_info[0, 3]) == Xo.shape[0]
    for i, nu in ((1, 0.8), (2, 2.5)):
        st, ll, g, F, b = res[i]
        assert st == 0 and ll == one[nu][0], (nu, ll, one[nu][0])
        np.testing.assert_array_equal(g, one[nu][1])
        np.testing.assert_array_equal(F, one[nu][2])
        assert int(BL.last_info[i, 3]) < Xo.shape[0] // 10


@pytest.mark.parametrize("form", SPLIT_FORMS)
@pytest.mark.parametrize("nu", [0.8, 1.7, 2.0])
def test_split_estimated_nu(form, nu):
    """An estimated nu in the split forms: at each theta the split kernels
    take float32 tables of D and g at nu and of the central difference dM/dnu
    (nu +- 1e-3) for the extra dSigma_nu a row.  Against the float64 form:
    the bounds of test_split_matches_float64.  At nu = 2.0 (within 1e-3 of an
    integer) there are no float32 tables: every block goes to the float64
    pass (counted as redone) and the result is the float64 form's to 1e-12.
    A batch of the problem gives the one-problem bits."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups
    Xo, y, Z, nn, theta = _inputs(3000, 4, 20, 1e-3, seed=91)
    th = np.concatenate([theta[:-1], [math.log(nu)], theta[-1:]])
    groups = _nn_groups(nn, 20)
    prob = DeviceProblem(Xo, y, Z, groups)
    a = prob.evaluate(th, None, estimate_nu=True)
    b = prob.evaluate(th, None, estimate_nu=True, precision=form, team_lanes=16)
    redone = int(prob.last_info[3])
    if nu == 2.0:
        assert redone == Xo.shape[0]
        assert abs(b[0] - a[0]) <= 1e-12 * abs(a[0]), (b[0], a[0])
        np.testing.assert_allclose(b[1], a[1], rtol=1e-10, atol=1e-10 * np.abs(a[1]).max())
        np.testing.assert_allclose(b[2], a[2], rtol=1e-10, atol=1e-10 * np.abs(a[2]).max())
    else:
        assert b[0] != a[0]  # the split form ran
        assert redone < Xo.shape[0] // 10
        assert abs(b[0] - a[0]) <= 5e-6 * abs(a[0]), (b[0], a[0])
        assert np.abs(b[1] - a[1]).max() <= 1e-3 * np.abs(a[1]).max()
        assert np.abs(b[2] - a[2]).max() <= 1e-3 * np.abs(a[2]).max()
        np.testing.assert_allclose(b[3], a[3], rtol=2e-4, atol=1e-6)
    BL = BatchedLikelihood([BatchProblem(Xo, y, Z, groups, nu=None, estimate_nu=True)],
                           precisions=(form,), team_lanes=16)
    st, ll, g, F, beta = BL.evaluate([th])[0]
    assert st == 0 and ll == b[0]
    np.testing.assert_array_equal(g, b[1])
    np.testing.assert_array_equal(F, b[2])


def test_split_estimated_nu_against_oracle(oracle):
    """The split form with an estimated nu (nu = 1.3) against the oracle
    (scipy's kv and the reference's central difference), with the bounds of
    test_split_against_oracle."""
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups
    Xo, yo, Zo, nn, theta = _inputs(1500, 3, 15, 1e-3, seed=92)
    th = np.concatenate([theta[:-1], [math.log(1.3)], theta[-1:]])
    groups = _nn_groups(nn, 15)
    prob = DeviceProblem(Xo, yo, Zo, groups)
    ll, g, F, b = prob.evaluate(th, None, estimate_nu=True, precision="split")
    assert ll != prob.evaluate(th, None, estimate_nu=True)[0]  # the split form ran
    ll_o, g_o, F_o, b_o = oracle.vecchia_loglik_np(th, Xo, yo, Zo, groups, None,
                                                    estimate_nu=True)[:4]
    assert abs(ll - ll_o) <= 1e-7 * abs(ll_o), (ll, ll_o)
    sd = np.sqrt(np.diag(F_o))
    assert np.all(np.abs(g - g_o) <= 1e-3 * sd), np.abs(g - g_o) / sd
    assert np.abs(F - F_o).max() <= 1e-5 * np.abs(F_o).max()
    np.testing.assert_allclose(b, b_o, rtol=1e-4, atol=1e-8)
