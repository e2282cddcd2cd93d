"""GPU likelihood / score / Fisher information (sv_vecchia_loglik).

Same properties as the reference's tests/test_likelihood.py (exact-GP
equality at m = n-1, analytic score vs central differences, a symmetric PSD
Fisher matrix, need_grad on/off agreement, the general Matern against the
closed forms, estimated nu), plus parity with the reference's own outputs
(tests/golden/likelihood.npz) and with the CPU oracle at larger sizes.
"""
import math

import numpy as np
import pytest
from scipy.spatial.distance import cdist

pytestmark = pytest.mark.gpu

LIK_CASES = ["toy_const", "toy_none", "toy_nograd", "toy_full", "nu05", "nu15", "nu25_pen",
             "nu08", "nu175", "estnu", "estnu_full", "c2like", "nug1e8"]


def _sv():
    import pyscaledvecchia_gb300 as sv
    from pyscaledvecchia_gb300._covariance import LOG2PI, _matern_corr
    from pyscaledvecchia_gb300.ordering import _nn_groups
    return sv, LOG2PI, _matern_corr, _nn_groups


def _dense_loglik(X, y, theta, corr):
    d = X.shape[1]
    s2, lam, tau = math.exp(theta[0]), np.exp(theta[1:1 + d]), math.exp(theta[-1])
    R = cdist(X / lam, X / lam)
    L = np.linalg.cholesky(s2 * (corr(R) + tau * np.eye(len(X))))
    z = np.linalg.solve(L, y)
    return -0.5 * (len(y) * math.log(2 * math.pi) + 2 * np.log(np.diag(L)).sum() + z @ z)


@pytest.fixture
def problem():
    rng = np.random.default_rng(11)
    n, d = 70, 3
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    theta = np.array([math.log(1.3), math.log(0.4), math.log(0.8), math.log(2.5),
                      math.log(0.04)])
    return X, y, theta


def _prep(X, theta, m, d):
    sv, _, _, _nn_groups = _sv()
    Xs = X / np.exp(theta[1:1 + d])
    order = sv.maximin_order(Xs)
    nn = sv.find_ordered_nn(Xs[order], m)
    return order, _nn_groups(nn, m)


def test_full_conditioning_equals_exact_gp(problem):
    sv, _, _matern_corr, _ = _sv()
    X, y, theta = problem
    n, d = X.shape
    order, groups = _prep(X, theta, n - 1, d)
    ll, _, _, _ = sv.vecchia_profile_loglik(theta, X[order], y[order], None, groups, 2.5)
    exact = _dense_loglik(X, y, theta, lambda r: _matern_corr(r, 2.5))
    assert abs(ll - exact) < 1e-7


@pytest.mark.parametrize("nu", [0.5, 1.5, 2.5, 0.8])
def test_score_matches_central_differences(problem, nu):
    sv, _, _, _ = _sv()
    X, y, theta = problem
    n, d = X.shape
    order, groups = _prep(X, theta, 9, d)
    Z = np.ones((n, 1))

    def f(th):
        return sv.vecchia_profile_loglik(th, X[order], y[order], Z[order], groups, nu)

    ll0, g0, M0, _ = f(theta)
    h = 1e-6
    num = np.array([(f(theta + h * e)[0] - f(theta - h * e)[0]) / (2 * h)
                    for e in np.eye(len(theta))])
    assert np.max(np.abs(g0 - num) / (1 + np.abs(num))) < 1e-5
    assert np.abs(M0 - M0.T).max() < 1e-6
    assert np.linalg.eigvalsh(0.5 * (M0 + M0.T)).min() > -1e-6


def test_loglik_same_with_and_without_score(problem):
    sv, _, _, _ = _sv()
    X, y, theta = problem
    order, groups = _prep(X, theta, 9, X.shape[1])
    a = sv.vecchia_profile_loglik(theta, X[order], y[order], None, groups, 2.5, need_grad=True)
    b = sv.vecchia_profile_loglik(theta, X[order], y[order], None, groups, 2.5, need_grad=False)
    assert b[1] is None and b[2] is None
    assert abs(a[0] - b[0]) < 1e-10


def test_general_matern_agrees_with_closed_forms():
    from pyscaledvecchia_gb300._covariance import _matern_corr, _matern_g
    from pyscaledvecchia_gb300._matern_general import _matern_corr_general, _matern_g_general
    r = np.linspace(1e-6, 6.0, 333)
    for nu in (0.5, 1.5, 2.5):
        np.testing.assert_allclose(_matern_corr_general(r, nu), _matern_corr(r, nu), atol=1e-10)
        keep = r > 0.01
        np.testing.assert_allclose(_matern_g_general(r, nu)[keep], _matern_g(r, nu)[keep],
                                   atol=1e-8)


def test_general_g_is_the_radial_derivative():
    from pyscaledvecchia_gb300._matern_general import _matern_corr_general, _matern_g_general
    r = np.linspace(0.05, 5.0, 250)
    for nu in (1.75, 0.8, 3.3):
        h = 1e-6
        num = (_matern_corr_general(r + h, nu) - _matern_corr_general(r - h, nu)) / (2 * h) / r
        rel = np.abs(num - _matern_g_general(r, nu)) / np.abs(num)
        assert rel.max() < 1e-6


def test_estimated_nu_score_and_fisher():
    sv, _, _, _ = _sv()
    rng = np.random.default_rng(5)
    n, d = 64, 3
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    Z = np.ones((n, 1))
    theta = np.array([math.log(1.4), math.log(0.3), math.log(0.7), math.log(0.6),
                      math.log(1.6), math.log(0.05)])
    order, groups = _prep(X, theta, 10, d)

    def f(th):
        return sv.vecchia_profile_loglik(th, X[order], y[order], Z[order], groups, nu=None,
                                         estimate_nu=True)

    _, g0, M0, _ = f(theta)
    h = 1e-6
    num = np.array([(f(theta + h * e)[0] - f(theta - h * e)[0]) / (2 * h)
                    for e in np.eye(len(theta))])
    assert np.max(np.abs(g0 - num) / (1 + np.abs(num))) < 1e-5
    assert np.abs(M0 - M0.T).max() < 1e-6
    assert np.linalg.eigvalsh(0.5 * (M0 + M0.T)).min() > -1e-6


def test_estimated_nu_full_conditioning_equals_exact_gp():
    sv, _, _, _ = _sv()
    from pyscaledvecchia_gb300._matern_general import _matern_corr_general
    rng = np.random.default_rng(3)
    n, d = 48, 2
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    theta = np.array([math.log(1.1), math.log(0.35), math.log(0.25), math.log(1.3),
                      math.log(0.03)])
    order, groups = _prep(X, theta, n - 1, d)
    ll, _, _, _ = sv.vecchia_profile_loglik(theta, X[order], y[order], None, groups, nu=None,
                                            estimate_nu=True)
    nu = math.exp(theta[1 + d])
    exact = _dense_loglik(X, y, np.delete(theta, 1 + d), lambda r: _matern_corr_general(r, nu))
    assert abs(ll - exact) < 1e-7


# ---------------------------------------------------------------------------
# parity with the reference's outputs on identical inputs
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", LIK_CASES)
def test_parity_with_reference(golden_likelihood, name):
    sv, _, _, _nn_groups = _sv()
    g = golden_likelihood
    X, y, Z, nn, theta = (g[name + s] for s in ("_X", "_y", "_Z", "_nn", "_theta"))
    m, nu, est, need_grad, vp, lvt = g[name + "_meta"]
    groups = _nn_groups(nn, int(m))
    out = sv.vecchia_profile_loglik(theta, X, y, Z if Z.shape[1] else None, groups,
                                    None if nu < 0 else float(nu), estimate_nu=bool(est),
                                    need_grad=bool(need_grad), var_penalty=vp, log_var_target=lvt)
    ll_ref = float(g[name + "_ll"])
    # float64 throughout; the ill-conditioned nugget-1e-8 case carries the
    # reference's own rounding (block condition numbers near 1e9)
    tol = 1e-7 if name == "nug1e8" else 1e-10
    assert abs(out[0] - ll_ref) <= tol * max(1.0, abs(ll_ref)), (out[0], ll_ref)
    if need_grad:
        gr, fi = g[name + "_grad"], g[name + "_fish"]
        gt = 1e-5 if name == "nug1e8" else 1e-8
        np.testing.assert_allclose(out[1], gr, rtol=gt, atol=gt * np.abs(gr).max())
        np.testing.assert_allclose(out[2], fi, rtol=gt, atol=gt * np.abs(fi).max())
    if g[name + "_beta"].size:
        np.testing.assert_allclose(out[3], g[name + "_beta"], rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("n,d,m,q,nu", [(5000, 10, 30, 1, 2.5), (3000, 4, 40, 5, 1.5),
                                         (2500, 6, 20, 0, 0.5), (1500, 3, 140, 1, 2.5)])
def test_parity_with_oracle_larger(oracle, n, d, m, q, nu):
    """Warp (k+1 <= 32) and CTA (k+1 > 32) block kernels against the oracle."""
    sv, _, _, _nn_groups = _sv()
    rng = np.random.default_rng(n + d)
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    Z = np.column_stack([np.ones(n), X])[:, :q] if q else None
    lam = np.exp(rng.uniform(math.log(0.1), math.log(5.0), d))
    theta = np.concatenate([[math.log(1.7)], np.log(lam), [math.log(2e-3)]])
    Xs = X / lam
    order = oracle.maximin_order(Xs)
    nn = oracle.ordered_nn(Xs[order], m)
    groups = _nn_groups(nn, m)
    Zo = Z[order] if q else None
    got = sv.vecchia_profile_loglik(theta, X[order], y[order], Zo, groups, nu)
    ref = oracle.vecchia_loglik(theta, X[order], y[order], Zo, groups, nu)
    assert abs(got[0] - ref[0]) <= 1e-10 * abs(ref[0])
    np.testing.assert_allclose(got[1], ref[1], rtol=1e-8, atol=1e-8 * np.abs(ref[1]).max())
    np.testing.assert_allclose(got[2], ref[2], rtol=1e-8, atol=1e-8 * np.abs(ref[2]).max())
    if q:
        np.testing.assert_allclose(got[3], ref[3], rtol=1e-8, atol=1e-10)


def test_chunk_jitter_matches_oracle(oracle):
    """Duplicated inputs with a tiny nugget make blocks singular; the whole
    chunk is refactored with the first jitter level at which all of its blocks
    succeed (_covariance.py:235-252)."""
    sv, _, _, _nn_groups = _sv()
    rng = np.random.default_rng(8)
    X0 = rng.random((300, 2))
    X = np.vstack([X0, X0[:40]])
    n = X.shape[0]
    y = rng.standard_normal(n)
    theta = np.array([0.0, math.log(0.5), math.log(0.5), math.log(1e-200)])
    order = oracle.maximin_order(X / 0.5)
    nn = oracle.ordered_nn((X / 0.5)[order], 10)
    groups = _nn_groups(nn, 10)
    got = sv.vecchia_profile_loglik(theta, X[order], y[order], np.ones((n, 1)), groups, 2.5)
    ref = oracle.vecchia_loglik(theta, X[order], y[order], np.ones((n, 1)), groups, 2.5)
    assert abs(got[0] - ref[0]) <= 1e-6 * abs(ref[0])


def test_bad_nu_raises():
    sv, _, _, _nn_groups = _sv()
    X = np.random.default_rng(0).random((10, 2))
    nn = sv.find_ordered_nn(X, 3)
    with pytest.raises(ValueError):
        sv.vecchia_profile_loglik(np.zeros(4), X, np.zeros(10), None, _nn_groups(nn, 3), -1.0)


def test_bad_conditioning_sets_raise(problem):
    """Rows or neighbours outside the data raise ValueError (checked while the
    block table is packed on the device, before any kernel reads them)."""
    sv, _, _, _ = _sv()
    X, y, theta = problem
    n, d = X.shape
    order, groups = _prep(X, theta, 8, d)
    Xo, yo, Z = X[order], y[order], np.ones((n, 1))
    for bad_value in (n, n + 7, -2, -1):
        bad = [(np.asarray(r).copy(), np.asarray(nb).copy()) for r, nb in groups]
        rows, nb = bad[-1]
        nb[len(rows) // 2, 0] = bad_value
        with pytest.raises(ValueError):
            sv.vecchia_profile_loglik(theta, Xo, yo, Z, bad, 2.5)
    bad = [(np.asarray(r).copy(), np.asarray(nb).copy()) for r, nb in groups]
    bad[-1][0][3] = n
    with pytest.raises(ValueError):
        sv.vecchia_profile_loglik(theta, Xo, yo, Z, bad, 2.5)
    # the good sets still evaluate afterwards
    assert np.isfinite(sv.vecchia_profile_loglik(theta, Xo, yo, Z, groups, 2.5)[0])


def test_group_order_and_large_blocks_pack_like_the_host(oracle):
    """Conditioning sets given in any group order, with blocks beyond a warp
    (k + 1 > 32), give the oracle's values through the device-packed table."""
    sv, _, _, _nn_groups = _sv()
    rng = np.random.default_rng(21)
    n, d, m = 1500, 3, 40
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    Z = np.ones((n, 1))
    nn = sv.find_ordered_nn(X, m)
    groups = _nn_groups(nn, m)
    theta = np.array([0.1, math.log(0.3), math.log(0.2), math.log(0.4), math.log(0.01)])
    ref = oracle.vecchia_loglik(theta, X, y, Z, groups, 2.5)
    shuffled = [groups[i] for i in rng.permutation(len(groups))]
    for gs in (groups, shuffled):
        ll, g, F, beta = sv.vecchia_profile_loglik(theta, X, y, Z, gs, 2.5)
        assert abs(ll - ref[0]) <= 1e-9 * abs(ref[0])
        np.testing.assert_allclose(g, ref[1], rtol=1e-8, atol=1e-8 * np.abs(ref[1]).max())


def test_device_chunk_ids_match_the_host_rule():
    """Chunk ids computed on the device (sv_chunk_ids) equal the host rule
    (chunk_ids: _chunks per group, groups numbered in their own order), for
    groups in order, shuffled, and with blocks beyond a warp moved last."""
    sv, _, _, _nn_groups = _sv()
    from pyscaledvecchia_gb300.likelihood import DeviceProblem, chunk_ids
    rng = np.random.default_rng(5)
    for n, d, m in ((3000, 3, 20), (2500, 2, 45)):
        X = rng.random((n, d))
        groups = _nn_groups(sv.find_ordered_nn(X, m), m)
        for gs in (groups, [groups[i] for i in rng.permutation(len(groups))]):
            prob = DeviceProblem(X, rng.standard_normal(n), None, gs)
            for Pc in (1, d + 2):
                got = prob.chunk_tensor(Pc).cpu().numpy()
                want = chunk_ids(prob._gid, prob._gk, prob._gl, Pc)
                np.testing.assert_array_equal(got, want)



def test_block_table_same_from_host_reads_and_copies(monkeypatch):
    """The block table packed from the groups' NumPy arrays read in place
    (where the device reads host memory) equals the one packed from device
    copies, including ragged groups, k > 31 and a bad index."""
    sv, _, _, _nn_groups = _sv()
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    rng = np.random.default_rng(9)
    n, d, m = 4000, 3, 40
    X = rng.random((n, d))
    groups = _nn_groups(sv.find_ordered_nn(X, m), m)
    y = rng.standard_normal(n)
    tables = []
    for direct in (True, False):
        monkeypatch.setattr(_lib, "_HOST_READABLE", direct)
        prob = DeviceProblem(X, y, None, groups)
        tables.append([t.cpu().numpy() for t in (prob.rowb, prob.kb, prob.nbr)])
        bad = [(g[0], g[1].copy()) for g in groups]
        bad[-1][1][5, 3] = n + 7
        with pytest.raises(ValueError):
            DeviceProblem(X, y, None, bad)
    for a, b in zip(*tables):
        np.testing.assert_array_equal(a, b)
