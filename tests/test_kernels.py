"""Device Bessel K_nu, elementwise Matern, block covariance, batched Cholesky
and triangular solves against SciPy / the reference's outputs."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bessel_k_against_scipy():
    from scipy.special import kv
    from pyscaledvecchia_gb300 import _lib
    lib, torch = _lib.device_ready()
    x = np.logspace(-7, 2.8, 5000)
    xd = _lib.to_dev(torch, x, np.float64)
    out = torch.empty_like(xd)
    for nu in (0.0, 0.3, 0.5, 0.8, 0.999, 1.5, 1.75, 2.5, 3.3, 6.1, 9.7, 10.001, 0.799, 0.801):
        rc = lib.sv_bessel_k(_lib.ptr(xd), x.size, nu, _lib.ptr(out), _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_bessel_k")
        ref = kv(nu, x)
        ok = ref > 1e-290
        rel = np.abs(out.cpu().numpy()[ok] - ref[ok]) / ref[ok]
        # scipy's kv (AMOS) itself carries up to ~1.5e-13 relative error here
        assert rel.max() < 5e-13, (nu, rel.max())


def test_matern_elementwise_vs_reference(golden_blocks):
    from pyscaledvecchia_gb300._covariance import _matern_corr, _matern_g
    from pyscaledvecchia_gb300._matern_general import _matern_corr_general, _matern_g_general
    g = golden_blocks
    r = g["r"]
    for nu in (0.5, 1.5, 2.5):
        np.testing.assert_allclose(_matern_corr(r, nu), g[f"Mc_{nu}"], rtol=1e-14, atol=1e-300)
        np.testing.assert_allclose(_matern_g(r, nu), g[f"gc_{nu}"], rtol=1e-14, atol=1e-300)
    for nu in (0.3, 0.5, 0.8, 1.5, 1.75, 2.5, 3.3, 6.1, 9.7):
        np.testing.assert_allclose(_matern_corr_general(r, nu), g[f"Mg_{nu}"], rtol=5e-13,
                                   atol=1e-300)
        # g near the r floor (1e-7) is ~1e9 and inherits scipy's kv error there
        np.testing.assert_allclose(_matern_g_general(r, nu), g[f"gg_{nu}"], rtol=2e-11,
                                   atol=1e-300)


def test_block_cov_vs_reference(golden_blocks):
    from pyscaledvecchia_gb300._covariance import _block_cov
    from pyscaledvecchia_gb300._matern_general import _block_cov_general
    g = golden_blocks
    Xb, ranges, mask = g["Xb"], g["ranges"], g["mask"]
    for nu in (0.5, 1.5, 2.5, 0.8, 1.75):
        S, dS = _block_cov(Xb, ranges, 1.3, 0.07, nu, derivs=True, nug_mask=mask)
        np.testing.assert_allclose(S, g[f"S_{nu}"], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(dS, g[f"dS_{nu}"], rtol=1e-11, atol=1e-13)
        S2, none = _block_cov(Xb, ranges, 1.3, 0.07, nu, derivs=False, nug_mask=mask)
        assert none is None
        np.testing.assert_allclose(S2, S)
    S, dS = _block_cov_general(Xb, ranges, 1.3, 0.07, 1.2, derivs=True, estimate_nu=True)
    np.testing.assert_allclose(S, g["S_est1.2"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(dS, g["dS_est1.2"], rtol=1e-8, atol=1e-10)


def test_batch_chol_and_solves():
    from pyscaledvecchia_gb300._covariance import _backsolve_LT, _batch_chol, _forward_solve
    rng = np.random.default_rng(0)
    A = rng.standard_normal((7, 33, 33))
    S = A @ A.transpose(0, 2, 1) + 33 * np.eye(33)
    L = _batch_chol(S)
    np.testing.assert_allclose(L, np.linalg.cholesky(S), rtol=1e-12, atol=1e-12)
    Bm = rng.standard_normal((7, 33, 3))
    X = _forward_solve(L, Bm)
    np.testing.assert_allclose(L @ X, Bm, atol=1e-10)
    Y = _backsolve_LT(L, Bm)
    np.testing.assert_allclose(L.transpose(0, 2, 1) @ Y, Bm, atol=1e-10)


def test_batch_chol_jitter_is_batch_wide():
    """A singular block forces one jitter level on every block of the batch:
    the first p in -12..-4 at which every block factorises, added to each
    block's diagonal as 10^p * mean(diag)."""
    from pyscaledvecchia_gb300._covariance import _batch_chol
    rng = np.random.default_rng(1)
    v = rng.standard_normal((5, 1))
    good = np.eye(5) + 0.1
    sing = v @ v.T  # rank one
    S = np.stack([good, sing])
    L = _batch_chol(S)
    scale = np.einsum("bii->b", S) / 5
    p_ref = None
    for p in range(-12, -3):
        try:
            np.linalg.cholesky(S + (10.0 ** p) * scale[:, None, None] * np.eye(5))
            p_ref = p
            break
        except np.linalg.LinAlgError:
            continue
    jit = (10.0 ** p_ref) * scale
    # both blocks carry the batch's jitter (backward error of the factor)
    for b in range(2):
        R = L[b] @ L[b].T - S[b]
        np.testing.assert_allclose(np.diag(R), jit[b], rtol=1e-3)
        off = R - np.diag(np.diag(R))
        assert np.abs(off).max() <= 1e-12 * scale[b]
    assert np.allclose(np.triu(L[0], 1), 0.0)
    with pytest.raises(np.linalg.LinAlgError):
        _batch_chol(np.stack([good, -np.eye(5)]))
    assert math.isfinite(float(L.sum()))
