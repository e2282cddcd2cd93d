"""Exact marginal variances of the joint predictive law (predict_joint(
exact_var=True)): diag((U_pp U_pp^T)^-1) from sv_joint_var_diag against the
dense S = U_pp^-T of gp.py:391-393 (the reference), formed on the CPU from
the same factor columns, and the panel split against one panel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fit(n=1500, d=3, seed=0):
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = np.sin(4 * X[:, 0]) + X[:, 1] * X[:, 2] + 0.05 * rng.standard_normal(n)
    gp = ScaledVecchiaGP(m_est=15, n_est=1000, var_correction=False).fit(X, y)
    return gp, rng.uniform(-0.05, 1.05, (2000, d))


def _dense_var(F):
    """(S**2).sum(1) with S = Lt^-1, Lt = U_pp^T built from the columns."""
    from scipy.linalg import solve_triangular
    ns, n, k = F["ns"], F["n"], F["k"]
    acol = F["acol"].cpu().numpy()
    nbr = F["nbr"].cpu().numpy()
    Lt = np.zeros((ns, ns))
    for c in range(ns):
        Lt[c, c] = acol[c, k]
        for s in range(k):
            ix = nbr[c, s]
            if ix >= n:
                Lt[c, ix - n] = acol[c, s]
    S = solve_triangular(Lt, np.eye(ns), lower=True)
    return (S ** 2).sum(1)


@pytest.mark.parametrize("m", [10, 40])
def test_joint_variance_against_the_dense_inverse(m):
    gp, Xte = _fit()
    Xs = (Xte - gp._lo) / gp._span
    F = gp._joint_factor_device(Xs, m)
    v = gp._joint_var_diag(F).cpu().numpy()
    ref = _dense_var(F)
    np.testing.assert_allclose(v, ref, rtol=1e-10, atol=0)


def test_panels_agree_with_one_panel():
    """Panels of 7 columns and fewer (the scratch holds 7 columns of every
    row) against the single panel of the whole lower triangle."""
    gp, Xte = _fit(seed=1)
    Xs = (Xte[:700] - gp._lo) / gp._span
    F = gp._joint_factor_device(Xs, 30)
    ns = F["ns"]
    one = gp._joint_var_diag(F, panel_bytes=8 * ns * ns).cpu().numpy()
    many = gp._joint_var_diag(F, panel_bytes=8 * ns * 7).cpu().numpy()
    np.testing.assert_allclose(many, one, rtol=1e-13, atol=0)


def test_too_small_panel_is_refused():
    import torch

    from pyscaledvecchia_gb300 import _lib
    lib, _ = _lib.device_ready()
    gp, Xte = _fit(seed=2)
    F = gp._joint_factor_device((Xte[:100] - gp._lo) / gp._span, 10)
    ns = F["ns"]
    panel = _lib.workspace(torch, 8 * (ns - 1))
    ws = _lib.workspace(torch, lib.sv_joint_solve_workspace_bytes(ns))
    v = torch.empty(ns, dtype=torch.float64, device="cuda")
    info = _lib.new_info(torch)
    rc = lib.sv_joint_var_diag(ns, F["n"], F["k"], F["k"], _lib.ptr(F["nbr"]), _lib.ptr(F["acol"]),
                               _lib.ptr(v), _lib.ptr(info), _lib.ptr(ws), ws.numel(), _lib.ptr(panel),
                               8 * (ns - 1), _lib.stream_handle(torch))
    assert rc == 5  # SV_ENOSPC
