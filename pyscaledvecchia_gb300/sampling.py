"""Unconditional Vecchia draws on the GPU.

y = U^-T eps, where U is the sparse inverse Cholesky factor whose column i
is a_i = L_i^-T e_K of block i (likelihood.py:27-29 of the reference); the
draw has covariance (U U^T)^-1, the Vecchia approximation of
sigma^2 [M_nu + tau I].  The reference only samples conditionally on data
(gp.py:395-401); synthetic problems drawn "from the method itself" need this
prior form.  Blocks come from sv_predict_blocks (nugget on every row), the
solve from sv_joint_solve.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .likelihood import matern_table_nu

__all__ = ["vecchia_prior_sample"]


def vecchia_prior_sample_device(torch, Xo_d, nn_d, theta, nu, eps_d):
    """Device form: Xo_d (n, d) in the ordering, nn_d (n, m+1) int64 from the
    ordered neighbour search, theta = [log s2, log lam_1..d, log tau],
    eps_d (n, nsim).  Returns y (n, nsim) on the device."""
    lib = _lib.load_library()
    n, d = Xo_d.shape
    m = nn_d.shape[1] - 1
    nsim = eps_d.shape[1]
    nbr = nn_d[:, 1:].to(torch.int32).contiguous() if m > 0 else \
        torch.full((n, 1), -1, dtype=torch.int32, device="cuda")
    k = max(m, 1)
    tgt = torch.arange(n, dtype=torch.int32, device="cuda")
    acol = torch.empty((n, k + 1), dtype=torch.float64, device="cuda")
    D = _lib.PredDesc()
    D.nall, D.nobs, D.nblk = n, n, n
    D.d, D.k, D.ldnbr = d, k, k
    D.general = int(nu not in (0.5, 1.5, 2.5))
    D.target_nugget = 1
    D.nu = float(nu)
    mtab = None
    if D.general and matern_table_nu(float(nu)):
        # M and g interpolated as the likelihood interpolates them
        mtab = torch.empty(int(lib.sv_matern_table_doubles()), dtype=torch.float64, device="cuda")
        _lib.check(lib, lib.sv_matern_table(float(nu), _lib.ptr(mtab), mtab.numel(),
                                            _lib.stream_handle(torch)), "sv_matern_table")
        D.matern_table = mtab.data_ptr()
    th = _lib.to_dev(torch, np.asarray(theta, dtype=np.float64), np.float64)
    info = _lib.new_info(torch)
    rc = lib.sv_predict_blocks(D, _lib.ptr(th), _lib.ptr(Xo_d), _lib.ptr(tgt), _lib.ptr(nbr),
                               None, None, None, _lib.ptr(acol), None, _lib.ptr(info),
                               _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_predict_blocks")
    y = torch.empty((n, nsim), dtype=torch.float64, device="cuda")
    info2 = _lib.new_info(torch)
    ws = _lib.workspace(torch, lib.sv_joint_solve_workspace_bytes(n))
    rc = lib.sv_joint_solve(n, 0, k, k, _lib.ptr(nbr), _lib.ptr(acol), _lib.ptr(eps_d), nsim,
                            _lib.ptr(y), _lib.ptr(info2), _lib.ptr(ws), ws.numel(),
                            _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_joint_solve")
    _lib.check_info(lib, info.cpu().numpy(), "sv_predict_blocks")
    _lib.check_info(lib, info2.cpu().numpy(), "sv_joint_solve")
    return y


def vecchia_prior_sample(Xo, nn, theta, nu, eps):
    """Host form of ``vecchia_prior_sample_device`` (NumPy in and out).

    Xo (n, d) inputs in the ordering, nn (n, m+1) from ``find_ordered_nn``,
    theta [log sigma^2, log lambda_1..d, log tau], eps (n,) or (n, nsim)
    standard normal draws.  Returns y with the shape of eps.
    """
    lib, torch = _lib.device_ready()
    eps = np.asarray(eps, dtype=np.float64)
    e2 = eps.reshape(eps.shape[0], -1)
    y = vecchia_prior_sample_device(torch, _lib.to_dev(torch, Xo, np.float64),
                                    _lib.to_dev(torch, np.asarray(nn, np.int64), np.int64),
                                    theta, nu, _lib.to_dev(torch, e2, np.float64))
    return y.cpu().numpy().reshape(eps.shape)
