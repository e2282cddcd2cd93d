"""Matern correlation and batched block linear algebra, on the GPU.

Drop-in counterparts of the reference's ``scaled_vecchia._covariance``
(jdtuck/pyscaledvecchia, src/scaled_vecchia/_covariance.py).  Every numeric
routine runs in libsvgpu.so (include/svgpu.h); NumPy arrays go in and come
out, as in the reference.

  LOG2PI, _matern_corr, _matern_g   _covariance.py:39, 49-72
  _check_nu                         _covariance.py:75-77
  _block_cov                        _covariance.py:150-198
  _forward_solve, _backsolve_LT     _covariance.py:205-232
  _batch_chol                       _covariance.py:235-252
  _chunks                           _covariance.py:255-259

The fused likelihood and prediction paths do not go through these
block-at-a-time helpers; they exist for callers of the reference's
block-level interface.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib

LOG2PI = math.log(2.0 * math.pi)
_SQRT3 = math.sqrt(3.0)
_SQRT5 = math.sqrt(5.0)


def _elementwise(r, nu, which, general):
    lib, torch = _lib.device_ready()
    r = np.asarray(r, dtype=float)
    flat = np.ascontiguousarray(r.reshape(-1))
    if flat.size == 0:
        return np.empty(r.shape)
    rd = _lib.to_dev(torch, flat, np.float64)
    out = torch.empty_like(rd)
    rc = lib.sv_matern_eval(_lib.ptr(rd), flat.size, float(nu), which, general, _lib.ptr(out),
                            _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_matern_eval")
    res = out.cpu().numpy().reshape(r.shape)
    return res[()] if res.ndim == 0 else res


def _matern_corr(r: np.ndarray, nu: float) -> np.ndarray:
    """M_nu(r): isotropic Matern correlation, closed form for nu = .5/1.5/2.5."""
    if nu not in (0.5, 1.5, 2.5):
        raise ValueError("nu must be one of 0.5, 1.5, 2.5")
    return _elementwise(r, nu, 0, 0)


def _matern_g(r: np.ndarray, nu: float) -> np.ndarray:
    """g(r) = M_nu'(r) / r  (finite at r=0 for nu >= 1.5)."""
    if nu not in (0.5, 1.5, 2.5):
        raise ValueError("nu must be one of 0.5, 1.5, 2.5")
    return _elementwise(r, nu, 1, 0)


def _check_nu(nu: float) -> None:
    if not (isinstance(nu, (int, float)) and nu > 0.0):
        raise ValueError("nu must be a positive number")


def _block_cov_device(Xb, ranges, variance, nugget, nu, derivs, nug_mask, general,
                      estimate_nu=False, nu_fd_h=1e-3):
    lib, torch = _lib.device_ready()
    Xb = np.ascontiguousarray(Xb, dtype=np.float64)
    B, K, d = Xb.shape
    P = d + 2 + (1 if estimate_nu else 0)
    rng = np.ascontiguousarray(ranges, dtype=np.float64).reshape(-1)
    if rng.shape[0] != d:
        raise ValueError("ranges must have one entry per input dimension")
    xd = _lib.to_dev(torch, Xb, np.float64)
    S = torch.empty((B, K, K), dtype=torch.float64, device="cuda")
    dS = torch.empty((B, P, K, K), dtype=torch.float64, device="cuda") if derivs else None
    md = None
    if nug_mask is not None:
        md = _lib.to_dev(torch, np.asarray(nug_mask, dtype=np.float64).reshape(B, K), np.float64)
    rc = lib.sv_block_cov(_lib.ptr(xd), B, K, d, rng.ctypes.data_as(_lib.c_vp), float(variance),
                          float(nugget), float(nu), int(general), int(bool(estimate_nu)),
                          float(nu_fd_h), _lib.ptr(md), _lib.ptr(S), _lib.ptr(dS),
                          _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_block_cov")
    return S.cpu().numpy(), (dS.cpu().numpy() if derivs else None)


def _block_cov(Xb, ranges, variance, nugget, nu, derivs=True, nug_mask=None):
    """Covariance matrices (and d/dlog-parameter derivatives) for a batch of blocks.

    Xb (B, K, d) raw coordinates, ranges (d,) lambda_l, variance sigma^2,
    nugget tau (relative), nu the Matern smoothness (0.5/1.5/2.5 closed form,
    any other positive value the Bessel form), nug_mask (B, K) or None.
    Returns Sigma (B, K, K) and dSigma (B, d+2, K, K) w.r.t. log sigma^2,
    log lambda_1..d, log tau (or None when derivs is False).
    """
    _check_nu(nu)
    general = nu not in (0.5, 1.5, 2.5)
    return _block_cov_device(Xb, ranges, variance, nugget, nu, derivs, nug_mask, general)


def _forward_solve(L: np.ndarray, Bm: np.ndarray) -> np.ndarray:
    """Solve L X = B for lower-triangular L. L:(b,K,K), B:(b,K,nrhs)."""
    return _trsm(L, Bm, "sv_forward_solve")


def _backsolve_LT(L: np.ndarray, Bm: np.ndarray) -> np.ndarray:
    """Solve L^T X = B for lower-triangular L."""
    return _trsm(L, Bm, "sv_backsolve_LT")


def _trsm(L, Bm, name):
    lib, torch = _lib.device_ready()
    L = np.ascontiguousarray(L, dtype=np.float64)
    Bm = np.ascontiguousarray(Bm, dtype=np.float64)
    b, K, nrhs = Bm.shape
    if L.shape != (b, K, K):
        raise ValueError("L must be (b, K, K) matching B (b, K, nrhs)")
    if b == 0 or nrhs == 0:
        return np.empty_like(Bm)
    Ld = _lib.to_dev(torch, L, np.float64)
    Bd = _lib.to_dev(torch, Bm, np.float64)
    Xd = torch.empty_like(Bd)
    rc = getattr(lib, name)(_lib.ptr(Ld), _lib.ptr(Bd), b, K, nrhs, _lib.ptr(Xd),
                            _lib.stream_handle(torch))
    _lib.check(lib, rc, name)
    return Xd.cpu().numpy()


def _batch_chol(Sigma: np.ndarray) -> np.ndarray:
    """Cholesky with escalating jitter (blocks can be near-singular).

    If any block of the batch fails, the whole batch is refactored with
    10^p * mean(diag) added to each block's diagonal, p = -12..-4, at the
    first p for which every block succeeds; otherwise LinAlgError.
    """
    lib, torch = _lib.device_ready()
    S = np.ascontiguousarray(Sigma, dtype=np.float64)
    B, K, K2 = S.shape
    if K != K2:
        raise ValueError("Sigma must be (B, K, K)")
    if B == 0:
        return np.empty_like(S)
    Sd = _lib.to_dev(torch, S, np.float64)
    Ld = torch.empty_like(Sd)
    info = _lib.new_info(torch)
    ws = _lib.workspace(torch, lib.sv_batch_chol_workspace_bytes(B))
    rc = lib.sv_batch_chol(_lib.ptr(Sd), B, K, _lib.ptr(Ld), _lib.ptr(info), _lib.ptr(ws),
                           ws.numel(), _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_batch_chol")
    _lib.check_info(lib, info.cpu().numpy(), "sv_batch_chol")
    return Ld.cpu().numpy()


def _chunks(n_rows: int, K: int, P: int, budget: int = 4_000_000):
    """Yield (start, end) row-slices sized so that K*K*P*chunk stays bounded."""
    step = max(1, budget // max(1, K * K * max(P, 1)))
    for a in range(0, n_rows, step):
        yield a, min(n_rows, a + step)
