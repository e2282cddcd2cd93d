"""CPU oracle for the scaled Vecchia hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
to check the device result, and by ``bench.py`` for its CPU baseline.  The product package
(pyscaledvecchia_gb300) never imports, loads or calls anything here.

Two layers, both restating the reference implementation
(jdtuck/pyscaledvecchia, src/scaled_vecchia/...):

* ``sv_oracle.c`` (built to oracle/_build/libsvoracle.so, OpenMP over blocks):
  exact maximin ordering (ordering.py:27-59), exact ordered kNN by
  (distance, index) (ordering.py:76-116), the closed-form-nu likelihood,
  score and Fisher information (likelihood.py:66-175 with the block kernels
  of _covariance.py:111-147, 205-252) and marginal prediction blocks
  (gp.py:242-277).
* NumPy/SciPy below: the general (Bessel, scipy.special.kv) Matern path
  (_matern_general.py:87-179) inside a per-block likelihood, the joint
  factor and sparse solves (gp.py:307-402).

Pinned against the golden vectors of tests/golden/ (generated by running the
reference itself, see tests/golden/make_golden.py): bit-exact maximin orders,
equal neighbour sets, and likelihood outputs to ~1e-12 relative.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsvoracle.so")
LOG2PI = math.log(2.0 * math.pi)

_lib = None


def build(force=False):
    """Compile sv_oracle.c with gcc (no FMA contraction, OpenMP)."""
    src = os.path.join(HERE, "sv_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared", "-fPIC",
           src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.or_maximin.argtypes = [vp, i64, i32, i64, vp]
        L.or_ordered_nn.argtypes = [vp, i64, i32, i32, i64, vp]
        L.or_knn_query.argtypes = [vp, i64, vp, i64, i32, i32, vp]
        L.or_vecchia_loglik.argtypes = [vp, vp, vp, vp, i64, i32, i32, vp, vp, vp, i32, i64, vp,
                                        dbl, i32, dbl, dbl, vp]
        L.or_vecchia_loglik.restype = i32
        L.or_predict_blocks.argtypes = [vp, vp, vp, i64, i32, i32, vp, vp, dbl, dbl, dbl, vp, vp]
        L.or_predict_blocks.restype = i32
        L.or_block_records.argtypes = [vp, vp, vp, vp, i64, i32, i32, vp, vp, vp, i32, i64, i64, vp,
                                       dbl, i32, vp, vp]
        L.or_block_records.restype = i32
        L.or_num_threads.restype = i32
        L.or_set_num_threads.argtypes = [i32]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def set_threads(t):
    lib().or_set_num_threads(int(t))


def num_threads():
    return int(lib().or_num_threads())


# ---------------------------------------------------------------------------
# ordering
# ---------------------------------------------------------------------------
def maximin_order(X, first=None):
    X = np.ascontiguousarray(X, dtype=np.float64)
    if first is None:
        first = int(np.argmin(((X - X.mean(0)) ** 2).sum(1)))  # ordering.py:72
    n, d = X.shape
    out = np.empty(n, dtype=np.int64)
    if n:
        lib().or_maximin(_p(X), n, d, int(first), _p(out))
    return out


def ordered_nn(X, m, start=0):
    X = np.ascontiguousarray(X, dtype=np.float64)
    n, d = X.shape
    nn = np.empty((n, m + 1), dtype=np.int64)
    if n:
        lib().or_ordered_nn(_p(X), n, d, int(m), int(start), _p(nn))
    return nn


def knn_query(Xref, Xq, k):
    Xref = np.ascontiguousarray(Xref, dtype=np.float64)
    Xq = np.ascontiguousarray(Xq, dtype=np.float64)
    nb = np.empty((Xq.shape[0], k), dtype=np.int64)
    lib().or_knn_query(_p(Xref), Xref.shape[0], _p(Xq), Xq.shape[0], Xq.shape[1], int(k), _p(nb))
    return nb


def nn_groups(nn, m):
    """ordering.py:119-127."""
    n = nn.shape[0]
    ks = np.minimum(np.arange(n), m)
    return [(np.where(ks == k)[0], nn[np.where(ks == k)[0], 1:k + 1]) for k in np.unique(ks)]


def _flatten_groups(groups, Pc=None):
    rows, kb, nbs, chunk = [], [], [], []
    cid = 0
    for r, nb in groups:
        r = np.asarray(r, dtype=np.int64)
        nb = np.asarray(nb, dtype=np.int64).reshape(len(r), -1)
        K = nb.shape[1] + 1
        rows.append(r)
        kb.append(np.full(len(r), nb.shape[1], dtype=np.int32))
        nbs.append(nb)
        if Pc is not None:
            step = max(1, 4_000_000 // max(1, K * K * max(Pc, 1)))  # _covariance.py:255-259
            ids = np.arange(len(r)) // step + cid
            cid = (ids.max() + 1) if len(r) else cid
            chunk.append(ids)
    kmax = max((nb.shape[1] for nb in nbs), default=0)
    B = sum(len(r) for r in rows)
    nbr = np.full((B, max(kmax, 1)), -1, dtype=np.int64)
    o = 0
    for nb in nbs:
        nbr[o:o + nb.shape[0], :nb.shape[1]] = nb
        o += nb.shape[0]
    chunk = np.concatenate(chunk).astype(np.int64) if Pc is not None and chunk else None
    return (np.concatenate(rows) if rows else np.zeros(0, np.int64),
            np.concatenate(kb) if kb else np.zeros(0, np.int32), nbr, chunk)


# ---------------------------------------------------------------------------
# likelihood
# ---------------------------------------------------------------------------
def vecchia_loglik(theta, Xo, yo, Zo, groups, nu, need_grad=True, var_penalty=0.0,
                   log_var_target=0.0, chunked=True):
    """C restatement of likelihood.py:66-175 for nu in {0.5, 1.5, 2.5}."""
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    Xo = np.ascontiguousarray(Xo, dtype=np.float64)
    yo = np.ascontiguousarray(yo, dtype=np.float64)
    n, d = Xo.shape
    has_Z = Zo is not None and Zo.shape[1] > 0
    q = Zo.shape[1] if has_Z else 0
    Zc = np.ascontiguousarray(Zo, dtype=np.float64) if has_Z else None
    P = d + 2
    rows, kb, nbr, chunk = _flatten_groups(groups, (P if need_grad else 1) if chunked else None)
    out = np.zeros(1 + P + P * P + q)
    rc = lib().or_vecchia_loglik(_p(theta), _p(Xo), _p(yo), _p(Zc), n, d, q, _p(rows), _p(kb),
                                 _p(nbr), nbr.shape[1], rows.shape[0], _p(chunk), float(nu),
                                 int(need_grad), float(var_penalty), float(log_var_target),
                                 _p(out))
    if rc == -1:
        raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
    if rc != 0:
        raise ValueError("unsupported sizes")
    ll = float(out[0])
    if need_grad:
        return ll, out[1:1 + P].copy(), out[1 + P:1 + P + P * P].reshape(P, P).copy(), \
            out[1 + P + P * P:].copy()
    return ll, None, None, out[1:1 + q].copy()


def matern_general(r, nu, deriv=False):
    """_matern_general.py:92-116 with scipy.special (M or g)."""
    from scipy.special import gammaln, kv
    r = np.asarray(r, dtype=float)
    rr = np.where(r < 1e-7, 1e-7, r)
    c = math.sqrt(2.0 * nu) * rr
    lc = (1.0 - nu) * math.log(2.0) - gammaln(nu)
    if not deriv:
        return np.where(r < 1e-7, 1.0, np.exp(lc + nu * np.log(c)) * kv(nu, c))
    val = -(math.sqrt(2.0 * nu) / rr) * np.exp(lc + nu * np.log(c)) * kv(nu - 1.0, c)
    return np.where(r < 1e-7, 0.0, val)


def matern_closed(r, nu, deriv=False):
    r = np.asarray(r, dtype=float)
    if nu == 0.5:
        if not deriv:
            return np.exp(-r)
        rs = np.where(r > 0, r, 1.0)
        return np.where(r > 0, -np.exp(-rs) / rs, 0.0)
    c = (math.sqrt(3.0) if nu == 1.5 else math.sqrt(5.0)) * r
    if nu == 1.5:
        return (1 + c) * np.exp(-c) if not deriv else -3.0 * np.exp(-c)
    return (1 + c + c * c / 3) * np.exp(-c) if not deriv else -(5 / 3) * (1 + c) * np.exp(-c)


def block_cov_np(Xb, ranges, variance, nugget, nu, derivs=True, nug_mask=None,
                 estimate_nu=False, h=1e-3):
    """Sigma and dSigma for one batch of blocks (any nu; scipy kv for the
    general form), rows [sigma^2, lambda_1..d, (nu), tau]."""
    B, K, d = Xb.shape
    U = Xb / ranges
    diff = U[:, :, None, :] - U[:, None, :, :]
    r = np.sqrt((diff ** 2).sum(-1))
    closed = (not estimate_nu) and nu in (0.5, 1.5, 2.5)
    Mf = (lambda rr, v: matern_closed(rr, v)) if closed else (lambda rr, v: matern_general(rr, v))
    gf = (lambda rr, v: matern_closed(rr, v, True)) if closed else \
        (lambda rr, v: matern_general(rr, v, True))
    M = Mf(r, nu)
    mask = np.ones((B, K)) if nug_mask is None else np.asarray(nug_mask, dtype=float)
    nugd = np.eye(K)[None] * (nugget * mask[:, :, None])
    S = variance * (M + nugd)
    if not derivs:
        return S, None
    P = d + 2 + (1 if estimate_nu else 0)
    dS = np.empty((B, P, K, K))
    dS[:, 0] = S
    g = gf(r, nu)
    for l in range(d):
        dS[:, 1 + l] = -variance * g * diff[..., l] ** 2
    p = 1 + d
    if estimate_nu:
        dS[:, p] = variance * nu * (matern_general(r, nu + h) - matern_general(r, nu - h)) / (2 * h)
        p += 1
    dS[:, p] = variance * nugd
    return S, dS


def _chol_jitter(S):
    """_covariance.py:235-252 for one batch."""
    try:
        return np.linalg.cholesky(S)
    except np.linalg.LinAlgError:
        pass
    scale = np.einsum("bii->b", S) / S.shape[-1]
    eye = np.eye(S.shape[-1])
    for p in range(-12, -3):
        try:
            return np.linalg.cholesky(S + (10.0 ** p) * scale[:, None, None] * eye)
        except np.linalg.LinAlgError:
            continue
    raise np.linalg.LinAlgError("block Cholesky failed even with jitter")


def vecchia_loglik_np(theta, Xo, yo, Zo, groups, nu, estimate_nu=False, need_grad=True,
                      var_penalty=0.0, log_var_target=0.0):
    """NumPy/SciPy restatement of likelihood.py:66-175 for any nu (small n)."""
    from scipy.linalg import solve_triangular
    theta = np.asarray(theta, dtype=float)
    n, d = Xo.shape
    variance = math.exp(theta[0])
    ranges = np.exp(theta[1:1 + d])
    if estimate_nu:
        nu = math.exp(theta[1 + d])
        nugget = math.exp(theta[2 + d])
        P = d + 3
    else:
        nugget = math.exp(theta[1 + d])
        P = d + 2
    has_Z = Zo is not None and Zo.shape[1] > 0
    q = Zo.shape[1] if has_Z else 0
    XtX, Zty, fish = np.zeros((q, q)), np.zeros(q), np.zeros((P, P))
    recs = []
    for rows, nb in groups:
        K = nb.shape[1] + 1
        idx = np.concatenate([nb, rows[:, None]], axis=1)
        step = max(1, 4_000_000 // max(1, K * K * (P if need_grad else 1)))
        for a0 in range(0, len(rows), step):
            blk = idx[a0:a0 + step]
            S, dS = block_cov_np(Xo[blk], ranges, variance, nugget, nu, derivs=need_grad,
                                 estimate_nu=estimate_nu)
            L = _chol_jitter(S)
            for b in range(blk.shape[0]):
                Lb = L[b]
                eK = np.zeros(K)
                eK[-1] = 1.0
                a = solve_triangular(Lb, eK, lower=True, trans="T")
                yv = yo[blk[b]]
                Zv = Zo[blk[b]] if has_Z else np.zeros((K, 0))
                yt, Zt = a @ yv, a @ Zv
                XtX += np.outer(Zt, Zt)
                Zty += Zt * yt
                W = None
                if need_grad:
                    rhs = np.einsum("pkl,l->kp", dS[b], a)
                    W = solve_triangular(Lb, rhs, lower=True).T
                    wK = W[:, -1]
                    fish += 0.5 * (2.0 * W @ W.T - np.outer(wK, wK))
                recs.append((Lb, W, yv, Zv))
    beta = np.linalg.solve(XtX + 1e-12 * np.eye(q), Zty) if has_Z else np.zeros(0)
    ll = -0.5 * n * LOG2PI
    grad = np.zeros(P)
    for Lb, W, yv, Zv in recs:
        resid = yv - (Zv @ beta if has_Z else 0.0)
        z = solve_triangular(Lb, resid, lower=True)
        zK = z[-1]
        ll -= 0.5 * (2.0 * math.log(Lb[-1, -1]) + zK ** 2)
        if need_grad:
            wK = W[:, -1]
            grad -= 0.5 * (wK * (1.0 + zK ** 2) - 2.0 * zK * (W @ z))
    if var_penalty > 0.0:
        excess = max(0.0, theta[0] - log_var_target)
        ll -= 0.5 * var_penalty * excess ** 2
        if need_grad:
            grad[0] -= var_penalty * excess
            if excess > 0.0:
                fish[0, 0] += var_penalty
    if not need_grad:
        return ll, None, None, beta
    return ll, grad, fish, beta


# ---------------------------------------------------------------------------
# prediction
# ---------------------------------------------------------------------------
def predict_marginal(X_tr, resid, Xq, theta, nu, m):
    """gp.py:242-277 (noise-free target), C restatement for closed-form nu."""
    d = X_tr.shape[1]
    ranges = np.exp(theta[1:1 + d])
    m = min(m, X_tr.shape[0])
    nb = knn_query(X_tr / ranges, Xq / ranges, m)
    mean, var = np.empty(Xq.shape[0]), np.empty(Xq.shape[0])
    rc = lib().or_predict_blocks(_p(np.ascontiguousarray(X_tr)), _p(np.ascontiguousarray(resid)),
                                 _p(np.ascontiguousarray(Xq)), Xq.shape[0], d, m, _p(nb),
                                 _p(np.ascontiguousarray(ranges)), math.exp(theta[0]),
                                 math.exp(theta[-1]), float(nu), _p(mean), _p(var))
    if rc != 0:
        raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
    return mean, var, nb


def joint_factor_np(X_obs, Xs, theta, nu, m):
    """gp.py:307-358: block columns of U for the observed-first ordering."""
    from scipy import sparse
    n, d = X_obs.shape
    ns = Xs.shape[0]
    ranges = np.exp(theta[1:1 + d])
    Xall = np.vstack([X_obs, Xs])
    Xsc = Xall / ranges
    order_obs = maximin_order(Xsc[:n])
    order_pred = maximin_order(Xsc[n:]) + n
    order = np.concatenate([order_obs, order_pred])
    k = min(m, n)
    nn = ordered_nn(Xsc[order], k, start=n)
    Xo = Xall[order]
    K = k + 1
    blk = np.concatenate([nn[n:, 1:K], np.arange(n, n + ns)[:, None]], axis=1)
    mask = np.ones((ns, K))
    mask[:, K - 1] = 0.0
    mask[:, :K - 1] = (blk[:, :K - 1] < n).astype(float)
    closed = nu in (0.5, 1.5, 2.5)
    S, _ = block_cov_np(Xo[blk], ranges, math.exp(theta[0]), math.exp(theta[-1]), nu,
                        derivs=False, nug_mask=mask, estimate_nu=False) if closed else \
        block_cov_np(Xo[blk], ranges, math.exp(theta[0]), math.exp(theta[-1]), nu,
                     derivs=False, nug_mask=mask)
    L = _chol_jitter(S)
    eK = np.zeros((ns, K, 1))
    eK[:, -1, 0] = 1.0
    from scipy.linalg import solve_triangular
    av = np.stack([solve_triangular(L[b], eK[b, :, 0], lower=True, trans="T") for b in range(ns)])
    U = sparse.coo_matrix((av.ravel(), (blk.ravel(), np.repeat(np.arange(ns), K))),
                          shape=(n + ns, ns)).tocsc()
    return U[:n, :], U[n:, :], order[n:] - n, order_obs, av, blk
