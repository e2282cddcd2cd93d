"""The scaled Vecchia GP emulator (Katzfuss, Guinness & Lawrence, 2020/2022)
with its hot path on the GPU.

Drop-in counterpart of the reference's ``scaled_vecchia.gp.ScaledVecchiaGP``
(src/scaled_vecchia/gp.py): the same dataclass fields, fitted attributes,
properties and methods, and the same host-side control (standardisation,
subsampling and every random draw come from NumPy exactly as in the
reference).  The numeric work runs in libsvgpu.so:

  fit            maximin ordering + ordered kNN in the scaled space
                 (gp.py:182-191), one fused likelihood/score/Fisher launch per
                 objective call (gp.py:196-209), Fisher scoring on the host
                 (optimize.py), variance correction (gp.py:410-425)
  predict        kNN query + noise-free prediction blocks (gp.py:242-304)
  predict_joint  observed-first maximin, ordered kNN of the prediction rows,
                 block columns of U and the sparse triangular solves
                 (gp.py:307-402)
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .likelihood import DeviceProblem
from .optimize import _fisher_scoring
from .ordering import (_nn_groups, knn_query_device, maximin_order, maximin_order_device,
                       ordered_nn_device)

__all__ = ["ScaledVecchiaGP"]


@dataclass
class ScaledVecchiaGP:
    """Gaussian-process emulator with a scaled Vecchia approximation.

    The fields are the reference model's settings, with the same names and
    defaults: how many nearest earlier points condition each point when the
    likelihood is evaluated (``m_est``) and when predicting (``m_pred``); how
    many rows the parameters are estimated on (``n_est``, a random subset when
    the data are larger); the Matern smoothness ``nu`` (a closed form for
    0.5, 1.5 and 2.5, the Bessel form for any other positive value, estimated
    when None); the mean model ``trend`` ('zero', 'constant' or 'linear' in
    the inputs); the relative ``nugget`` (estimated when None, held at the
    given value otherwise); the ``var_penalty`` pulling log sigma^2 towards
    the data's variance; ``var_correction`` (fit the predictive-variance
    factor b on an inner split); ``lambda_max`` (the largest range before an
    input counts as irrelevant); the Fisher-scoring budget ``max_iter`` and
    tolerance ``tol``; the seed of every random draw (``random_state``).

    One setting has no counterpart in the reference: ``precision``, the
    arithmetic of the likelihood blocks in fit and of the prediction blocks:
    "float64" (the reference's) or "split" (block entries assembled in
    float32 from centred coordinates and the correlation deficit, the
    factorisation, solves and sums in float64; ill-conditioned blocks are
    redone in float64).  The likelihood takes the split form for the closed
    forms, for a fixed nu of the library's float32 table (at most 8 and at
    least 1e-3 from an integer) and for an estimated nu whose value and
    value +- 1e-3 are such (at each iterate), the prediction blocks for the
    closed forms; any other nu runs in float64.
    """

    m_est: int = 30
    m_pred: int = 140
    n_est: int = 5000
    nu: float | None = 2.5
    trend: str = "constant"
    nugget: float | None = None
    var_penalty: float = 1.0
    var_correction: bool = True
    lambda_max: float = 1e3
    max_iter: int = 40
    tol: float = 1e-4
    random_state: int | None = 0
    verbose: bool = False
    precision: str = "float64"

    # fitted state -----------------------------------------------------------
    X_: np.ndarray = field(default=None, init=False, repr=False)
    y_: np.ndarray = field(default=None, init=False, repr=False)
    theta_: np.ndarray = field(default=None, init=False, repr=False)
    beta_: np.ndarray = field(default=None, init=False, repr=False)
    b_: float = field(default=1.0, init=False)
    d_: int = field(default=None, init=False, repr=False)
    _estimate_nu: bool = field(default=False, init=False, repr=False)
    _nu_fit: float = field(default=None, init=False, repr=False)
    # (nu, device Matern table) of the last general nu predicted with
    _mtab_cache: tuple = field(default=None, init=False, repr=False, compare=False)

    def _precision(self):
        if self.precision not in ("float64", "split"):
            raise ValueError("precision must be 'float64' or 'split'")
        return self.precision

    # ---------------- basis / scaling helpers ------------------------------
    def _design(self, X):
        if self.trend == "zero":
            return np.zeros((X.shape[0], 0))
        if self.trend == "constant":
            return np.ones((X.shape[0], 1))
        if self.trend == "linear":
            return np.column_stack([np.ones(X.shape[0]), X])
        raise ValueError("trend must be 'zero', 'constant' or 'linear'")

    @property
    def variance_(self):
        return math.exp(self.theta_[0])

    @property
    def ranges_(self):
        return np.exp(self.theta_[1:1 + self.d_])

    @property
    def relevance_(self):
        """1 / lambda_l -- how strongly input l affects the response."""
        return 1.0 / self.ranges_

    @property
    def nu_(self):
        """Matern smoothness used: the fixed ``nu`` or the fitted value."""
        return self._nu_fit

    @property
    def nugget_(self):
        return math.exp(self.theta_[-1])

    def _clip_theta(self, theta, d, estimate_nu):
        hi = math.log(self.lambda_max) if np.isfinite(self.lambda_max) else np.inf
        theta[1:1 + d] = np.clip(theta[1:1 + d], math.log(1e-8), hi)
        if estimate_nu:
            theta[1 + d] = np.clip(theta[1 + d], math.log(0.3), math.log(10.0))
        theta[-1] = np.clip(theta[-1], math.log(1e-12), math.log(1e3))
        return theta

    # ---------------- fitting ----------------------------------------------
    def fit(self, X, y):
        st = self._fit_prepare(X, y)
        d, estimate_nu = st["d"], st["estimate_nu"]
        theta = st["theta0"]
        state = {}

        def rebuild(th):
            order, groups = self._order_and_neighbours(st["Xe"], th, d, st["m"])
            state["order"] = order
            state["groups"] = groups
            state["prob"] = DeviceProblem(st["Xe"][order], st["ye"][order], st["Ze"][order], groups)

        rebuild(theta)
        last_ranges = np.exp(theta[1:1 + d]).copy()

        nev = [0]

        def objective(th):
            nev[0] += 1
            th = self._objective_theta(th, d, estimate_nu)
            ll, g, M, beta = state["prob"].evaluate(
                th, self.nu, estimate_nu=estimate_nu, need_grad=True,
                var_penalty=self.var_penalty, log_var_target=st["log_var_target"],
                precision=self._precision())
            g, M = self._freeze_nugget(g, M)
            return ll, g, M, beta

        def reorder_hook(th, k):
            nonlocal last_ranges
            r = self._reorder_ranges(th, d, estimate_nu, last_ranges, k)
            if r is None:
                return False
            rebuild(th)
            last_ranges = r.copy()
            return True

        theta, ll, beta = _fisher_scoring(
            theta, objective, max_iter=self.max_iter, tol=self.tol,
            verbose=self.verbose, reorder_hook=reorder_hook)
        split = self._precision() != "float64"
        self.fit_stats_ = {"split": nev[0] if split else 0, "float64": 0 if split else nev[0]}
        return self._fit_finish(st, theta, ll, beta)

    # ---------------- pieces of fit shared with the batched fitter ----------
    def _fit_prepare(self, X, y):
        """Standardisation, subsample and initial theta (gp.py:139-177)."""
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=float)
        y = np.asarray(y, dtype=float).ravel()
        n, d = X.shape
        if y.shape[0] != n:
            raise ValueError("X and y have incompatible shapes")

        estimate_nu = self.nu is None
        self._estimate_nu = estimate_nu
        self.d_ = d

        self._lo = X.min(0)
        self._span = np.where(X.max(0) - X.min(0) > 0, X.max(0) - X.min(0), 1.0)
        self._ymu = y.mean()
        self._ysd = y.std() if y.std() > 0 else 1.0

        self.X_ = (X - self._lo) / self._span
        self.y_ = (y - self._ymu) / self._ysd

        rng = np.random.default_rng(self.random_state)
        if self.n_est is not None and n > self.n_est:
            sub = rng.choice(n, self.n_est, replace=False)
        else:
            sub = np.arange(n)
        Xe, ye = self.X_[sub], self.y_[sub]
        Ze = self._design(Xe)
        m = min(self.m_est, len(sub) - 1)

        P0 = d + 2 + (1 if estimate_nu else 0)
        theta = np.empty(P0)
        theta[0] = math.log(max(ye.var(), 1e-8))
        theta[1:1 + d] = math.log(0.2 * math.sqrt(d))
        fixed_nug = self.nugget is not None
        if estimate_nu:
            theta[1 + d] = math.log(1.5)
        theta[-1] = math.log(self.nugget if fixed_nug else 0.1)
        theta = self._clip_theta(theta, d, estimate_nu)
        return {"n": n, "d": d, "estimate_nu": estimate_nu, "rng": rng, "Xe": Xe, "ye": ye,
                "Ze": Ze, "m": m, "theta0": theta,
                "log_var_target": math.log(max(ye.var(), 1e-8))}

    @staticmethod
    def _order_and_neighbours(Xe, th, d, m):
        """Maximin ordering and neighbours in the scaled space (gp.py:182-191);
        the scaled inputs are formed with the reference's own expression so
        the exact searches see the same bits."""
        lib, torch = _lib.device_ready()
        Xs = Xe / np.exp(th[1:1 + d])
        first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
        Xs_dev = _lib.to_dev(torch, Xs, np.float64)
        order_d, info = maximin_order_device(torch, Xs_dev, first)
        nn_d, info2 = ordered_nn_device(torch, Xs_dev[order_d].contiguous(), m)
        order = order_d.cpu().numpy()
        nn = nn_d.cpu().numpy()
        _lib.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
        _lib.check_info(lib, info2.cpu().numpy(), "sv_ordered_knn")
        return order, _nn_groups(nn, m)

    def _objective_theta(self, th, d, estimate_nu):
        """theta as the objective sees it: clipped, nugget held (gp.py:197-199)."""
        th = self._clip_theta(np.array(th, dtype=float), d, estimate_nu)
        if self.nugget is not None:
            th[-1] = math.log(self.nugget)
        return th

    def _freeze_nugget(self, g, M):
        """Fixed nugget: zero its score and decouple its Fisher row (gp.py:206-208)."""
        if g is not None and self.nugget is not None:
            g = g.copy()
            g[-1] = 0.0
            M = M.copy()
            M[-1, :] = 0.0
            M[:, -1] = 0.0
            M[-1, -1] = 1.0
        return g, M

    def _reorder_ranges(self, th, d, estimate_nu, last_ranges, k):
        """Ranges to reorder with, or None when they moved less than 1e-3 in
        log scale since the last ordering (gp.py:211-221)."""
        r = np.exp(self._clip_theta(np.array(th), d, estimate_nu)[1:1 + d])
        if np.max(np.abs(np.log(r / last_ranges))) < 1e-3:
            return None
        if self.verbose:
            print(f"    [reorder at iter {k}] ranges = "
                  + np.array2string(r, precision=3))
        return r

    def _fit_finish(self, st, theta, ll, beta):
        """Fitted attributes and the variance correction (gp.py:227-239)."""
        d, estimate_nu = st["d"], st["estimate_nu"]
        theta = self._clip_theta(np.array(theta), d, estimate_nu)
        if self.nugget is not None:
            theta[-1] = math.log(self.nugget)
        self.theta_ = theta
        self.beta_ = beta
        self.loglik_ = ll
        self._nu_fit = math.exp(theta[1 + d]) if estimate_nu else self.nu

        self.b_ = 1.0
        if self.var_correction and st["n"] >= 200:
            self.b_ = self._estimate_b(st["rng"])
        return self

    # ---------------- prediction -------------------------------------------
    def _pred_theta(self):
        """[log s2, log lambda, log tau] on the device (the nu row dropped)."""
        d = self.d_
        th = np.concatenate([self.theta_[:1 + d], self.theta_[-1:]])
        return th

    def _general(self):
        return self.nu_ not in (0.5, 1.5, 2.5)

    def _matern_table(self):
        """Device Matern table of a general fitted nu (sv_matern_table: the
        table the likelihood interpolates M and g from), built once per nu;
        None for the closed forms and a nu outside the tables' range (K_nu
        per entry)."""
        from .likelihood import matern_table_nu
        nu = float(self.nu_)
        if not self._general() or not matern_table_nu(nu):
            return None
        cache = getattr(self, "_mtab_cache", None)
        if cache is not None and cache[0] == nu:
            return cache[1]
        lib, torch = _lib.device_ready()
        t = torch.empty(int(lib.sv_matern_table_doubles()), dtype=torch.float64, device="cuda")
        _lib.check(lib, lib.sv_matern_table(nu, _lib.ptr(t), t.numel(), _lib.stream_handle(torch)),
                   "sv_matern_table")
        self._mtab_cache = (nu, t)
        return t

    def _predict_scaled(self, Xs_std, X_tr, y_tr_resid, m, noise_free=True):
        """Marginal Vecchia predictions conditioning on the m nearest training
        inputs.  Exact mean and variance of the Vecchia predictive law."""
        lib, torch = _lib.device_ready()
        d = X_tr.shape[1]
        ranges = self.ranges_
        m = min(m, X_tr.shape[0])
        nq = Xs_std.shape[0]
        ntr = X_tr.shape[0]
        Xtr_d = _lib.to_dev(torch, X_tr, np.float64)
        Xq_d = _lib.to_dev(torch, Xs_std, np.float64)
        # neighbours in the scaled space, inputs scaled as gp.py:253-254 does
        nb, info = knn_query_device(torch, _lib.to_dev(torch, X_tr / ranges, np.float64),
                                    _lib.to_dev(torch, Xs_std / ranges, np.float64), m)
        Xall = torch.cat([Xtr_d, Xq_d]).contiguous()
        tgt = torch.arange(ntr, ntr + nq, dtype=torch.int32, device="cuda")
        nbr = nb.to(torch.int32).contiguous()
        resid = _lib.to_dev(torch, y_tr_resid, np.float64)
        mean = torch.empty(nq, dtype=torch.float64, device="cuda")
        var = torch.empty(nq, dtype=torch.float64, device="cuda")
        D = _lib.PredDesc()
        D.nall, D.nobs, D.nblk = ntr + nq, (ntr if noise_free else ntr + nq), nq
        D.d, D.k, D.ldnbr = d, m, m
        D.general, D.nu = int(self._general()), float(self.nu_)
        D.precision = int(self._precision() == "split")
        mtab = self._matern_table()
        D.matern_table = mtab.data_ptr() if mtab is not None else None
        th = _lib.to_dev(torch, self._pred_theta(), np.float64)
        info2 = _lib.new_info(torch)
        rc = lib.sv_predict_blocks(D, _lib.ptr(th), _lib.ptr(Xall), _lib.ptr(tgt), _lib.ptr(nbr),
                                   _lib.ptr(resid), _lib.ptr(mean), _lib.ptr(var), None, None,
                                   _lib.ptr(info2), _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_predict_blocks")
        res = torch.cat([mean, var]).cpu().numpy()
        _lib.check_info(lib, info.cpu().numpy(), "sv_knn_query")
        inf2 = info2.cpu().numpy()
        _lib.check_info(lib, inf2, "sv_predict_blocks")
        self.pred_stats_ = {"blocks": int(nq), "redone_float64": int(inf2[3])}
        return res[:nq], res[nq:]

    def predict(self, Xstar, return_std=False, return_var=False, m=None):
        """Marginal predictive mean (and sd/variance) at new inputs."""
        self._check_fitted()
        Xstar = np.ascontiguousarray(np.atleast_2d(Xstar), dtype=float)
        Xs = (Xstar - self._lo) / self._span
        m = self.m_pred if m is None else m

        Z_tr = self._design(self.X_)
        resid = self.y_ - (Z_tr @ self.beta_ if self.beta_.size else 0.0)
        mu, va = self._predict_scaled(Xs, self.X_, resid, m)
        Zs = self._design(Xs)
        if self.beta_.size:
            mu = mu + Zs @ self.beta_

        mean = self._ymu + self._ysd * mu
        if not (return_std or return_var):
            return mean
        var = (self._ysd ** 2) * self.b_ * va
        if return_var:
            return mean, var
        return mean, np.sqrt(var)

    # ---------------- joint prediction (Sec. 3.3) ---------------------------
    def _joint_factor_device(self, Xs, m):
        """Block columns of the sparse inverse Cholesky factor of the combined
        (observations first) ordering, on the device."""
        lib, torch = _lib.device_ready()
        n, d = self.X_.shape
        ns = Xs.shape[0]
        ranges = self.ranges_
        Xall = np.vstack([self.X_, Xs])
        Xsc = Xall / ranges
        order_obs = maximin_order(Xsc[:n])
        order_pred = maximin_order(Xsc[n:]) + n
        order = np.concatenate([order_obs, order_pred])
        Xo_sc = _lib.to_dev(torch, Xsc[order], np.float64)
        k = min(m, n)
        nn, info = ordered_nn_device(torch, Xo_sc, k, start=n)
        K = k + 1
        nbr = nn[n:, 1:K].to(torch.int32).contiguous()
        Xo = _lib.to_dev(torch, Xall[order], np.float64)
        tgt = torch.arange(n, n + ns, dtype=torch.int32, device="cuda")
        Z_tr = self._design(self.X_)
        resid = self.y_ - (Z_tr @ self.beta_ if self.beta_.size else 0.0)
        resid_d = _lib.to_dev(torch, resid[order_obs], np.float64)
        acol = torch.empty((ns, K), dtype=torch.float64, device="cuda")
        rhs = torch.empty(ns, dtype=torch.float64, device="cuda")
        D = _lib.PredDesc()
        D.nall, D.nobs, D.nblk = n + ns, n, ns
        D.d, D.k, D.ldnbr = d, k, k
        D.general, D.nu = int(self._general()), float(self.nu_)
        D.precision = int(self._precision() == "split")
        mtab = self._matern_table()
        D.matern_table = mtab.data_ptr() if mtab is not None else None
        th = _lib.to_dev(torch, self._pred_theta(), np.float64)
        info2 = _lib.new_info(torch)
        rc = lib.sv_predict_blocks(D, _lib.ptr(th), _lib.ptr(Xo), _lib.ptr(tgt), _lib.ptr(nbr),
                                   _lib.ptr(resid_d), None, None, _lib.ptr(acol), _lib.ptr(rhs),
                                   _lib.ptr(info2), _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_predict_blocks")
        _lib.check_info(lib, info.cpu().numpy(), "sv_ordered_knn")
        _lib.check_info(lib, info2.cpu().numpy(), "sv_predict_blocks")
        perm = order[n:] - n
        return dict(n=n, ns=ns, k=k, nbr=nbr, acol=acol, rhs=rhs, perm=perm,
                    order_obs=order_obs)

    def _joint_factor(self, Xs, m):
        """Sparse inverse-Cholesky columns for the prediction block, as scipy
        sparse matrices (U_op, U_pp, perm, order_obs) like the reference."""
        from scipy import sparse
        F = self._joint_factor_device(Xs, m)
        n, ns, k = F["n"], F["ns"], F["k"]
        K = k + 1
        a = F["acol"].cpu().numpy()
        nb = F["nbr"].cpu().numpy().astype(np.int64)
        rows = np.concatenate([nb, (n + np.arange(ns))[:, None]], axis=1)
        cols = np.repeat(np.arange(ns), K)
        U = sparse.coo_matrix((a.ravel(), (rows.ravel(), cols)), shape=(n + ns, ns)).tocsc()
        return U[:n, :], U[n:, :], F["perm"], F["order_obs"]

    def _joint_solve(self, F, R):
        """Solve U_pp^T X = R (R: (ns, nrhs) device tensor) on the device."""
        lib, torch = _lib.device_ready()
        ns, nrhs = R.shape
        X = torch.empty_like(R)
        info = _lib.new_info(torch)
        ws = _lib.workspace(torch, lib.sv_joint_solve_workspace_bytes(ns))
        rc = lib.sv_joint_solve(ns, F["n"], F["k"], F["k"], _lib.ptr(F["nbr"]), _lib.ptr(F["acol"]),
                                _lib.ptr(R), nrhs, _lib.ptr(X), _lib.ptr(info), _lib.ptr(ws),
                                ws.numel(), _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_joint_solve")
        return X, info

    def _joint_var_diag(self, F, panel_bytes=None):
        """diag((U_pp U_pp^T)^-1) in the elimination ordering (device tensor).
        The panel scratch holds at most a quarter of the free device memory
        (and never more than the whole lower triangle needs)."""
        lib, torch = _lib.device_ready()
        ns = F["ns"]
        if panel_bytes is None:
            free = torch.cuda.mem_get_info()[0]
            panel_bytes = min(8 * ns * ns, max(8 * ns, free // 4))
        panel = _lib.workspace(torch, int(panel_bytes))
        ws = _lib.workspace(torch, lib.sv_joint_solve_workspace_bytes(ns))
        v = torch.empty(ns, dtype=torch.float64, device="cuda")
        info = _lib.new_info(torch)
        rc = lib.sv_joint_var_diag(ns, F["n"], F["k"], F["k"], _lib.ptr(F["nbr"]), _lib.ptr(F["acol"]),
                                   _lib.ptr(v), _lib.ptr(info), _lib.ptr(ws), ws.numel(),
                                   _lib.ptr(panel), panel.numel(), _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_joint_var_diag")
        _lib.check_info(lib, info.cpu().numpy(), "sv_joint_var_diag")
        return v

    def predict_joint(self, Xstar, m=None, n_sim=0, exact_var=False,
                      random_state=None):
        """Joint Vecchia predictive distribution (Sec. 3.3).

        Returns a dict with 'mean', optionally 'var' and 'samples' (n_sim, n*).
        """
        self._check_fitted()
        lib, torch = _lib.device_ready()
        Xstar = np.ascontiguousarray(np.atleast_2d(Xstar), dtype=float)
        Xs = (Xstar - self._lo) / self._span
        m = self.m_pred if m is None else m
        ns = Xs.shape[0]

        F = self._joint_factor_device(Xs, m)
        perm = F["perm"]
        inv = np.empty(ns, dtype=np.int64)
        inv[perm] = np.arange(ns)

        X, info = self._joint_solve(F, F["rhs"].reshape(ns, 1).contiguous())
        mu_ord = X.reshape(-1).cpu().numpy()
        _lib.check_info(lib, info.cpu().numpy(), "sv_joint_solve")
        mu = mu_ord[inv]
        Zs = self._design(Xs)
        if self.beta_.size:
            mu = mu + Zs @ self.beta_
        out = {"mean": self._ymu + self._ysd * mu}

        rng = np.random.default_rng(self.random_state if random_state is None
                                    else random_state)
        if exact_var:
            # diag((U_pp U_pp^T)^-1) = (S**2).sum(1), S = U_pp^-T (gp.py:391-393),
            # from rows of S in column panels, never the whole of S at once
            v = self._joint_var_diag(F).cpu().numpy()[inv]
            out["var"] = (self._ysd ** 2) * self.b_ * v
        if n_sim > 0:
            eps = rng.standard_normal((ns, n_sim))
            E = _lib.to_dev(torch, eps, np.float64)
            dr_d, info = self._joint_solve(F, E)
            dr = dr_d.cpu().numpy()[inv]
            _lib.check_info(lib, info.cpu().numpy(), "sv_joint_solve")
            samples = (mu[:, None] + math.sqrt(self.b_) * dr).T
            out["samples"] = self._ymu + self._ysd * samples
            if "var" not in out:
                out["var"] = out["samples"].var(0, ddof=1)
        return out

    def sample_joint(self, Xstar, n_sim=100, m=None, random_state=None):
        """Draw joint sample paths from the predictive distribution."""
        return self.predict_joint(Xstar, m=m, n_sim=n_sim,
                                  random_state=random_state)["samples"]

    # ---------------- variance correction ----------------------------------
    def _estimate_b(self, rng):
        """Sec. 3.4: b minimising the negative log score on an inner split."""
        n = self.X_.shape[0]
        n_in = min(2000, n // 5)
        idx = rng.permutation(n)
        te, tr = idx[:n_in], idx[n_in:]
        Z_tr = self._design(self.X_[tr])
        resid = self.y_[tr] - (Z_tr @ self.beta_ if self.beta_.size else 0.0)
        mu, va = self._predict_scaled(self.X_[te], self.X_[tr], resid,
                                      min(self.m_pred, len(tr)))
        if self.beta_.size:
            mu = mu + self._design(self.X_[te]) @ self.beta_
        va = np.maximum(va, 1e-300)
        b = float(np.mean((self.y_[te] - mu) ** 2 / va))
        return max(b, 1e-8)

    def _check_fitted(self):
        if self.theta_ is None:
            raise RuntimeError("call .fit(X, y) first")

    def summary(self):
        """A text report of the fitted model: its settings, the Vecchia
        log-likelihood of the standardised responses, the variance, smoothness,
        nugget and variance factor, and each input's relevance 1/lambda."""
        self._check_fitted()
        how = "estimated" if self._estimate_nu else "fixed"
        nu_set = "estimate" if self.nu is None else self.nu
        rows = [
            f"ScaledVecchiaGP  nu={nu_set}  m_est={self.m_est}  m_pred={self.m_pred}  "
            f"trend={self.trend!r}",
            f"  loglik (Vecchia, standardised y)  {self.loglik_:.3f}",
            f"  variance sigma^2                  {self.variance_:.6g}",
            f"  smoothness nu ({how:9s})        {self.nu_:.4g}",
            f"  relative nugget                   {self.nugget_:.6g}",
            f"  variance factor b                 {self.b_:.4g}",
            "  relevance 1/lambda per input (inputs scaled to the unit box):",
        ]
        rows += [f"    x{j:<3d} {r:12.4f}" for j, r in enumerate(self.relevance_)]
        return "\n".join(rows)
