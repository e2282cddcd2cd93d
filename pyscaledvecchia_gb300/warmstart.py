"""Learned warm start for Fisher scoring (no counterpart in the reference).

A DeepSets set encoder (sv_encoder.cu: per-point MLP 32 -> 128 -> 128 with
GELU, mean pool, head 128 -> 128 -> 16; bfloat16 weights, float32
accumulation) reads a 512-point subsample of a fit's standardised
estimation set (x in the unit box, y centred and scaled, as gp.py:151-157
prepares them) and predicts the standardised log-parameters
[log sigma^2, log lambda_1..d, log tau] at which Fisher scoring starts.
Per point it sees x (zero padded to 12 columns) and y, and for the point's
nearest neighbour in the whole estimation set the distance, the difference
of y and its square and the 12 coordinate gaps |dx_l|: with x and y alone
mean pooling sees only first-order moments, which barely identify the nugget
or the per-dimension ranges (trained on 50,000 problems, such an encoder
stayed within 14 % of the loss of predicting the prior means and saved no
Fisher-scoring evaluations); differences between near neighbours carry both.
Only the starting point of gp.py:169-177 moves: the iteration, its stopping
rule and the converged likelihood are unchanged, and the default start
stays the fallback (no encoder, d > 12, or a non-finite prediction).

Training data are problems the method draws itself: X uniform in [0,1]^d,
y a Vecchia draw (the unconditional sample_joint prior) with Matern 2.5 and
known parameters; the targets are those parameters expressed in the
standardised frame the fit works in (lambda / span of each column,
sigma^2 / var(y), tau unchanged).  Forward, backward and Adam run in the
library's kernels.
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import _lib

__all__ = ["SetEncoder", "draw_training_problems", "draw_problems", "problem_features",
           "evaluate_warm_start", "DEFAULT_WEIGHTS"]

S_POINTS = 512
MAX_D = 12
N_FEAT = 32
N_OUT = 16
TAU_INDEX = 13
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart.npz")


def _subsample(n, seed, S=S_POINTS):
    c = min(n, S)
    return np.sort(np.random.default_rng(seed).choice(n, c, replace=False)) if n > S else np.arange(n)


def problem_features(Xstd, ystd, seed=0, S=S_POINTS, X_dev=None):
    """(S, 32) float64 features and the number of valid points of one set: a
    seeded subsample of min(n, S) rows; columns 0..11 x (zero padded), 12 y,
    13 the distance to the row's nearest neighbour among all n rows, 14 the y
    difference to it, 15 its square, 16..27 the coordinate gaps |dx_l|, and
    28..30 the same distance, difference and square for the second nearest
    neighbour.  The neighbour search runs on the device (sv_knn_query)."""
    from .ordering import knn_query_device
    lib, torch = _lib.device_ready()
    Xstd = np.ascontiguousarray(Xstd, dtype=np.float64)
    ystd = np.asarray(ystd, dtype=np.float64).reshape(-1)
    n, d = Xstd.shape
    if d > MAX_D:
        raise ValueError("the encoder takes at most 12 input dimensions")
    idx = _subsample(n, seed, S)
    c = idx.shape[0]
    f = np.zeros((S, N_FEAT))
    f[:c, :d] = Xstd[idx]
    f[:c, MAX_D] = ystd[idx]
    if n > 1:
        Xd = X_dev if X_dev is not None else _lib.to_dev(torch, Xstd, np.float64)
        kq = min(3, n)
        nb, info = knn_query_device(torch, Xd, _lib.to_dev(torch, Xstd[idx], np.float64), kq)
        nb = nb.cpu().numpy()
        _lib.check_info(lib, info.cpu().numpy(), "sv_knn_query")
        # drop the row itself (ties at distance 0 may put it second)
        own = nb == idx[:, None]
        first = np.where(own[:, 0], nb[:, 1], nb[:, 0])
        dx = Xstd[first] - Xstd[idx]
        dy = ystd[first] - ystd[idx]
        f[:c, 13] = np.sqrt((dx * dx).sum(1))
        f[:c, 14] = dy
        f[:c, 15] = dy * dy
        f[:c, 16:16 + d] = np.abs(dx)
        if kq == 3:
            second = np.where(own[:, 0] | own[:, 1], nb[:, 2], nb[:, 1])
            dx2 = Xstd[second] - Xstd[idx]
            dy2 = ystd[second] - ystd[idx]
            f[:c, 28] = np.sqrt((dx2 * dx2).sum(1))
            f[:c, 29] = dy2
            f[:c, 30] = dy2 * dy2
    return f, c


def targets_of(theta_std, d):
    """Target vector and loss weights of a problem with standardised
    log-parameters theta_std = [log s2, log lambda_1..d, log tau]."""
    t = np.zeros(N_OUT)
    w = np.zeros(N_OUT)
    t[0] = theta_std[0]
    t[1:1 + d] = theta_std[1:1 + d]
    t[TAU_INDEX] = theta_std[-1]
    w[0] = 1.0
    w[1:1 + d] = 1.0
    w[TAU_INDEX] = 1.0
    return t, w


def standardise(X, y):
    """gp.py:151-157: unit-box inputs, centred and scaled responses."""
    lo = X.min(0)
    span = np.where(X.max(0) - X.min(0) > 0, X.max(0) - X.min(0), 1.0)
    ysd = y.std() if y.std() > 0 else 1.0
    return (X - lo) / span, (y - y.mean()) / ysd, span, ysd


def _draw_specs(rng, B, n, d_range, lam_range, tau_range, s2_range):
    """B problem specifications (d, X, lambda, tau, sigma^2, eps, eps2)."""
    spec = []
    for _ in range(B):
        d = int(rng.integers(d_range[0], d_range[1] + 1))
        X = rng.random((n, d))
        lam = np.exp(rng.uniform(math.log(lam_range[0]), math.log(lam_range[1]), d))
        tau = float(np.exp(rng.uniform(math.log(tau_range[0]), math.log(tau_range[1]))))
        s2 = float(np.exp(rng.uniform(math.log(s2_range[0]), math.log(s2_range[1]))))
        spec.append((d, X, lam, tau, s2, rng.standard_normal(n), rng.standard_normal(n)))
    return spec


def _draw_responses(spec, n, m):
    """y of every specified problem: one batched device reorder orders them
    all, one prior draw draws them all (see draw_training_problems)."""
    lib, torch = _lib.device_ready()
    from .batched import BatchedLikelihood, BatchProblem, ordered_groups
    from .sampling import vecchia_prior_sample_device
    B = len(spec)
    tau0 = 1e-8
    mm = min(m, n - 1)
    BL = BatchedLikelihood([BatchProblem(sp[1], np.zeros(n), None, ordered_groups(n, mm))
                            for sp in spec], need_grad=False, chunked=False)
    BL.set_sources([sp[1] for sp in spec], [np.zeros(n)] * B, [None] * B, [mm] * B)
    orders = BL.reorder(list(range(B)),
                        [np.concatenate([[0.0], np.log(sp[2]), [math.log(sp[3])]]) for sp in spec],
                        return_orders=True)
    Xall = BL.X.cpu().numpy()
    nbr = BL.nbr.cpu().numpy().astype(np.int64)
    N = B * n
    Xs = np.zeros((N, MAX_D))
    nn = np.full((N, mm + 1), -1, dtype=np.int64)
    for p, sp in enumerate(spec):
        d, lam = sp[0], sp[2]
        xo = int(BL.x_off[p])
        Xs[p * n:(p + 1) * n, :d] = Xall[xo:xo + n * d].reshape(n, d) / lam
        o = int(BL.blk_off[p])
        loc = nbr[o:o + n, :mm]
        nn[p * n:(p + 1) * n, 0] = np.arange(p * n, (p + 1) * n)
        nn[p * n:(p + 1) * n, 1:] = np.where(loc >= 0, loc + p * n, -1)
    eps = np.concatenate([sp[5] for sp in spec]).reshape(N, 1)
    th = np.concatenate([[0.0], np.zeros(MAX_D), [math.log(tau0)]])
    f = vecchia_prior_sample_device(torch, _lib.to_dev(torch, Xs, np.float64),
                                    _lib.to_dev(torch, nn, np.int64), th, 2.5,
                                    _lib.to_dev(torch, eps, np.float64)).reshape(-1).cpu().numpy()
    ys = []
    for p, sp in enumerate(spec):
        d, X, lam, tau, s2, _, e2 = sp
        yo = math.sqrt(s2) * (f[p * n:(p + 1) * n] + math.sqrt(max(tau - tau0, 0.0)) * e2)
        y = np.empty(n)
        y[orders[p]] = yo
        ys.append(y)
    return ys


def draw_problems(nprob, seed=0, n=2000, d_range=(3, 12), lam_range=(0.05, 100.0),
                  tau_range=(1e-8, 1e-1), s2_range=(0.1, 10.0), m=30, chunk=512):
    """(Xs, ys) of nprob problems drawn as draw_training_problems draws them
    (the held-out problems of the warm-start evaluation)."""
    rng = np.random.default_rng(seed)
    Xs, ys = [], []
    for c0 in range(0, nprob, chunk):
        spec = _draw_specs(rng, min(chunk, nprob - c0), n, d_range, lam_range, tau_range, s2_range)
        ys += _draw_responses(spec, n, m)
        Xs += [sp[1] for sp in spec]
    return Xs, ys


def draw_training_problems(nprob, seed=0, n=2000, d_range=(3, 12), lam_range=(0.05, 100.0),
                           tau_range=(1e-8, 1e-1), s2_range=(0.1, 10.0), m=30, chunk=512,
                           fit_targets=False):
    """Problems drawn by the method itself: returns (features (nprob, S, 32),
    counts (nprob,), targets (nprob, 16), weights (nprob, 16), dims (nprob,)).

    y is a Vecchia prior draw (Matern 2.5, m neighbours) in the exact maximin
    order of the scaled inputs.  Chunks of problems are ordered by one
    batched device reorder; one draw then serves the whole chunk: every
    problem's rows are pre-scaled by its own lambda (zero padded to 12
    columns) so all share lambda = 1, the draw uses sigma^2 = 1 and
    tau0 = 1e-8, and each problem's own nugget enters as independent noise
    (sigma^2 (M + tau0 I) + sigma^2 (tau - tau0) I = sigma^2 (M + tau I)).

    fit_targets: the targets are the fitted parameters instead of the
    generating ones -- each chunk is fitted with fit_batched (split
    precision with float64 polish, nugget estimated, nu = 2.5, n_est = None),
    so the encoder learns where Fisher scoring ends, clipped ranges of
    irrelevant inputs included."""
    _lib.device_ready()
    rng = np.random.default_rng(seed)
    feats = np.zeros((nprob, S_POINTS, N_FEAT))
    cnt = np.zeros(nprob, dtype=np.int32)
    tg = np.zeros((nprob, N_OUT))
    wt = np.zeros((nprob, N_OUT))
    dims = np.zeros(nprob, dtype=np.int64)
    for c0 in range(0, nprob, chunk):
        B = min(chunk, nprob - c0)
        spec = _draw_specs(rng, B, n, d_range, lam_range, tau_range, s2_range)
        ys = _draw_responses(spec, n, m)
        fitted = None
        if fit_targets:
            from .fit_batched import fit_batched
            from .gp import ScaledVecchiaGP
            models = [ScaledVecchiaGP(m_est=m, n_est=None, nu=2.5, var_correction=False) for _ in spec]
            fitted = fit_batched(models, [sp[1] for sp in spec], ys, precision="split")
        for p, sp in enumerate(spec):
            d, X, lam, tau, s2, _, e2 = sp
            Xstd, ystd, span, ysd = standardise(X, ys[p])
            if fitted is not None:
                th_std = np.asarray(fitted[p].theta_, dtype=np.float64)
            else:
                th_std = np.concatenate([[math.log(s2) - 2.0 * math.log(ysd)], np.log(lam / span),
                                         [math.log(tau)]])
            i = c0 + p
            feats[i], cnt[i] = problem_features(Xstd, ystd, seed=i)
            tg[i], wt[i] = targets_of(th_std, d)
            dims[i] = d
    return feats, cnt, tg, wt, dims


def init_params(seed=0):
    """Float32 parameters: He-normal weights, zero biases (the targets are
    normalised, so zero is their training mean)."""
    from_rng = np.random.default_rng(seed)
    H = 128
    parts = [
        from_rng.standard_normal((H, N_FEAT)) * math.sqrt(2.0 / N_FEAT), np.zeros(H),
        from_rng.standard_normal((H, H)) * math.sqrt(2.0 / H), np.zeros(H),
        from_rng.standard_normal((H, H)) * math.sqrt(2.0 / H), np.zeros(H),
        from_rng.standard_normal((N_OUT, H)) * math.sqrt(1.0 / H) * 0.1,
    ]
    parts.append(np.zeros(N_OUT))  # targets are normalised: zero mean
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


class SetEncoder:
    """Device-resident encoder parameters and the calls around them.

    The network predicts normalised targets: output o is (t_o - mu_o) / sd_o
    with mu, sd taken from the training set and kept with the weights."""

    def __init__(self, params=None, seed=0, t_mu=None, t_sd=None):
        lib, torch = _lib.device_ready()
        self.lib, self.torch = lib, torch
        self.nparam = int(lib.sv_encoder_param_count())
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32).reshape(-1)
        if p.shape[0] != self.nparam:
            raise ValueError("parameter vector has the wrong length")
        self.p = torch.from_numpy(p.copy()).to("cuda")
        self.pb = torch.empty(self.nparam, dtype=torch.int16, device="cuda")
        self._st = _lib.stream_handle(torch)
        _lib.check(lib, lib.sv_encoder_to_bf16(_lib.ptr(self.p), _lib.ptr(self.pb), self.nparam, self._st),
                   "sv_encoder_to_bf16")
        self._ws = None
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.step = 0
        self.t_mu = np.zeros(N_OUT) if t_mu is None else np.asarray(t_mu, dtype=np.float64)
        self.t_sd = np.ones(N_OUT) if t_sd is None else np.asarray(t_sd, dtype=np.float64)

    # ---------------------------------------------------------------- io
    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        z = np.load(path)
        return cls(params=z["params"], t_mu=z["t_mu"] if "t_mu" in z.files else None,
                   t_sd=z["t_sd"] if "t_sd" in z.files else None)

    def save(self, path, **extra):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, params=self.p.cpu().numpy(), t_mu=self.t_mu, t_sd=self.t_sd, **extra)

    def set_target_scaling(self, targets, weights):
        """mu, sd of every output over the training sets that use it."""
        w = np.asarray(weights) > 0
        t = np.asarray(targets, dtype=np.float64)
        for o in range(N_OUT):
            if w[:, o].any():
                self.t_mu[o] = t[w[:, o], o].mean()
                self.t_sd[o] = max(t[w[:, o], o].std(), 1e-3)

    def params(self):
        return self.p.cpu().numpy()

    # ---------------------------------------------------------------- device
    def pack(self, feats):
        """(nset, S, 16) float64 host features -> bfloat16 device tensor."""
        torch = self.torch
        f = _lib.to_dev(torch, np.ascontiguousarray(feats, dtype=np.float64), np.float64)
        x = torch.empty(f.numel(), dtype=torch.int16, device="cuda")
        _lib.check(self.lib, self.lib.sv_encoder_pack(_lib.ptr(f), f.numel(), _lib.ptr(x), self._st),
                   "sv_encoder_pack")
        return x

    def _workspace(self, nset, S, train):
        nb = int(self.lib.sv_encoder_workspace_bytes(nset, S, int(train)))
        if nb == 0:
            raise ValueError("invalid encoder batch shape")
        if self._ws is None or self._ws.numel() < nb:
            self._ws = _lib.workspace(self.torch, nb)
        return self._ws

    def forward_dev(self, x, cnt_d, nset, S=S_POINTS, variant="tcgen05"):
        torch = self.torch
        out = torch.empty((nset, N_OUT), dtype=torch.float32, device="cuda")
        ws = self._workspace(nset, S, False)
        v = {"tcgen05": 0, "mma_sync": 1}[variant]
        rc = self.lib.sv_encoder_forward(nset, S, _lib.ptr(x), _lib.ptr(cnt_d), _lib.ptr(self.p),
                                         _lib.ptr(self.pb), _lib.ptr(out), v, _lib.ptr(ws), ws.numel(),
                                         self._st)
        _lib.check(self.lib, rc, "sv_encoder_forward")
        return out

    def forward(self, feats, cnt, variant="tcgen05"):
        """Encoder outputs (nset, 16) for host features; variant "tcgen05"
        (inference kernels) or "mma_sync" (the training forward)."""
        x = self.pack(feats)
        cnt_d = _lib.to_dev(self.torch, np.asarray(cnt, dtype=np.int32), np.int32)
        return self.forward_dev(x, cnt_d, feats.shape[0], feats.shape[1],
                                variant).cpu().numpy().astype(np.float64)

    def predict(self, feats, cnt, variant="tcgen05"):
        """Targets in log-parameter units: the normalised outputs scaled back."""
        return self.forward(feats, cnt, variant) * self.t_sd + self.t_mu

    def loss_grad_dev(self, x, cnt_d, tgt_d, wts_d, nset, S=S_POINTS):
        torch = self.torch
        out = torch.empty((nset, N_OUT), dtype=torch.float32, device="cuda")
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        grad = torch.empty(self.nparam, dtype=torch.float32, device="cuda")
        ws = self._workspace(nset, S, True)
        rc = self.lib.sv_encoder_backward(nset, S, _lib.ptr(x), _lib.ptr(cnt_d), _lib.ptr(self.p),
                                          _lib.ptr(self.pb), _lib.ptr(tgt_d), _lib.ptr(wts_d),
                                          _lib.ptr(out), _lib.ptr(loss), _lib.ptr(grad), _lib.ptr(ws),
                                          ws.numel(), self._st)
        _lib.check(self.lib, rc, "sv_encoder_backward")
        return loss, out, grad

    def loss_grad(self, feats, cnt, targets, weights):
        t = self.torch
        x = self.pack(feats)
        cnt_d = _lib.to_dev(t, np.asarray(cnt, dtype=np.int32), np.int32)
        tg = _lib.to_dev(t, np.asarray(targets, dtype=np.float32), np.float32)
        wt = _lib.to_dev(t, np.asarray(weights, dtype=np.float32), np.float32)
        loss, out, grad = self.loss_grad_dev(x, cnt_d, tg, wt, feats.shape[0], feats.shape[1])
        return float(loss.item()), out.cpu().numpy(), grad.cpu().numpy()

    def adam_step(self, grad, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step += 1
        rc = self.lib.sv_encoder_adam(_lib.ptr(self.p), _lib.ptr(grad), _lib.ptr(self.m), _lib.ptr(self.v),
                                      _lib.ptr(self.pb), self.nparam, lr, beta1, beta2, eps, self.step,
                                      weight_decay, self._st)
        _lib.check(self.lib, rc, "sv_encoder_adam")

    def train(self, feats, cnt, targets, weights, epochs=30, batch=256, lr=1e-3, seed=0,
              lr_final=1e-5, log=None):
        """Mini-batch Adam with a cosine learning-rate schedule; the whole
        training set stays on the device.  Returns the per-epoch mean loss."""
        torch = self.torch
        N = feats.shape[0]
        x = self.pack(feats).reshape(N, -1)
        cnt_d = _lib.to_dev(torch, np.asarray(cnt, dtype=np.int32), np.int32)
        w = np.asarray(weights, dtype=np.float64)
        wn = w / np.maximum(w.sum(1, keepdims=True), 1.0)  # mean over a set's outputs
        tn = (np.asarray(targets, dtype=np.float64) - self.t_mu) / self.t_sd
        tg_d = _lib.to_dev(torch, tn.astype(np.float32), np.float32)
        # mean over the batch's sets (every batch holds exactly `batch` sets)
        wt_d = _lib.to_dev(torch, (wn / batch).astype(np.float32), np.float32)
        rng = np.random.default_rng(seed)
        nb = max(1, N // batch)
        total = epochs * nb
        hist = []
        it = 0
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(N)).to("cuda")
            acc = 0.0
            for j in range(nb):
                idx = perm[j * batch:(j + 1) * batch]
                bs = batch
                lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / total))
                loss, _, grad = self.loss_grad_dev(x[idx].contiguous(), cnt_d[idx].contiguous(),
                                                   tg_d[idx].contiguous(), wt_d[idx].contiguous(), bs)
                self.adam_step(grad, lr_t)
                acc += float(loss.item())
                it += 1
            hist.append(acc / nb)
            if log:
                log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.5f}")
        return hist

    # ---------------------------------------------------------------- use
    def initial_thetas(self, estimation_sets):
        """Starting log-parameters for fits.  estimation_sets: list of
        (Xe_std, ye_std) as the fit prepares them (gp.py:156-165).  Returns a
        list of [log s2, log lambda_1..d, log tau] arrays, None where the
        encoder does not apply (d > 12) or predicts a non-finite value."""
        ok = [i for i, (X, _) in enumerate(estimation_sets) if X.shape[1] <= MAX_D]
        res = [None] * len(estimation_sets)
        if not ok:
            return res
        feats = np.zeros((len(ok), S_POINTS, N_FEAT))
        cnt = np.zeros(len(ok), dtype=np.int32)
        for j, i in enumerate(ok):
            X, y = estimation_sets[i]
            feats[j], cnt[j] = problem_features(X, y, seed=i)
        out = self.predict(feats, cnt)
        for j, i in enumerate(ok):
            d = estimation_sets[i][0].shape[1]
            th = np.concatenate([[out[j, 0]], out[j, 1:1 + d], [out[j, TAU_INDEX]]])
            if np.all(np.isfinite(th)):
                res[i] = th
        return res


def evaluate_warm_start(enc, nprob=1000, seed=1, n=2000, precisions=("float64", "split"),
                        tol_ll=1e-6):
    """Held-out comparison of the encoder's start with the default start:
    nprob problems drawn as the training problems are (another seed), each
    fitted with fit_batched (nugget estimated, nu = 2.5, n_est = None, no
    variance correction) from the default start, from the encoder's start,
    and in the judged form (both, the larger loglik kept).  Per precision:
    wall time of each form, objective evaluations per fit, and how the warm
    fits' converged loglik compares with the default fits' (within tol_ll,
    better, worse)."""
    import time

    import torch

    from .fit_batched import fit_batched
    from .gp import ScaledVecchiaGP
    t0 = time.time()
    Xs, ys = draw_problems(nprob, seed=seed, n=n)
    out = {"problems": nprob, "n": n, "seed": seed, "draw_s": time.time() - t0}

    def models():
        return [ScaledVecchiaGP(n_est=None, nu=2.5, var_correction=False) for _ in Xs]

    def timed(**kw):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fit_batched(models(), Xs, ys, **kw)
        torch.cuda.synchronize()
        return r, time.perf_counter() - t

    def evals(fits):
        return np.array([g.fit_stats_["split"] + g.fit_stats_["float64"] for g in fits], dtype=float)

    fit_batched(models()[:4], Xs[:4], ys[:4], precision="float64", warm_start=enc)  # warm-up
    for prec in precisions:
        base, tb = timed(precision=prec)
        warm, tw = timed(precision=prec, warm_start=enc)
        judged, tj = timed(precision=prec, warm_start=enc, warm_judge=True)
        dll = np.array([w.loglik_ - b.loglik_ for w, b in zip(warm, base)])
        djl = np.array([j.loglik_ - b.loglik_ for j, b in zip(judged, base)])
        eb, ew = evals(base), evals(warm)
        out[prec] = {
            "default_s": tb, "warm_s": tw, "judged_s": tj,
            "default_fits_per_s": nprob / tb, "warm_fits_per_s": nprob / tw,
            "judged_fits_per_s": nprob / tj,
            "evals_default_mean": float(eb.mean()), "evals_warm_mean": float(ew.mean()),
            "evals_default_median": float(np.median(eb)), "evals_warm_median": float(np.median(ew)),
            "frac_warm_within_tol": float(np.mean(np.abs(dll) < tol_ll)),
            "frac_warm_better": float(np.mean(dll >= tol_ll)),
            "frac_warm_worse": float(np.mean(dll <= -tol_ll)),
            "warm_dll_median": float(np.median(dll)),
            "frac_judged_within_tol": float(np.mean(np.abs(djl) < tol_ll)),
            "frac_judged_better": float(np.mean(djl >= tol_ll)),
            "judged_min_dll": float(djl.min()),
        }
    return out


def main(argv=None):
    """Train the encoder on problems drawn by the method and save it:
    python -m pyscaledvecchia_gb300.warmstart --problems 50000 --out <path>"""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--problems", type=int, default=50000)
    ap.add_argument("--n", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--fit-targets", action="store_true",
                    help="train on the fitted parameters of every drawn problem")
    ap.add_argument("--evaluate", type=int, default=0,
                    help="only compare the saved encoder's start with the default start on this "
                         "many held-out problems (evaluate_warm_start) and exit")
    ap.add_argument("--eval-out", default=None, help="JSON file for the --evaluate results")
    ap.add_argument("--infer", type=int, default=0,
                    help="only run the inference forward (tcgen05) on this many random sets "
                         "with the saved weights, timed, and exit")
    a = ap.parse_args(argv)
    if a.evaluate:
        import json
        res = evaluate_warm_start(SetEncoder.load(a.out), nprob=a.evaluate, seed=a.seed + 1, n=a.n)
        print(json.dumps(res, indent=1))
        if a.eval_out:
            with open(a.eval_out, "w") as fh:
                json.dump(res, fh, indent=1)
        return
    if a.infer:
        import torch
        enc = SetEncoder.load(a.out) if os.path.exists(a.out) else SetEncoder(seed=a.seed)
        rng = np.random.default_rng(a.seed)
        feats = np.zeros((a.infer, S_POINTS, N_FEAT))
        feats[:, :, :MAX_D] = rng.random((a.infer, S_POINTS, MAX_D))
        feats[:, :, MAX_D] = rng.standard_normal((a.infer, S_POINTS))
        x = enc.pack(feats)
        cnt = _lib.to_dev(torch, np.full(a.infer, S_POINTS, dtype=np.int32), np.int32)
        for variant in ("tcgen05", "mma_sync"):
            for _ in range(3):
                enc.forward_dev(x, cnt, a.infer, variant=variant)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                enc.forward_dev(x, cnt, a.infer, variant=variant)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 10
            flops = 2.0 * a.infer * S_POINTS * (N_FEAT * 128 + 128 * 128)
            print(f"{variant}: {a.infer} sets x {S_POINTS} points: {ms:.3f} ms per forward, "
                  f"{flops / ms / 1e9:.1f} TFLOP/s in the per-point layers (incl. head)")
        return
    t0 = time.time()
    feats, cnt, tg, wt, dims = draw_training_problems(a.problems, seed=a.seed, n=a.n,
                                                      fit_targets=a.fit_targets)
    t_draw = time.time() - t0
    # the last 2 % are held out
    nval = max(1, a.problems // 50)
    tr = slice(0, a.problems - nval)
    va = slice(a.problems - nval, a.problems)
    enc = SetEncoder(seed=a.seed)
    enc.set_target_scaling(tg[tr], wt[tr])
    t0 = time.time()
    hist = enc.train(feats[tr], cnt[tr], tg[tr], wt[tr], epochs=a.epochs, batch=a.batch, lr=a.lr,
                     seed=a.seed, lr_final=a.lr * 0.02, log=print)
    t_train = time.time() - t0
    pred = enc.predict(feats[va], cnt[va])
    err = (pred - tg[va]) ** 2
    errp = (enc.t_mu - tg[va]) ** 2
    val = {}
    for name, ix in (("log_s2", [0]), ("log_lambda", list(range(1, 1 + MAX_D))), ("log_tau", [TAU_INDEX])):
        m = wt[va][:, ix] > 0
        val[name] = (float(err[:, ix][m].mean()), float(errp[:, ix][m].mean()))
        print(f"held out {name}: MSE {val[name][0]:.3f} (predicting the training mean: {val[name][1]:.3f})")
    enc.save(a.out, loss=np.array(hist), problems=a.problems, n=a.n, epochs=a.epochs,
             draw_s=t_draw, train_s=t_train,
             val=np.array([[v[0], v[1]] for v in val.values()]))
    print(f"drew {a.problems} problems in {t_draw:.1f}s, trained {a.epochs} epochs in {t_train:.1f}s")


if __name__ == "__main__":
    main()
