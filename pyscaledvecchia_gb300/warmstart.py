"""Learned warm start for Fisher scoring (no counterpart in the reference).

A DeepSets set encoder (sv_encoder.cu: per-point MLP 16 -> 128 -> 128 with
GELU, mean pool, head 128 -> 128 -> 16; bfloat16 weights, float32
accumulation) reads a 512-point subsample of a fit's standardised
estimation set (x in the unit box, y centred and scaled, as gp.py:151-157
prepares them) and predicts the standardised log-parameters
[log sigma^2, log lambda_1..d, log tau] at which Fisher scoring starts.
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

__all__ = ["SetEncoder", "draw_training_problems", "problem_features", "DEFAULT_WEIGHTS"]

S_POINTS = 512
MAX_D = 12
N_FEAT = 16
N_OUT = 16
TAU_INDEX = 13
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart.npz")


def problem_features(Xstd, ystd, seed=0, S=S_POINTS):
    """(S, 16) float64 features and the number of valid points: a seeded
    subsample of min(n, S) rows, x zero padded to 12 columns, y in column 12."""
    Xstd = np.asarray(Xstd, dtype=np.float64)
    n, d = Xstd.shape
    if d > MAX_D:
        raise ValueError("the encoder takes at most 12 input dimensions")
    c = min(n, S)
    idx = np.sort(np.random.default_rng(seed).choice(n, c, replace=False)) if n > S else np.arange(n)
    f = np.zeros((S, N_FEAT))
    f[:c, :d] = Xstd[idx]
    f[:c, MAX_D] = np.asarray(ystd, dtype=np.float64).reshape(-1)[idx]
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


def draw_training_problems(nprob, seed=0, n=2000, d_range=(3, 12), lam_range=(0.05, 100.0),
                           tau_range=(1e-8, 1e-1), s2_range=(0.1, 10.0), m=30):
    """Problems drawn by the method itself: returns (features (nprob, S, 16),
    counts (nprob,), targets (nprob, 16), weights (nprob, 16), dims (nprob,)).
    y is an unconditional Vecchia draw (Matern 2.5, m neighbours) in the
    exact maximin order of the scaled inputs."""
    lib, torch = _lib.device_ready()
    from .ordering import maximin_order_device, ordered_nn_device
    from .sampling import vecchia_prior_sample_device
    rng = np.random.default_rng(seed)
    feats = np.zeros((nprob, S_POINTS, N_FEAT))
    cnt = np.zeros(nprob, dtype=np.int32)
    tg = np.zeros((nprob, N_OUT))
    wt = np.zeros((nprob, N_OUT))
    dims = np.zeros(nprob, dtype=np.int64)
    for i in range(nprob):
        d = int(rng.integers(d_range[0], d_range[1] + 1))
        X = rng.random((n, d))
        lam = np.exp(rng.uniform(math.log(lam_range[0]), math.log(lam_range[1]), d))
        tau = float(np.exp(rng.uniform(math.log(tau_range[0]), math.log(tau_range[1]))))
        s2 = float(np.exp(rng.uniform(math.log(s2_range[0]), math.log(s2_range[1]))))
        eps = rng.standard_normal(n)
        Xs = X / lam
        first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
        Xs_d = _lib.to_dev(torch, Xs, np.float64)
        order_d, info = maximin_order_device(torch, Xs_d, first)
        nn_d, info2 = ordered_nn_device(torch, Xs_d[order_d].contiguous(), min(m, n - 1))
        order = order_d.cpu().numpy()
        _lib.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
        _lib.check_info(lib, info2.cpu().numpy(), "sv_ordered_knn")
        theta = np.concatenate([[math.log(s2)], np.log(lam), [math.log(tau)]])
        yo = vecchia_prior_sample_device(torch, _lib.to_dev(torch, X[order], np.float64), nn_d,
                                         theta, 2.5, _lib.to_dev(torch, eps.reshape(n, 1), np.float64))
        y = np.empty(n)
        y[order] = yo.reshape(-1).cpu().numpy()
        Xstd, ystd, span, ysd = standardise(X, y)
        th_std = np.concatenate([[math.log(s2) - 2.0 * math.log(ysd)], np.log(lam / span), [math.log(tau)]])
        feats[i], cnt[i] = problem_features(Xstd, ystd, seed=i)
        tg[i], wt[i] = targets_of(th_std, d)
        dims[i] = d
    return feats, cnt, tg, wt, dims


def init_params(seed=0):
    """Float32 parameters: He-normal weights, zero hidden biases, output bias
    at the centre of the training priors (log lambda ~ 0.8, log tau ~ -10.4)."""
    from_rng = np.random.default_rng(seed)
    H = 128
    parts = [
        from_rng.standard_normal((H, N_FEAT)) * math.sqrt(2.0 / 14.0), np.zeros(H),
        from_rng.standard_normal((H, H)) * math.sqrt(2.0 / H), np.zeros(H),
        from_rng.standard_normal((H, H)) * math.sqrt(2.0 / H), np.zeros(H),
        from_rng.standard_normal((N_OUT, H)) * math.sqrt(1.0 / H) * 0.1,
    ]
    b4 = np.zeros(N_OUT)
    b4[1:1 + MAX_D] = 0.5 * (math.log(0.05) + math.log(100.0))
    b4[TAU_INDEX] = 0.5 * (math.log(1e-8) + math.log(1e-1))
    parts.append(b4)
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


class SetEncoder:
    """Device-resident encoder parameters and the calls around them."""

    def __init__(self, params=None, seed=0):
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

    # ---------------------------------------------------------------- io
    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        z = np.load(path)
        return cls(params=z["params"])

    def save(self, path, **extra):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, params=self.p.cpu().numpy(), **extra)

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
        tg_d = _lib.to_dev(torch, np.asarray(targets, dtype=np.float32), np.float32)
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
        out = self.forward(feats, cnt)
        for j, i in enumerate(ok):
            d = estimation_sets[i][0].shape[1]
            th = np.concatenate([[out[j, 0]], out[j, 1:1 + d], [out[j, TAU_INDEX]]])
            if np.all(np.isfinite(th)):
                res[i] = th
        return res


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
    ap.add_argument("--infer", type=int, default=0,
                    help="only run the inference forward (tcgen05) on this many random sets "
                         "with the saved weights, timed, and exit")
    a = ap.parse_args(argv)
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
    feats, cnt, tg, wt, dims = draw_training_problems(a.problems, seed=a.seed, n=a.n)
    t_draw = time.time() - t0
    enc = SetEncoder(seed=a.seed)
    t0 = time.time()
    hist = enc.train(feats, cnt, tg, wt, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed,
                     log=print)
    t_train = time.time() - t0
    enc.save(a.out, loss=np.array(hist), problems=a.problems, n=a.n, epochs=a.epochs,
             draw_s=t_draw, train_s=t_train)
    print(f"drew {a.problems} problems in {t_draw:.1f}s, trained {a.epochs} epochs in {t_train:.1f}s")


if __name__ == "__main__":
    main()
