"""Warm-start set encoder (sv_encoder.cu, warmstart.py) against its CPU
oracle (oracle/encoder.py).

CPU: the oracle's chain rule against central differences of its own exact
(unrounded) network, and the bfloat16 rounding against hand-made values.
GPU: forward outputs, loss, every gradient block and an Adam step of the
kernels against the oracle on the same bfloat16 inputs and weights; ragged
sets (points not a multiple of the tile); training lowers the loss; and
with the shipped weights, fits started from the encoder's prediction need
fewer Fisher-scoring evaluations than the default start.
"""
import math
import os

import numpy as np
import pytest


def _setup(nset=5, S=256, seed=0):
    from oracle import encoder as E
    rng = np.random.default_rng(seed)
    p = np.concatenate([rng.standard_normal(int(np.prod(shp))) * (0.3 if name[0] == "W" else 0.1)
                        for name, shp in E.LAYOUT]).astype(np.float32)
    cnt = rng.integers(S // 3, S + 1, nset).astype(np.int32)
    cnt[0] = S
    cnt[-1] = min(S, 129)  # one point into the second tile (S > 128)
    f = np.zeros((nset, S, 32))
    for b in range(nset):
        d = int(rng.integers(3, 13))
        f[b, :cnt[b], :d] = rng.random((cnt[b], d))
        f[b, :cnt[b], 12] = rng.standard_normal(cnt[b])
        f[b, :cnt[b], 13] = rng.random(cnt[b]) * 0.3          # neighbour distance
        f[b, :cnt[b], 14] = rng.standard_normal(cnt[b]) * 0.5  # y difference
        f[b, :cnt[b], 15] = f[b, :cnt[b], 14] ** 2
        f[b, :cnt[b], 16:16 + d] = rng.random((cnt[b], d)) * 0.2
    tgt = rng.standard_normal((nset, 16)) * 2
    w = (rng.random((nset, 16)) > 0.3).astype(np.float64) / nset
    return E, p, f, cnt, tgt, w


def test_oracle_gradient_matches_finite_differences():
    E, p, f, cnt, tgt, w = _setup(nset=3, S=128, seed=1)
    x = f  # exact network: no rounding anywhere
    p64 = p.astype(np.float64)
    loss, _, g = E.loss_and_grad(p64, x, cnt, tgt, w, rounding=False)
    rng = np.random.default_rng(2)
    for _ in range(6):
        v = rng.standard_normal(p64.shape[0])
        h = 1e-6
        lp = E.loss_and_grad(p64 + h * v, x, cnt, tgt, w, rounding=False)[0]
        lm = E.loss_and_grad(p64 - h * v, x, cnt, tgt, w, rounding=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g @ v) <= 1e-6 * max(1.0, abs(fd)), (fd, g @ v)


def test_oracle_bf16_rounding():
    """bfloat16 keeps 7 fraction bits: one ulp at 1.0 is 2^-7."""
    from oracle import encoder as E
    u = 2.0 ** -8
    vals = np.array([1.0, 1 + u, 1 + 3 * u, 1 + u + u / 16, 1 + u - u / 16, -3.14159265, 65504.0],
                    dtype=np.float32)
    want = [1.0, 1.0, 1 + 4 * u, 1 + 2 * u, 1.0, -3.140625, 65536.0]
    np.testing.assert_array_equal(E.bf16(vals), want)  # ties go to the even neighbour


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["mma_sync", "tcgen05"])
def test_forward_matches_oracle(variant):
    from pyscaledvecchia_gb300.warmstart import SetEncoder
    E, p, f, cnt, tgt, w = _setup()
    enc = SetEncoder(params=p)
    out = enc.forward(f, cnt, variant=variant)
    ref = E.forward(p, E.pack(f), cnt)
    assert _rel(out, ref) < 1e-4
    np.testing.assert_allclose(out, ref, rtol=2e-3, atol=2e-3)


@pytest.mark.gpu
def test_tcgen05_and_mma_sync_forwards_agree():
    """Same bfloat16 operands, float32 accumulation in both: agreement to
    float32 rounding (plus the odd h1 rounding flip)."""
    from pyscaledvecchia_gb300.warmstart import SetEncoder
    E, p, f, cnt, tgt, w = _setup(nset=7, S=512, seed=9)
    enc = SetEncoder(params=p)
    a = enc.forward(f, cnt, variant="tcgen05")
    b = enc.forward(f, cnt, variant="mma_sync")
    assert _rel(a, b) < 2e-5


@pytest.mark.gpu
def test_loss_and_gradient_match_oracle():
    from pyscaledvecchia_gb300.warmstart import SetEncoder
    E, p, f, cnt, tgt, w = _setup(seed=3)
    enc = SetEncoder(params=p)
    loss, out, g = enc.loss_grad(f, cnt, tgt, w)
    rl, rout, rg = E.loss_and_grad(p, E.pack(f), cnt, tgt, w)
    assert abs(loss - rl) <= 1e-4 * abs(rl)
    o = 0
    for name, shp in E.LAYOUT:
        n = int(np.prod(shp))
        gb, rb = g[o:o + n], rg[o:o + n]
        assert _rel(gb, rb) < 3e-3, (name, _rel(gb, rb))
        assert gb @ rb / (np.linalg.norm(gb) * np.linalg.norm(rb)) > 0.99999, name
        o += n


@pytest.mark.gpu
def test_adam_step_matches_oracle():
    from pyscaledvecchia_gb300.warmstart import SetEncoder
    E, p, f, cnt, tgt, w = _setup(seed=4)
    enc = SetEncoder(params=p)
    _, _, g = enc.loss_grad(f, cnt, tgt, w)
    import torch
    gd = torch.from_numpy(g.astype(np.float32)).to("cuda")
    enc.adam_step(gd, 1e-3, weight_decay=1e-4)
    enc.adam_step(gd, 1e-3, weight_decay=1e-4)
    pr, m, v = p.astype(np.float64), np.zeros(p.shape[0]), np.zeros(p.shape[0])
    for step in (1, 2):
        pr, m, v = E.adam(pr, g.astype(np.float64), m, v, 1e-3, 0.9, 0.999, 1e-8, step, 1e-4)
    np.testing.assert_allclose(enc.params(), pr, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_training_fits_a_small_set():
    """The kernels' gradient and Adam drive the training loss of a small
    set of problems drawn by the method well down (what generalises is the
    held-out warm-start test's business)."""
    from pyscaledvecchia_gb300.warmstart import SetEncoder, draw_training_problems
    feats, cnt, tg, wt, dims = draw_training_problems(64, seed=11, n=600)
    enc = SetEncoder(seed=1)
    hist = enc.train(feats, cnt, tg, wt, epochs=80, batch=16, lr=3e-3, lr_final=3e-4)
    assert hist[-1] < 0.8 * hist[0], hist


def _heldout(nprob, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nprob):
        d = int(rng.integers(3, 9))
        n = 1000
        X = rng.random((n, d))
        lam = np.exp(rng.uniform(math.log(0.05), math.log(100.0), d))
        out.append((X, lam, float(np.exp(rng.uniform(math.log(1e-6), math.log(1e-2)))), d, rng))
    return out


@pytest.mark.gpu
def test_warm_start_gain_on_heldout_problems():
    """Shipped weights (trained on the fitted parameters of 50,000 problems
    drawn by the method), held-out problems drawn the same way: the
    encoder's start lies much closer to where Fisher scoring converges than
    the default start and the fits need fewer objective evaluations; the
    judged form (both starts, the better converged loglik kept) is never
    worse than the default start."""
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    from pyscaledvecchia_gb300.fit_batched import fit_batched
    from pyscaledvecchia_gb300.warmstart import DEFAULT_WEIGHTS, SetEncoder
    assert os.path.exists(DEFAULT_WEIGHTS), "trained encoder weights are missing"
    enc = SetEncoder.load()
    import torch
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device, ordered_nn_device
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample_device
    _lib.device_ready()
    Xs, ys = [], []
    for X, lam, tau, d, rng in _heldout(32, 12345):
        n = X.shape[0]
        Xs_ = X / lam
        first = int(np.argmin(((Xs_ - Xs_.mean(0)) ** 2).sum(1)))
        xd = _lib.to_dev(torch, Xs_, np.float64)
        od, _ = maximin_order_device(torch, xd, first)
        nd, _ = ordered_nn_device(torch, xd[od].contiguous(), 30)
        o = od.cpu().numpy()
        th = np.concatenate([[0.0], np.log(lam), [math.log(tau)]])
        yo = vecchia_prior_sample_device(torch, _lib.to_dev(torch, X[o], np.float64), nd, th, 2.5,
                                         _lib.to_dev(torch, rng.standard_normal((n, 1)), np.float64))
        y = np.empty(n)
        y[o] = yo.reshape(-1).cpu().numpy()
        Xs.append(X)
        ys.append(y)

    def models():
        return [ScaledVecchiaGP(n_est=None, var_correction=False) for _ in Xs]

    base = fit_batched(models(), Xs, ys, precision="float64")
    warm = fit_batched(models(), Xs, ys, precision="float64", warm_start=enc)
    # starting points: the default theta0 and the encoder's (clipped as fit does)
    d0, dw = [], []
    for X, y, b in zip(Xs, ys, base):
        g = ScaledVecchiaGP(n_est=None, var_correction=False)
        st = g._fit_prepare(X, y)
        th_w = enc.initial_thetas([(st["Xe"], st["ye"])])[0]
        t0w = g._clip_theta(np.concatenate([th_w[:1 + st["d"]], th_w[-1:]]), st["d"], False)
        d0.append(np.sum((st["theta0"] - b.theta_) ** 2))
        dw.append(np.sum((t0w - b.theta_) ** 2))
    d0, dw = np.array(d0), np.array(dw)
    eb = np.array([g.fit_stats_["float64"] for g in base])
    ew = np.array([g.fit_stats_["float64"] for g in warm])
    print(f"start-to-optimum distance^2: default {d0.mean():.2f}, encoder {dw.mean():.2f}; "
          f"objective evaluations: default {eb.mean():.2f}, encoder {ew.mean():.2f}")
    # measured with the shipped weights (32 problems): distance^2 136.8 -> 51.2,
    # evaluations 24.5 -> 22.3
    assert dw.mean() < 0.5 * d0.mean(), (dw.mean(), d0.mean())
    assert ew.mean() < 0.95 * eb.mean(), (ew.mean(), eb.mean())
    # Fisher scoring with reorders at the iterates is path dependent: another
    # start can end on another ordering and another local optimum (measured:
    # better in about half of the problems, worse in the other half), which
    # is what warm_start="judged" is for
    dll = np.array([w.loglik_ - b.loglik_ for w, b in zip(warm, base)])
    print(f"warm - default loglik: median {np.median(dll):.3g}, better in {np.mean(dll > 1e-6):.2f}, "
          f"worse in {np.mean(dll < -1e-6):.2f}")
    judged = fit_batched(models(), Xs, ys, precision="float64", warm_start=enc, warm_judge=True)
    for j, b, w in zip(judged, base, warm):
        assert j.loglik_ == max(b.loglik_, w.loglik_)
