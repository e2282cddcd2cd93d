"""Benchmark: scaled Vecchia log-likelihood + score + Fisher evaluation.

Workload (one "step"): the profile log-likelihood, its score and the Fisher
information of a scaled Vecchia model with n = 200,000 points in d = 10,
m = 30 neighbours (K = 31 blocks, P = 12 parameters), Matern nu = 2.5,
sigma^2 = 2, tau = 1e-3, lambda log-uniform in [0.05, 50], X uniform in
[0,1]^10 (seed 1), y an unconditional Vecchia draw y = U^-T eps (computed
on the host with NumPy, the same arrays in both arms); the ordering and
neighbour sets are the exact maximin / kNN of the scaled inputs.  The timed
form is the split form: float32 distances, Matern assembly, dSigma.a and
Fisher / score Gram products, float64 LDL^T, triangular solves,
log-determinant and likelihood sums.  Throughput unit: conditioning blocks
per second (one block per point).  Synthetic data (the reference publishes
no dataset or numbers).

  value : device-resident inputs, one sv_vecchia_loglik per step, CUDA
          events on the launching stream, L2 flushed (256 MB write) between
          steps and excluded from the step time
  e2e   : the public call vecchia_profile_loglik(theta, X, y, Z, groups, nu,
          precision="split") on host NumPy arrays (conditioning-set packing,
          host->device copies, kernels, device->host read of the results)

``--impl reference`` times the reference algorithm's CPU form on the host
cores instead: the C restatement of its Numba loops (oracle/sv_oracle.c,
OpenMP over blocks, every host thread), on the same ordered inputs.

Multi-GPU (torchrun, N > 1): every rank evaluates its own independent
problem (seed 1 + rank), there is no data-path collective; value = all
ranks' blocks / the slowest rank's time (weak scaling).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Vecchia fits/s, chosen vs plain form on GB300 at |dloglik|<1e-6; blocks/s"
# DRAM bytes (read + write) per block of one k_block_split64<16> launch at the
# default size (n = 200,000): an ncu capture of that launch (one pass,
# dram__bytes_read.sum 45.10 MB + dram__bytes_write.sum 132.88 MB) divided by
# its 200,000 blocks
SPLIT64_TRAFFIC_PER_BLOCK = 889.9
# the exact maximin order of the default workload, computed once by the
# oracle (tests/golden/make_c2_order.py)
C2_ORDER = os.path.join(ROOT, "tests", "golden", "c2_order.npz")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=200_000)
    ap.add_argument("--d", type=int, default=10)
    ap.add_argument("--m", type=int, default=30)
    ap.add_argument("--nu", type=float, default=2.5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fits-problems", type=int, default=256,
                    help="problems of the batched-fits workload (0 = skip it)")
    ap.add_argument("--fits-dump", default="",
                    help="write per-problem results of the batched-fits workload to this .npz")
    ap.add_argument("--no-predict", action="store_true", help="skip the prediction workload")
    ap.add_argument("--no-c1", action="store_true", help="skip the n = 2000 fit + predict workload")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the other precision forms and smoothness values of the evaluation")
    ap.add_argument("--kernel-case", default="",
                    choices=["", "pred", "pred64", "tree", "jvar", "nu08", "nu08s"],
                    help="run one small case of a kernel for a profiler capture and exit: "
                         "pred / pred64 (sv_predict_blocks, split / float64, 20,000 blocks of "
                         "141), tree (tree-form maximin, 100,000 rows, d = 10), jvar "
                         "(sv_joint_var_diag, 5,000 points), nu08 / nu08s (the float64 / "
                         "split evaluation at fixed nu = 0.8 with its Matern table, 20,000 "
                         "rows of the benchmark's distribution, three calls)")
    return ap.parse_args()


def kernel_case(name):
    """Small cases for profiler captures (a few hundred MB on the device)."""
    import torch

    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    from pyscaledvecchia_gb300 import _lib as L
    from pyscaledvecchia_gb300.ordering import knn_query_device, maximin_order_device
    lib, _ = L.device_ready()
    if name in ("pred", "pred64"):
        rng = np.random.default_rng(0)
        ntr, nte, d, m = 100_000, 20_000, 6, 140
        Xtr, Xte = rng.random((ntr, d)), rng.random((nte, d))
        # the fitted parameters of the prediction workload (standardised frame)
        theta = np.array([-0.38, -2.30, -1.63, -0.93, -0.17, 1.96, 6.9, -5.87])
        ranges = np.exp(theta[1:1 + d])
        nb, _ = knn_query_device(torch, L.to_dev(torch, Xtr / ranges, np.float64),
                                 L.to_dev(torch, Xte / ranges, np.float64), m)
        Xall = torch.cat([L.to_dev(torch, Xtr, np.float64), L.to_dev(torch, Xte, np.float64)])
        tgt = torch.arange(ntr, ntr + nte, dtype=torch.int32, device="cuda")
        nbr = nb.to(torch.int32).contiguous()
        rd = L.to_dev(torch, rng.standard_normal(ntr), np.float64)
        th = L.to_dev(torch, theta, np.float64)
        D = L.PredDesc()
        D.nall, D.nobs, D.nblk = ntr + nte, ntr, nte
        D.d, D.k, D.ldnbr = d, m, m
        D.general, D.nu, D.precision = 0, 2.5, int(name == "pred")
        mean = torch.empty(nte, dtype=torch.float64, device="cuda")
        var = torch.empty_like(mean)
        info = L.new_info(torch)
        for _ in range(3):
            L.check(lib, lib.sv_predict_blocks(D, L.ptr(th), L.ptr(Xall), L.ptr(tgt), L.ptr(nbr),
                                               L.ptr(rd), L.ptr(mean), L.ptr(var), None, None,
                                               L.ptr(info), L.stream_handle(torch)),
                    "sv_predict_blocks")
        torch.cuda.synchronize()
        L.check_info(lib, info.cpu().numpy(), "sv_predict_blocks")
    elif name == "tree":
        n, d = 100_000, 10
        rng = np.random.default_rng(1)
        Xs = rng.random((n, d)) / np.exp(rng.uniform(math.log(0.05), math.log(50.0), d))
        first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
        _, info = maximin_order_device(torch, L.to_dev(torch, Xs, np.float64), first, 16)
        torch.cuda.synchronize()
        L.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
    elif name == "jvar":
        rng = np.random.default_rng(2)
        X = rng.random((20_000, 4))
        y = np.sin(5 * X[:, 0]) + X[:, 1] + 0.1 * rng.standard_normal(20_000)
        gp = ScaledVecchiaGP(m_est=20, n_est=2000, var_correction=False).fit(X, y)
        F = gp._joint_factor_device((rng.random((5000, 4)) - gp._lo) / gp._span, 40)
        gp._joint_var_diag(F)
        torch.cuda.synchronize()
    elif name in ("nu08", "nu08s"):
        from pyscaledvecchia_gb300.likelihood import DeviceProblem
        from pyscaledvecchia_gb300.ordering import _nn_groups, ordered_nn_device
        n, d, m = 20_000, 10, 30
        X, lam, theta, eps = make_inputs(n, d, 1)
        Xs = X / lam
        first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
        Xs_d = L.to_dev(torch, Xs, np.float64)
        o, _ = maximin_order_device(torch, Xs_d, first)
        nn, _ = ordered_nn_device(torch, Xs_d[o].contiguous(), m)
        order = o.cpu().numpy()
        prob = DeviceProblem(X[order], eps, np.ones((n, 1)), _nn_groups(nn.cpu().numpy(), m))
        prec = "split" if name == "nu08s" else "float64"
        for _ in range(3):
            prob.evaluate(theta, 0.8, precision=prec, team_lanes=16 if prec == "split" else 0)
        torch.cuda.synchronize()
    print(json.dumps({"kernel_case": name, "status": "ok"}))


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_inputs(n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    lam = np.exp(rng.uniform(math.log(0.05), math.log(50.0), d))
    theta = np.concatenate([[math.log(2.0)], np.log(lam), [math.log(1e-3)]])
    eps = rng.standard_normal(n)
    return X, lam, theta, eps


def matern_closed(nu, r):
    if nu == 0.5:
        return np.exp(-r)
    if nu == 1.5:
        c = math.sqrt(3.0) * r
        return (1.0 + c) * np.exp(-c)
    c = math.sqrt(5.0) * r
    return (1.0 + c + c * c / 3.0) * np.exp(-c)


def vecchia_response(Xo, nn, theta, nu, eps, chunk=4096):
    """Unconditional Vecchia draw y = U^-T eps on the host (NumPy): column i
    of U is a_i = L_i^-T e_K of block (neighbours of i, i) with covariance
    sigma^2 (M_nu + tau I), so y_i = (eps_i - sum_j a_ij y_j) / a_ii in row
    order.  The benchmark's response in both arms (identical arrays)."""
    n, d = Xo.shape
    m = nn.shape[1] - 1
    s2, lam, tau = math.exp(theta[0]), np.exp(theta[1:1 + d]), math.exp(theta[-1])
    U = Xo / lam
    a_self = np.empty(n)
    a_nb = np.zeros((n, max(m, 1)))
    for k in range(0, m + 1):
        rows = np.arange(k, k + 1) if k < m else np.arange(m, n)
        rows = rows[rows < n]
        for c0 in range(0, rows.shape[0], chunk):
            r = rows[c0:c0 + chunk]
            blk = np.concatenate([nn[r, 1:k + 1], r[:, None]], axis=1)  # (B, k+1)
            P = U[blk] - U[r][:, None, :]  # centred on the block's own point
            q = (P * P).sum(-1)
            D = np.sqrt(np.maximum(q[:, :, None] + q[:, None, :] - 2.0 * (P @ np.transpose(P, (0, 2, 1))),
                                   0.0))
            S = s2 * (matern_closed(nu, D) + tau * np.eye(k + 1))
            L = np.linalg.cholesky(S)
            e = np.zeros((r.shape[0], k + 1, 1))
            e[:, k, 0] = 1.0
            a = np.linalg.solve(np.transpose(L, (0, 2, 1)), e)[:, :, 0]
            a_self[r] = a[:, k]
            a_nb[r, :k] = a[:, :k]
    y = np.empty(n)
    for i in range(n):
        k = min(i, m)
        s = eps[i]
        if k:
            s -= a_nb[i, :k] @ y[nn[i, 1:k + 1]]
        y[i] = s / a_self[i]
    return y


def nn_digest(nn):
    return hashlib.sha256(np.ascontiguousarray(nn, dtype=np.int32).tobytes()).hexdigest()


def c2_fixture(n, d, m, seed):
    """(order, neighbour-table digest) of the oracle for the default
    workload, or None for other sizes."""
    if (n, d, m, seed) != (200_000, 10, 30, 1) or not os.path.exists(C2_ORDER):
        return None
    f = np.load(C2_ORDER)
    return f["order"].astype(np.int64), str(f["nn_sha256"])


def block_flops(kb, P):
    """float64 flops per block of size K = k+1: LDL^T K^3/3, a = L^-T e_K,
    W = L^-1 (dS a) for P rows, z = L^-1 y: K^3/3 + (P+2) K^2."""
    K = kb.astype(np.float64) + 1.0
    return float(np.sum(K ** 3 / 3.0 + (P + 2) * K ** 2))


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "25"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def wait_first(self, timeout=5.0):
        """Block until nvidia-smi has written its first sample (it takes a
        while to start), so that the samples cover the whole timed region."""
        t0 = time.perf_counter()
        while self.p is not None and time.perf_counter() - t0 < timeout:
            try:
                if os.path.getsize(self.f.name) > 0:
                    return
            except OSError:
                return
            time.sleep(0.01)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak(lib, torch, probe="fp64"):
    """TFLOP/s of the float64 (probe="fp64") or float32 ("fp32") FMA probe:
    8 independent FMA chains in each of sv_fp64_probe_threads() threads,
    best of three timed launches after a warm-up."""
    from pyscaledvecchia_gb300 import _lib
    nthr = int(lib.sv_fp64_probe_threads())
    dt = torch.float64 if probe == "fp64" else torch.float32
    fn = lib.sv_fp64_fma_probe if probe == "fp64" else lib.sv_fp32_fma_probe
    out = torch.empty(nthr, dtype=dt, device="cuda")
    iters = 4096 if probe == "fp64" else 65536
    st = _lib.stream_handle(torch)
    fn(_lib.ptr(out), iters, st)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn(_lib.ptr(out), iters, st)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, 2.0 * 8 * iters * nthr / (ms * 1e-3) / 1e12)
    return best


def errors_vs(ref, got):
    """Per-output error of (ll, grad, fisher, beta) against a float64
    reference: ll relative; score in units of its standard deviation
    sqrt(F_ii) (the score is a sum of zero-mean terms); Fisher relative to
    its largest entry; beta relative."""
    ll0, g0, F0, b0 = ref
    ll1, g1, F1, b1 = got
    sd = np.sqrt(np.maximum(np.diag(F0), 1e-300))
    return {"ll_rel": abs(ll1 - ll0) / abs(ll0),
            "score_in_sd": float(np.max(np.abs(g1 - g0) / sd)),
            "fisher_rel_max": float(np.abs(F1 - F0).max() / np.abs(F0).max()),
            "beta_rel": float(np.max(np.abs(b1 - b0) / np.maximum(np.abs(b0), 1e-300)))}


def cpu_reference_eval(Xo, yo, Zo, groups, theta, nu, threads):
    from oracle import oracle
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    out = oracle.vecchia_loglik(theta, Xo, yo, Zo, groups, nu)
    return time.perf_counter() - t0, out


# ---------------------------------------------------------------------------
# C1: plain single fit + predict, n = 2000
# ---------------------------------------------------------------------------
def c1_inputs():
    """X_train 2000 x 8 and X_test 500 x 8 uniform in [0,1]^8 (seed 0); y an
    exact GP draw (dense Cholesky) of sigma^2 = 1, Matern 2.5, relative nugget
    1e-4, lambda = (0.2, 0.3, 0.5, 1, 2, 5, 50, 100), constant mean 0.5, drawn
    jointly at the training and test points."""
    rng = np.random.default_rng(0)
    Xtr = rng.random((2000, 8))
    Xte = rng.random((500, 8))
    lam = np.array([0.2, 0.3, 0.5, 1.0, 2.0, 5.0, 50.0, 100.0])
    Xa = np.vstack([Xtr, Xte]) / lam
    r = np.sqrt(((Xa[:, None, :] - Xa[None, :, :]) ** 2).sum(-1))
    S = matern_closed(2.5, r) + 1e-4 * np.eye(Xa.shape[0])
    y = 0.5 + np.linalg.cholesky(S) @ rng.standard_normal(Xa.shape[0])
    return Xtr, y[:2000], Xte, y[2000:]


C1_SETTINGS = dict(m_est=30, m_pred=140, n_est=2000, nu=2.5, trend="constant", nugget=None)
C1_WORKLOAD = ("fit + predict, n_train 2000 x 8, n_test 500, Matern 2.5, exact GP draw "
               "(tau 1e-4), m_est 30, m_pred 140, n_est 2000, constant trend, nugget estimated")


def run_c1(make_model, reps):
    Xtr, ytr, Xte, yte = c1_inputs()
    make_model().fit(Xtr[:500], ytr[:500])  # warm-up (library, allocations)
    tf, tp, res = [], [], None
    for _ in range(reps):
        t0 = time.perf_counter()
        gp = make_model().fit(Xtr, ytr)
        t1 = time.perf_counter()
        mu, sd = gp.predict(Xte, return_std=True)
        t2 = time.perf_counter()
        tf.append(t1 - t0)
        tp.append(t2 - t1)
        res = (gp, mu, sd)
    gp, mu, sd = res
    t = float(np.mean(tf) + np.mean(tp))
    return {"workload": C1_WORKLOAD, "fit_s": float(np.mean(tf)), "predict_s": float(np.mean(tp)),
            "fit_predict_s": t, "fits_per_s": 1.0 / t, "loglik": float(gp.loglik_),
            "theta": [float(v) for v in gp.theta_], "b": float(gp.b_),
            "rmse_test": float(np.sqrt(np.mean((mu - yte) ** 2))), "reps": reps}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    X, lam, theta, eps = make_inputs(args.n, args.d, 1)
    Xs = X / lam
    fx = c2_fixture(args.n, args.d, args.m, 1)
    t0 = time.perf_counter()
    if fx is not None:
        order = fx[0]  # the oracle's own maximin order, computed once
        src = "oracle maximin order (tests/golden/c2_order.npz)"
    else:
        order = oracle.maximin_order(Xs)
        src = "oracle maximin order"
    t_order = time.perf_counter() - t0
    t0 = time.perf_counter()
    nn = oracle.ordered_nn(Xs[order], args.m)
    t_nn = time.perf_counter() - t0
    nn_ok = (nn_digest(nn) == fx[1]) if fx is not None else None
    groups = oracle.nn_groups(nn, args.m)
    Xo, Zo = np.ascontiguousarray(X[order]), np.ones((args.n, 1))
    yo = vecchia_response(Xo, nn, theta, 2.5, eps)
    for _ in range(args.warmup):
        cpu_reference_eval(Xo, yo, Zo, groups, theta, args.nu, threads)
    ts, out = [], None
    for _ in range(args.steps):
        t, out = cpu_reference_eval(Xo, yo, Zo, groups, theta, args.nu, threads)
        ts.append(t)
    t = float(np.mean(ts))
    v = args.n / t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "blocks/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; y = Vecchia draw computed on the host, the same arrays as "
                "the GPU arm)",
        "config": {"workload": f"loglik+score+Fisher, n={args.n}, d={args.d}, m={args.m}, "
                               f"nu={args.nu}", "n": args.n, "d": args.d, "m": args.m,
                   "nu": args.nu, "ordering": src},
        "cpu_baseline": {"value": v, "unit": "blocks/s", "cores": threads, "kind": "port",
                         "sample": f"full evaluation of all {args.n} blocks per step "
                                   "(C restatement of the reference's Numba loops, OpenMP)"},
        "e2e": {"value": v, "unit": "blocks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "extra": {"ll": out[0], "order_s": t_order, "knn_s": t_nn,
                  "nn_matches_oracle_fixture": nn_ok},
    }
    if not args.no_c1:
        from oracle.fit import OracleGP
        line["extra"]["c1"] = run_c1(lambda: OracleGP(**C1_SETTINGS), reps=1)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# C3: batched fits
# ---------------------------------------------------------------------------
def make_fit_problems(nprob, seed=2):
    """The batched-fits workload: nprob independent problems, n log-uniform
    in [500, 20000], d uniform in {3..12}, m in {10, 20, 30}, X uniform in
    [0,1]^d, lambda log-uniform in [0.05, 100], Matern 2.5 Vecchia draws
    (sigma^2 = 1); the first half hold a fixed nugget of 1e-8 (and are drawn
    with tau = 1e-8), the second half estimate it (drawn with tau
    log-uniform in [1e-4, 1e-1])."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nprob):
        n = int(round(math.exp(rng.uniform(math.log(500), math.log(20000)))))
        d = int(rng.integers(3, 13))
        m = int(rng.choice([10, 20, 30]))
        X = rng.random((n, d))
        lam = np.exp(rng.uniform(math.log(0.05), math.log(100.0), d))
        fixed = i < nprob // 2
        tau = 1e-8 if fixed else float(np.exp(rng.uniform(math.log(1e-4), math.log(1e-1))))
        eps = rng.standard_normal(n)
        out.append(dict(n=n, d=d, m=m, X=X, lam=lam, tau=tau, fixed=fixed, eps=eps))
    return out


def draw_fit_responses(torch, lib, probs):
    """y of every problem: unconditional Vecchia draw in its own maximin
    order (the method's sample_joint prior), returned in the rows' order."""
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device, ordered_nn_device
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample_device
    ys = []
    for pr in probs:
        X, lam, n, m = pr["X"], pr["lam"], pr["n"], pr["m"]
        Xs = X / lam
        first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
        Xs_d = _lib.to_dev(torch, Xs, np.float64)
        order_d, info = maximin_order_device(torch, Xs_d, first)
        _lib.check_info(lib, info.cpu().numpy(), "maximin")
        nn_d, info = ordered_nn_device(torch, Xs_d[order_d].contiguous(), m)
        _lib.check_info(lib, info.cpu().numpy(), "knn")
        order = order_d.cpu().numpy()
        theta = np.concatenate([[0.0], np.log(lam), [math.log(pr["tau"])]])
        yo = vecchia_prior_sample_device(torch, _lib.to_dev(torch, X[order], np.float64), nn_d, theta,
                                         2.5, _lib.to_dev(torch, pr["eps"].reshape(n, 1), np.float64))
        y = np.empty(n)
        y[order] = yo.reshape(-1).cpu().numpy()
        ys.append(y)
    return ys


def _form_stats(ref, models, t, nprob):
    ll_r = np.array([g.loglik_ for g in ref])
    ll_m = np.array([g.loglik_ for g in models])
    dll = ll_m - ll_r
    rel = np.abs(dll) / np.maximum(np.abs(ll_r), 1.0)
    same = sum(bool(np.array_equal(a.theta_, b.theta_) and a.loglik_ == b.loglik_)
               for a, b in zip(ref, models))
    ev = np.array([g.fit_stats_["split"] + g.fit_stats_["float64"] for g in models])
    return {"fits_per_s": nprob / t, "s": t, "objective_evals_mean": float(ev.mean()),
            "dll_abs_max": float(np.abs(dll).max()), "dll_abs_median": float(np.median(np.abs(dll))),
            "dll_rel_max": float(rel.max()),
            "frac_abs_dll_below_1e-6": float(np.mean(np.abs(dll) < 1e-6)),
            "frac_not_worse_than_plain": float(np.mean(dll >= -1e-6 * np.maximum(np.abs(ll_r), 1.0))),
            "bitwise_equal_to_plain": int(same)}


def run_fits(torch, lib, nprob, dump=""):
    """Batched-fits workload.  Forms: plain (ScaledVecchiaGP.fit one problem
    at a time, float64, default start, no graphs); batched_float64
    (fit_batched: all problems per launch, CUDA-graph replay, batched device
    reorders, float64 evaluations: the plain form's iterates bit for bit);
    batched_split (split-precision iterations + float64 polish); and, when
    trained weights ship, batched_split_warm (the same from the encoder's
    starting point).  "chosen" is the fastest form whose loglik agrees with
    the plain form's within 1e-6 on every problem."""
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    from pyscaledvecchia_gb300.fit_batched import fit_batched
    from pyscaledvecchia_gb300 import warmstart
    probs = make_fit_problems(nprob)
    t0 = time.perf_counter()
    ys = draw_fit_responses(torch, lib, probs)
    t_draw = time.perf_counter() - t0

    def model(pr):
        return ScaledVecchiaGP(m_est=pr["m"], n_est=None, nu=2.5,
                               nugget=1e-8 if pr["fixed"] else None, var_correction=False)

    enc = warmstart.SetEncoder.load() if os.path.exists(warmstart.DEFAULT_WEIGHTS) else None
    Xs = [pr["X"] for pr in probs]
    # warm-up of every path on two small problems (library load, graphs)
    small = sorted(range(nprob), key=lambda i: probs[i]["n"])[:2]
    for i in small:
        model(probs[i]).fit(Xs[i], ys[i])
    for prec in ("float64", "split"):
        fit_batched([model(probs[i]) for i in small], [Xs[i] for i in small], [ys[i] for i in small],
                    precision=prec, warm_start=enc)
    torch.cuda.synchronize()

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    def sched(st):
        return {k: (float(v) if isinstance(v, float) else v) for k, v in st.items()
                if k not in ("batch", "thetas")}

    plain, t_plain = timed(lambda: [model(pr).fit(X, y) for pr, X, y in zip(probs, Xs, ys)])
    forms = {}
    st64 = {}
    b64, t = timed(lambda: fit_batched([model(pr) for pr in probs], Xs, ys, precision="float64",
                                       stats=st64))
    forms["batched_float64"] = _form_stats(plain, b64, t, nprob)
    forms["batched_float64"]["schedule"] = sched(st64)
    st = {}
    spl, t = timed(lambda: fit_batched([model(pr) for pr in probs], Xs, ys, precision="split", stats=st))
    forms["batched_split"] = _form_stats(plain, spl, t, nprob)
    forms["batched_split"]["schedule"] = sched(st)
    if enc is not None:
        stw = {}
        warm, t = timed(lambda: fit_batched([model(pr) for pr in probs], Xs, ys, precision="split",
                                            warm_start=enc, stats=stw))
        forms["batched_split_warm"] = _form_stats(plain, warm, t, nprob)
        forms["batched_split_warm"]["schedule"] = sched(stw)
        # both starts per model in one float64 batch, the better converged
        # loglik kept: never below the plain fit (whose path is the default one)
        judged, t = timed(lambda: fit_batched([model(pr) for pr in probs], Xs, ys, precision="float64",
                                              warm_start=enc, warm_judge=True))
        forms["batched_float64_warm_judged"] = _form_stats(plain, judged, t, nprob)
        dj = np.array([a.loglik_ - b.loglik_ for a, b in zip(judged, plain)])
        forms["batched_float64_warm_judged"]["frac_better_than_plain"] = float(np.mean(dj > 1e-6))
        forms["batched_float64_warm_judged"]["dll_median_where_better"] = (
            float(np.median(dj[dj > 1e-6])) if np.any(dj > 1e-6) else 0.0)

    # split form vs float64 at every final state of the split fits (same ordering)
    BL = st["batch"]
    th_obj = [g._objective_theta(t_, g.d_, False) for g, t_ in zip(spl, st["thetas"])]
    r64 = BL.evaluate(th_obj, active=np.ones(nprob, bool), precision="float64")
    r32 = BL.evaluate(th_obj, active=np.ones(nprob, bool), precision="split")
    e_ll = max(abs(a[1] - b[1]) / abs(b[1]) for a, b in zip(r32, r64))
    # score error in units of its standard deviation sqrt(F_ii) (the score
    # itself is ~0 at the optimum, so a relative error says nothing there)
    e_g = max(float(np.max(np.abs(a[2] - b[2]) / np.sqrt(np.maximum(np.diag(b[3]), 1e-300))))
              for a, b in zip(r32, r64))
    e_f = max(float(np.abs(a[3] - b[3]).max() / max(np.abs(b[3]).max(), 1e-300)) for a, b in zip(r32, r64))
    e_b = max(float(np.abs(a[4] - b[4]).max() / max(np.abs(b[4]).max(), 1e-300)) for a, b in zip(r32, r64))
    if dump:
        np.savez_compressed(
            dump, n=np.array([p["n"] for p in probs]), d=np.array([p["d"] for p in probs]),
            m=np.array([p["m"] for p in probs]), fixed=np.array([p["fixed"] for p in probs]),
            ll_plain=np.array([g.loglik_ for g in plain]), ll_b64=np.array([g.loglik_ for g in b64]),
            ll_split=np.array([g.loglik_ for g in spl]),
            evals_plain=np.array([g.fit_stats_["float64"] for g in plain]),
            evals_split=np.array([g.fit_stats_["split"] for g in spl]),
            evals_polish=np.array([g.fit_stats_["float64"] for g in spl]),
            **({"ll_warm": np.array([g.loglik_ for g in warm]),
                "evals_warm": np.array([g.fit_stats_["split"] + g.fit_stats_["float64"] for g in warm])}
               if enc is not None else {}))
    ok = [k for k, v in forms.items() if v["frac_abs_dll_below_1e-6"] == 1.0 or
          v["dll_rel_max"] < 1e-6]
    # forms whose loglik is never below the plain form's (within 1e-6)
    not_worse = [k for k, v in forms.items() if v["frac_not_worse_than_plain"] == 1.0]
    chosen = max(ok, key=lambda k: forms[k]["fits_per_s"]) if ok else None
    fastest = max(forms, key=lambda k: forms[k]["fits_per_s"])
    return {
        "workload": f"{nprob} independent fits, n log-U[500,20000] (total "
                    f"{sum(p['n'] for p in probs)} points), d U{{3..12}}, m in {{10,20,30}}, "
                    "nu = 2.5, half fixed nugget 1e-8, n_est = None, var_correction off",
        "plain_fits_per_s": nprob / t_plain, "plain_s": t_plain,
        "plain_objective_evals_mean": float(np.mean([g.fit_stats_["float64"] for g in plain])),
        "forms": forms,
        "chosen_form": chosen, "chosen_fits_per_s": forms[chosen]["fits_per_s"] if chosen else None,
        "chosen_speedup": (forms[chosen]["fits_per_s"] * t_plain / nprob) if chosen else None,
        "fastest_form": fastest, "fastest_speedup": forms[fastest]["fits_per_s"] * t_plain / nprob,
        "never_worse_forms": not_worse,
        "split_vs_float64_at_final_state": {"ll_rel_max": e_ll, "score_err_max_in_sd": e_g,
                                            "fisher_rel_max": e_f, "beta_rel_max": e_b},
        "draw_s": t_draw,
    }


# ---------------------------------------------------------------------------
# C4: prediction and joint sampling
# ---------------------------------------------------------------------------
def c4_inputs(torch):
    """The prediction workload's data: n_train = 100,000 points in [0,1]^6,
    y a Matern-2.5 Vecchia draw (m = 30) with lambda = (0.1, 0.2, 0.4, 0.8,
    5, 100), sigma^2 = 1, tau = 1e-6, and 50,000 test points in
    [-0.1, 1.1]^6 (seed 3).  Returns (X, y, Xte)."""
    from pyscaledvecchia_gb300 import _lib as L
    from pyscaledvecchia_gb300.ordering import maximin_order_device, ordered_nn_device
    from pyscaledvecchia_gb300.sampling import vecchia_prior_sample_device
    rng = np.random.default_rng(3)
    ntr, nte, d = 100_000, 50_000, 6
    X = rng.random((ntr, d))
    Xte = rng.uniform(-0.1, 1.1, (nte, d))
    lam = np.array([0.1, 0.2, 0.4, 0.8, 5.0, 100.0])
    eps = rng.standard_normal(ntr)
    Xs = X / lam
    first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
    Xs_d = L.to_dev(torch, Xs, np.float64)
    od, _ = maximin_order_device(torch, Xs_d, first)
    nd, _ = ordered_nn_device(torch, Xs_d[od].contiguous(), 30)
    o = od.cpu().numpy()
    th = np.concatenate([[0.0], np.log(lam), [math.log(1e-6)]])
    yo = vecchia_prior_sample_device(torch, L.to_dev(torch, X[o], np.float64), nd, th, 2.5,
                                     L.to_dev(torch, eps.reshape(ntr, 1), np.float64))
    y = np.empty(ntr)
    y[o] = yo.reshape(-1).cpu().numpy()
    return X, y, Xte


def run_predict(torch, lib, check_oracle=True):
    """Prediction and joint sampling on c4_inputs: the default fit (m_est 30,
    n_est 5000, variance correction b on the reference's inner split); then
    the 50,000 test points: marginal mean/sd with m_pred = 140 (141-point
    blocks) in float64 and in the split form (float32 assembly, float64
    LDL^T and solves), their differences and their errors against the
    oracle on a sample of 2,000 points, and 100 joint sample paths."""
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    X, y, Xte = c4_inputs(torch)
    nte = Xte.shape[0]

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    gp = ScaledVecchiaGP(m_est=30, m_pred=140, nu=2.5)
    _, t_fit = timed(lambda: gp.fit(X, y))
    res = {"workload": "n_train 100000 x 6, n_test 50000, m_pred 140, 100 joint paths, nu 2.5",
           "fit_s": t_fit, "b": float(gp.b_), "fitted_ranges": [float(v) for v in gp.ranges_],
           "nugget": float(gp.nugget_)}
    K = 141
    flops = K ** 3 / 3 + K ** 2  # LDL^T and the solve of one block (float64)
    pred = {}
    for prec in ("float64", "split"):
        gp.precision = prec
        gp.predict(Xte[:2000], return_std=True)  # warm-up
        (mu, sd), t = timed(lambda: gp.predict(Xte, return_std=True))
        ms = predict_kernel_ms(torch, lib, gp, Xte)
        pred[prec] = (mu, sd)
        res[prec] = {"predict_s": t, "predict_points_per_s": nte / t, "kernel_ms": ms,
                     "kernel_fp64_tflops": nte * flops / (ms * 1e-3) / 1e12,
                     "blocks_redone_in_float64": gp.pred_stats_["redone_float64"],
                     "sd_finite": bool(np.all(np.isfinite(sd)))}
    mu64, sd64 = pred["float64"]
    mu32, sd32 = pred["split"]
    res["split_vs_float64"] = pred_errors(mu32, sd32, mu64, sd64)
    if check_oracle:
        # the oracle (C restatement of gp.py:242-277, OpenMP on the host's
        # cores) on every 25th test point, against which both forms are compared
        from oracle import oracle
        oracle.build()
        oracle.set_threads(os.cpu_count() or 1)
        sub = np.arange(0, nte, 25)
        Xs_te = (Xte[sub] - gp._lo) / gp._span
        Ztr = gp._design(gp.X_)
        resid = gp.y_ - (Ztr @ gp.beta_ if gp.beta_.size else 0.0)
        t0 = time.perf_counter()
        mo, vo, _ = oracle.predict_marginal(gp.X_, resid, Xs_te, gp._pred_theta(), 2.5, 140)
        t_or = time.perf_counter() - t0
        mo = gp._ymu + gp._ysd * (mo + (gp._design(Xs_te) @ gp.beta_ if gp.beta_.size else 0.0))
        so = gp._ysd * np.sqrt(gp.b_ * vo)
        res["oracle_sample"] = f"every 25th test point ({sub.size}), {os.cpu_count()} threads"
        res["oracle_points_per_s"] = sub.size / t_or
        for prec in ("float64", "split"):
            res[prec + "_vs_oracle"] = pred_errors(pred[prec][0][sub], pred[prec][1][sub], mo, so)
    gp.precision = "float64"
    samples, t_joint = timed(lambda: gp.sample_joint(Xte, n_sim=100, random_state=0))
    res["sample_joint_s"] = t_joint
    res["samples_shape"] = list(samples.shape)
    # exact marginal variances of the joint law, diag((U_pp U_pp^T)^-1)
    # (gp.py:391-393 forms the dense 50,000 x 50,000 U_pp^-T for this)
    F = gp._joint_factor_device((Xte - gp._lo) / gp._span, gp.m_pred)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    v = gp._joint_var_diag(F)
    torch.cuda.synchronize()
    res["exact_var_diag_s"] = time.perf_counter() - t0
    res["exact_var_finite_positive"] = bool(torch.all(v > 0).item() and torch.isfinite(v).all().item())
    return res


def pred_errors(mu, sd, mu_ref, sd_ref):
    """Prediction differences in units of the reference sd: |mean - mean_ref|
    / sd_ref and |sd - sd_ref| / sd_ref (median, 99th percentile, max)."""
    em = np.abs(mu - mu_ref) / sd_ref
    es = np.abs(sd - sd_ref) / sd_ref

    def q(e):
        return [float(np.median(e)), float(np.quantile(e, 0.99)), float(e.max())]
    return {"mean_err_over_sd": q(em), "sd_rel_err": q(es), "points": int(mu.shape[0])}


def predict_kernel_ms(torch, lib, gp, Xte, reps=5):
    """Device time of the prediction-block launch alone (sv_predict_blocks,
    the model's precision) on the whole test set: neighbours searched once,
    CUDA events around each launch on the launching stream, median of reps."""
    from pyscaledvecchia_gb300 import _lib as L
    from pyscaledvecchia_gb300.ordering import knn_query_device
    Xs_te = (Xte - gp._lo) / gp._span
    Ztr = gp._design(gp.X_)
    resid = gp.y_ - (Ztr @ gp.beta_ if gp.beta_.size else 0.0)
    ntr, d = gp.X_.shape
    nte = Xs_te.shape[0]
    m = min(gp.m_pred, ntr)
    nb, _ = knn_query_device(torch, L.to_dev(torch, gp.X_ / gp.ranges_, np.float64),
                             L.to_dev(torch, Xs_te / gp.ranges_, np.float64), m)
    Xall = torch.cat([L.to_dev(torch, gp.X_, np.float64), L.to_dev(torch, Xs_te, np.float64)])
    tgt = torch.arange(ntr, ntr + nte, dtype=torch.int32, device="cuda")
    nbr = nb.to(torch.int32).contiguous()
    rd = L.to_dev(torch, resid, np.float64)
    th = L.to_dev(torch, gp._pred_theta(), np.float64)
    D = L.PredDesc()
    D.nall, D.nobs, D.nblk = ntr + nte, ntr, nte
    D.d, D.k, D.ldnbr = d, m, m
    D.general, D.nu = int(gp._general()), float(gp.nu_)
    D.precision = int(gp.precision == "split")
    mean = torch.empty(nte, dtype=torch.float64, device="cuda")
    var = torch.empty_like(mean)
    info = L.new_info(torch)
    st = torch.cuda.current_stream()
    ts = []
    for _ in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        rc = lib.sv_predict_blocks(D, L.ptr(th), L.ptr(Xall), L.ptr(tgt), L.ptr(nbr), L.ptr(rd),
                                   L.ptr(mean), L.ptr(var), None, None, L.ptr(info),
                                   L.stream_handle(torch))
        e1.record(st)
        torch.cuda.synchronize()
        L.check(lib, rc, "sv_predict_blocks")
        ts.append(e0.elapsed_time(e1))
    L.check_info(lib, info.cpu().numpy(), "sv_predict_blocks")
    return float(np.median(ts[1:]))


# ---------------------------------------------------------------------------
# C2 at the other smoothness values, and the Bessel K_nu against scipy
# ---------------------------------------------------------------------------
def bessel_error(torch, lib, Xo, nn, theta, nu, nblk=2000, seed=5):
    """Largest relative error of the device K_nu (sv_bessel_k) against
    scipy.special.kv on this workload's own arguments: c = sqrt(2 nu) r for
    every pair of nblk random blocks (r floored at 1e-7 as in
    _matern_general.py:92-116)."""
    from scipy.special import kv

    from pyscaledvecchia_gb300 import _lib
    n, d = Xo.shape
    U = Xo / np.exp(theta[1:1 + d])
    rng = np.random.default_rng(seed)
    rows = rng.choice(np.arange(nn.shape[1], n), nblk, replace=False)
    blk = np.concatenate([nn[rows, 1:], rows[:, None]], axis=1)
    P = U[blk]
    r = np.sqrt(((P[:, :, None, :] - P[:, None, :, :]) ** 2).sum(-1))
    iu = np.triu_indices(blk.shape[1], 1)
    c = math.sqrt(2.0 * nu) * np.maximum(r[:, iu[0], iu[1]].ravel(), 1e-7)
    xd = _lib.to_dev(torch, c, np.float64)
    out = torch.empty_like(xd)
    rc = lib.sv_bessel_k(_lib.ptr(xd), c.shape[0], float(nu), _lib.ptr(out), _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_bessel_k")
    got = out.cpu().numpy()
    ref = kv(nu, c)
    ok = ref > 0
    return {"args": int(c.shape[0]), "c_min": float(c.min()), "c_max": float(c.max()),
            "max_rel_err_vs_scipy_kv": float(np.max(np.abs(got[ok] - ref[ok]) / ref[ok])),
            "underflow_both_zero": int(np.sum((ref == 0) & (got == 0)))}


def main():
    args = parse()
    if args.kernel_case:
        kernel_case(args.kernel_case)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)

    import pyscaledvecchia_gb300 as sv
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups, maximin_order_device, ordered_nn_device

    lib, _ = _lib.device_ready()
    n, d, m, nu = args.n, args.d, args.m, args.nu
    seed = 1 + rank
    X, lam, theta, eps = make_inputs(n, d, seed)

    # ---- setup: exact ordering and neighbours on the GPU, the response on the host
    Xs = X / lam
    first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
    Xs_d = _lib.to_dev(torch, Xs, np.float64)
    # the ordering kernels' first launch (module load, launch set-up) outside
    # the timing: the grid and tree forms on 30,000 rows
    for fl in (4, 16):
        _, info = maximin_order_device(torch, Xs_d[:30_000].contiguous(), 0, fl)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    order_d, info = maximin_order_device(torch, Xs_d, first)
    torch.cuda.synchronize()
    t_maximin = time.perf_counter() - t0
    _lib.check_info(lib, info.cpu().numpy(), "maximin")
    t0 = time.perf_counter()
    nn_d, info = ordered_nn_device(torch, Xs_d[order_d].contiguous(), m)
    torch.cuda.synchronize()
    t_knn = time.perf_counter() - t0
    _lib.check_info(lib, info.cpu().numpy(), "knn")
    # the same rows through the tree form of the maximin (the route beyond the
    # grid form's shared memory), and the tree form at a million rows
    t0 = time.perf_counter()
    order_t, info = maximin_order_device(torch, Xs_d, first, 16)
    torch.cuda.synchronize()
    t_tree = time.perf_counter() - t0
    _lib.check_info(lib, info.cpu().numpy(), "maximin")
    tree_same = bool(torch.equal(order_t, order_d))
    maximin_tree = {"rows": n, "tree_s": t_tree, "default_route_s": t_maximin,
                    "same_order_as_default_route": tree_same}
    if not args.no_forms:
        X1, lam1, _, _ = make_inputs(1_000_000, d, seed + 100)
        Xs1 = X1 / lam1
        f1 = int(np.argmin(((Xs1 - Xs1.mean(0)) ** 2).sum(1)))
        Xs1_d = _lib.to_dev(torch, Xs1, np.float64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        o1, info = maximin_order_device(torch, Xs1_d, f1)
        torch.cuda.synchronize()
        maximin_tree["rows_1M_s"] = time.perf_counter() - t0
        _lib.check_info(lib, info.cpu().numpy(), "maximin")
        del Xs1_d, o1
    order = order_d.cpu().numpy()
    nn = nn_d.cpu().numpy()
    fx = c2_fixture(n, d, m, seed)
    order_ok = bool(np.array_equal(order, fx[0])) if fx is not None else None
    nn_ok = (nn_digest(nn) == fx[1]) if fx is not None else None
    Xo = np.ascontiguousarray(X[order])
    yo = vecchia_response(Xo, nn, theta, 2.5, eps)
    Zo = np.ones((n, 1))
    groups = _nn_groups(nn, m)
    prob = DeviceProblem(Xo, yo, Zo, groups)
    P = d + 2
    th_d = _lib.to_dev(torch, theta, np.float64)
    kb = np.minimum(np.arange(n), m)
    flops = block_flops(kb, P)
    launches_per_step = prob.kernel_launches("split", nu=nu)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def time_form(precision, lanes, steps, warmup, nu_=None):
        nu_ = nu if nu_ is None else nu_
        for _ in range(warmup):
            prob.launch(th_d, P, nu_, False, True, 0.0, 0.0, True, precision=precision,
                        team_lanes=lanes)
        torch.cuda.synchronize()
        evs = []
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prob.launch(th_d, P, nu_, False, True, 0.0, 0.0, True, precision=precision,
                        team_lanes=lanes)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    # team width of the split kernels: the fastest on this problem
    def best_width(prec):
        ms = {w: float(np.median(time_form(prec, w, 2, 1))) for w in (4, 8, 16, 32)}
        return min(ms, key=ms.get), ms
    best_lanes, lane_ms = best_width("split")
    res64 = prob.evaluate(theta, nu)
    res = prob.evaluate(theta, nu, precision="split", team_lanes=best_lanes)

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.wait_first()
    step_ms = time_form("split", best_lanes, args.steps, args.warmup)
    clk = clocks.stop()
    t_step = float(np.mean(step_ms)) * 1e-3
    if world > 1:
        tt = torch.tensor([t_step], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step = float(tt.item())
    value = world * n / t_step

    # ---- e2e through the public API on host arrays
    h2d = Xo.nbytes + yo.nbytes + Zo.nbytes + prob.nblk * (4 + 4 + 4 * prob.ldnbr + 4) + 8 * len(theta)
    d2h = 8 * (1 + P + P * P + 1) + 16
    for _ in range(2):
        sv.vecchia_profile_loglik(theta, Xo, yo, Zo, groups, nu, precision="split")
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ll_e2e = sv.vecchia_profile_loglik(theta, Xo, yo, Zo, groups, nu, precision="split")[0]
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / args.steps
    if world > 1:
        tt = torch.tensor([t_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.item())

    if rank != 0:
        torch.distributed.destroy_process_group()
        return

    # ---- the other forms and smoothness values of the same workload
    forms = {}
    if not args.no_forms:
        ms64 = float(np.mean(time_form("float64", 0, max(2, args.steps // 2), 1)))
        forms["float64"] = {"ms": ms64, "blocks_per_s": n / (ms64 * 1e-3)}
        df_lanes, df_ms = best_width("split_df")
        res_df = prob.evaluate(theta, nu, precision="split_df", team_lanes=df_lanes)
        forms["split_df"] = {"ms": df_ms[df_lanes], "blocks_per_s": n / (df_ms[df_lanes] * 1e-3),
                             "team_lanes": df_lanes, "team_lanes_ms": df_ms,
                             "factorisation": "double-float (float32 pairs, ~46 bits)",
                             "errors_vs_float64_form": errors_vs(res64, res_df)}
        for nu_o in (1.5,):
            ms_s = float(np.mean(time_form("split", best_lanes, max(2, args.steps // 2), 1, nu_o)))
            ms_f = float(np.mean(time_form("float64", 0, max(2, args.steps // 2), 1, nu_o)))
            r_s = prob.evaluate(theta, nu_o, precision="split", team_lanes=best_lanes)
            r_f = prob.evaluate(theta, nu_o)
            forms[f"nu{nu_o}"] = {"split_ms": ms_s, "split_blocks_per_s": n / (ms_s * 1e-3),
                                  "float64_ms": ms_f, "float64_blocks_per_s": n / (ms_f * 1e-3),
                                  "split_errors_vs_float64_form": errors_vs(r_f, r_s)}
        # linear trend (gp.py:99-100: Z = [1, x], q = d + 1 = 11 columns of
        # the GLS profiling gathered per block, likelihood.py:129-134)
        Zl = np.concatenate([np.ones((n, 1)), Xo], axis=1)
        prob_l = DeviceProblem(Xo, yo, Zl, groups)
        tl = {}
        for prec in ("split", "float64"):
            for _ in range(2):
                prob_l.launch(th_d, P, nu, False, True, 0.0, 0.0, True, precision=prec,
                              team_lanes=best_lanes if prec == "split" else 0)
            torch.cuda.synchronize()
            ev = []
            for _ in range(max(2, args.steps // 2)):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                prob_l.launch(th_d, P, nu, False, True, 0.0, 0.0, True, precision=prec,
                              team_lanes=best_lanes if prec == "split" else 0)
                e1.record(stream)
                ev.append((e0, e1))
            torch.cuda.synchronize()
            tl[prec] = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        rl_s = prob_l.evaluate(theta, nu, precision="split", team_lanes=best_lanes)
        rl_f = prob_l.evaluate(theta, nu)
        forms["trend_linear"] = {"q": int(Zl.shape[1]), "split_ms": tl["split"],
                                 "split_blocks_per_s": n / (tl["split"] * 1e-3),
                                 "float64_ms": tl["float64"],
                                 "float64_blocks_per_s": n / (tl["float64"] * 1e-3),
                                 "split_errors_vs_float64_form": errors_vs(rl_f, rl_s)}
        del prob_l
        # fixed nu = 0.8: general smoothness.  The split form assembles from
        # the call's float32 Matern table (deficit and g), the float64 form
        # takes M and g from its float64 table; both tables are built from the
        # device K_nu.  The per-entry Bessel routine (a batched evaluation
        # without tables) once, as the float64 table's check
        ms08s = float(np.mean(time_form("split", best_lanes, max(2, args.steps // 2), 1, 0.8)))
        r_s08 = prob.evaluate(theta, 0.8, precision="split", team_lanes=best_lanes)
        redone08 = int(prob.last_info[3])
        ms08 = float(np.mean(time_form("float64", 0, max(2, args.steps // 2), 1, 0.8)))
        from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem
        r_tab = prob.evaluate(theta, 0.8)
        BL08 = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=0.8)], matern_tables=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st08, *r_bes = BL08.evaluate([theta])[0]
        torch.cuda.synchronize()
        ms_bes = (time.perf_counter() - t0) * 1e3
        del BL08
        forms["nu0.8"] = {"split_ms": ms08s, "split_blocks_per_s": n / (ms08s * 1e-3),
                          "split_blocks_redone_in_float64": redone08,
                          "split_errors_vs_float64_form": errors_vs(r_tab, r_s08),
                          "float64_ms": ms08, "float64_blocks_per_s": n / (ms08 * 1e-3),
                          "kernel": "split: float32 deficit and g from an 8-term float32 "
                                    "Chebyshev table; float64: M and g from a 16-term float64 "
                                    "table; both of the device K_nu for the fixed nu",
                          "per_entry_bessel_ms": ms_bes,
                          "table_vs_per_entry_bessel": errors_vs(tuple(r_bes), r_tab),
                          "bessel_k": bessel_error(torch, lib, Xo, nn, theta, 0.8)}
        # estimated nu (the reference's nu=None; log nu in theta at nu = 1.3):
        # M and g at nu and M at nu +- h (the central difference for dM/dnu)
        # from the evaluation's three tables; the per-entry Bessel routine (a
        # batched evaluation without tables) once, as their check
        nu_e = 1.3
        th_e = np.concatenate([theta[:-1], [math.log(nu_e)], theta[-1:]])
        th_e_d = _lib.to_dev(torch, th_e, np.float64)
        prob.launch(th_e_d, P + 1, None, True, True, 0.0, 0.0, True)
        torch.cuda.synchronize()
        ev = []
        for _ in range(max(2, args.steps // 2)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prob.launch(th_e_d, P + 1, None, True, True, 0.0, 0.0, True)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        ms_et = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        r_et = prob.evaluate(th_e, None, estimate_nu=True)
        # the split form: float32 tables of D, g and dM/dnu at this theta
        prob.launch(th_e_d, P + 1, None, True, True, 0.0, 0.0, True, precision="split",
                    team_lanes=best_lanes)
        torch.cuda.synchronize()
        ev = []
        for _ in range(max(2, args.steps // 2)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prob.launch(th_e_d, P + 1, None, True, True, 0.0, 0.0, True, precision="split",
                        team_lanes=best_lanes)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        ms_es = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        r_es = prob.evaluate(th_e, None, estimate_nu=True, precision="split", team_lanes=best_lanes)
        redone_e = int(prob.last_info[3])
        BLe = BatchedLikelihood([BatchProblem(Xo, yo, Zo, groups, nu=None, estimate_nu=True)],
                                matern_tables=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st_e, *r_eb = BLe.evaluate([th_e])[0]
        torch.cuda.synchronize()
        ms_eb = (time.perf_counter() - t0) * 1e3
        del BLe
        forms["nu_estimated"] = {"nu": nu_e, "split_ms": ms_es,
                                 "split_blocks_per_s": n / (ms_es * 1e-3),
                                 "split_blocks_redone_in_float64": redone_e,
                                 "split_errors_vs_float64_form": errors_vs(r_et, r_es),
                                 "float64_ms": ms_et,
                                 "float64_blocks_per_s": n / (ms_et * 1e-3),
                                 "kernel": "split: float32 tables of D, g and dM/dnu; float64: M and "
                                           "g at nu and M at nu +- h from three Chebyshev tables; "
                                           "all of the device K_nu",
                                 "per_entry_bessel_ms": ms_eb,
                                 "table_vs_per_entry_bessel": errors_vs(tuple(r_eb), r_et)}

    peak = measured_peak(lib, torch, "fp64")
    peak32 = measured_peak(lib, torch, "fp32")
    achieved = flops / t_step / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": "blocks/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 distances/Matern/dSigma.a/Gram + f64 LDL^T, solves, log-determinant, "
                 "likelihood sums (split form)",
        "data": "synthetic (seeded; y = Vecchia draw computed on the host, the same arrays as "
                "the reference arm)",
        "config": {"workload": f"loglik+score+Fisher, n={n}, d={d}, m={m}, nu={nu}, split form",
                   "n": n, "d": d, "m": m, "nu": nu, "blocks_per_step": n,
                   "l2": "flushed between steps (256 MB write, outside the step time)",
                   "parallelism": f"{world} independent problem(s), one per GPU"},
        "e2e": {"value": world * n / t_e2e, "unit": "blocks/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches_per_step * args.steps),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": (SPLIT64_TRAFFIC_PER_BLOCK * n
                                 if SPLIT64_TRAFFIC_PER_BLOCK and n == 200000 else None),
                     "peak_source": "float64 FMA probe measured in this run (sv_fp64_fma_probe); "
                                    "MEASURED_PEAKS.json has no float64 figure",
                     "basis": "achieved = K^3/3 + (P+2)K^2 float64 flops per block (LDL^T, a, "
                              "W, z) / mean step time (the whole evaluation, of which the block "
                              "kernel is the dominant launch); traffic = DRAM bytes per block of "
                              "an ncu capture of the block kernel at this size x blocks",
                     "fp32_probe_tflops": peak32},
        "clocks": clk,
        "extra": {"ll_split": res[0], "ll_float64": res64[0], "ll_e2e": ll_e2e,
                  "split_errors_vs_float64_form": errors_vs(res64, res),
                  "blocks_refactored_in_float64": int(prob.last_info[3]),
                  "team_lanes_ms": lane_ms, "team_lanes": best_lanes,
                  "maximin_s": t_maximin, "knn_s": t_knn, "maximin_tree": maximin_tree,
                  "order_matches_oracle": order_ok, "nn_matches_oracle": nn_ok,
                  "step_ms_all": step_ms, "forms": forms},
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        from oracle import oracle
        oracle.build()
        tcpu, out = cpu_reference_eval(Xo, yo, Zo, groups, theta, nu, threads)
        line["cpu_baseline"] = {"value": n / tcpu, "unit": "blocks/s", "cores": threads,
                                "kind": "port",
                                "sample": f"one full evaluation of all {n} blocks "
                                          "(C restatement of the reference's Numba loops, OpenMP)"}
        line["extra"]["ll_cpu"] = out[0]
        line["extra"]["split_errors_vs_oracle"] = errors_vs(out, res)
        line["extra"]["float64_errors_vs_oracle"] = errors_vs(out, res64)
    if not args.no_c1:
        from pyscaledvecchia_gb300 import ScaledVecchiaGP
        line["c1"] = run_c1(lambda: ScaledVecchiaGP(**C1_SETTINGS), reps=3)
    if args.fits_problems > 0:
        line["fits"] = run_fits(torch, lib, args.fits_problems, args.fits_dump)
    if not args.no_predict:
        line["predict"] = run_predict(torch, lib, check_oracle=not args.no_cpu_baseline)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
