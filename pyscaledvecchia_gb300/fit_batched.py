"""Fit many ScaledVecchiaGP models together (batched Fisher scoring).

Each model is fitted exactly as ScaledVecchiaGP.fit does (gp.py:138-239):
the same standardisation, subsample, initial theta, clipping, nugget freeze,
reorders at iterations 2, 4, 8, 16 and variance correction.  What changes is
the schedule: every model's Fisher-scoring iteration runs as a generator
(optimize.fisher_scoring_steps), and each round answers the pending
objective requests of all models with one batched likelihood launch per
precision (sv_vecchia_loglik_batched), replayed from a CUDA graph.

precision="split" runs the iterations on the split-precision kernels
(float32 assembly, float64 factorisation; "split_df": double-float
factorisation) and then continues each model in float64 from where it
stopped ("polish", no reorders) until the float64 iteration stops too, so the
reported loglik, theta and beta are float64 results.  precision="float64" runs float64
throughout (the fitted theta then follows the reference's own iteration).
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .batched import BatchedLikelihood, BatchProblem, ordered_groups
from .optimize import EVAL_FAILED, fisher_scoring_steps

__all__ = ["fit_batched"]


class _Fit:
    """Host state of one model in a batched fit."""

    def __init__(self, model, X, y, theta0=None):
        self.model = model
        self.st = model._fit_prepare(X, y)
        self.d = self.st["d"]
        self.est = self.st["estimate_nu"]
        if theta0 is not None:
            th = np.array(theta0, dtype=float).reshape(-1)
            if th.shape[0] != self.st["theta0"].shape[0]:
                raise ValueError("initial theta has the wrong length")
            self.st["theta0"] = model._clip_theta(th, self.d, self.est)
        self.last_ranges = np.exp(self.st["theta0"][1:1 + self.d]).copy()
        self.phase = "main"
        self.gen = None
        self.msg = None
        self.result = None
        self.evals = {"split": 0, "float64": 0}
        self.iters = 0

    def problem(self):
        """The problem with the ordered-search block layout; its rows and
        neighbours are filled in by the first rebuild."""
        st = self.st
        n = st["Xe"].shape[0]
        return BatchProblem(st["Xe"], st["ye"], st["Ze"], ordered_groups(n, st["m"]),
                            nu=self.model.nu, estimate_nu=self.est,
                            var_penalty=self.model.var_penalty,
                            log_var_target=st["log_var_target"])


def fit_batched(models, Xs, ys, *, precision="split", graphs=True, init_thetas=None,
                warm_start=None, warm_judge=False, team_lanes=0, polish_iter=5, verbose=False,
                stats=None, overlap_reorders=True):
    """Fit ``models[i]`` to ``(Xs[i], ys[i])`` for every i, together.

    models : ScaledVecchiaGP instances (each keeps its own settings)
    precision : "split" (split-precision iterations + float64 polish),
            "split_df" (the same on the double-float split kernel) or
            "float64" (every evaluation in float64: the fitted parameters are
            bit for bit those of ScaledVecchiaGP.fit)
    polish_iter : float64 Fisher-scoring iterations after the split phase
            (it re-anchors the split iterate in float64; near parameter
            clips the iteration can crawl for its whole budget)
    graphs : replay each batched evaluation from a captured CUDA graph
    init_thetas : optional per-model starting log-parameters (a warm start);
            None entries use the model's default initialisation
    warm_start : optional warmstart.SetEncoder; its prediction from each
            model's standardised estimation set is the starting point
            (fixed nuggets and an estimated nu keep their default entries;
            models it does not apply to keep the default start)
    warm_judge : with warm_start, fit every model from both starts in the
            same batch and keep the fit with the larger converged loglik
            (the default start on ties): Fisher scoring with reorders at the
            iterates is path dependent, and this way the network moves only
            the starting point and never makes the answer worse
    stats : optional dict that receives the schedule's counters (rounds,
            batched launches, reorder calls, seconds in each part) and the
            batch itself under "batch" (for diagnostics)
    overlap_reorders : rebuild the problems that asked for a reorder on a
            side stream while the others' evaluation round runs; they join
            the next round.  Every problem takes the same steps either way
            (its own evaluations and reorders in its own order), so the
            fitted parameters are the same bit for bit
    Returns the list of fitted models.  Per-model counters are left in
    ``model.fit_stats_`` (objective evaluations per precision).
    """
    import time
    t_start = time.perf_counter()
    cnt = {"rounds": 0, "launches": 0, "reorder_calls": 0, "reordered_problems": 0,
           "t_setup": 0.0, "t_reorder": 0.0, "t_eval": 0.0, "t_host": 0.0}
    if precision not in ("split", "split_df", "float64"):
        raise ValueError("precision must be 'split', 'split_df' or 'float64'")
    if not (len(models) == len(Xs) == len(ys)):
        raise ValueError("models, Xs and ys must have the same length")
    if len(models) == 0:
        return []
    _lib.device_ready()
    fits = [_Fit(mdl, X, y, None if init_thetas is None else init_thetas[i])
            for i, (mdl, X, y) in enumerate(zip(models, Xs, ys))]
    owner = list(range(len(fits)))
    if warm_start is not None and warm_judge:
        # second copy of every fit: the warm start goes to the copies
        fits = fits + [_Fit(mdl, X, y, None if init_thetas is None else init_thetas[i])
                       for i, (mdl, X, y) in enumerate(zip(models, Xs, ys))]
        owner = owner + list(range(len(models)))
    nmod = len(models)
    if warm_start is not None:
        t_ws = time.perf_counter()
        tgt = fits[nmod:] if warm_judge else fits
        pred = warm_start.initial_thetas([(f.st["Xe"], f.st["ye"]) for f in tgt])
        for f, th in zip(tgt, pred):
            if th is None:
                continue
            t0 = f.st["theta0"].copy()
            t0[:1 + f.d] = th[:1 + f.d]
            if f.model.nugget is None:
                t0[-1] = th[-1]
            f.st["theta0"] = f.model._clip_theta(t0, f.d, f.est)
            f.last_ranges = np.exp(f.st["theta0"][1:1 + f.d]).copy()
        cnt["t_warm_start"] = time.perf_counter() - t_ws
    precs = (precision, "float64") if precision != "float64" else ("float64",)
    BL = BatchedLikelihood([f.problem() for f in fits], need_grad=True, precisions=precs,
                           team_lanes=team_lanes)
    BL.set_sources([f.st["Xe"] for f in fits], [f.st["ye"] for f in fits],
                   [f.st["Ze"] for f in fits], [f.st["m"] for f in fits])

    import torch
    side = torch.cuda.Stream() if overlap_reorders else None

    def rebuild(ids, thetas, deferred=False):
        """gp.py:182-191 for several fits: one batched device call for the
        problems that fit a cluster, the one-problem path for the rest.
        deferred: the device call on the side stream, returned unfinished
        (a function that waits for it), or None when there was none."""
        t0 = time.perf_counter()
        cnt["reorder_calls"] += 1
        cnt["reordered_problems"] += len(ids)
        dev = [(i, th) for i, th in zip(ids, thetas) if BL.device_reorderable(i)]
        finish = None
        if dev:
            if deferred:
                side.wait_stream(torch.cuda.current_stream())
                finish = BL.reorder([i for i, _ in dev], [th for _, th in dev], stream=side,
                                    deferred=True)
            else:
                BL.reorder([i for i, _ in dev], [th for _, th in dev])
        for i, th in zip(ids, thetas):
            if BL.device_reorderable(i):
                continue
            f = fits[i]
            order, groups = f.model._order_and_neighbours(f.st["Xe"], th, f.d, f.st["m"])
            BL.update_problem(i, f.st["Xe"][order], f.st["ye"][order], f.st["Ze"][order], groups)
        cnt["t_reorder"] += time.perf_counter() - t0
        return finish

    rebuild(list(range(len(fits))), [f.st["theta0"] for f in fits])
    if graphs:
        for p in precs:
            BL.capture(p)

    cnt["t_setup"] = time.perf_counter() - t_start - cnt["t_reorder"]
    main_prec = precs[0]
    for f in fits:
        f.gen = fisher_scoring_steps(f.st["theta0"], max_iter=f.model.max_iter,
                                     tol=f.model.tol, verbose=verbose and f.model.verbose)
        f.msg = next(f.gen)
        f.prec = main_prec

    def advance(f, reply):
        try:
            f.msg = f.gen.send(reply)
        except StopIteration as stop:
            theta, ll, beta = stop.value
            if f.phase == "main" and precision != "float64":
                # float64 polish from the split iterate, no reorders
                f.phase = "polish"
                f.prec = "float64"
                f.gen = fisher_scoring_steps(theta, max_iter=min(f.model.max_iter, polish_iter),
                                             tol=f.model.tol, reorder=False)
                f.msg = next(f.gen)
            else:
                f.phase = "done"
                f.msg = None
                f.result = (theta, ll, beta)

    nprob = len(fits)
    inflight = None  # (fits being rebuilt on the side stream, the wait for it)
    while True:
        # reorder requests (gp.py:211-221): the ones whose ranges moved are
        # rebuilt together in one batched call (on the side stream, those
        # fits sitting out this round, when overlap_reorders)
        while inflight is None:
            req = [i for i, f in enumerate(fits) if f.msg is not None and f.msg[0] == "reorder"]
            if not req:
                break
            todo, ths = [], []
            for i in req:
                f = fits[i]
                _, th, k = f.msg
                r = f.model._reorder_ranges(th, f.d, f.est, f.last_ranges, k)
                if r is None:
                    advance(f, False)
                    continue
                todo.append(i)
                ths.append(th)
                f.last_ranges = r.copy()
            if todo:
                if overlap_reorders:
                    finish = rebuild(todo, ths, deferred=True)
                    inflight = (todo, finish)
                    break
                rebuild(todo, ths)
                for i in todo:
                    advance(fits[i], True)
        waiting = set(inflight[0]) if inflight is not None else set()
        pend = [i for i, f in enumerate(fits)
                if f.msg is not None and f.msg[0] != "reorder" and i not in waiting]
        if not pend:
            if inflight is not None:
                todo, finish = inflight
                inflight = None
                t0 = time.perf_counter()
                if finish is not None:
                    finish()
                cnt["t_reorder"] += time.perf_counter() - t0
                for i in todo:
                    advance(fits[i], True)
                continue
            if any(f.msg is not None for f in fits):
                continue
            break
        thetas = [None] * nprob
        masks = {p: np.zeros(nprob, dtype=bool) for p in precs}
        for i in pend:
            f = fits[i]
            thetas[i] = f.model._objective_theta(f.msg[1], f.d, f.est)
            masks[f.prec][i] = True
        t0 = time.perf_counter()
        BL.set_theta(thetas)
        for p in precs:
            if masks[p].any():
                BL.set_active(masks[p], p)
        for p in precs:
            if masks[p].any():
                BL.run(p)
                cnt["launches"] += 1
        out, info = BL.fetch()
        cnt["rounds"] += 1
        cnt["t_eval"] += time.perf_counter() - t0
        for i in pend:
            f = fits[i]
            st, ll, g, M, beta = BL.unpack(out, info, i)
            f.evals["float64" if f.prec == "float64" else "split"] += 1
            if st == _lib.SV_ECHOL:
                advance(f, EVAL_FAILED)
                continue
            if st != _lib.SV_OK:
                _lib.check_info(BL.lib, info[i], "sv_vecchia_loglik_batched")
            g, M = f.model._freeze_nugget(g, M)
            advance(f, (ll, g, M, beta))
        if inflight is not None:
            # the side stream's rebuild: its fits take the next round
            todo, finish = inflight
            inflight = None
            t0 = time.perf_counter()
            if finish is not None:
                finish()
            cnt["t_reorder"] += time.perf_counter() - t0
            for i in todo:
                advance(fits[i], True)

    cnt["t_total"] = time.perf_counter() - t_start
    cnt["t_host"] = cnt["t_total"] - cnt["t_setup"] - cnt["t_reorder"] - cnt["t_eval"]
    if stats is not None:
        stats.update(cnt)
        stats["batch"] = BL
        stats["thetas"] = [f.result[0] for f in fits]
    best = {}
    for i, f in enumerate(fits):
        o = owner[i]
        if o not in best or f.result[1] > best[o].result[1]:
            best[o] = f
    for o, f in best.items():
        theta, ll, beta = f.result
        f.model._fit_finish(f.st, theta, ll, beta)
        ev = {"split": 0, "float64": 0}
        for i, g in enumerate(fits):
            if owner[i] == o:
                for k in ev:
                    ev[k] += g.evals[k]
        f.model.fit_stats_ = ev
    return models
