"""Several GPUs, one process each: the likelihood of one problem split by
blocks, and batched fits split by problem.

No counterpart in the reference, which runs on one host; the arithmetic is
the reference's (likelihood.py:66-175, gp.py:138-239) unchanged.

One problem across ranks (``ShardedLikelihood``): Vecchia blocks are
independent given the ordering and neighbour sets, so each rank evaluates
the blocks of its share of the evaluation's reduction partitions (contiguous
runs of blocks, fixed by the block count; sv_loglik_shard_sizes) with the
same kernels as one GPU would, and four stages exchange what the passes of
likelihood.py share, each by an element-wise all-reduce:
  1. the jitter level each chunk needs (MAX; the reference retries a whole
     chunk with its largest level, _covariance.py:235-259, and a chunk may
     straddle ranks);
  2. the pass-1 partial sums of every partition (log L_KK, Z'y, Z'Z and the
     Fisher information; SUM of rows that only one rank fills);
  3. the pass-2 partial sums once every rank has solved for beta
     (likelihood.py:146-162; SUM likewise);
  4. the totals, the variance penalty and beta.
A partition's partial sums are the same bits whichever rank computes them
and the SUM exchanges add exact zeros, so the sharded result is bit for bit
that of one GPU (tested on one GPU by running the shards' stages in turn,
and with world_size-2 gloo process groups on CPU with the oracle as each
rank's evaluator).

Batched fits across ranks (``fit_batched_sharded``): problems are
independent, so each rank fits its share with ``fit_batched`` and the fitted
parameters are exchanged afterwards; the share balances the estimated cost
sum over blocks of K^3 by longest-processing-time assignment.  Each fit is
the one-GPU fit bit for bit.

Every GPU holds the whole problem (X, y, Z and the block table: 45.6 MB at
n = 200,000, d = 10, m = 30); only the block work is divided.  Exchanges
are torch.distributed all-reduces (NCCL between GPUs); no kernel reads
another GPU's memory.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

__all__ = ["ShardedLikelihood", "DeviceShard", "sharded_evaluate", "partition_range",
           "problem_cost", "assign_problems", "fit_batched_sharded"]


def partition_range(nparts, rank, world):
    """The contiguous run [begin, end) of nparts partitions that rank owns."""
    return (nparts * rank) // world, (nparts * (rank + 1)) // world


def _torch_allreduce(group):
    import torch.distributed as dist

    def allreduce(t, op):
        dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM, group=group)
        return t
    return allreduce


def sharded_evaluate(ev, theta, allreduce):
    """The four stages of a sharded evaluation on stage evaluator ``ev``
    (``DeviceShard``, or a CPU stand-in with the same methods), exchanging
    through ``allreduce(tensor, op)`` (op "max" or "sum", in place).
    Returns what ``ev.stage4`` returns."""
    cm = allreduce(ev.stage1(theta), "max")
    p1 = allreduce(ev.stage2(cm), "sum")
    p2 = allreduce(ev.stage3(p1), "sum")
    return ev.stage4(p2)


class DeviceShard:
    """One rank's share of a one-problem evaluation on its GPU: the blocks of
    reduction partitions [part_begin, part_end) of ``prob`` (a
    likelihood.DeviceProblem holding the whole problem) through
    sv_vecchia_loglik_stage.  Exchange buffers are device tensors."""

    def __init__(self, prob, part_begin, part_end, nu, P, estimate_nu=False, need_grad=True,
                 var_penalty=0.0, log_var_target=0.0, precision="float64", team_lanes=0):
        from .likelihood import _PRECISION
        self.prob, self.torch, self.lib = prob, prob.torch, prob.lib
        torch, lib = self.torch, self.lib
        self.P, self.nu, self.estimate_nu, self.need_grad = P, nu, estimate_nu, need_grad
        D = _lib.LoglikDesc()
        D.n, D.nblk, D.nblk_warp = prob.n, prob.nblk, prob.nblk_warp
        D.d, D.q, D.ldnbr, D.kmax = prob.d, prob.q, prob.ldnbr, prob.kmax
        D.need_grad, D.estimate_nu, D.chunked = int(bool(need_grad)), int(bool(estimate_nu)), 1
        D.precision, D.team_lanes = _PRECISION[precision], int(team_lanes)
        D.nu = float(nu) if nu is not None else 1.0
        D.var_penalty, D.log_var_target = float(var_penalty), float(log_var_target)
        self.desc = D
        parts, l1, l2 = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _lib.check(lib, lib.sv_loglik_shard_sizes(D, ctypes.byref(parts), ctypes.byref(l1),
                                                  ctypes.byref(l2)), "sv_loglik_shard_sizes")
        self.parts, self.len1, self.len2 = parts.value, l1.value, l2.value
        if not (0 <= part_begin <= part_end <= self.parts):
            raise ValueError("partition range outside the problem's partitions")
        self.pb, self.pe = int(part_begin), int(part_end)
        self.ws = _lib.workspace(torch, lib.sv_loglik_workspace_bytes(D))
        self.chunk = prob.chunk_tensor(P if need_grad else 1)
        self.out = torch.empty(1 + P + P * P + prob.q, dtype=torch.float64, device="cuda")
        self.info = _lib.new_info(torch)

    def _stage(self, stage, cm, p1, p2):
        P_ = _lib.ptr
        pr = self.prob
        rc = self.lib.sv_vecchia_loglik_stage(
            self.desc, stage, self.pb, self.pe, P_(self.theta), P_(pr.X), P_(pr.y), P_(pr.Z),
            P_(pr.rowb), P_(pr.kb), P_(pr.nbr), P_(self.chunk), P_(cm), P_(p1), P_(p2),
            P_(self.out), P_(self.info), P_(self.ws), self.ws.numel(), _lib.stream_handle(self.torch))
        _lib.check(self.lib, rc, "sv_vecchia_loglik_stage")

    def stage1(self, theta):
        torch = self.torch
        self.theta = _lib.to_dev(torch, np.asarray(theta, dtype=np.float64)[:self.P], np.float64)
        self.cm = torch.zeros(max(self.prob.nblk, 1), dtype=torch.int32, device="cuda")
        self.p1 = torch.zeros((self.parts, self.len1), dtype=torch.float64, device="cuda")
        self.p2 = torch.zeros((self.parts, self.len2), dtype=torch.float64, device="cuda")
        self._stage(1, self.cm, self.p1, self.p2)
        return self.cm

    def stage2(self, chunk_max):
        self._stage(2, chunk_max, self.p1, self.p2)
        return self.p1

    def stage3(self, part1):
        self._stage(3, self.cm, part1, self.p2)
        return self.p2

    def stage4(self, part2):
        self._stage(4, self.cm, self.p1, part2)
        return self.out, self.info


class ShardedLikelihood:
    """vecchia_profile_loglik of one problem on the GPUs of a process group:
    this rank evaluates its share of the blocks (``partition_range``) and the
    ranks exchange partial sums; every rank returns the same (ll, grad,
    fisher, beta), bit for bit the one-GPU result.  Xo, yo, Zo, groups as
    for vecchia_profile_loglik, the same on every rank."""

    def __init__(self, Xo, yo, Zo, groups, group=None):
        import torch.distributed as dist
        from .likelihood import DeviceProblem
        self.prob = DeviceProblem(Xo, yo, Zo, groups)
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self._shards = {}

    def evaluate(self, theta, nu, estimate_nu=False, need_grad=True, var_penalty=0.0,
                 log_var_target=0.0, precision="float64", team_lanes=0):
        import torch.distributed as dist
        theta = np.asarray(theta, dtype=float).reshape(-1)
        d = self.prob.d
        P = d + 3 if estimate_nu else d + 2
        key = (float(nu) if nu is not None else None, bool(estimate_nu), bool(need_grad),
               float(var_penalty), float(log_var_target), precision, int(team_lanes))
        if key not in self._shards:
            sh = DeviceShard(self.prob, 0, 0, nu, P, estimate_nu, need_grad, var_penalty,
                             log_var_target, precision, team_lanes)
            sh.pb, sh.pe = partition_range(sh.parts, self.rank, self.world)
            self._shards[key] = sh
        sh = self._shards[key]
        out, info = sharded_evaluate(sh, theta, _torch_allreduce(self.group))
        dist.all_reduce(info, op=dist.ReduceOp.MAX, group=self.group)
        res = out.cpu().numpy()
        _lib.check_info(self.prob.lib, info.cpu().numpy(), "sv_vecchia_loglik_stage")
        q = self.prob.q
        beta = res[1 + P + P * P:1 + P + P * P + q].copy()
        if not need_grad:
            return float(res[0]), None, None, beta
        return (float(res[0]), res[1:1 + P].copy(), res[1 + P:1 + P + P * P].reshape(P, P).copy(),
                beta)


# ---------------------------------------------------------------------------
# batched fits by problem
# ---------------------------------------------------------------------------
def problem_cost(n, m_est, n_est):
    """Estimated evaluation cost of a fit: the sum over its blocks of K^3
    (the factorisation's share), for the rows it fits (n_est subsample) and
    its neighbour count."""
    n_eff = min(n, n_est) if n_est is not None else n
    m = max(min(m_est, n_eff - 1), 0)
    small = sum((k + 1) ** 3 for k in range(min(m, n_eff)))
    return float(small + max(n_eff - m, 0) * (m + 1) ** 3)


def assign_problems(costs, world):
    """Rank of every problem: longest processing time first (costs
    descending, ties by index), each to the least-loaded rank (ties to the
    lowest rank).  Deterministic, so every rank computes the same table."""
    load = [0.0] * world
    owner = [0] * len(costs)
    for i in sorted(range(len(costs)), key=lambda j: (-costs[j], j)):
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += costs[i]
    return owner


_FITTED = ("theta_", "beta_", "loglik_", "b_", "_nu_fit")


def fit_batched_sharded(models, Xs, ys, group=None, fit_fn=None, rank=None, world=None,
                        allgather=None, **kw):
    """``fit_batched`` with the models divided among the ranks of a process
    group: every rank fits its share (``assign_problems`` on
    ``problem_cost``) and receives the others' fitted parameters, so every
    rank returns all models fitted.  ``fit_fn`` (default fit_batched) is the
    fitting routine; ``rank``, ``world`` and ``allgather`` (a list of every
    rank's object) default to those of torch.distributed on ``group``.
    Keyword arguments go to fit_fn."""
    if fit_fn is None:
        from .fit_batched import fit_batched as fit_fn
    if allgather is None or rank is None or world is None:
        import torch.distributed as dist
        rank = dist.get_rank(group) if rank is None else rank
        world = dist.get_world_size(group) if world is None else world
        if allgather is None:
            def allgather(obj):
                out = [None] * world
                dist.all_gather_object(out, obj, group=group)
                return out
    costs = [problem_cost(np.asarray(X).shape[0], m.m_est, m.n_est) for m, X in zip(models, Xs)]
    owner = assign_problems(costs, world)
    mine = [i for i in range(len(models)) if owner[i] == rank]
    if mine:
        fit_fn([models[i] for i in mine], [Xs[i] for i in mine], [ys[i] for i in mine], **kw)
    payload = {i: {k: getattr(models[i], k) for k in _FITTED + ("fit_stats_",)
                   if hasattr(models[i], k)} for i in mine}
    for part in allgather(payload):
        for i, st in part.items():
            if owner[i] == rank:
                continue
            m = models[i]
            m._fit_prepare(Xs[i], ys[i])  # standardisation of the model's own data (host)
            for k, v in st.items():
                setattr(m, k, v)
    return models
