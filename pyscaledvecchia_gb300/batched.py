"""Many independent Vecchia likelihoods evaluated together on the GPU.

The reference fits one problem at a time (gp.py:138-239); the per-problem
arithmetic here is still likelihood.py:66-175, but the blocks of all
problems go through one set of kernel launches (sv_vecchia_loglik_batched):
each problem keeps its own inputs, conditioning sets, parameters, outputs
and status words, and a per-block problem index lets the block kernels mix
problems freely.  Problems can be switched off per call (``active``), so a
captured CUDA graph of one evaluation can be replayed while problems finish
at different times.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._covariance import _check_nu
from .likelihood import _PRECISION, _SPLIT, _WARP_K, chunk_ids, pack_groups
from .ordering import _nn_groups

_POOL = None


def _host_pool():
    """Worker threads for per-problem host arithmetic (numpy), created once."""
    global _POOL
    if _POOL is None:
        import concurrent.futures as cf
        _POOL = cf.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))
    return _POOL


__all__ = ["BatchProblem", "BatchedLikelihood", "ordered_groups"]


class OrderedGroups(list):
    """The _nn_groups structure (ordering.py:119-127) of an ordered
    m-neighbour search over n rows, with placeholder (zero) neighbour
    indices: row i alone in group i for i < m, rows m..n-1 in group m.  The
    layout a device reorder fills in; BatchedLikelihood packs it without
    walking the groups."""

    def __init__(self, n, m):
        n, m = int(n), int(m)
        zero = np.zeros(1, dtype=np.int64)
        groups = [(np.array([k], dtype=np.int64), np.broadcast_to(zero, (1, k)))
                  for k in range(min(n, m))]
        if n > m:
            groups.append((np.arange(m, n, dtype=np.int64), np.broadcast_to(zero, (n - m, m))))
        super().__init__(groups)
        self.n, self.m = n, m


def ordered_groups(n, m):
    """The _nn_groups structure of an ordered m-neighbour search over n rows
    (row i has min(i, m) neighbours), with placeholder neighbour indices."""
    return OrderedGroups(n, m)


def _pack_ordered(n, m):
    """pack_groups of OrderedGroups(n, m) (m + 1 <= 32: no reordering of
    large blocks), built directly: block i = row i with min(i, m)
    neighbours, group i for i < m, group m for the rest.  The neighbour table
    is None: its placeholders (row 0) are written straight into the batch's
    table, and a device reorder writes every row's neighbours."""
    kb = np.minimum(np.arange(n), m).astype(np.int32)
    rowb = np.arange(n, dtype=np.int32)
    gk = list(range(min(n, m))) + ([m] if n > m else [])
    gl = [1] * min(n, m) + ([n - m] if n > m else [])
    return rowb, kb, None, kb.copy(), gk, gl


@dataclass
class BatchProblem:
    """One likelihood of a batch: inputs in Vecchia order plus the settings
    of vecchia_profile_loglik (likelihood.py:66-75)."""
    Xo: np.ndarray
    yo: np.ndarray
    Zo: Optional[np.ndarray]
    groups: list
    nu: Optional[float] = 2.5
    estimate_nu: bool = False
    var_penalty: float = 0.0
    log_var_target: float = 0.0


class BatchedLikelihood:
    """Device-resident inputs of a batch of likelihood problems.

    Layout in device memory: X, y and Z of all problems concatenated
    (row-major per problem), blocks of problem p contiguous at
    [blk_off_p, blk_off_p + nblk_p) with row indices local to the problem,
    neighbour lists padded to the batch's largest k.  ``theta`` is
    (nprob, Pmax), ``out`` (nprob, 1 + Pmax + Pmax^2 + qmax), ``info``
    (nprob, 4).
    """

    def __init__(self, problems, need_grad=True, chunked=True, precisions=("float64",),
                 team_lanes=0, split_rho_min=0.0, matern_tables=True):
        for pr in precisions:
            if pr not in _PRECISION:
                raise ValueError("precision must be 'float64', 'split' or 'split_df'")
        if len(problems) == 0:
            raise ValueError("a batch needs at least one problem")
        lib, torch = _lib.device_ready()
        self.lib, self.torch = lib, torch
        self.nprob = len(problems)
        self.need_grad = bool(need_grad)
        self.chunked = bool(chunked)
        self.precisions = tuple(precisions)
        self.team_lanes = int(team_lanes)
        self.split_rho_min = float(split_rho_min)

        self.n = np.empty(self.nprob, dtype=np.int64)
        self.d = np.empty(self.nprob, dtype=np.int64)
        self.q = np.empty(self.nprob, dtype=np.int64)
        self.P = np.empty(self.nprob, dtype=np.int64)
        self.estimate_nu = np.zeros(self.nprob, dtype=bool)
        xs, ys, zs = [], [], []
        packs = []
        for i, pr in enumerate(problems):
            X = np.ascontiguousarray(pr.Xo, dtype=np.float64)
            if X.ndim != 2:
                raise ValueError("X must be two-dimensional")
            y = np.ascontiguousarray(pr.yo, dtype=np.float64).reshape(-1)
            if y.shape[0] != X.shape[0]:
                raise ValueError("X and y have incompatible shapes")
            Z = None
            if pr.Zo is not None and np.asarray(pr.Zo).ndim == 2 and np.asarray(pr.Zo).shape[1] > 0:
                Z = np.ascontiguousarray(pr.Zo, dtype=np.float64)
                if Z.shape[0] != X.shape[0]:
                    raise ValueError("X and Z have incompatible shapes")
            if not pr.estimate_nu:
                _check_nu(pr.nu)
            self.n[i], self.d[i] = X.shape
            self.q[i] = Z.shape[1] if Z is not None else 0
            self.estimate_nu[i] = bool(pr.estimate_nu)
            self.P[i] = self.d[i] + 2 + (1 if pr.estimate_nu else 0)
            xs.append(X.reshape(-1))
            ys.append(y)
            if Z is not None:
                zs.append(Z.reshape(-1))
            if isinstance(pr.groups, OrderedGroups) and pr.groups.n == X.shape[0] and pr.groups.m + 1 <= _WARP_K:
                packs.append(_pack_ordered(pr.groups.n, pr.groups.m))
            else:
                packs.append(pack_groups(pr.groups, X.shape[0]))
        self.dmax = int(self.d.max())
        self.qmax = int(self.q.max())
        self.any_est = bool(self.estimate_nu.any())
        # a fixed nu without a closed form, or an estimated nu, in some
        # problem: the evaluation interpolates its Matern from per-problem
        # tables (matern_tables=False keeps the per-entry Bessel routine: the
        # check of the tables)
        self.general_nu = matern_tables and any(
            pr.estimate_nu or float(pr.nu) not in (0.5, 1.5, 2.5) for pr in problems)
        self.Pmax = self.dmax + 2 + (1 if self.any_est else 0)
        self.ostride = 1 + self.Pmax + self.Pmax * self.Pmax + self.qmax

        nblk = np.array([pk[0].shape[0] for pk in packs], dtype=np.int64)
        self.blk_off = np.concatenate([[0], np.cumsum(nblk)[:-1]]).astype(np.int64)
        self.nblk = nblk
        self.total_blocks = int(nblk.sum())
        self.kmax = max((int(pk[1].max()) if pk[1].shape[0] else 0) for pk in packs)
        self.ldnbr = max(self.kmax, 1)
        B = self.total_blocks
        rowb = np.empty(B, dtype=np.int32)
        kb = np.empty(B, dtype=np.int32)
        nbr = np.full((B, self.ldnbr), -1, dtype=np.int32)
        bprob = np.empty(B, dtype=np.int32)
        chunk = np.empty(B, dtype=np.int32)
        nchunk = 0
        for i, (rb, k, nb, gid, gk, gl) in enumerate(packs):
            o, c = int(self.blk_off[i]), rb.shape[0]
            rowb[o:o + c] = rb
            kb[o:o + c] = k
            if nb is not None:
                nbr[o:o + c, :nb.shape[1]] = nb
            else:  # ordered layout: row 0 as every neighbour placeholder
                mm = int(k.max()) if c else 0
                for r in range(min(c, mm)):
                    nbr[o + r, :r] = 0
                if c > mm:
                    nbr[o + mm:o + c, :mm] = 0
            bprob[o:o + c] = i
            ids = chunk_ids(gid, gk, gl, int(self.P[i]) if self.need_grad else 1)
            chunk[o:o + c] = ids + nchunk
            nchunk += int(ids.max()) + 1 if c else 0
        big = (kb + 1) > _WARP_K
        wlist = np.flatnonzero(~big).astype(np.int32)
        clist = np.flatnonzero(big).astype(np.int32)
        self.nwarp, self.ncta = wlist.shape[0], clist.shape[0]
        # one team width per launch of a split form: the given one, else the
        # autotuner's choice for the problem with the most blocks of at most
        # 32 points
        self._lanes = {prec: self.team_lanes for prec in self.precisions}
        for prec in self.precisions:
            if (prec in _SPLIT and self.team_lanes == 0 and self.nwarp > 0
                    and self.Pmax + 1 + self.qmax <= 32):
                from . import autotune
                wp = bprob[wlist]
                i = int(np.argmax(np.bincount(wp, minlength=self.nprob)))
                Kw = int(kb[wlist][wp == i].max()) + 1
                self._lanes[prec] = autotune.team_lanes(Kw, int(self.d[i]), int(self.q[i]),
                                                        self.need_grad, precision=prec)

        xlen = np.array([a.shape[0] for a in xs], dtype=np.int64)
        self.x_off = np.concatenate([[0], np.cumsum(xlen)[:-1]]).astype(np.int64)
        self.y_off = np.concatenate([[0], np.cumsum(self.n)[:-1]]).astype(np.int64)
        zlen = self.n * self.q
        self.z_off = np.concatenate([[0], np.cumsum(zlen)[:-1]]).astype(np.int64)
        self.nx = int(xlen.sum())

        dev = lambda a, t: _lib.to_dev(torch, a, t)
        self.X = dev(np.concatenate(xs), np.float64)
        self.y = dev(np.concatenate(ys), np.float64)
        self.Z = dev(np.concatenate(zs), np.float64) if zs else None
        self.rowb = dev(rowb, np.int32)
        self.kb = dev(kb, np.int32)
        self.nbr = dev(nbr, np.int32)
        self.bprob = dev(bprob, np.int32)
        self.wlist = dev(wlist, np.int32) if self.nwarp else None
        self.clist = dev(clist, np.int32) if self.ncta else None
        self.chunk = dev(chunk, np.int32) if self.chunked else None

        # problem table (host copy kept for the per-call skip flags)
        self._descs = (_lib.ProbDesc * self.nprob)()
        for i, pr in enumerate(problems):
            D = self._descs[i]
            D.n, D.x_off, D.y_off, D.z_off = int(self.n[i]), int(self.x_off[i]), int(self.y_off[i]), int(self.z_off[i])
            D.blk_off, D.nblk = int(self.blk_off[i]), int(self.nblk[i])
            D.d, D.q, D.estimate_nu, D.skip = int(self.d[i]), int(self.q[i]), int(bool(pr.estimate_nu)), 0
            D.nu = float(pr.nu) if pr.nu is not None else 1.0
            D.var_penalty, D.log_var_target = float(pr.var_penalty), float(pr.log_var_target)

        self._theta_host = torch.zeros((self.nprob, self.Pmax), dtype=torch.float64).pin_memory()
        self.theta = torch.zeros((self.nprob, self.Pmax), dtype=torch.float64, device="cuda")
        self.out = torch.zeros((self.nprob, self.ostride), dtype=torch.float64, device="cuda")
        self.info = torch.zeros((self.nprob, 4), dtype=torch.int32, device="cuda")
        self._res_host = torch.empty(self.nprob * self.ostride, dtype=torch.float64).pin_memory()
        self._info_host = torch.empty(self.nprob * 4, dtype=torch.int32).pin_memory()

        # one launch mode per precision: its own batch descriptor, problem
        # table (skip flags), staging buffer and graph; data and workspace shared
        self._modes = {}
        wsb = 0
        for prec in self.precisions:
            Bd = _lib.BatchDesc()
            Bd.nprob, Bd.nblk, Bd.nwarp, Bd.ncta, Bd.nx = self.nprob, B, self.nwarp, self.ncta, self.nx
            Bd.dmax, Bd.qmax, Bd.kmax, Bd.ldnbr = self.dmax, self.qmax, self.kmax, self.ldnbr
            Bd.need_grad, Bd.any_estimate_nu, Bd.chunked = int(self.need_grad), int(self.any_est), int(self.chunked)
            Bd.precision, Bd.team_lanes = _PRECISION[prec], self._lanes[prec]
            Bd.theta_stride, Bd.out_stride = self.Pmax, self.ostride
            Bd.general_nu = int(self.general_nu)
            Bd.split_rho_min = self.split_rho_min
            Bd.nblk_max = int(self.nblk.max())
            wsb = max(wsb, int(lib.sv_loglik_batched_workspace_bytes(Bd)))
            nb = ctypes.sizeof(self._descs)
            self._modes[prec] = {
                "bdesc": Bd, "graph": None, "active": None,
                "host": torch.empty(nb, dtype=torch.uint8).pin_memory(),
                "descs": torch.empty(nb, dtype=torch.uint8, device="cuda")}
            self.set_active(np.ones(self.nprob, dtype=bool), prec)
        self.ws = _lib.workspace(torch, wsb)

    # ---------------------------------------------------------------- inputs
    def set_active(self, active, precision=None):
        """Problems the given mode evaluates in the following launches (bool
        per problem); the others keep their previous out and info entries."""
        prec = precision or self.precisions[0]
        mode = self._modes[prec]
        a = np.asarray(active, dtype=bool).reshape(-1)
        if a.shape[0] != self.nprob:
            raise ValueError("active needs one flag per problem")
        if mode["active"] is not None and np.array_equal(a, mode["active"]):
            return
        mode["active"] = a.copy()
        for i in range(self.nprob):
            self._descs[i].skip = 0 if a[i] else 1
        # the staging buffer may still be in an earlier copy's flight
        self.torch.cuda.current_stream().synchronize()
        ctypes.memmove(mode["host"].data_ptr(), ctypes.addressof(self._descs), ctypes.sizeof(self._descs))
        mode["descs"].copy_(mode["host"], non_blocking=True)

    def set_theta(self, thetas):
        """thetas: per-problem vectors (>= P_p entries; None leaves a row as is)."""
        self.torch.cuda.current_stream().synchronize()
        th = self._theta_host.numpy()
        for i in range(self.nprob):
            if thetas[i] is None:
                continue
            v = np.asarray(thetas[i], dtype=np.float64).reshape(-1)
            P = int(self.P[i])
            if v.shape[0] < P:
                raise ValueError(f"theta of problem {i} has too few entries")
            th[i, :P] = v[:P]
        self.theta.copy_(self._theta_host, non_blocking=True)

    def update_problem(self, i, Xo, yo, Zo, groups):
        """Replace problem i's inputs and conditioning sets in place (after a
        reorder).  The block structure (k of every block) must be unchanged,
        as it is for every maximin reorder of the same rows."""
        torch = self.torch
        n, d = int(self.n[i]), int(self.d[i])
        X = np.ascontiguousarray(Xo, dtype=np.float64)
        if X.shape != (n, d):
            raise ValueError("reordered inputs must keep the problem's shape")
        rb, k, nb, *_ = pack_groups(groups, n)
        o, c = int(self.blk_off[i]), int(self.nblk[i])
        if rb.shape[0] != c or not np.array_equal(self.kb[o:o + c].cpu().numpy(), k):
            raise ValueError("reordered conditioning sets change the block structure")
        xo = int(self.x_off[i])
        self.X[xo:xo + n * d].copy_(torch.from_numpy(X.reshape(-1)))
        yo_ = int(self.y_off[i])
        self.y[yo_:yo_ + n].copy_(torch.from_numpy(np.ascontiguousarray(yo, dtype=np.float64).reshape(-1)))
        q = int(self.q[i])
        if q:
            zo = int(self.z_off[i])
            self.Z[zo:zo + n * q].copy_(torch.from_numpy(np.ascontiguousarray(Zo, dtype=np.float64).reshape(-1)))
        self.rowb[o:o + c].copy_(torch.from_numpy(rb))
        full = np.full((c, self.ldnbr), -1, dtype=np.int32)
        full[:, :nb.shape[1]] = nb
        self.nbr[o:o + c].copy_(torch.from_numpy(full))

    # --------------------------------------------------------------- reorder
    def set_sources(self, Xe, ye, Ze, ms):
        """Keep every problem's rows in subsample order on the device for
        device reorders (``reorder``): Xe[i] (n_i x d_i), ye[i], Ze[i] (or
        None) and its neighbour count ms[i].  The problem's blocks must have
        the layout of an ordered search (block i = row i with min(i, m)
        neighbours), as ordered_groups builds it."""
        torch = self.torch
        rowb = self.rowb.cpu().numpy()
        kb = self.kb.cpu().numpy()
        self._Xe_host = []
        for i in range(self.nprob):
            n, d, m = int(self.n[i]), int(self.d[i]), int(ms[i])
            o = int(self.blk_off[i])
            if (int(self.nblk[i]) != n or not np.array_equal(rowb[o:o + n], np.arange(n))
                    or not np.array_equal(kb[o:o + n], np.minimum(np.arange(n), m))):
                raise ValueError(f"problem {i} does not have the ordered-search block layout")
            X = np.ascontiguousarray(Xe[i], dtype=np.float64)
            if X.shape != (n, d):
                raise ValueError(f"source rows of problem {i} have the wrong shape")
            self._Xe_host.append(X)
        self.m = np.asarray(ms, dtype=np.int64)
        self.Xe = _lib.to_dev(torch, np.concatenate([x.reshape(-1) for x in self._Xe_host]), np.float64)
        self.ye = _lib.to_dev(torch, np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1) for v in ye]),
                              np.float64)
        zs = [np.asarray(Ze[i], dtype=np.float64).reshape(-1) for i in range(self.nprob) if self.q[i] > 0]
        self.Ze = _lib.to_dev(torch, np.concatenate(zs), np.float64) if zs else None
        self._max_rows = {}
        self._ro_ws = None
        self._ro_info = torch.zeros((self.nprob, 4), dtype=torch.int32, device="cuda")
        self._ro_order = torch.empty(int(self.n.sum()), dtype=torch.int64, device="cuda")

    def device_reorderable(self, i):
        """Whether problem i fits the batched (one-cluster) maximin."""
        d = int(self.d[i])
        if d not in self._max_rows:
            self._max_rows[d] = int(self.lib.sv_maximin_cluster_max_rows(d))
        return int(self.n[i]) <= self._max_rows[d]

    def reorder(self, ids, thetas, return_orders=False, maximin_flags=0, stream=None,
                deferred=False):
        """Rebuild the Vecchia structure of problems ``ids`` at their
        parameters (gp.py:182-191) on the device: scaled inputs, maximin
        order, reordered X/y/Z and neighbour columns.  ``thetas[j]`` belongs
        to ``ids[j]``.  Returns the orders (list of int64 arrays) on request.
        maximin_flags are test aids that give the same orders by other
        routes: 1 ranks every choice of pivot by exact square roots, 2 takes
        one pivot per pass by a full scan of the problem's points.
        stream: the CUDA stream of the work (default: the current one);
        deferred: return at once a function that waits for the work and
        checks its status (the problems' buffers must not be read before)."""
        lib, torch = self.lib, self.torch
        ids = [int(i) for i in ids]
        if not ids:
            return [] if return_orders else None
        probs = (_lib.ReorderProb * len(ids))()
        ranges = np.ones((len(ids), self.dmax), dtype=np.float64)
        for i in ids:
            if not self.device_reorderable(i):
                raise ValueError(f"problem {i} is too large for the batched maximin")

        def first_row(j):
            i = ids[j]
            d = int(self.d[i])
            r = np.exp(np.asarray(thetas[j], dtype=float)[1:1 + d])  # gp.py:183
            Xs = self._Xe_host[i] / r                                # gp.py:184
            return r, int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))  # ordering.py:72

        # the host's share (numpy, which releases the interpreter lock in
        # these array operations): the problems' first rows side by side
        firsts = list(_host_pool().map(first_row, range(len(ids)))) if len(ids) > 1 \
            else [first_row(0)]
        for j, i in enumerate(ids):
            d = int(self.d[i])
            r, first = firsts[j]
            ranges[j, :d] = r
            P = probs[j]
            P.n, P.xe_off, P.ye_off, P.ze_off = int(self.n[i]), int(self.x_off[i]), int(self.y_off[i]), int(self.z_off[i])
            P.x_off, P.y_off, P.z_off = int(self.x_off[i]), int(self.y_off[i]), int(self.z_off[i])
            P.blk_off, P.first = int(self.blk_off[i]), first
            P.d, P.q, P.m, P.flags = d, int(self.q[i]), int(self.m[i]), int(maximin_flags) & 3
        D = _lib.ReorderDesc()
        D.nprob, D.dmax, D.ldnbr = len(ids), self.dmax, self.ldnbr
        nbytes = int(lib.sv_reorder_batched_workspace_bytes(D, ctypes.cast(probs, ctypes.c_void_p)))
        if nbytes == 0:
            raise ValueError("invalid reorder request")
        if self._ro_ws is None or self._ro_ws.numel() < nbytes:
            self._ro_ws = _lib.workspace(torch, nbytes)
        P_ = _lib.ptr
        sh = ctypes.c_void_p(stream.cuda_stream) if stream is not None else _lib.stream_handle(torch)
        rc = lib.sv_reorder_batched(D, ctypes.cast(probs, ctypes.c_void_p),
                                    ranges.ctypes.data_as(ctypes.c_void_p), P_(self.Xe), P_(self.ye),
                                    P_(self.Ze), P_(self.X), P_(self.y), P_(self.Z), P_(self.nbr),
                                    P_(self._ro_order), P_(self._ro_info), P_(self._ro_ws),
                                    self._ro_ws.numel(), sh)
        _lib.check(lib, rc, "sv_reorder_batched")
        if deferred:
            done = torch.cuda.Event()
            done.record(stream if stream is not None else torch.cuda.current_stream())
            nids = len(ids)

            def finish():
                done.synchronize()
                inf = self._ro_info[:nids].cpu().numpy()
                for j in range(nids):
                    _lib.check_info(lib, inf[j], "sv_reorder_batched")
            return finish
        info = self._ro_info[:len(ids)].cpu().numpy()
        for j in range(len(ids)):
            _lib.check_info(lib, info[j], "sv_reorder_batched")
        if not return_orders:
            return None
        allo = self._ro_order.cpu().numpy()
        out, off = [], 0
        for i in ids:
            n = int(self.n[i])
            out.append(allo[off:off + n].copy())
            off += n
        return out

    # ---------------------------------------------------------------- launch
    def launch(self, precision=None, stream=None):
        """Enqueue one evaluation of the mode's active problems (kernels and
        memsets only)."""
        lib, P = self.lib, _lib.ptr
        mode = self._modes[precision or self.precisions[0]]
        st = stream if stream is not None else _lib.stream_handle(self.torch)
        rc = lib.sv_vecchia_loglik_batched(
            mode["bdesc"], P(mode["descs"]), P(self.theta), P(self.X), P(self.y), P(self.Z),
            P(self.rowb), P(self.kb), P(self.nbr), P(self.bprob), P(self.wlist), P(self.clist),
            P(self.chunk), P(self.out), P(self.info), P(self.ws), self.ws.numel(), st)
        _lib.check(lib, rc, "sv_vecchia_loglik_batched")

    def capture(self, precision=None):
        """Capture one evaluation of a mode as a CUDA graph (replayed by ``run``)."""
        torch = self.torch
        prec = precision or self.precisions[0]
        # warm-up launch outside the capture (it sets the kernels' attributes)
        # with every problem switched off, so it does no evaluation work
        saved = self._modes[prec]["active"].copy()
        self.set_active(np.zeros(self.nprob, dtype=bool), prec)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch(prec)
        torch.cuda.current_stream().wait_stream(s)
        self.set_active(saved, prec)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self.launch(prec)
        self._modes[prec]["graph"] = g
        return g

    def run(self, precision=None):
        """One evaluation: graph replay when captured, else direct launches."""
        mode = self._modes[precision or self.precisions[0]]
        if mode["graph"] is not None:
            mode["graph"].replay()
        else:
            self.launch(precision)

    def fetch(self):
        """Copy out and info to the host; returns (out (nprob, ostride), info (nprob, 4))."""
        torch = self.torch
        self._res_host.copy_(self.out.reshape(-1), non_blocking=True)
        self._info_host.copy_(self.info.reshape(-1), non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return (self._res_host.numpy().reshape(self.nprob, self.ostride).copy(),
                self._info_host.numpy().reshape(self.nprob, 4).copy())

    def unpack(self, out, info, i):
        """Problem i's (status, ll, grad, fisher, beta) from fetched arrays."""
        P, q = int(self.P[i]), int(self.q[i])
        r = out[i]
        st = int(info[i, 0])
        ll = float(r[0])
        beta = r[1 + P + P * P:1 + P + P * P + q].copy()
        if not self.need_grad:
            return st, ll, None, None, beta
        return st, ll, r[1:1 + P].copy(), r[1 + P:1 + P + P * P].reshape(P, P).copy(), beta

    def evaluate(self, thetas, active=None, precision=None):
        """Evaluate the active problems at ``thetas``; returns a list with,
        per problem, (status, ll, grad, fisher, beta) or None when inactive.
        status is 0 (SV_OK) or an SV_* code (2 = Cholesky failed even with
        jitter, as numpy.linalg.LinAlgError in the reference)."""
        prec = precision or self.precisions[0]
        if active is not None:
            self.set_active(active, prec)
        self.set_theta(thetas)
        self.run(prec)
        out, info = self.fetch()
        self.last_info = info
        act = self._modes[prec]["active"]
        return [self.unpack(out, info, i) if act[i] else None for i in range(self.nprob)]
