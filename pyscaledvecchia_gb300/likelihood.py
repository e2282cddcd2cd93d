"""Profile Vecchia log-likelihood, score and Fisher information on the GPU.

Drop-in counterpart of the reference's ``scaled_vecchia.likelihood``
(src/scaled_vecchia/likelihood.py:66-175).  For block U_i = (c(i), i) with
covariance S = L L' and a = L^-T e_K (the block's column of the sparse inverse
Cholesky factor):

    l_i          = -1/2 (log 2 pi + 2 log L_KK + z_K^2),   z = L^-1 r
    dl_i/dth_j   = -1/2 [ w^j_K (1 + z_K^2) - 2 z_K (w^j . z) ]
    I_i[j, k]    =  1/2 [ 2 (w^j . w^k) - w^j_K w^k_K ],   w^j = L^-1 (dS_j a)

with the trend coefficients beta profiled out by GLS on the whitened
columns a.y, a.Z.  All of it runs in the fused block kernels of
libsvgpu.so (sv_vecchia_loglik); the host only packs the conditioning sets.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._covariance import _check_nu, _chunks

__all__ = ["vecchia_profile_loglik"]

_WARP_K = 32  # blocks with K = k+1 <= 32 run one per warp, larger ones one per CTA
_PRECISION = {"float64": 0, "split": 1, "split_df": 2}
_SPLIT = ("split", "split_df")


def matern_table_nu(nu, estimate_nu=False):
    """Whether the library interpolates this fixed nu's Matern from a
    per-evaluation table (no closed form, nu <= 10, and sqrt(2 nu) 1e-7 >=
    2^-40)."""
    if (estimate_nu or nu is None or not 0.0 < nu <= 10.0
            or float(nu) in (0.5, 1.5, 2.5)):
        return False
    return math.frexp(math.sqrt(2.0 * nu) * 1e-7)[1] - 1 >= -40


def split_nu(nu, estimate_nu=False):
    """Whether the split forms assemble this nu in float32: a closed form
    (0.5, 1.5, 2.5), or a fixed nu of the library's float32 table (at most 8
    and at least 1e-3 from an integer: near an integer the table's series
    loses its digits).  Any other fixed nu runs the float64 kernels.  An
    estimated nu takes the split kernels, which decide at each theta (nu,
    nu - 1e-3 and nu + 1e-3 with float32 tables, or the float64 pass)."""
    if estimate_nu:
        return True
    if nu is None:
        return False
    if float(nu) in (0.5, 1.5, 2.5):
        return True
    return (matern_table_nu(nu) and float(nu) <= 8.0
            and abs(float(nu) - round(float(nu))) >= 1e-3)


def pack_groups(groups, n=None):
    """Flatten ``_nn_groups`` output into per-block arrays.

    Returns (rowb int32 (B,), kb int32 (B,), nbr int32 (B, kmax), group_k list,
    group_len list) with warp-sized blocks first (stable).
    """
    rows_l, k_l, nb_l = [], [], []
    for rows, nb in groups:
        rows = np.asarray(rows, dtype=np.int64).reshape(-1)
        nb = np.asarray(nb, dtype=np.int64).reshape(rows.shape[0], -1)
        rows_l.append(rows)
        k_l.append(nb.shape[1])
        nb_l.append(nb)
    B = int(sum(r.shape[0] for r in rows_l))
    kmax = max(k_l) if k_l else 0
    rowb = np.empty(B, dtype=np.int32)
    kb = np.empty(B, dtype=np.int32)
    nbr = np.full((B, max(kmax, 1)), -1, dtype=np.int32)
    gid = np.empty(B, dtype=np.int32)
    o = 0
    for g, (rows, k, nb) in enumerate(zip(rows_l, k_l, nb_l)):
        c = rows.shape[0]
        rowb[o:o + c] = rows
        kb[o:o + c] = k
        if k:
            nbr[o:o + c, :k] = nb
        gid[o:o + c] = g
        o += c
    # padding is -1, so plain extrema check every entry
    if n is not None and B and (rowb.min() < 0 or rowb.max() >= n or
                                (kmax and (nbr.max() >= n or nbr.min() < -1))):
        raise ValueError("conditioning sets reference rows outside the data")
    big = (kb + 1) > _WARP_K
    if big.any() and not np.all(np.diff(big.astype(np.int8)) >= 0):
        perm = np.argsort(big, kind="stable")
        rowb, kb, nbr, gid = rowb[perm], kb[perm], nbr[perm], gid[perm]
    return rowb, kb, nbr, gid, k_l, [r.shape[0] for r in rows_l]


def chunk_ids(gid, group_k, group_len, Pc):
    """Jitter-sharing chunk of every block: the reference factorises each group
    in chunks of ``_chunks(len(rows), K, Pc)`` rows and retries a whole chunk
    with the same jitter (_covariance.py:235-259, likelihood.py:114)."""
    ids_per_group = []
    nxt = 0
    for k, ln in zip(group_k, group_len):
        ids = np.empty(ln, dtype=np.int32)
        for a0, a1 in _chunks(ln, k + 1, Pc):
            ids[a0:a1] = nxt
            nxt += 1
        ids_per_group.append(ids)
    if gid.shape[0] == 0:
        return np.zeros(0, dtype=np.int32)
    flat = np.concatenate(ids_per_group)
    if np.all(np.diff(gid) >= 0):
        # groups in order (no warp/CTA regrouping): block b is the flat entry b
        return flat.astype(np.int32)
    # rank of each block inside its group (the stable warp/CTA split keeps it)
    sort_idx = np.argsort(gid, kind="stable")
    first = np.searchsorted(gid[sort_idx], np.arange(len(group_k)))
    rank = np.empty(gid.shape[0], dtype=np.int64)
    rank[sort_idx] = np.arange(gid.shape[0]) - first[gid[sort_idx]]
    offs = np.concatenate([[0], np.cumsum(group_len)])[:-1].astype(np.int64)
    return flat[offs[gid] + rank].astype(np.int32)


class DeviceProblem:
    """Device-resident inputs of one likelihood (X, y, Z in Vecchia order and
    the packed conditioning sets), reused across objective evaluations."""

    def __init__(self, Xo, yo, Zo, groups):
        lib, torch = _lib.device_ready()
        self.lib, self.torch = lib, torch
        Xo = np.ascontiguousarray(Xo, dtype=np.float64)
        self.n, self.d = Xo.shape
        yo = np.ascontiguousarray(yo, dtype=np.float64).reshape(-1)
        if yo.shape[0] != self.n:
            raise ValueError("X and y have incompatible shapes")
        self.has_Z = Zo is not None and np.asarray(Zo).ndim == 2 and np.asarray(Zo).shape[1] > 0
        self.q = int(np.asarray(Zo).shape[1]) if self.has_Z else 0
        # the packing kernel first: it reads the groups while the host waits
        # in the copies of X, y and Z
        pending = self._pack_on_device(groups)
        self.X = _lib.to_dev(torch, Xo, np.float64)
        self.y = _lib.to_dev(torch, yo, np.float64)
        self.Z = _lib.to_dev(torch, np.asarray(Zo, dtype=np.float64), np.float64) if self.has_Z else None
        if pending is not None:
            torch.cuda.current_stream().wait_stream(pending[1])
            if int(pending[0].item()):  # waits for the packing
                raise ValueError("conditioning sets reference rows outside the data")
        del pending
        self._chunks = {}
        self._ws = None
        self.out = None
        self.info = _lib.new_info(torch)

    def _pack_on_device(self, groups):
        """Enqueue the block table of ``pack_groups`` built on the device
        (sv_pack_blocks) from the groups' own arrays, on the library's side
        stream: warp-sized groups first, group order kept.  Returns (bad flag,
        side stream, arrays the kernel reads): the current stream must wait
        for the side stream before the tables or the flag are used, and the
        arrays must live until then (flag nonzero: a row or neighbour index
        outside the data); None when there are no blocks."""
        torch, lib = self.torch, self.lib
        rows_l, nb_l = [], []
        for rows, nb in groups:
            rows = np.ascontiguousarray(rows, dtype=np.int64).reshape(-1)
            nb = np.ascontiguousarray(nb, dtype=np.int64).reshape(rows.shape[0], -1)
            rows_l.append(rows)
            nb_l.append(nb)
        gk = [nb.shape[1] for nb in nb_l]
        gl = [r.shape[0] for r in rows_l]
        order = [g for g in range(len(gk)) if gk[g] + 1 <= _WARP_K] + \
                [g for g in range(len(gk)) if gk[g] + 1 > _WARP_K]
        B = int(sum(gl))
        kmax = max(gk) if gk else 0
        self.nblk = B
        self.kmax = kmax if B else 0
        self.nblk_warp = int(sum(gl[g] for g in range(len(gk)) if gk[g] + 1 <= _WARP_K))
        self.ldnbr = max(kmax, 1)
        self.rowb = torch.empty(max(B, 1), dtype=torch.int32, device="cuda")[:B]
        self.kb = torch.empty(max(B, 1), dtype=torch.int32, device="cuda")[:B]
        self.nbr = torch.empty((max(B, 1), self.ldnbr), dtype=torch.int32, device="cuda")[:B]
        self._order = order
        self._gk, self._gl = gk, gl
        self._goff = [0] * len(gk)  # first block of each group in the packed table
        if B == 0:
            return None
        bad = torch.empty(1, dtype=torch.int32, device="cuda")
        side = _lib.side_stream(torch)
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            return self._pack_enqueue(groups_arrays=(rows_l, nb_l), order=order, gl=gl, gk=gk,
                                      bad=bad, side=side)

    def _pack_enqueue(self, groups_arrays, order, gl, gk, bad, side):
        """sv_pack_blocks on the current (side) stream; see _pack_on_device."""
        torch, lib = self.torch, self.lib
        rows_l, nb_l = groups_arrays
        desc = (_lib.PackGroup * len(order))()
        if _lib.device_reads_host_memory(lib):
            # the packing kernel reads the groups' own arrays over the
            # chip-to-chip link: no copies (the arrays are returned to the
            # caller, which keeps them until it has waited for the packing)
            src = {g: (rows_l[g].ctypes.data, nb_l[g].ctypes.data) for g in order}
            keep = None
        else:
            # small groups travel in one copy, large ones in their own
            small = [g for g in order if gl[g] * max(gk[g], 1) < 65536]
            src, keep = {}, []
            if small:
                flat = np.concatenate([np.concatenate([rows_l[g], nb_l[g].reshape(-1)]) for g in small])
                fd = _lib.to_dev(torch, flat, np.int64)
                keep.append(fd)
                base, o = fd.data_ptr(), 0
                for g in small:
                    c, k = gl[g], gk[g]
                    src[g] = (base + 8 * o, base + 8 * (o + c))
                    o += c + c * k
            for g in order:
                if g not in src:
                    r_d, nb_d = _lib.to_dev(torch, rows_l[g], np.int64), _lib.to_dev(torch, nb_l[g], np.int64)
                    keep += [r_d, nb_d]
                    src[g] = (r_d.data_ptr(), nb_d.data_ptr())
        o = 0
        for j, g in enumerate(order):
            self._goff[g] = o
            d = desc[j]
            d.rows = src[g][0] if gl[g] else None
            d.nb = src[g][1] if gl[g] * gk[g] else None
            d.count, d.out_off, d.k = gl[g], o, gk[g]
            o += gl[g]
        rc = lib.sv_pack_blocks(ctypes.cast(desc, ctypes.c_void_p), len(order), self.n, self.ldnbr,
                                _lib.ptr(self.rowb), _lib.ptr(self.kb), _lib.ptr(self.nbr), _lib.ptr(bad),
                                _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_pack_blocks")
        return bad, side, (rows_l, nb_l, src if keep is None else keep, desc)

    @property
    def _gid(self):
        """Group of every packed block (host form, for checks of the device tables)."""
        order = self._order
        return np.repeat(np.asarray(order, dtype=np.int32),
                         np.asarray([self._gl[g] for g in order], dtype=np.int64))

    def kernel_launches(self, precision="float64", chunked=True, estimate_nu=False, nu=2.5):
        """Number of library kernels one evaluation launches."""
        warp = self.nblk_warp > 0
        cta = self.nblk > self.nblk_warp
        split = (precision in _SPLIT and split_nu(nu, estimate_nu)
                 and self.d + 3 + self.q <= 32)
        n = (1 if warp else 0) + (1 if cta else 0)
        if estimate_nu or matern_table_nu(nu):
            n += 2 if split else 1  # the Matern tables: float64, and float32 for the split kernels
        if split and warp:
            n += 1  # coordinate pre-pass
        if chunked:
            n += 1 + (1 if warp else 0) + (1 if cta else 0)
        if split and warp:
            n += 1  # float64 re-evaluation of flagged blocks
        return n + 2 + 4  # status/parameter set-up, then the four reduction kernels

    def chunk_tensor(self, Pc):
        """Chunk of every block (chunk_ids), computed on the device from the
        groups' sizes and _chunks' row counts (sv_chunk_ids)."""
        if Pc not in self._chunks:
            torch, lib = self.torch, self.lib
            G = len(self._gk)
            desc = (_lib.ChunkGroup * max(G, 1))()
            base = 0
            for g in range(G):
                k, ln = self._gk[g], self._gl[g]
                step = max(1, 4_000_000 // max(1, (k + 1) * (k + 1) * max(Pc, 1)))  # _chunks
                desc[g].count, desc[g].out_off = ln, self._goff[g]
                desc[g].base, desc[g].step = base, step
                base += (ln + step - 1) // step
            ids = torch.empty(max(self.nblk, 1), dtype=torch.int32, device="cuda")[:self.nblk]
            rc = lib.sv_chunk_ids(ctypes.cast(desc, ctypes.c_void_p), G, _lib.ptr(ids),
                                  _lib.stream_handle(torch))
            _lib.check(lib, rc, "sv_chunk_ids")
            self._chunks[Pc] = ids
        return self._chunks[Pc]

    def launch(self, theta_dev, P, nu, estimate_nu, need_grad, var_penalty, log_var_target,
               chunked=True, stream=None, precision="float64", team_lanes=0):
        """Enqueue one evaluation; results land in self.out / self.info.

        precision "float64" is the reference's arithmetic; "split" computes
        distances, Matern terms, dSigma.a and the Gram products (trace
        contractions) in float32, the factorisation, solves, log-determinant
        and the likelihood sums in float64; "split_df" is "split" with the
        factorisation and solves in double-float (float32 pairs, about 46
        bits) instead of float64.  The split forms take a closed-form nu or a
        fixed nu of the float32 table (split_nu); other cases, and blocks that
        are ill-conditioned or outside float32's exponent range, are evaluated
        in float64 by the library."""
        torch, lib = self.torch, self.lib
        if (precision in _SPLIT and not team_lanes and self.nblk_warp > 0
                and split_nu(nu, estimate_nu) and self.d + 3 + self.q <= 32):
            from . import autotune
            team_lanes = autotune.team_lanes(min(self.kmax + 1, 32), self.d, self.q, need_grad,
                                             precision=precision)
        D = _lib.LoglikDesc()
        D.n, D.nblk, D.nblk_warp = self.n, self.nblk, self.nblk_warp
        D.d, D.q, D.ldnbr, D.kmax = self.d, self.q, self.ldnbr, self.kmax
        D.need_grad, D.estimate_nu = int(bool(need_grad)), int(bool(estimate_nu))
        D.chunked = int(bool(chunked))
        D.precision = _PRECISION[precision]
        D.team_lanes = int(team_lanes)
        D.nu = float(nu) if nu is not None else 1.0
        D.var_penalty, D.log_var_target = float(var_penalty), float(log_var_target)
        nbytes = lib.sv_loglik_workspace_bytes(D)
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = _lib.workspace(torch, nbytes)
        nout = 1 + P + P * P + self.q
        if self.out is None or self.out.numel() != nout:
            self.out = torch.empty(nout, dtype=torch.float64, device="cuda")
        chunk = self.chunk_tensor(P if need_grad else 1) if chunked else None
        st = stream if stream is not None else _lib.stream_handle(torch)
        rc = lib.sv_vecchia_loglik(D, _lib.ptr(theta_dev), _lib.ptr(self.X), _lib.ptr(self.y),
                                   _lib.ptr(self.Z), _lib.ptr(self.rowb), _lib.ptr(self.kb),
                                   _lib.ptr(self.nbr), _lib.ptr(chunk), _lib.ptr(self.out),
                                   _lib.ptr(self.info), _lib.ptr(self._ws), self._ws.numel(), st)
        _lib.check(lib, rc, "sv_vecchia_loglik")

    def evaluate(self, theta, nu, estimate_nu=False, need_grad=True, var_penalty=0.0,
                 log_var_target=0.0, chunked=True, precision="float64", team_lanes=0):
        torch = self.torch
        theta = np.asarray(theta, dtype=float).reshape(-1)
        d = self.d
        P = d + 3 if estimate_nu else d + 2
        if theta.shape[0] < P:
            raise ValueError("theta has too few entries for this input dimension")
        if not estimate_nu:
            _check_nu(nu)
        th = _lib.to_dev(torch, theta[:P], np.float64)
        self.launch(th, P, nu, estimate_nu, need_grad, var_penalty, log_var_target, chunked,
                    precision=precision, team_lanes=team_lanes)
        res = torch.cat([self.out, self.info.to(torch.float64)]).cpu().numpy()
        nout = 1 + P + P * P + self.q
        self.last_info = res[nout:].astype(np.int64)
        _lib.check_info(self.lib, self.last_info, "sv_vecchia_loglik")
        ll = float(res[0])
        beta = res[1 + P + P * P:nout].copy() if self.has_Z else np.zeros(0)
        if not need_grad:
            return ll, None, None, beta
        grad = res[1:1 + P].copy()
        fish = res[1 + P:1 + P + P * P].reshape(P, P).copy()
        return ll, grad, fish, beta


def vecchia_profile_loglik(theta, Xo, yo, Zo, groups, nu, estimate_nu=False,
                           need_grad=True, var_penalty=0.0, log_var_target=0.0, *,
                           precision="float64"):
    """Profile Vecchia loglikelihood, its gradient and the Fisher information.

    theta : (P,) log-scale parameters [log sigma^2, log lambda_1..d, log tau]
            (P = d+2), or [log sigma^2, log lambda_1..d, log nu, log tau]
            (P = d+3) with ``estimate_nu``.
    Xo, yo, Zo : inputs, responses and trend design (or None) in Vecchia order.
    groups : output of ``ordering._nn_groups``.
    nu : fixed Matern smoothness (ignored with ``estimate_nu``).
    precision (keyword only, not in the reference): "float64" (default, the
            reference's arithmetic), "split" (float32 assembly and Gram
            products, float64 factorisation, solves and log-determinant) or
            "split_df" (the same with a double-float factorisation; see
            DeviceProblem.launch).
    Returns (ll, grad, fisher, beta); grad and fisher are None when
    ``need_grad`` is False.  Raises numpy.linalg.LinAlgError when a block
    cannot be factorised even with jitter.
    """
    theta = np.asarray(theta, dtype=float)
    if precision not in _PRECISION:
        raise ValueError("precision must be 'float64', 'split' or 'split_df'")
    prob = DeviceProblem(Xo, yo, Zo, groups)
    return prob.evaluate(theta, nu, estimate_nu=estimate_nu, need_grad=need_grad,
                         var_penalty=var_penalty, log_var_target=log_var_target,
                         precision=precision)

