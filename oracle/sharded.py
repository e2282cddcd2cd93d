"""CPU stage evaluator of the sharded likelihood, on the oracle.

TEST INFRASTRUCTURE ONLY: the evaluator each rank of the world_size-2 gloo
test runs in place of a GPU (tests/test_sharding.py).  The product package
never imports it.

It restates the two passes of likelihood.py:66-175 (the reference) over
per-block records (oracle/sv_oracle.c, or_block_records) in the four stages
of pyscaledvecchia_gb300.sharding.sharded_evaluate:
  stage 1  records of the shard's blocks at jitter level 0; the largest level
           of every chunk among them (the caller takes the MAX over ranks);
  stage 2  blocks whose chunk needs a larger level are redone at that level
           (the chunk-wide jitter of _covariance.py:235-252); pass-1 partial
           sums (log L_KK, Z'y, Z'Z, Fisher) of the shard's partitions;
  stage 3  beta = solve(Z'Z + 1e-12 I, Z'y) from all partitions' sums
           (likelihood.py:146); pass-2 partial sums (likelihood.py:149-162);
  stage 4  ll, score, Fisher and beta, with the variance penalty
           (likelihood.py:165-171).
Partitions are the device's: max(8, ceil(nblk / 1024)) runs of ceil(nblk /
parts) blocks.  Every sum runs in a fixed order (blocks of a partition in
order, then partitions in order), so one rank and several ranks give the
same bits.
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle


def red_parts(nblk):
    return int(min(4096, max(8, (nblk + 1023) // 1024)))


class OracleShard:
    def __init__(self, Xo, yo, Zo, groups, nu, part_begin, part_end, var_penalty=0.0,
                 log_var_target=0.0):
        self.Xo = np.ascontiguousarray(Xo, dtype=np.float64)
        self.yo = np.ascontiguousarray(yo, dtype=np.float64)
        self.n, self.d = self.Xo.shape
        self.q = Zo.shape[1] if Zo is not None else 0
        self.Zo = np.ascontiguousarray(Zo, dtype=np.float64) if self.q else None
        self.P = self.d + 2
        self.nu = nu
        self.var_penalty, self.log_var_target = var_penalty, log_var_target
        rows, kb, nbr, chunk = oracle._flatten_groups(groups, self.P)
        self.rows, self.kb, self.nbr, self.chunk = rows, kb, nbr, chunk
        self.nblk = rows.shape[0]
        self.parts = red_parts(self.nblk)
        self.per = -(-self.nblk // self.parts)
        self.pb, self.pe = part_begin, part_end
        self.b0 = min(part_begin * self.per, self.nblk)
        self.b1 = min(part_end * self.per, self.nblk)
        q, P = self.q, self.P
        self.len1 = 1 + q + q * q + P * P
        self.len2 = 1 + P

    def _records(self, theta, b0, b1, force=None):
        cs = 3 + 2 * self.q + 2 * self.P + self.P * self.q + self.P * self.P
        rec = np.zeros((max(b1 - b0, 1), cs))
        lev = np.zeros(max(b1 - b0, 1), dtype=np.int32)
        if b1 > b0:
            f = None if force is None else np.ascontiguousarray(force, dtype=np.int32)
            rc = oracle.lib().or_block_records(
                oracle._p(np.ascontiguousarray(theta, dtype=np.float64)), oracle._p(self.Xo),
                oracle._p(self.yo), oracle._p(self.Zo), self.n, self.d, self.q, oracle._p(self.rows),
                oracle._p(self.kb), oracle._p(self.nbr), self.nbr.shape[1], b0, b1, oracle._p(f),
                float(self.nu), 1, oracle._p(rec), oracle._p(lev))
            if rc < 0:
                raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
        return rec[:b1 - b0], lev[:b1 - b0]

    def stage1(self, theta):
        self.theta = np.asarray(theta, dtype=np.float64)
        self.rec, self.lev = self._records(self.theta, self.b0, self.b1)
        cm = np.zeros(self.nblk, dtype=np.int32)
        for b in range(self.b0, self.b1):
            c = self.chunk[b]
            cm[c] = max(cm[c], self.lev[b - self.b0])
        return cm

    def stage2(self, chunk_max):
        need = [b for b in range(self.b0, self.b1) if chunk_max[self.chunk[b]] > self.lev[b - self.b0]]
        for b in need:
            r, lv = self._records(self.theta, b, b + 1, [chunk_max[self.chunk[b]]])
            self.rec[b - self.b0] = r[0]
        q = self.q
        part1 = np.zeros((self.parts, self.len1))
        for p in range(self.pb, self.pe):
            s = np.zeros(self.len1)
            for b in range(p * self.per, min((p + 1) * self.per, self.nblk)):
                c = self.rec[b - self.b0]
                ay, aZ = c[1], c[2:2 + q]
                s[0] += c[0]
                s[1:1 + q] += aZ * ay
                s[1 + q:1 + q + q * q] += np.outer(aZ, aZ).ravel()
                s[1 + q + q * q:] += c[3 + 2 * q + 2 * self.P + self.P * q:]
            part1[p] = s
        return part1

    def stage3(self, part1):
        q, P = self.q, self.P
        tot = np.zeros(self.len1)
        for p in range(self.parts):
            tot += part1[p]
        self.sum1 = tot
        self.beta = np.linalg.solve(tot[1 + q:1 + q + q * q].reshape(q, q) + 1e-12 * np.eye(q),
                                    tot[1:1 + q]) if q else np.zeros(0)
        part2 = np.zeros((self.parts, self.len2))
        for p in range(self.pb, self.pe):
            s = np.zeros(self.len2)
            for b in range(p * self.per, min((p + 1) * self.per, self.nblk)):
                c = self.rec[b - self.b0]
                zK = c[2 + q] - c[3 + q:3 + 2 * q] @ self.beta
                s[0] -= 0.5 * (2.0 * c[0] + zK * zK)
                wK = c[3 + 2 * q:3 + 2 * q + P]
                wzy = c[3 + 2 * q + P:3 + 2 * q + 2 * P]
                wzZ = c[3 + 2 * q + 2 * P:3 + 2 * q + 2 * P + P * q].reshape(P, q)
                wz = wzy - wzZ @ self.beta
                s[1:] -= 0.5 * (wK * (1.0 + zK * zK) - 2.0 * zK * wz)
            part2[p] = s
        return part2

    def stage4(self, part2):
        q, P = self.q, self.P
        tot = np.zeros(self.len2)
        for p in range(self.parts):
            tot += part2[p]
        ll = -0.5 * self.n * math.log(2.0 * math.pi) + tot[0]
        g = tot[1:].copy()
        F = self.sum1[1 + q + q * q:].reshape(P, P).copy()
        if self.var_penalty > 0.0:
            ex = max(self.theta[0] - self.log_var_target, 0.0)
            ll -= 0.5 * self.var_penalty * ex * ex
            g[0] -= self.var_penalty * ex
            if ex > 0.0:
                F[0, 0] += self.var_penalty
        return ll, g, F, self.beta.copy()
