"""Oracle ordering and neighbour sets of the benchmark's n = 200,000 workload.

The exact maximin ordering of 200,000 points in d = 10 takes the oracle
(oracle/sv_oracle.c, a single-threaded restatement of ordering.py:27-59)
several minutes, too long to repeat in every test run or benchmark start.
This script computes it once for the seeded inputs of ``bench.make_inputs``
(n = 200,000, d = 10, seed 1; X uniform in [0,1]^10, lambda log-uniform in
[0.05, 50]; scaled inputs X / lambda, first point by ordering.py:72) and
stores:

  order      int32 (200000,)  the oracle's maximin order
  nn_sha256  the SHA-256 of the oracle's ordered 30-neighbour table of the
             reordered inputs (int32, row-major (200000, 31), -1 padding)

Used by tests/test_c2_parity.py (the device ordering and neighbour search
against the oracle at the benchmark's size) and by ``bench.py --impl
reference`` (the reference arm evaluates the same ordered inputs as the
GPU arm).  Run from the repository root: python tests/golden/make_c2_order.py
"""
import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from bench import make_inputs  # noqa: E402
from oracle import oracle  # noqa: E402

N, D, M, SEED = 200_000, 10, 30, 1


def nn_digest(nn):
    return hashlib.sha256(np.ascontiguousarray(nn, dtype=np.int32).tobytes()).hexdigest()


def main():
    X, lam, _, _ = make_inputs(N, D, SEED)
    Xs = X / lam
    t0 = time.time()
    order = oracle.maximin_order(Xs)
    t1 = time.time()
    nn = oracle.ordered_nn(Xs[order], M)
    t2 = time.time()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c2_order.npz")
    np.savez_compressed(out, order=order.astype(np.int32), nn_sha256=np.array(nn_digest(nn)),
                        n=N, d=D, m=M, seed=SEED)
    print(f"maximin {t1 - t0:.1f} s, neighbours {t2 - t1:.1f} s -> {out}")


if __name__ == "__main__":
    main()
