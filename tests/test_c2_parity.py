"""Ordering and neighbour sets at the benchmark's own size.

The benchmark's workload (n = 200,000 points in d = 10, seed 1, X / lambda
with lambda log-uniform in [0.05, 50]) is ordered on the GPU by the grid
form of the pass maximin (beyond one thread-block cluster) and searched by
the ordered neighbour kernel (m = 30).  tests/golden/c2_order.npz holds the
oracle's exact maximin order of those inputs and the SHA-256 of the oracle's
ordered 30-neighbour table (tests/golden/make_c2_order.py; the oracle is
pinned to the reference's own orders in tests/test_oracle_golden.py).  Both
must be reproduced exactly: the order as an array, the neighbour table bit
for bit (neighbours nearest first, ties to the smaller index, -1 padding).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_maximin_and_neighbours_match_the_oracle_at_200k():
    import sys
    sys.path.insert(0, ROOT)
    import torch

    from bench import c2_fixture, make_inputs, nn_digest
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device, ordered_nn_device
    n, d, m, seed = 200_000, 10, 30, 1
    fx = c2_fixture(n, d, m, seed)
    assert fx is not None, "tests/golden/c2_order.npz is missing"
    lib, _ = _lib.device_ready()
    X, lam, _, _ = make_inputs(n, d, seed)
    Xs = X / lam
    first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
    assert n > lib.sv_maximin_cluster_max_rows(d)  # the grid form's route
    Xs_d = _lib.to_dev(torch, Xs, np.float64)
    order_d, info = maximin_order_device(torch, Xs_d, first)
    _lib.check_info(lib, info.cpu().numpy(), "maximin")
    np.testing.assert_array_equal(order_d.cpu().numpy(), fx[0])
    nn_d, info = ordered_nn_device(torch, Xs_d[order_d].contiguous(), m)
    _lib.check_info(lib, info.cpu().numpy(), "knn")
    assert nn_digest(nn_d.cpu().numpy()) == fx[1]


def test_tree_form_maximin_at_200k():
    """The tree form (the route beyond the grid form's shared memory) on the
    same 200,000 rows gives the oracle's order too."""
    import sys
    sys.path.insert(0, ROOT)
    import torch

    from bench import c2_fixture, make_inputs
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device
    n, d, m, seed = 200_000, 10, 30, 1
    fx = c2_fixture(n, d, m, seed)
    assert fx is not None, "tests/golden/c2_order.npz is missing"
    lib, _ = _lib.device_ready()
    X, lam, _, _ = make_inputs(n, d, seed)
    Xs = X / lam
    first = int(np.argmin(((Xs - Xs.mean(0)) ** 2).sum(1)))
    order_d, info = maximin_order_device(torch, _lib.to_dev(torch, Xs, np.float64), first, 16)
    _lib.check_info(lib, info.cpu().numpy(), "maximin")
    np.testing.assert_array_equal(order_d.cpu().numpy(), fx[0])
