"""Batched device rebuild of many problems' Vecchia structure
(sv_reorder_batched: gp.py:182-191 per problem).

Every problem's maximin order, reordered X/y/Z and neighbour columns must
equal, bit for bit, the one-problem path (maximin_order + find_ordered_nn +
_nn_groups, themselves pinned to the reference), whatever else shares the
call: problems of every cluster size (1 to 8 CTAs), several dimensions and
neighbour counts, trend columns, and a subset of the batch.  The
one-problem maximin also runs through the cluster kernel for such sizes;
the grid-wide kernel keeps its own oracle case above the cluster limit.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems():
    from pyscaledvecchia_gb300.batched import BatchProblem, ordered_groups
    specs = [(1, 700, 3, 10, 1), (2, 5200, 7, 30, 1), (3, 20000, 12, 20, 0), (4, 1500, 5, 40, 2),
             (5, 9000, 10, 10, 1), (6, 2, 4, 1, 1), (7, 12000, 3, 30, 1)]
    probs, raw, thetas = [], [], []
    for seed, n, d, m, q in specs:
        rng = np.random.default_rng(seed)
        X = rng.random((n, d))
        y = rng.standard_normal(n)
        Z = None if q == 0 else np.column_stack([np.ones(n)] + [X[:, :q - 1]] if q > 1 else [np.ones(n)])
        m = min(m, n - 1)
        th = np.concatenate([[0.1], rng.uniform(math.log(0.05), math.log(100.0), d), [math.log(1e-3)]])
        probs.append(BatchProblem(X, y, Z, ordered_groups(n, m)))
        raw.append((X, y, Z, m))
        thetas.append(th)
    return probs, raw, thetas


def _expected(X, y, Z, m, th):
    from pyscaledvecchia_gb300 import find_ordered_nn, maximin_order
    d = X.shape[1]
    Xs = X / np.exp(th[1:1 + d])
    order = maximin_order(Xs)
    nn = find_ordered_nn(Xs[order], m)
    return order, nn


def test_batched_reorder_matches_single_problem_path():
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    probs, raw, thetas = _problems()
    BL = BatchedLikelihood(probs)
    BL.set_sources([r[0] for r in raw], [r[1] for r in raw], [r[2] for r in raw], [r[3] for r in raw])
    ids = list(range(len(probs)))
    orders = BL.reorder(ids, thetas, return_orders=True)
    Xd, yd = BL.X.cpu().numpy(), BL.y.cpu().numpy()
    Zd = BL.Z.cpu().numpy() if BL.Z is not None else None
    nbr = BL.nbr.cpu().numpy()
    for i, ((X, y, Z, m), th) in enumerate(zip(raw, thetas)):
        order, nn = _expected(X, y, Z, m, th)
        np.testing.assert_array_equal(orders[i], order)
        n, d = X.shape
        xo = int(BL.x_off[i])
        np.testing.assert_array_equal(Xd[xo:xo + n * d].reshape(n, d), X[order])
        np.testing.assert_array_equal(yd[int(BL.y_off[i]):int(BL.y_off[i]) + n], y[order])
        if Z is not None:
            q = Z.shape[1]
            zo = int(BL.z_off[i])
            np.testing.assert_array_equal(Zd[zo:zo + n * q].reshape(n, q), Z[order])
        o = int(BL.blk_off[i])
        got = nbr[o:o + n]
        want = np.full((n, BL.ldnbr), -1, dtype=np.int64)
        want[:, :m] = nn[:, 1:m + 1]
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("flags", [1, 2])
def test_other_maximin_routes_give_the_same_orders(flags):
    """Ranking every pivot choice by exact square roots (the route taken when
    candidates' squared distances lie within a few ulps) and taking one pivot
    per pass by a full scan (the route taken when no batch of pivots is
    certain) give the same orders as the default passes."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    probs, raw, thetas = _problems()
    BL = BatchedLikelihood(probs)
    BL.set_sources([r[0] for r in raw], [r[1] for r in raw], [r[2] for r in raw], [r[3] for r in raw])
    ids = list(range(len(probs)))
    a = BL.reorder(ids, thetas, return_orders=True)
    b = BL.reorder(ids, thetas, return_orders=True, maximin_flags=flags)
    for i, (x, y) in enumerate(zip(a, b)):
        np.testing.assert_array_equal(x, y)
        order, _ = _expected(*raw[i], thetas[i])
        np.testing.assert_array_equal(y, order)


def test_lattice_ties_through_the_cluster_kernel(oracle):
    """Exact ties (a lattice) and duplicates through the cluster maximin,
    by every route, against the oracle."""
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem, ordered_groups
    g = np.arange(30, dtype=float)
    X = np.array([[a, b] for a in g for b in g])
    X = np.vstack([X, X[::11]]) / 7.0
    n = X.shape[0]
    BL = BatchedLikelihood([BatchProblem(X, np.zeros(n), None, ordered_groups(n, 5))])
    BL.set_sources([X], [np.zeros(n)], [None], [5])
    ref = oracle.maximin_order(X)
    for flags in (0, 1, 2):
        o = BL.reorder([0], [np.zeros(4)], return_orders=True, maximin_flags=flags)[0]
        np.testing.assert_array_equal(o, ref)


def test_batched_reorder_subset_leaves_others():
    from pyscaledvecchia_gb300.batched import BatchedLikelihood
    probs, raw, thetas = _problems()
    BL = BatchedLikelihood(probs)
    BL.set_sources([r[0] for r in raw], [r[1] for r in raw], [r[2] for r in raw], [r[3] for r in raw])
    X0, nbr0 = BL.X.cpu().numpy().copy(), BL.nbr.cpu().numpy().copy()
    BL.reorder([1, 4], [thetas[1], thetas[4]])
    X1, nbr1 = BL.X.cpu().numpy(), BL.nbr.cpu().numpy()
    for i in range(len(probs)):
        n, d = raw[i][0].shape
        xo, o = int(BL.x_off[i]), int(BL.blk_off[i])
        if i in (1, 4):
            order, nn = _expected(*raw[i], thetas[i])
            np.testing.assert_array_equal(X1[xo:xo + n * d].reshape(n, d), raw[i][0][order])
        else:
            np.testing.assert_array_equal(X1[xo:xo + n * d], X0[xo:xo + n * d])
            np.testing.assert_array_equal(nbr1[o:o + n], nbr0[o:o + n])


def test_cluster_limits_and_grid_kernel_case(oracle):
    """Above one cluster's shared memory the one-problem maximin runs the
    grid-wide kernel; both sides of the limit agree with the oracle."""
    import pyscaledvecchia_gb300 as sv
    from pyscaledvecchia_gb300 import _lib
    lib, _ = _lib.device_ready()
    d = 64
    lim = int(lib.sv_maximin_cluster_max_rows(d))
    assert 1000 < lim < 20000
    rng = np.random.default_rng(5)
    for n in (lim, lim + 500):
        X = rng.random((n, d)) / np.exp(rng.uniform(-1, 1, d))
        np.testing.assert_array_equal(sv.maximin_order(X), oracle.maximin_order(X))


def test_reorder_rejects_oversized_problem():
    from pyscaledvecchia_gb300.batched import BatchedLikelihood, BatchProblem, ordered_groups
    from pyscaledvecchia_gb300 import _lib
    lib, _ = _lib.device_ready()
    n = int(lib.sv_maximin_cluster_max_rows(2)) + 10
    X = np.random.default_rng(0).random((n, 2))
    BL = BatchedLikelihood([BatchProblem(X, np.zeros(n), None, ordered_groups(n, 5))])
    BL.set_sources([X], [np.zeros(n)], [None], [5])
    assert not BL.device_reorderable(0)
    with pytest.raises(ValueError):
        BL.reorder([0], [np.zeros(4)])
