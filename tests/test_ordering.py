"""GPU maximin ordering (sv_maximin_order) and neighbour searches
(sv_ordered_knn, sv_knn_query).

Covers the properties of the reference's tests/test_ordering.py
(permutation, determinism, brute-force neighbour sets, self column and -1
padding, ``start``), bit-exact agreement with the reference's own orders
(tests/golden/ordering.npz, including lattice ties and duplicate points) and
with the oracle at sizes the reference cannot reach.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sv():
    import pyscaledvecchia_gb300 as sv
    return sv


def test_order_is_a_permutation():
    X = np.random.default_rng(1).random((257, 5))
    o = _sv().maximin_order(X)
    assert sorted(o.tolist()) == list(range(257))


def test_order_is_deterministic():
    X = np.random.default_rng(2).random((90, 2))
    np.testing.assert_array_equal(_sv().maximin_order(X), _sv().maximin_order(X))


def test_neighbours_match_brute_force():
    sv = _sv()
    rng = np.random.default_rng(7)
    n, d, m = 150, 3, 9
    X = rng.random((n, d))
    Xo = X[sv.maximin_order(X)]
    nn = sv.find_ordered_nn(Xo, m)
    for i in range(1, n):
        k = min(i, m)
        dist = np.linalg.norm(Xo[:i] - Xo[i], axis=1)
        assert set(np.argsort(dist)[:k].tolist()) == set(nn[i, 1:k + 1].tolist()), i


def test_self_column_and_padding():
    X = np.random.default_rng(3).random((40, 2))
    nn = _sv().find_ordered_nn(X, 6)
    assert np.array_equal(nn[:, 0], np.arange(40))
    assert np.all(nn[0, 1:] == -1)
    assert np.sum(nn[3, 1:] != -1) == 3


def test_start_gives_the_same_sets():
    sv = _sv()
    X = np.random.default_rng(4).random((80, 3))
    full = sv.find_ordered_nn(X, 7, start=0)
    part = sv.find_ordered_nn(X, 7, start=50)
    assert np.array_equal(full[50:], part[50:])
    assert np.all(part[1:50, 1:] == -1)


def test_maximin_bit_exact_vs_reference(golden_ordering):
    g = golden_ordering
    names = sorted({k[3:-2] for k in g.files if k.startswith("mm_") and k.endswith("_X")})
    for nm in names:
        first = 17 if nm == "first" else None
        np.testing.assert_array_equal(_sv().maximin_order(g[f"mm_{nm}_X"], first),
                                      g[f"mm_{nm}_order"], err_msg=nm)


def test_neighbour_sets_vs_reference(golden_ordering):
    g = golden_ordering
    names = sorted({k[3:-2] for k in g.files if k.startswith("nn_") and k.endswith("_X")})
    for nm in names:
        X, ref = g[f"nn_{nm}_X"], g[f"nn_{nm}_nn"]
        m, start = (int(v) for v in g[f"nn_{nm}_meta"])
        got = _sv().find_ordered_nn(X, m, start=start)
        np.testing.assert_array_equal(got[:, 0], ref[:, 0])
        for i in range(X.shape[0]):
            assert set(got[i, 1:].tolist()) == set(ref[i, 1:].tolist()), (nm, i)


@pytest.mark.parametrize("n,d", [(2000, 8), (20000, 10), (6000, 3), (3000, 12)])
def test_maximin_bit_exact_vs_oracle(oracle, n, d):
    rng = np.random.default_rng(n + d)
    lam = np.exp(rng.uniform(np.log(0.05), np.log(50.0), d))
    X = rng.random((n, d)) / lam
    np.testing.assert_array_equal(_sv().maximin_order(X), oracle.maximin_order(X))


def test_maximin_ties_and_duplicates(oracle):
    g = np.arange(25, dtype=float)
    X = np.array([[a, b] for a in g for b in g])          # lattice: many exact ties
    X = np.vstack([X, X[::7]])                            # and exact duplicates
    np.testing.assert_array_equal(_sv().maximin_order(X), oracle.maximin_order(X))


def _maximin_routed(X, flags):
    import torch
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device
    lib, _ = _lib.device_ready()
    first = int(np.argmin(((X - X.mean(0)) ** 2).sum(1)))
    o, info = maximin_order_device(torch, _lib.to_dev(torch, X, np.float64), first, flags)
    _lib.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
    return o.cpu().numpy()


@pytest.mark.parametrize("flags", [4, 5, 6, 1, 2, 16, 17, 18])
def test_maximin_routes_vs_oracle(oracle, flags):
    """The grid form (flag 4: lists through global memory behind a grid
    barrier, one CTA per SM from 9,728 rows), the tree form (flag 16: one CTA
    over a 32-ary tree of the rows) and the exact-root and tie-pass routes
    (flags 1, 2, alone and with either form) give the reference's order on
    random rows, a lattice with duplicates and rows on a coarse grid of
    values."""
    rng = np.random.default_rng(11)
    g = np.arange(30, dtype=float)
    lattice = np.array([[a, b] for a in g for b in g])
    cases = [rng.random((12000, 4)) / np.exp(rng.uniform(-1, 1, 4)),
             np.vstack([lattice, lattice[::9]]) / 7.0,
             np.round(rng.random((2500, 3)) * 12) / 3.0,
             rng.random((700, 64))]
    for X in cases:
        np.testing.assert_array_equal(_maximin_routed(X, flags), oracle.maximin_order(X))


def test_maximin_form_limits():
    from pyscaledvecchia_gb300 import _lib
    lib, _ = _lib.device_ready()
    for d in (2, 10, 64):
        assert lib.sv_maximin_grid_max_rows(d) > lib.sv_maximin_cluster_max_rows(d)
        assert lib.sv_maximin_max_rows(d) == 2 ** 31 - 1
    assert lib.sv_maximin_grid_max_rows(10) > 500_000


@pytest.mark.parametrize("n,d,m,start", [(20000, 10, 30, 0), (5000, 3, 140, 0),
                                         (4000, 6, 25, 1500), (3000, 2, 8, 0)])
def test_ordered_knn_exact_vs_oracle(oracle, n, d, m, start):
    rng = np.random.default_rng(3 * n + d)
    X = rng.random((n, d))
    got = _sv().find_ordered_nn(X, m, start=start)
    ref = oracle.ordered_nn(X, m, start)
    np.testing.assert_array_equal(got, ref)  # same (distance, index) order


def test_knn_query_exact_vs_oracle(oracle):
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import knn_query_device
    lib, torch = _lib.device_ready()
    rng = np.random.default_rng(9)
    Xr = rng.random((12000, 6))
    Xq = rng.uniform(-0.1, 1.1, (3000, 6))
    nb, info = knn_query_device(torch, _lib.to_dev(torch, Xr, np.float64),
                                _lib.to_dev(torch, Xq, np.float64), 140)
    _lib.check_info(lib, info.cpu().numpy(), "knn")
    np.testing.assert_array_equal(nb.cpu().numpy(), oracle.knn_query(Xr, Xq, 140))


@pytest.mark.parametrize("k", [48, 140, 300])
def test_large_k_lattice_ties_and_duplicates(oracle, k):
    """Large k (one warp per query, a float32-bounded superset settled by
    exact keys): lattice rows with exact ties and duplicated rows, ordered
    and query searches, against the oracle."""
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import knn_query_device
    lib, torch = _lib.device_ready()
    g = np.arange(11, dtype=float)
    X = np.array([[a, b, c] for a in g for b in g for c in g]) / 3.0
    X = np.vstack([X, X[::5]])
    rng = np.random.default_rng(1)
    X = X[rng.permutation(len(X))]
    np.testing.assert_array_equal(_sv().find_ordered_nn(X, k, start=200), oracle.ordered_nn(X, k, 200))
    Xq = np.vstack([X[:300], rng.uniform(-0.5, 4.0, (300, 3))])
    nb, info = knn_query_device(torch, _lib.to_dev(torch, X, np.float64), _lib.to_dev(torch, Xq, np.float64), k)
    _lib.check_info(lib, info.cpu().numpy(), "knn")
    np.testing.assert_array_equal(nb.cpu().numpy(), oracle.knn_query(X, Xq, k))


def test_knn_lattice_ties(oracle):
    g = np.arange(12, dtype=float)
    X = np.array([[a, b, c] for a in g for b in g for c in g])
    rng = np.random.default_rng(0)
    X = X[rng.permutation(len(X))]
    np.testing.assert_array_equal(_sv().find_ordered_nn(X, 20), oracle.ordered_nn(X, 20))
