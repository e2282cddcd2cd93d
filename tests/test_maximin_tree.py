"""The tree form of the exact maximin (sv_maximin_order beyond the grid
form's shared memory, or flag 16): the same order as the grid form where both
run, and at a million rows the properties every maximin order has.

The tree form is pinned to the oracle on random rows, lattices with
duplicates and coarse grids of values (tests/test_ordering.py, flags 16-18)
and at the benchmark's 200,000 rows (tests/test_c2_parity.py)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rows(n, d, seed):
    rng = np.random.default_rng(seed)
    lam = np.exp(rng.uniform(math.log(0.05), math.log(50.0), d))
    return rng.random((n, d)) / lam


def _order(X, flags):
    import torch

    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device
    lib, _ = _lib.device_ready()
    first = int(np.argmin(((X - X.mean(0)) ** 2).sum(1)))
    Xd = _lib.to_dev(torch, X, np.float64)
    o, info = maximin_order_device(torch, Xd, first, flags)
    _lib.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
    return o, Xd, first


def test_tree_form_equals_grid_form_at_500k():
    X = _rows(500_000, 10, 3)
    from pyscaledvecchia_gb300 import _lib
    lib = _lib.load_library()
    assert X.shape[0] <= lib.sv_maximin_grid_max_rows(10)
    tree, _, _ = _order(X, 16)
    grid, _, _ = _order(X, 4)
    np.testing.assert_array_equal(tree.cpu().numpy(), grid.cpu().numpy())


def test_tree_form_at_a_million_rows():
    """1,000,000 rows in d = 10 (the default route there): a permutation
    starting at the given first row, and the distance of each row to the rows
    before it (the ordered 1-nearest-neighbour search, exact) never grows
    along the order: the maximin distances of the reference's loop."""
    import torch

    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import ordered_nn_device
    lib = _lib.load_library()
    n, d = 1_000_000, 10
    X = _rows(n, d, 5)
    assert n > lib.sv_maximin_grid_max_rows(d)
    o, Xd, first = _order(X, 0)
    order = o.cpu().numpy()
    assert order[0] == first
    assert np.array_equal(np.sort(order), np.arange(n))
    Xo = Xd[o].contiguous()
    nn, info = ordered_nn_device(torch, Xo, 1)
    _lib.check_info(lib, info.cpu().numpy(), "knn")
    j = nn[1:, 1].cpu().numpy()
    Xh = Xo.cpu().numpy()
    s = np.zeros(n - 1)
    for l in range(d):  # the reference's sequential sum (ordering.py:52-57)
        df = Xh[1:, l] - Xh[j, l]
        s += df * df
    dist = np.sqrt(s)
    assert np.all(np.diff(dist) <= 0.0), int(np.argmax(np.diff(dist) > 0))
