"""Host-side rules of the likelihood path (CPU): the conditioning-set groups
of ordering.py:119-127, the jitter-sharing chunk rule of _covariance.py:255-259
(which blocks a failed factorisation retries together, so it decides the
numbers returned) and the block table handed to the device."""
import numpy as np
import pytest

from pyscaledvecchia_gb300._covariance import _chunks
from pyscaledvecchia_gb300.likelihood import chunk_ids, pack_groups
from pyscaledvecchia_gb300.ordering import _nn_groups


def _toy_nn(n, m, seed=0):
    # nn[i] = [i, neighbours of i among rows < i] as find_ordered_nn returns it
    rng = np.random.default_rng(seed)
    nn = np.full((n, m + 1), -1, dtype=np.int64)
    for i in range(n):
        nn[i, 0] = i
        k = min(i, m)
        if k:
            nn[i, 1:k + 1] = rng.choice(i, size=k, replace=False)
    return nn


def test_chunk_rule_sizes():
    # rows per chunk: 4e6 // (K^2 P): 346 at K = 31 with the score (P = 12),
    # 4162 without (P = 1), 201 at K = 141
    for (K, P, step) in ((31, 12, 346), (31, 1, 4162), (141, 1, 201)):
        sl = list(_chunks(10_000, K, P))
        assert sl[0] == (0, step)
        assert all(b - a == step for a, b in sl[:-1])
        assert sl[-1][1] == 10_000
        assert all(sl[i][1] == sl[i + 1][0] for i in range(len(sl) - 1))
    assert list(_chunks(0, 31, 12)) == []
    assert list(_chunks(5, 10_000, 100)) == [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5)]  # at least one row


def test_nn_groups_split_rows_by_conditioning_size():
    n, m = 50, 6
    nn = _toy_nn(n, m)
    groups = _nn_groups(nn, m)
    assert [g[1].shape[1] for g in groups] == list(range(m + 1))
    for k, (rows, nb) in enumerate(groups):
        want_rows = np.arange(k, k + 1) if k < m else np.arange(m, n)
        np.testing.assert_array_equal(rows, want_rows)
        np.testing.assert_array_equal(nb, nn[rows, 1:k + 1])


def test_pack_groups_block_table():
    n, m = 80, 40  # k up to 40: blocks of K > 32 go after the warp-sized ones
    nn = _toy_nn(n, m, seed=1)
    groups = _nn_groups(nn, m)
    rowb, kb, nbr, gid, gk, gl = pack_groups(groups, n)
    assert rowb.shape[0] == n and sorted(rowb.tolist()) == list(range(n))
    big = kb + 1 > 32
    assert not np.any(np.diff(big.astype(np.int8)) < 0)  # warp-sized blocks first
    for b in range(n):
        i, k = int(rowb[b]), int(kb[b])
        assert k == min(i, m)
        np.testing.assert_array_equal(nbr[b, :k], nn[i, 1:k + 1])
        assert np.all(nbr[b, k:] == -1)
        assert gk[gid[b]] == k
    assert sum(gl) == n
    bad = [(g[0], g[1].copy()) for g in groups]
    bad[-1][1][0, 0] = n
    with pytest.raises(ValueError):
        pack_groups(bad, n)


def test_chunk_ids_number_chunks_group_by_group():
    gk, gl = [0, 1, 30], [1, 1, 1000]
    gid = np.repeat(np.arange(3, dtype=np.int32), gl)
    ids = chunk_ids(gid, gk, gl, 12)
    # groups of one row are one chunk each; K = 31 with P = 12: 346 rows per chunk
    assert ids[0] == 0 and ids[1] == 1
    big = ids[2:]
    np.testing.assert_array_equal(big, 2 + np.arange(1000) // 346)


def test_matern_table_gates_follow_the_library():
    """The host's gates (which fixed nu gets Matern tables, which takes the
    split forms) use the library's limits: the float64 tables up to
    kMtabNuMax, the float32 ones up to kFtabNuMax and at least 1e-3 from an
    integer (csrc/sv_matern.cuh), an estimated nu always (decided on the
    device at each theta)."""
    import os
    import re

    from pyscaledvecchia_gb300.likelihood import matern_table_nu, split_nu
    src = open(os.path.join(os.path.dirname(__file__), os.pardir, "pyscaledvecchia_gb300",
                            "csrc", "sv_matern.cuh")).read()
    mtab_max = float(re.search(r"kMtabNuMax = ([0-9.]+);", src).group(1))
    ftab_max = float(re.search(r"kFtabNuMax = ([0-9.]+);", src).group(1))
    assert (mtab_max, ftab_max) == (10.0, 8.0)
    for nu in (0.5, 1.5, 2.5):
        assert not matern_table_nu(nu) and split_nu(nu)
    assert matern_table_nu(0.8) and split_nu(0.8)
    assert matern_table_nu(mtab_max) and not matern_table_nu(mtab_max + 0.5)
    assert split_nu(ftab_max - 0.5) and not split_nu(ftab_max + 0.5)
    assert matern_table_nu(2.0) and not split_nu(2.0)          # within 1e-3 of an integer
    assert not split_nu(1.0005) and split_nu(1.002)
    assert not matern_table_nu(1e-12)                         # below the tables' first octave
    assert not matern_table_nu(0.8, estimate_nu=True)         # estimated: built per theta
    assert split_nu(None, estimate_nu=True) and not split_nu(None)
