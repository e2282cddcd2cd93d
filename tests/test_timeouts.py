"""Bounded device waits that run out, on purpose, through test aids.

Every spin-wait in the library's kernels has an iteration limit after which
the kernel records SV_ETIMEOUT and returns instead of waiting on.  Two waits
are made to run out here by a flag that nothing then sets (no fault, no trap,
no endless loop):
  * the grid barrier of the grid-form maximin (sv_maximin_order_flags bit 3:
    one CTA does not arrive at the first barrier; every CTA's wait runs out
    after 4096 polls and every CTA returns);
  * the row-dependency wait of the sparse triangular solve
    (sv_joint_solve_flags bit 0: row 0 never publishes its result; the rows
    that depend on it give up after 4096 polls, the others finish).
The call returns SV_OK at launch; the status arrives in the info words, the
Python layer maps it to RuntimeError, and the next normal call on the same
device gives the normal result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_grid_maximin_barrier_wait_runs_out(oracle):
    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import maximin_order_device
    lib, torch = _lib.device_ready()
    rng = np.random.default_rng(4)
    X = rng.random((12000, 4))
    first = int(np.argmin(((X - X.mean(0)) ** 2).sum(1)))
    Xd = _lib.to_dev(torch, X, np.float64)
    _, info = maximin_order_device(torch, Xd, first, flags=4 | 8)
    info = info.cpu().numpy()
    assert int(info[0]) == _lib.SV_ETIMEOUT
    with pytest.raises(RuntimeError):
        _lib.check_info(lib, info, "sv_maximin_order")
    # the device is still usable: the grid form gives the oracle's order
    order, info = maximin_order_device(torch, Xd, first, flags=4)
    _lib.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
    np.testing.assert_array_equal(order.cpu().numpy(), oracle.maximin_order(X, first))


def _chain_problem(n, k):
    """A lower-bidiagonal-like dependency: row c depends on rows c-1..c-k."""
    nbr = np.full((n, k), -1, dtype=np.int32)
    for c in range(n):
        for i in range(k):
            if c - 1 - i >= 0:
                nbr[c, i] = c - 1 - i
    rng = np.random.default_rng(0)
    acol = rng.uniform(0.1, 0.3, (n, k + 1))
    acol[:, k] = rng.uniform(1.0, 2.0, n)
    return nbr, acol


def _solve(torch, lib, nbr, acol, R, flags):
    from pyscaledvecchia_gb300 import _lib
    n, k = nbr.shape
    nrhs = R.shape[1]
    X = torch.empty((n, nrhs), dtype=torch.float64, device="cuda")
    info = _lib.new_info(torch)
    ws = _lib.workspace(torch, lib.sv_joint_solve_workspace_bytes(n))
    nbr_d, acol_d, R_d = (_lib.to_dev(torch, nbr, np.int32), _lib.to_dev(torch, acol, np.float64),
                          _lib.to_dev(torch, R, np.float64))
    rc = lib.sv_joint_solve_flags(n, 0, k, k, _lib.ptr(nbr_d), _lib.ptr(acol_d), _lib.ptr(R_d),
                                  nrhs, _lib.ptr(X), _lib.ptr(info), _lib.ptr(ws), ws.numel(), flags,
                                  _lib.stream_handle(torch))
    assert rc == _lib.SV_OK
    return X.cpu().numpy(), info.cpu().numpy()


def test_joint_solve_row_wait_runs_out():
    from pyscaledvecchia_gb300 import _lib
    lib, torch = _lib.device_ready()
    n, k = 3000, 3
    nbr, acol = _chain_problem(n, k)
    R = np.random.default_rng(1).standard_normal((n, 4))
    _, info = _solve(torch, lib, nbr, acol, R, flags=1)
    assert int(info[0]) == _lib.SV_ETIMEOUT
    assert int(info[1]) >= 1  # a row that waited on row 0 or on a row behind it
    with pytest.raises(RuntimeError):
        _lib.check_info(lib, info, "sv_joint_solve")
    # the next normal call solves the system
    X, info = _solve(torch, lib, nbr, acol, R, flags=0)
    _lib.check_info(lib, info, "sv_joint_solve")
    ref = np.zeros_like(R)
    for c in range(n):
        s = R[c].copy()
        for i in range(k):
            if nbr[c, i] >= 0:
                s -= acol[c, i] * ref[nbr[c, i]]
        ref[c] = s / acol[c, k]
    np.testing.assert_allclose(X, ref, rtol=1e-12, atol=1e-12)
