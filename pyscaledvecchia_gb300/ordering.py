"""Maximin ordering and ordered nearest neighbours on the GPU.

Drop-in counterpart of the reference's ``scaled_vecchia.ordering``
(src/scaled_vecchia/ordering.py):

  maximin_order     ordering.py:62-73 (the farthest-point loop of :27-59 runs
                    in sv_maximin_order; ``first`` is chosen on the host with
                    the reference's own NumPy expression, :72)
  find_ordered_nn   ordering.py:76-116 (sv_ordered_knn)
  _nn_groups        ordering.py:119-127 (host bookkeeping)

Both searches are exact: the ordering reproduces the reference's IEEE
sequential float64 arithmetic and tie-breaking bit for bit, and neighbour
sets are the exact (distance, index) nearest sets.
"""
from __future__ import annotations

import numpy as np

from . import _lib

__all__ = ["maximin_order", "find_ordered_nn"]


def maximin_order_device(torch, Xd, first: int, flags: int = 0):
    """Maximin permutation of the rows of a device (n, d) float64 tensor.
    ``flags`` (test aids, same order): 1 ranks every pivot choice by exact
    roots, 2 takes pivots by tie passes only, 4 forces the grid form, 16 the
    tree form; 8 (with 4) makes the grid barrier's bounded wait run out
    (SV_ETIMEOUT in info)."""
    lib = _lib.load_library()
    n, d = Xd.shape
    order = torch.empty(n, dtype=torch.int64, device="cuda")
    info = _lib.new_info(torch)
    ws = _lib.workspace(torch, lib.sv_maximin_workspace_bytes_flags(n, d, int(flags)))
    if flags:
        rc = lib.sv_maximin_order_flags(_lib.ptr(Xd), n, d, int(first), _lib.ptr(order), _lib.ptr(info),
                                        _lib.ptr(ws), ws.numel(), int(flags), _lib.stream_handle(torch))
    else:
        rc = lib.sv_maximin_order(_lib.ptr(Xd), n, d, int(first), _lib.ptr(order), _lib.ptr(info),
                                  _lib.ptr(ws), ws.numel(), _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_maximin_order")
    return order, info


def maximin_order(X: np.ndarray, first: int | None = None) -> np.ndarray:
    """Exact maximum-minimum-distance ordering.

    Sequentially picks the point farthest from the set already chosen.  The
    first point is the one closest to the centroid.
    """
    X = np.ascontiguousarray(X, dtype=np.float64)
    if first is None:
        first = int(np.argmin(((X - X.mean(0)) ** 2).sum(1)))
    lib, torch = _lib.device_ready()
    n = X.shape[0]
    if n == 0:
        return np.empty(0, dtype=np.int64)
    Xd = _lib.to_dev(torch, X, np.float64)
    order, info = maximin_order_device(torch, Xd, first)
    out = order.cpu().numpy()
    _lib.check_info(lib, info.cpu().numpy(), "sv_maximin_order")
    return out


def ordered_nn_device(torch, Xd, m: int, start: int = 0):
    lib = _lib.load_library()
    n, d = Xd.shape
    nn = torch.empty((n, m + 1), dtype=torch.int64, device="cuda")
    info = _lib.new_info(torch)
    ws = _lib.workspace(torch, lib.sv_ordered_knn_workspace_bytes(n, d))
    rc = lib.sv_ordered_knn(_lib.ptr(Xd), n, d, int(m), int(start), _lib.ptr(nn), _lib.ptr(info),
                            _lib.ptr(ws), ws.numel(), _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_ordered_knn")
    return nn, info


def find_ordered_nn(X: np.ndarray, m: int, start: int = 0,
                    block_size: int = 1024) -> np.ndarray:
    """For each i, the min(i, m) nearest neighbours among indices < i.

    Column 0 is i itself, columns 1..k the neighbours (nearest first; ties go
    to the smaller index), entries beyond min(i, m) are -1.  ``start`` skips
    rows whose neighbours are not needed.  ``block_size`` is accepted for
    signature compatibility; the device search has no row blocking.
    """
    del block_size
    X = np.ascontiguousarray(X, dtype=float)
    lib, torch = _lib.device_ready()
    n = X.shape[0]
    if n == 0:
        return np.full((0, m + 1), -1, dtype=np.int64)
    Xd = _lib.to_dev(torch, X, np.float64)
    nn, info = ordered_nn_device(torch, Xd, int(m), int(start))
    out = nn.cpu().numpy()
    _lib.check_info(lib, info.cpu().numpy(), "sv_ordered_knn")
    return out


def knn_query_device(torch, Xref_d, Xq_d, k: int):
    """k nearest rows of Xref for every row of Xq (sorted), device tensors."""
    lib = _lib.load_library()
    nr, d = Xref_d.shape
    nq = Xq_d.shape[0]
    nb = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    info = _lib.new_info(torch)
    ws = _lib.workspace(torch, lib.sv_knn_query_workspace_bytes(nr, nq, d))
    rc = lib.sv_knn_query(_lib.ptr(Xref_d), nr, _lib.ptr(Xq_d), nq, d, int(k), _lib.ptr(nb),
                          _lib.ptr(info), _lib.ptr(ws), ws.numel(), _lib.stream_handle(torch))
    _lib.check(lib, rc, "sv_knn_query")
    return nb, info


def _nn_groups(nn: np.ndarray, m: int):
    """Split rows by conditioning-set size so each group can be batched."""
    n = nn.shape[0]
    ks = np.minimum(np.arange(n), m)
    groups = []
    for k in np.unique(ks):
        rows = np.where(ks == k)[0]
        groups.append((rows, nn[rows, 1:k + 1]))
    return groups
