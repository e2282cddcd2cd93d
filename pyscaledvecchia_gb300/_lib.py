"""ctypes binding of libsvgpu.so and the device-memory plumbing around it.

Device buffers are torch CUDA tensors (torch is used only for allocation,
streams and host<->device copies); every computation runs in the library's
own sm_103a kernels.  There is no CPU fallback: without a CUDA device or
without the built library every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

SV_OK, SV_EINVAL, SV_ECHOL, SV_ETIMEOUT, SV_ECUDA, SV_ENOSPC = range(6)

_lock = threading.Lock()
_lib = None

c_i32, c_i64, c_dbl, c_sz, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t, ctypes.c_void_p


class LoglikDesc(ctypes.Structure):
    """Mirror of sv_loglik_desc (include/svgpu.h)."""
    _fields_ = [("n", c_i64), ("nblk", c_i64), ("nblk_warp", c_i64),
                ("d", c_i32), ("q", c_i32), ("ldnbr", c_i32), ("kmax", c_i32),
                ("need_grad", c_i32), ("estimate_nu", c_i32), ("chunked", c_i32),
                ("precision", c_i32), ("team_lanes", c_i32), ("split_rho_min", c_dbl),
                ("nu", c_dbl), ("var_penalty", c_dbl),
                ("log_var_target", c_dbl)]


class ProbDesc(ctypes.Structure):
    """Mirror of sv_prob_desc (include/svgpu.h)."""
    _fields_ = [("n", c_i64), ("x_off", c_i64), ("y_off", c_i64), ("z_off", c_i64),
                ("blk_off", c_i64), ("nblk", c_i64), ("d", c_i32), ("q", c_i32),
                ("estimate_nu", c_i32), ("skip", c_i32), ("nu", c_dbl), ("var_penalty", c_dbl),
                ("log_var_target", c_dbl)]


class BatchDesc(ctypes.Structure):
    """Mirror of sv_batch_desc (include/svgpu.h)."""
    _fields_ = [("nprob", c_i64), ("nblk", c_i64), ("nwarp", c_i64), ("ncta", c_i64),
                ("nx", c_i64), ("dmax", c_i32), ("qmax", c_i32), ("kmax", c_i32),
                ("ldnbr", c_i32), ("need_grad", c_i32), ("any_estimate_nu", c_i32),
                ("chunked", c_i32), ("precision", c_i32), ("team_lanes", c_i32),
                ("theta_stride", c_i32), ("out_stride", c_i32), ("general_nu", c_i32),
                ("split_rho_min", c_dbl), ("nblk_max", c_i64)]


class ReorderProb(ctypes.Structure):
    """Mirror of sv_reorder_prob (include/svgpu.h)."""
    _fields_ = [("n", c_i64), ("xe_off", c_i64), ("ye_off", c_i64), ("ze_off", c_i64),
                ("x_off", c_i64), ("y_off", c_i64), ("z_off", c_i64), ("blk_off", c_i64),
                ("first", c_i64), ("d", c_i32), ("q", c_i32), ("m", c_i32), ("flags", c_i32)]


class PackGroup(ctypes.Structure):
    """Mirror of sv_pack_group (include/svgpu.h)."""
    _fields_ = [("rows", c_vp), ("nb", c_vp), ("count", c_i64), ("out_off", c_i64),
                ("k", c_i32), ("pad", c_i32)]


class ChunkGroup(ctypes.Structure):
    """Mirror of sv_chunk_group (include/svgpu.h)."""
    _fields_ = [("count", c_i64), ("out_off", c_i64), ("base", c_i32), ("step", c_i32)]


class ReorderDesc(ctypes.Structure):
    """Mirror of sv_reorder_desc (include/svgpu.h)."""
    _fields_ = [("nprob", c_i64), ("dmax", c_i32), ("ldnbr", c_i32)]


class PredDesc(ctypes.Structure):
    """Mirror of sv_pred_desc (include/svgpu.h)."""
    _fields_ = [("nall", c_i64), ("nobs", c_i64), ("nblk", c_i64), ("d", c_i32), ("k", c_i32),
                ("ldnbr", c_i32), ("general", c_i32), ("target_nugget", c_i32),
                ("precision", c_i32), ("nu", c_dbl), ("split_rho_min", c_dbl),
                ("matern_table", c_vp)]


# SV_ABI_VERSION of include/svgpu.h that the structures above mirror
ABI_VERSION = 4

# name -> (restype, argtypes); every symbol declared in include/svgpu.h
SIGNATURES = {
    "sv_status_string": (ctypes.c_char_p, [c_i32]),
    "sv_abi_version": (c_i32, []),
    "sv_last_cuda_error": (c_i32, []),
    "sv_maximin_workspace_bytes": (c_sz, [c_i64, c_i32]),
    "sv_maximin_order": (c_i32, [c_vp, c_i64, c_i32, c_i64, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "sv_maximin_order_flags": (c_i32, [c_vp, c_i64, c_i32, c_i64, c_vp, c_vp, c_vp, c_sz, c_i32, c_vp]),
    "sv_maximin_max_rows": (c_i64, [c_i32]),
    "sv_maximin_grid_max_rows": (c_i64, [c_i32]),
    "sv_maximin_workspace_bytes_flags": (c_sz, [c_i64, c_i32, c_i32]),
    "sv_ordered_knn_workspace_bytes": (c_sz, [c_i64, c_i32]),
    "sv_ordered_knn": (c_i32, [c_vp, c_i64, c_i32, c_i32, c_i64, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "sv_knn_query_workspace_bytes": (c_sz, [c_i64, c_i64, c_i32]),
    "sv_knn_query": (c_i32, [c_vp, c_i64, c_vp, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "sv_maximin_cluster_max_rows": (c_i64, [c_i32]),
    "sv_reorder_batched_workspace_bytes": (c_sz, [ctypes.POINTER(ReorderDesc), c_vp]),
    "sv_reorder_batched": (c_i32, [ctypes.POINTER(ReorderDesc), c_vp, c_vp] + [c_vp] * 10 + [c_sz, c_vp]),
    "sv_loglik_workspace_bytes": (c_sz, [ctypes.POINTER(LoglikDesc)]),
    "sv_pack_blocks": (c_i32, [c_vp, c_i32, c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "sv_chunk_ids": (c_i32, [c_vp, c_i32, c_vp, c_vp]),
    "sv_vecchia_loglik": (c_i32, [ctypes.POINTER(LoglikDesc), c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                  c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "sv_loglik_shard_sizes": (c_i32, [ctypes.POINTER(LoglikDesc), c_vp, c_vp, c_vp]),
    "sv_vecchia_loglik_stage": (c_i32, [ctypes.POINTER(LoglikDesc), c_i32, c_i32, c_i32] + [c_vp] * 14
                                + [c_sz, c_vp]),
    "sv_loglik_batched_workspace_bytes": (c_sz, [ctypes.POINTER(BatchDesc)]),
    "sv_vecchia_loglik_batched": (c_i32, [ctypes.POINTER(BatchDesc)] + [c_vp] * 15 + [c_sz, c_vp]),
    "sv_vecchia_loglik_noalloc": (c_i32, [ctypes.POINTER(LoglikDesc), c_vp, c_vp, c_vp, c_vp, c_vp,
                                          c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "sv_encoder_param_count": (c_i64, []),
    "sv_encoder_workspace_bytes": (c_sz, [c_i64, c_i32, c_i32]),
    "sv_encoder_pack": (c_i32, [c_vp, c_i64, c_vp, c_vp]),
    "sv_encoder_to_bf16": (c_i32, [c_vp, c_vp, c_i64, c_vp]),
    "sv_encoder_forward": (c_i32, [c_i64, c_i32] + [c_vp] * 5 + [c_i32, c_vp, c_sz, c_vp]),
    "sv_encoder_backward": (c_i32, [c_i64, c_i32] + [c_vp] * 10 + [c_sz, c_vp]),
    "sv_encoder_adam": (c_i32, [c_vp] * 5 + [c_i64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_float, c_i32, ctypes.c_float, c_vp]),
    "sv_matern_eval": (c_i32, [c_vp, c_i64, c_dbl, c_i32, c_i32, c_vp, c_vp]),
    "sv_matern_table_doubles": (c_i64, []),
    "sv_matern_table": (c_i32, [c_dbl, c_vp, c_i64, c_vp]),
    "sv_bessel_k": (c_i32, [c_vp, c_i64, c_dbl, c_vp, c_vp]),
    "sv_block_cov": (c_i32, [c_vp, c_i64, c_i32, c_i32, c_vp, c_dbl, c_dbl, c_dbl, c_i32, c_i32,
                             c_dbl, c_vp, c_vp, c_vp, c_vp]),
    "sv_batch_chol_workspace_bytes": (c_sz, [c_i64]),
    "sv_batch_chol": (c_i32, [c_vp, c_i64, c_i32, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "sv_forward_solve": (c_i32, [c_vp, c_vp, c_i64, c_i32, c_i32, c_vp, c_vp]),
    "sv_backsolve_LT": (c_i32, [c_vp, c_vp, c_i64, c_i32, c_i32, c_vp, c_vp]),
    "sv_predict_blocks": (c_i32, [ctypes.POINTER(PredDesc), c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                  c_vp, c_vp, c_vp, c_vp, c_vp]),
    "sv_joint_solve_workspace_bytes": (c_sz, [c_i64]),
    "sv_fp64_probe_threads": (c_i64, []),
    "sv_fp64_fma_probe": (c_i32, [c_vp, c_i32, c_vp]),
    "sv_fp32_fma_probe": (c_i32, [c_vp, c_i32, c_vp]),
    "sv_device_reads_host_memory": (c_i32, [c_vp]),
    "sv_joint_solve": (c_i32, [c_i64, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp,
                               c_vp, c_sz, c_vp]),
    "sv_joint_solve_flags": (c_i32, [c_i64, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp,
                                     c_vp, c_vp, c_sz, c_i32, c_vp]),
    "sv_joint_var_diag": (c_i32, [c_i64, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz,
                                  c_vp, c_sz, c_vp]),
}


def library_path() -> str:
    return _build.LIBPATH


def load_library(check_current: bool = True):
    """dlopen libsvgpu.so and attach the prototypes (no CUDA call is made)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIBPATH
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        if check_current and not _build.is_current():
            raise RuntimeError(f"{path} is stale relative to csrc/: rebuild it")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.sv_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{path} implements interface version {lib.sv_abi_version()}, "
                               f"these bindings version {ABI_VERSION}: rebuild it")
        _lib = lib
        return lib


def _torch():
    import torch
    return torch


def device_ready():
    """Load the library and make sure a CUDA device is present (else raise)."""
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("scaled Vecchia GPU kernels need a CUDA device; none is available")
    return load_library(), torch


def stream_handle(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def to_dev(torch, arr, dtype):
    """numpy -> device tensor (contiguous).  A plain copy from pageable
    memory: over the GB300's chip-to-chip link it takes half the time of a
    copy staged through pinned memory (48 MB: 0.29 ms against 0.57 ms)."""
    a = np.ascontiguousarray(arr, dtype=dtype)
    return torch.from_numpy(a).to("cuda")


_HOST_READABLE = None    # None: ask the current device; True / False: fixed
_HOST_READABLE_DEV = {}  # device index -> answer
_SIDE = {}               # device index -> side stream


def side_stream(torch):
    """A second stream of the library on the current device, for work that
    may overlap the host's copies on the current stream (created on first
    use)."""
    dev = torch.cuda.current_device()
    s = _SIDE.get(dev)
    if s is None:
        s = _SIDE[dev] = torch.cuda.Stream(device=dev)
    return s


def device_reads_host_memory(lib):
    """True when kernels may read ordinary NumPy memory directly (the current
    device reports coherent pageable access through the host's page
    tables)."""
    if _HOST_READABLE is not None:
        return _HOST_READABLE
    dev = _torch().cuda.current_device()
    v = _HOST_READABLE_DEV.get(dev)
    if v is None:
        c = ctypes.c_int32(0)
        check(lib, lib.sv_device_reads_host_memory(ctypes.byref(c)), "sv_device_reads_host_memory")
        v = _HOST_READABLE_DEV[dev] = bool(c.value)
    return v


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else ctypes.c_void_p(0)


def new_info(torch):
    return torch.zeros(4, dtype=torch.int32, device="cuda")


def workspace(torch, nbytes):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")


def check(lib, rc, what):
    """Map a returned status to the reference's exceptions."""
    if rc == SV_OK:
        return
    msg = lib.sv_status_string(rc).decode()
    if rc == SV_EINVAL:
        raise ValueError(f"{what}: {msg}")
    if rc == SV_ECHOL:
        raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
    if rc == SV_ECUDA:
        raise RuntimeError(f"{what}: CUDA error {lib.sv_last_cuda_error()}")
    raise RuntimeError(f"{what}: {msg}")


def check_info(lib, info_host, what):
    st = int(info_host[0])
    if st == SV_OK:
        return
    if st == SV_ECHOL:
        raise np.linalg.LinAlgError("block Cholesky failed even with jitter")
    if st == SV_ETIMEOUT:
        raise RuntimeError(f"{what}: a bounded device wait ran out (row/step {int(info_host[1])})")
    check(lib, st, what)
