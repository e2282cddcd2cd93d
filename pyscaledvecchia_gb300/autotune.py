"""Team-width autotuner of the split-precision block kernels.

The split kernels (csrc/sv_loglik_split64.cu, float64 factorisation, and
csrc/sv_loglik_split.cu, double-float factorisation) give every conditioning
block a team of G lanes (4, 8, 16 or 32; 32/G blocks per warp).  The fastest
G depends on the kernel, the block size K = m + 1, the input dimension d and
the number of right-hand sides: measured on GB300 with the double-float
factorisation, 8 lanes beat 16 by 24 % at d = 3, m = 10 and by 14 % at d = 3,
m = 20, while 16 is the fastest at m = 30 and for every d >= 6.

``team_lanes(K, d, q, need_grad, precision)`` times the four widths on a
synthetic problem of that shape the first time the shape is seen on a device
(exact nearest-neighbour conditioning sets of uniform points, about 24,000
blocks, best of three evaluations per width) and keeps the choice in memory
and in a JSON file: ``$SV_AUTOTUNE_CACHE``, else
``~/.cache/pyscaledvecchia_gb300/team_lanes.json``, keyed by device name,
precision form and shape.  A width other than 16 is taken only when it is more than 3 % faster,
so that timing noise does not flip choices.  ``SV_AUTOTUNE=0`` turns
measurement off (16 lanes).

The team width changes the order of a block's float32 / double-float
operations, so split-form results can differ between widths at the level of
the split form's own rounding; pass ``team_lanes`` explicitly for results
that must not depend on the cache.  The float64 form has no team width.
"""
import json
import math
import os
import tempfile
import threading

import numpy as np

WIDTHS = (4, 8, 16, 32)
DEFAULT = 16
_MARGIN = 0.03
_lock = threading.Lock()
_mem = {}
_file_loaded = False


def cache_path():
    p = os.environ.get("SV_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "pyscaledvecchia_gb300", "team_lanes.json")


def shape_key(device, K, d, q, need_grad, precision="split"):
    return f"{device}|{precision}|K={int(K)}|d={int(d)}|q={int(q)}|grad={int(bool(need_grad))}"


def _load_file():
    global _file_loaded
    if _file_loaded:
        return
    _file_loaded = True
    try:
        with open(cache_path()) as f:
            data = json.load(f)
        if isinstance(data, dict):
            for k, v in data.items():
                if isinstance(v, int) and v in WIDTHS:
                    _mem.setdefault(k, v)
    except (OSError, ValueError):
        pass


def _save_file():
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path), prefix=".team_lanes.")
        with os.fdopen(fd, "w") as f:
            json.dump(_mem, f, indent=0, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home keeps the in-memory choice


def choose(times):
    """The width to use from {width: ms}: the fastest, unless the default is
    within the margin of it (the default when nothing was measured)."""
    if not times:
        return DEFAULT
    best = min(times, key=times.get)
    if DEFAULT in times and times[DEFAULT] <= (1.0 + _MARGIN) * times[best]:
        return DEFAULT
    return best


def measure(K, d, q, need_grad, precision="split", nblocks=24000, seed=0):
    """{width: ms} of one evaluation in the given split form of a synthetic
    problem with blocks of K points in d dimensions and q trend columns."""
    from . import _lib
    from .likelihood import DeviceProblem
    from .ordering import _nn_groups, find_ordered_nn
    _, torch = _lib.device_ready()
    m = max(int(K) - 1, 0)
    n = max(int(nblocks), m + 1)
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    Z = np.ones((n, q)) if q > 0 else None
    groups = _nn_groups(find_ordered_nn(X, m), m)
    prob = DeviceProblem(X, y, Z, groups)
    P = d + 2
    theta = np.concatenate([[0.0], np.full(d, math.log(0.3)), [math.log(1e-3)]])
    th = _lib.to_dev(torch, theta, np.float64)
    times = {}
    for w in WIDTHS:
        def run():
            prob.launch(th, P, 2.5, False, need_grad, 0.0, 0.0, True, precision=precision, team_lanes=w)
        try:
            run()
            torch.cuda.synchronize()
        except (ValueError, RuntimeError):
            continue  # a width the library refuses for this shape is not a candidate
        best = float("inf")
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        times[w] = best
    return times


def team_lanes(K, d, q, need_grad, precision="split", measure_fn=None, device=None):
    """Team width for blocks of up to K points (K <= 32) in d dimensions with
    q trend columns in the given split form ("split" or "split_df")."""
    if os.environ.get("SV_AUTOTUNE", "1") == "0":
        return DEFAULT
    if K <= 1:
        return DEFAULT
    if device is None:
        from . import _lib
        _, torch = _lib.device_ready()
        if torch.cuda.is_current_stream_capturing():
            return _mem.get(shape_key(torch.cuda.get_device_name(torch.cuda.current_device()),
                                      K, d, q, need_grad, precision), DEFAULT)
        device = torch.cuda.get_device_name(torch.cuda.current_device())
    key = shape_key(device, K, d, q, need_grad, precision)
    with _lock:
        _load_file()
        if key in _mem:
            return _mem[key]
    times = (measure_fn or measure)(K, d, q, need_grad, precision=precision)
    w = choose(times)
    with _lock:
        _mem[key] = w
        _save_file()
    return w
