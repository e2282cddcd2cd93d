"""sv_vecchia_loglik_noalloc: the likelihood evaluation for callers that
cannot allocate device memory (an application whose own fixed pool owns the
GPU's memory, or a loop that must not call cudaMalloc because it synchronises
the device and can fail under memory pressure).  Its scratch is a fixed array
inside the library instead of a caller-provided workspace; its results must
be those of sv_vecchia_loglik on the same inputs.

Two calls in a row on different problems (the second also uses the CTA
kernel, K = 41) check that the contents the first call leaves in the shared
array do not leak into the second; the same for the split forms, whose
scratch also holds the float32 coordinate pairs and which run the jitter
fix-up and float64 re-evaluation passes, the last call filling most of the
array.  Collected last so that a run stopping at the first failure has run
every other test.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(seed, n, d, m):
    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups, find_ordered_nn, maximin_order
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = rng.standard_normal(n)
    lam = np.exp(rng.uniform(math.log(0.1), math.log(3.0), d))
    theta = np.concatenate([[math.log(1.4)], np.log(lam), [math.log(3e-3)]])
    order = maximin_order(X / lam)
    nn = find_ordered_nn((X / lam)[order], m)
    prob = DeviceProblem(X[order], y[order], np.ones((n, 1)), _nn_groups(nn, m))
    return prob, theta


def _desc(prob, P, precision=0):
    from pyscaledvecchia_gb300 import _lib
    D = _lib.LoglikDesc()
    D.n, D.nblk, D.nblk_warp = prob.n, prob.nblk, prob.nblk_warp
    D.d, D.q, D.ldnbr, D.kmax = prob.d, prob.q, prob.ldnbr, prob.kmax
    D.need_grad, D.estimate_nu, D.chunked, D.precision = 1, 0, 1, precision
    D.team_lanes = 16
    D.nu, D.var_penalty, D.log_var_target = 2.5, 0.0, 0.0
    return D


def _noalloc_call(prob, theta, precision=0):
    from pyscaledvecchia_gb300 import _lib
    lib, torch = _lib.device_ready()
    P = prob.d + 2
    D = _desc(prob, P, precision)
    th = _lib.to_dev(torch, theta, np.float64)
    out = torch.empty(1 + P + P * P + prob.q, dtype=torch.float64, device="cuda")
    info = _lib.new_info(torch)
    chunk = prob.chunk_tensor(P)
    rc = lib.sv_vecchia_loglik_noalloc(D, _lib.ptr(th), _lib.ptr(prob.X), _lib.ptr(prob.y),
                                       _lib.ptr(prob.Z), _lib.ptr(prob.rowb), _lib.ptr(prob.kb),
                                       _lib.ptr(prob.nbr), _lib.ptr(chunk), _lib.ptr(out),
                                       _lib.ptr(info), _lib.stream_handle(torch))
    assert rc == 0, lib.sv_status_string(rc)
    res = out.cpu().numpy()
    assert int(info.cpu().numpy()[0]) == 0
    return res[0], res[1:1 + P], res[1 + P:1 + P + P * P].reshape(P, P), res[1 + P + P * P:]


def test_noalloc_matches_workspace_entry_point_on_two_calls():
    for seed, n, d, m in ((1, 3000, 5, 20), (2, 1500, 3, 40)):
        prob, theta = _problem(seed, n, d, m)
        ll0, g0, F0, b0 = prob.evaluate(theta, 2.5)
        ll, g, F, b = _noalloc_call(prob, theta)
        assert abs(ll - ll0) <= 1e-10 * abs(ll0)
        np.testing.assert_allclose(g, g0, rtol=1e-8, atol=1e-8 * np.abs(g0).max())
        np.testing.assert_allclose(F, F0, rtol=1e-8, atol=1e-8 * np.abs(F0).max())
        np.testing.assert_allclose(b, b0, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("form,code", [("split", 1), ("split_df", 2)])
def test_noalloc_split_forms_on_two_calls(form, code):
    """The split forms (float32 assembly; float64 or double-float
    factorisation): the first problem has a fixed nugget of 1e-8, so blocks
    fall below the pivot-ratio test and are re-evaluated in float64; the
    second (n = 30,000, d = 10, m = 30) fills most of the fixed array."""
    from pyscaledvecchia_gb300 import _lib
    lib, _ = _lib.device_ready()
    cases = ((4, 2500, 3, 20, 1e-8), (5, 30000, 10, 30, 1e-3))
    for seed, n, d, m, tau in cases:
        prob, theta = _problem(seed, n, d, m)
        theta[-1] = math.log(tau)
        if n == 30000:
            need = lib.sv_loglik_workspace_bytes(_desc(prob, d + 2, code))
            assert 0.8 * (32 << 20) < need <= (32 << 20)
        ll0, g0, F0, b0 = prob.evaluate(theta, 2.5, precision=form, team_lanes=16)
        aux0 = int(prob.last_info[3])
        ll, g, F, b = _noalloc_call(prob, theta, code)
        if n == 2500:
            assert aux0 > 0  # the float64 re-evaluation pass ran
        assert abs(ll - ll0) <= 1e-10 * abs(ll0)
        np.testing.assert_allclose(g, g0, rtol=1e-8, atol=1e-8 * np.abs(g0).max())
        np.testing.assert_allclose(F, F0, rtol=1e-8, atol=1e-8 * np.abs(F0).max())
        np.testing.assert_allclose(b, b0, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("code", [0, 1])
def test_noalloc_call_captured_in_a_graph(code):
    """After the first call on a device (the scratch address lookup), the
    call enqueues only kernels (the problem descriptor goes in by value, the
    status words are cleared by a kernel): captured in a CUDA graph it
    replays with new parameters and gives the bits of direct calls."""
    from pyscaledvecchia_gb300 import _lib
    lib, torch = _lib.device_ready()
    prob, theta = _problem(6, 2000, 4, 15)
    _noalloc_call(prob, theta, code)
    P = prob.d + 2
    D = _desc(prob, P, code)
    th = _lib.to_dev(torch, theta, np.float64)
    out = torch.empty(1 + P + P * P + prob.q, dtype=torch.float64, device="cuda")
    info = _lib.new_info(torch)
    chunk = prob.chunk_tensor(P)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = lib.sv_vecchia_loglik_noalloc(D, _lib.ptr(th), _lib.ptr(prob.X), _lib.ptr(prob.y),
                                           _lib.ptr(prob.Z), _lib.ptr(prob.rowb), _lib.ptr(prob.kb),
                                           _lib.ptr(prob.nbr), _lib.ptr(chunk), _lib.ptr(out),
                                           _lib.ptr(info), _lib.stream_handle(torch))
    assert rc == 0, lib.sv_status_string(rc)
    rng = np.random.default_rng(0)
    for _ in range(3):
        t = theta + rng.uniform(-0.2, 0.2, theta.shape)
        th.copy_(torch.from_numpy(t))
        g.replay()
        torch.cuda.synchronize()
        assert int(info.cpu().numpy()[0]) == 0
        got = out.cpu().numpy()
        ll, gr, F, b = _noalloc_call(prob, t, code)
        want = np.concatenate([[ll], gr, F.ravel(), b])
        np.testing.assert_array_equal(got, want)


def test_noalloc_rejects_problems_beyond_the_fixed_scratch():
    from pyscaledvecchia_gb300 import _lib
    lib, torch = _lib.device_ready()
    prob, theta = _problem(3, 500, 4, 10)
    D = _desc(prob, 6)
    D.nblk = D.nblk_warp = 40_000_000  # needs far more than 32 MiB of scratch
    assert lib.sv_loglik_workspace_bytes(D) > (32 << 20)
    info = _lib.new_info(torch)
    rc = lib.sv_vecchia_loglik_noalloc(D, None, None, None, None, None, None, None, None, None,
                                       _lib.ptr(info), _lib.stream_handle(torch))
    assert rc == _lib.SV_ENOSPC
