"""Several ranks: one problem's likelihood split by blocks, batched fits split
by problem (pyscaledvecchia_gb300/sharding.py).

On CPU, world_size-2 gloo process groups run the exchanges with the oracle
as each rank's evaluator (oracle/sharded.py: the two passes of
likelihood.py:66-175 over per-block records, partitioned as the device
partitions them): two ranks give the bits of one rank, and the oracle's own
likelihood to rounding, also when chunk-wide jitter spans the ranks.
Problem-sharded fits give every rank every model, each fitted as one rank
would.  On the GPU, the shards of one problem run their stages in turn on the
one device (nothing waits on another launch) and must give the bits of
sv_vecchia_loglik.  Unmeasured on hardware with more than one GPU.
"""
import math
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem(case):
    """Ordered inputs from the oracle: ``plain`` is a smooth problem; ``jitter``
    has duplicated rows and a 1e-20 nugget, so some blocks need jitter and
    the chunk (one chunk spans the whole problem at this K) straddles ranks."""
    import sys
    sys.path.insert(0, ROOT)
    from oracle import oracle
    rng = np.random.default_rng(7)
    n, d, m = 3000, 3, 8
    X = rng.random((n, d))
    tau = 1e-3
    if case == "jitter":
        X[1500:1600] = X[100:200]  # duplicated rows
        tau = 1e-20  # below float64's resolution of the diagonal: singular blocks
    lam = np.array([0.3, 0.5, 0.8])
    theta = np.concatenate([[math.log(1.3)], np.log(lam), [math.log(tau)]])
    order = oracle.maximin_order(X / lam)
    nn = oracle.ordered_nn((X / lam)[order], m)
    y = rng.standard_normal(n)
    return X[order], y[order], np.ones((n, 1)), oracle.nn_groups(nn, m), theta


def _np_allreduce(arr, op):
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(arr)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return arr


def _worker(rank, world, port, outdir, case):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        from oracle.sharded import OracleShard, red_parts
        from pyscaledvecchia_gb300.sharding import partition_range, sharded_evaluate
        Xo, yo, Zo, groups, theta = _problem(case)
        nblk = Xo.shape[0]
        pb, pe = partition_range(red_parts(nblk), rank, world)
        ev = OracleShard(Xo, yo, Zo, groups, 2.5, pb, pe, var_penalty=1.0, log_var_target=-0.2)
        ll, g, F, beta = sharded_evaluate(ev, theta, _np_allreduce)
        np.savez(os.path.join(outdir, f"{case}_{world}_{rank}.npz"), ll=ll, g=g, F=F, beta=beta,
                 lev=ev.lev)
    finally:
        dist.destroy_process_group()


def _run(world, outdir, case):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port(), str(outdir), case), nprocs=world, join=True)


@pytest.mark.parametrize("case", ["plain", "jitter"])
def test_two_ranks_give_the_one_rank_bits(tmp_path, case):
    _run(1, tmp_path, case)
    _run(2, tmp_path, case)
    one = np.load(tmp_path / f"{case}_1_0.npz")
    for r in range(2):
        two = np.load(tmp_path / f"{case}_2_{r}.npz")
        for k in ("ll", "g", "F", "beta"):
            np.testing.assert_array_equal(two[k], one[k], err_msg=f"{case} rank {r} {k}")
    if case == "jitter":
        assert one["lev"].max() > 0  # some blocks needed jitter
    # and the oracle's own likelihood to rounding
    import sys
    sys.path.insert(0, ROOT)
    from oracle import oracle
    Xo, yo, Zo, groups, theta = _problem(case)
    ll0, g0, F0, b0 = oracle.vecchia_loglik(theta, Xo, yo, Zo, groups, 2.5, var_penalty=1.0,
                                            log_var_target=-0.2)
    assert abs(float(one["ll"]) - ll0) <= 1e-11 * abs(ll0)
    np.testing.assert_allclose(one["g"], g0, rtol=1e-9, atol=1e-9 * np.abs(g0).max())
    np.testing.assert_allclose(one["F"], F0, rtol=1e-10, atol=1e-10 * np.abs(F0).max())
    np.testing.assert_allclose(one["beta"], b0, rtol=1e-10, atol=1e-12)


def test_partitions_and_problem_assignment():
    from pyscaledvecchia_gb300.sharding import assign_problems, partition_range, problem_cost
    for nparts in (8, 9, 195, 4096):
        for world in (1, 2, 3, 8):
            rs = [partition_range(nparts, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == nparts
            assert all(rs[r][1] == rs[r + 1][0] for r in range(world - 1))
    costs = [problem_cost(n, m, None) for n, m in ((20000, 30), (500, 10), (8000, 20), (7000, 20),
                                                   (600, 30), (19000, 10))]
    assert problem_cost(100, 30, None) == sum((k + 1) ** 3 for k in range(30)) + 70 * 31 ** 3
    assert problem_cost(20000, 30, 5000) == problem_cost(5000, 30, None)
    owner = assign_problems(costs, 2)
    load = [sum(c for c, o in zip(costs, owner) if o == r) for r in range(2)]
    # Graham's bound for longest-processing-time assignment on two ranks:
    # at most 7/6 of the optimum, which is at least max(sum / 2, largest cost)
    assert max(load) <= (7.0 / 6.0) * max(sum(costs) / 2, max(costs)) * (1 + 1e-12)
    assert assign_problems(costs, 2) == owner  # deterministic


def _fit_worker(rank, world, port, outdir):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        from oracle.fit import OracleGP
        from pyscaledvecchia_gb300 import ScaledVecchiaGP
        from pyscaledvecchia_gb300.sharding import fit_batched_sharded
        rng = np.random.default_rng(3)
        Xs, ys, models = [], [], []
        for i in range(5):
            n = 150 + 60 * i
            X = rng.random((n, 2))
            Xs.append(X)
            ys.append(np.sin(3 * X[:, 0]) + 0.3 * X[:, 1] + 0.05 * rng.standard_normal(n))
            models.append(ScaledVecchiaGP(m_est=8, m_pred=15, n_est=None, var_correction=False))

        def oracle_fit(ms, Xl, yl):
            # the CPU stand-in for fit_batched: each model fitted by the oracle
            for mdl, X, y in zip(ms, Xl, yl):
                o = OracleGP(m_est=mdl.m_est, m_pred=mdl.m_pred, n_est=mdl.n_est, nu=mdl.nu,
                             var_correction=mdl.var_correction).fit(X, y)
                mdl._fit_prepare(X, y)
                mdl.theta_, mdl.beta_, mdl.loglik_, mdl.b_ = o.theta_, o.beta_, o.loglik_, o.b_
                mdl._nu_fit = mdl.nu
            return ms

        fit_batched_sharded(models, Xs, ys, fit_fn=oracle_fit)
        np.savez(os.path.join(outdir, f"fit_{world}_{rank}.npz"),
                 theta=np.array([m.theta_ for m in models], dtype=object),
                 ll=np.array([m.loglik_ for m in models]),
                 X0=np.array([m.X_[0] for m in models]))
    finally:
        dist.destroy_process_group()


def test_problem_sharded_fits_give_every_rank_every_model(tmp_path):
    import torch.multiprocessing as mp
    for world in (1, 2):
        mp.spawn(_fit_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    one = np.load(tmp_path / "fit_1_0.npz", allow_pickle=True)
    for r in range(2):
        two = np.load(tmp_path / f"fit_2_{r}.npz", allow_pickle=True)
        np.testing.assert_array_equal(two["ll"], one["ll"])
        np.testing.assert_array_equal(two["X0"], one["X0"])
        for a, b in zip(two["theta"], one["theta"]):
            np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("nu", [2.5, 0.8, None])
@pytest.mark.parametrize("precision", ["float64", "split"])
@pytest.mark.parametrize("nshard", [2, 3])
def test_device_shards_give_the_one_gpu_bits(precision, nshard, nu):
    """Shards of one problem run stage by stage on the one GPU, the exchanges
    done in between (MAX of the chunk tables, SUM of the partial-sum rows):
    the result is sv_vecchia_loglik's bit for bit, for a problem whose
    duplicated rows need chunk-wide jitter as well; at nu = 0.8 and with nu
    estimated (None: nu = 1.3 in theta) each shard builds the Matern tables
    in its first stage and its later passes read them."""
    import torch

    from pyscaledvecchia_gb300.likelihood import DeviceProblem
    from pyscaledvecchia_gb300.ordering import _nn_groups, find_ordered_nn, maximin_order
    from pyscaledvecchia_gb300.sharding import DeviceShard, partition_range
    rng = np.random.default_rng(11)
    for n, d, m, dup in ((20000, 10, 30, False), (12000, 3, 20, True)):
        X = rng.random((n, d))
        tau = 1e-3
        if dup:
            X[6000:6300] = X[300:600]
            tau = 1e-20
        lam = np.exp(rng.uniform(math.log(0.1), math.log(2.0), d))
        est = nu is None
        theta = np.concatenate([[math.log(1.7)], np.log(lam), [math.log(1.3)] if est else [],
                                [math.log(tau)]])
        order = maximin_order(X / lam)
        nn = find_ordered_nn((X / lam)[order], m)
        y = rng.standard_normal(n)
        prob = DeviceProblem(X[order], y[order], np.ones((n, 1)), _nn_groups(nn, m))
        P = d + 3 if est else d + 2
        ref = prob.evaluate(theta, nu, estimate_nu=est, precision=precision, team_lanes=16)
        probe = DeviceShard(prob, 0, 0, nu, P, estimate_nu=est, precision=precision, team_lanes=16)
        shards = [DeviceShard(prob, *partition_range(probe.parts, r, nshard), nu, P, estimate_nu=est,
                              precision=precision, team_lanes=16) for r in range(nshard)]
        cm = [s.stage1(theta) for s in shards]
        cmax = torch.stack(cm).max(dim=0).values.contiguous()
        p1 = [s.stage2(cmax.clone()) for s in shards]
        p1s = sum(p1[1:], p1[0].clone())
        p2 = [s.stage3(p1s.clone()) for s in shards]
        p2s = sum(p2[1:], p2[0].clone())
        outs = [s.stage4(p2s.clone())[0].cpu().numpy() for s in shards]
        for o in outs:
            assert o[0] == ref[0]
            np.testing.assert_array_equal(o[1:1 + P], ref[1])
            np.testing.assert_array_equal(o[1 + P:1 + P + P * P].reshape(P, P), ref[2])
            np.testing.assert_array_equal(o[1 + P + P * P:], ref[3])
        if dup:
            assert int(prob.last_info[2]) > 0  # chunk-wide jitter was used
