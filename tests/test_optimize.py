"""Fisher scoring (optimize.py:11-73) against traces recorded from the
reference on deterministic toy objectives: every evaluated theta, every
reorder call and the result must agree bit for bit, including the ridged
direction, the gradient fallback, LinAlgError tries and reorders."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

sys.path.insert(0, GOLDEN)
import toy_objectives as T  # noqa: E402

from pyscaledvecchia_gb300.optimize import (EVAL_FAILED, _fisher_scoring,  # noqa: E402
                                            fisher_scoring_steps)


@pytest.fixture(scope="module")
def golden_optimize():
    return load_golden("optimize")


@pytest.mark.parametrize("name", list(T.CASES))
def test_fisher_scoring_trace_matches_reference(golden_optimize, name):
    z = golden_optimize
    toy, theta0, max_step = T.make(name)
    np.testing.assert_array_equal(theta0, z[f"{name}_theta0"])
    th, ll, beta = _fisher_scoring(theta0, toy.objective, max_iter=25, tol=1e-6,
                                   reorder_hook=toy.reorder_hook, max_step=max_step)
    trace = np.array(toy.trace)
    assert trace.shape == z[f"{name}_trace"].shape
    np.testing.assert_array_equal(trace, z[f"{name}_trace"])
    np.testing.assert_array_equal(np.array([k for k, _ in toy.reorders]), z[f"{name}_reorder_k"])
    np.testing.assert_array_equal(np.array([t for _, t in toy.reorders]).reshape(len(toy.reorders), -1),
                                  z[f"{name}_reorder_th"])
    np.testing.assert_array_equal(th, z[f"{name}_theta"])
    assert ll == float(z[f"{name}_ll"])
    np.testing.assert_array_equal(beta, z[f"{name}_beta"])


def test_generator_interleaved_drivers_agree():
    """Two problems advanced alternately through the generator give the same
    traces as each driven alone (the batched fitter's schedule)."""
    names = ["smooth", "failing"]
    solo = {}
    for nm in names:
        toy, th0, ms = T.make(nm)
        solo[nm] = (_fisher_scoring(th0, toy.objective, max_iter=25, tol=1e-6,
                                    reorder_hook=toy.reorder_hook, max_step=ms), np.array(toy.trace))
    toys, gens, msgs, res = {}, {}, {}, {}
    for nm in names:
        toy, th0, ms = T.make(nm)
        toys[nm] = toy
        gens[nm] = fisher_scoring_steps(th0, max_iter=25, tol=1e-6, max_step=ms)
        msgs[nm] = next(gens[nm])
    while msgs:
        for nm in list(msgs):
            msg = msgs[nm]
            if msg[0] == "eval":
                try:
                    reply = toys[nm].objective(msg[1])
                except np.linalg.LinAlgError:
                    reply = EVAL_FAILED
            else:
                reply = toys[nm].reorder_hook(msg[1], msg[2])
            try:
                msgs[nm] = gens[nm].send(reply)
            except StopIteration as stop:
                res[nm] = stop.value
                del msgs[nm]
    for nm in names:
        (th, ll, beta), trace = solo[nm]
        np.testing.assert_array_equal(np.array(toys[nm].trace), trace)
        np.testing.assert_array_equal(res[nm][0], th)
        assert res[nm][1] == ll


def test_first_evaluation_failure_raises():
    def bad(th):
        raise np.linalg.LinAlgError("no")
    with pytest.raises(np.linalg.LinAlgError):
        _fisher_scoring(np.zeros(3), bad)
