"""The split form of the prediction blocks (ScaledVecchiaGP(precision=
"split"), sv_pred_desc.precision = 1) against the float64 form and the
oracle.

The split form assembles the entries below the diagonal in float32 (centred
coordinates as (hi, lo) pairs, the correlation deficit 1 - M) and keeps the
diagonal, the LDL^T and every solve in float64 (gp.py:257-276 of the
reference in float64 throughout).  Errors are stated in units of the
predictive sd: |mean_split - mean_64| / sd and |sd_split - sd_64| / sd.
"""
import math
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# measured at the benchmark's prediction workload (100,000 training points in
# d = 6, 50,000 test points, m_pred = 140, fitted nugget 2.8e-3): mean error
# 2.6e-5 sd at the median, 1.3e-4 at the 99th percentile, 2.5e-4 at most; sd
# relative error 1.1e-6, 5.6e-6, 9.0e-6 (the float32 rounding of the
# correlation deficits, about 6e-8 relative, times the blocks' conditioning;
# (hi, lo) coordinates instead of plain float32 ones changed nothing).  The
# bounds leave about 4x room.
MEAN_TOL_MAX, MEAN_TOL_MEDIAN = 1e-3, 1e-4
SD_TOL_MAX = 5e-5


def _errors(mu, sd, mu_ref, sd_ref):
    return np.abs(mu - mu_ref) / sd_ref, np.abs(sd - sd_ref) / sd_ref


def _scaled_inputs(gp, Xte):
    Xs = (Xte - gp._lo) / gp._span
    Ztr = gp._design(gp.X_)
    resid = gp.y_ - (Ztr @ gp.beta_ if gp.beta_.size else 0.0)
    return Xs, resid


@pytest.fixture(scope="module")
def c4_fit():
    sys.path.insert(0, ROOT)
    import torch

    from bench import c4_inputs
    from pyscaledvecchia_gb300 import ScaledVecchiaGP, _lib
    _lib.device_ready()
    X, y, Xte = c4_inputs(torch)
    gp = ScaledVecchiaGP(m_est=30, m_pred=140, nu=2.5).fit(X, y)
    return gp, Xte[:20000]


def test_split_predictions_at_the_benchmark_size(c4_fit):
    """20,000 of the benchmark's test points, 141-point blocks: the split
    form against the float64 form, and both against the oracle on 800 of
    them (its own neighbour search, float64 blocks)."""
    from oracle import oracle
    gp, Xte = c4_fit
    Xs, resid = _scaled_inputs(gp, Xte)
    gp.precision = "float64"
    mu64, va64 = gp._predict_scaled(Xs, gp.X_, resid, 140)
    gp.precision = "split"
    mu32, va32 = gp._predict_scaled(Xs, gp.X_, resid, 140)
    assert gp.pred_stats_["blocks"] == Xte.shape[0]
    gp.precision = "float64"
    em, es = _errors(mu32, np.sqrt(va32), mu64, np.sqrt(va64))
    print(f"split vs float64: mean/sd median {np.median(em):.3g} max {em.max():.3g}; "
          f"sd rel max {es.max():.3g}; redone in float64 {gp.pred_stats_['redone_float64']}")
    assert np.median(em) < MEAN_TOL_MEDIAN and em.max() < MEAN_TOL_MAX
    assert es.max() < SD_TOL_MAX
    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    sub = np.arange(0, Xte.shape[0], 25)
    Xs, resid = _scaled_inputs(gp, Xte[sub])
    mo, vo, _ = oracle.predict_marginal(gp.X_, resid, Xs, gp._pred_theta(), 2.5, 140)
    em, es = _errors(mu64[sub], np.sqrt(va64[sub]), mo, np.sqrt(vo))
    assert em.max() < 1e-9 and es.max() < 1e-9
    em, es = _errors(mu32[sub], np.sqrt(va32[sub]), mo, np.sqrt(vo))
    assert em.max() < MEAN_TOL_MAX and es.max() < SD_TOL_MAX


def _small(nu, n=3000, d=3, seed=0, noise=0.2):
    """A smooth response with noise: the fitted nugget keeps the blocks'
    pivot ratios well above the split form's threshold (with noise 0.01
    the fitted nugget drives every block below it, and the split setting
    redoes them all in float64)."""
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    rng = np.random.default_rng(seed)
    X = rng.random((n, d))
    y = np.sin(4 * X[:, 0]) + np.cos(3 * X[:, 1]) * X[:, 2] + noise * rng.standard_normal(n)
    gp = ScaledVecchiaGP(m_est=20, n_est=1500, nu=nu, var_correction=False).fit(X, y)
    return gp, rng.uniform(-0.05, 1.05, (1500, d))


@pytest.mark.parametrize("nu", [0.5, 1.5, 2.5])
@pytest.mark.parametrize("m", [20, 60])
def test_split_predictions_small(nu, m):
    """Warp-team blocks (m = 20: 21 points) and CTA blocks (m = 60) for each
    closed form."""
    gp, Xte = _small(nu)
    mu64, sd64 = gp.predict(Xte, return_std=True, m=m)
    gp.precision = "split"
    mu32, sd32 = gp.predict(Xte, return_std=True, m=m)
    assert gp.pred_stats_["redone_float64"] < Xte.shape[0] // 10
    em, es = _errors(mu32, sd32, mu64, sd64)
    assert em.max() < MEAN_TOL_MAX and es.max() < SD_TOL_MAX, (em.max(), es.max())


@pytest.mark.parametrize("nu", [1.75, 9.3])
def test_bessel_nu(nu):
    """A general nu: 1.75 has a float32 table (the split blocks take it,
    within this file's bounds, warp and CTA blocks); 9.3 has none (above 8),
    so the split setting predicts in float64, bit for bit."""
    gp, Xte = _small(nu, n=1500)
    for m in (30, 60):
        mu64, sd64 = gp.predict(Xte, return_std=True, m=m)
        gp.precision = "split"
        mu32, sd32 = gp.predict(Xte, return_std=True, m=m)
        gp.precision = "float64"
        if nu > 8.0:
            np.testing.assert_array_equal(mu32, mu64)
            np.testing.assert_array_equal(sd32, sd64)
            assert gp.pred_stats_["redone_float64"] == 0
            continue
        assert np.any(mu32 != mu64)  # the split form ran
        assert gp.pred_stats_["redone_float64"] < Xte.shape[0] // 10
        em, es = _errors(mu32, sd32, mu64, sd64)
        assert em.max() < MEAN_TOL_MAX and es.max() < SD_TOL_MAX, (em.max(), es.max())


@pytest.mark.parametrize("m", [20, 60])
def test_guard_redoes_every_block_in_float64(m):
    """split_rho_min = 2: even the first pivot (d_0 = Sigma_00) falls below
    it, so every block is redone in float64: the results are the float64
    form's bit for bit and info[SV_INFO_AUX] counts every block."""
    import torch

    from pyscaledvecchia_gb300 import _lib
    from pyscaledvecchia_gb300.ordering import knn_query_device
    lib, _ = _lib.device_ready()
    gp, Xte = _small(2.5)
    Xs, resid = _scaled_inputs(gp, Xte)
    ntr, d = gp.X_.shape
    nte = Xs.shape[0]
    nb, _ = knn_query_device(torch, _lib.to_dev(torch, gp.X_ / gp.ranges_, np.float64),
                             _lib.to_dev(torch, Xs / gp.ranges_, np.float64), m)
    Xall = torch.cat([_lib.to_dev(torch, gp.X_, np.float64), _lib.to_dev(torch, Xs, np.float64)])
    tgt = torch.arange(ntr, ntr + nte, dtype=torch.int32, device="cuda")
    nbr = nb.to(torch.int32).contiguous()
    rd = _lib.to_dev(torch, resid, np.float64)
    th = _lib.to_dev(torch, gp._pred_theta(), np.float64)
    out = {}
    for prec, rho in ((0, 0.0), (1, 2.0), (1, 0.0)):
        D = _lib.PredDesc()
        D.nall, D.nobs, D.nblk = ntr + nte, ntr, nte
        D.d, D.k, D.ldnbr = d, m, m
        D.general, D.nu, D.precision, D.split_rho_min = 0, 2.5, prec, rho
        mean = torch.empty(nte, dtype=torch.float64, device="cuda")
        var = torch.empty_like(mean)
        acol = torch.empty((nte, m + 1), dtype=torch.float64, device="cuda")
        info = _lib.new_info(torch)
        rc = lib.sv_predict_blocks(D, _lib.ptr(th), _lib.ptr(Xall), _lib.ptr(tgt), _lib.ptr(nbr),
                                   _lib.ptr(rd), _lib.ptr(mean), _lib.ptr(var), _lib.ptr(acol), None,
                                   _lib.ptr(info), _lib.stream_handle(torch))
        _lib.check(lib, rc, "sv_predict_blocks")
        inf = info.cpu().numpy()
        _lib.check_info(lib, inf, "sv_predict_blocks")
        out[(prec, rho)] = (mean.cpu().numpy(), var.cpu().numpy(), acol.cpu().numpy(), int(inf[3]))
    ref, guarded, split = out[(0, 0.0)], out[(1, 2.0)], out[(1, 0.0)]
    for a, b in zip(ref[:3], guarded[:3]):
        np.testing.assert_array_equal(a, b)
    assert ref[3] == 0 and guarded[3] == nte
    # the default threshold keeps most blocks in the split form
    assert split[3] < nte // 2
    assert math.isfinite(float(split[1].sum()))


def test_split_predictions_general_nu():
    """A general fitted nu (0.8): the split prediction blocks take the float32
    part of the model's Matern table (sv_matern_table) and stay within this
    file's bounds of the float64 predictions; a nu without a float32 table
    (2.0, within 1e-3 of an integer) predicts in float64 in both forms."""
    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    rng = np.random.default_rng(21)
    X = rng.random((3000, 3))
    y = np.sin(4 * X[:, 0]) + X[:, 1] ** 2 + 0.05 * rng.standard_normal(3000)
    Xq = rng.random((1000, 3))
    for nu in (0.8, 2.0):
        gp = ScaledVecchiaGP(nu=nu, m_est=20, m_pred=60, var_correction=False).fit(X, y)
        mu64, sd64 = gp.predict(Xq, return_std=True)
        gp.precision = "split"
        mu, sd = gp.predict(Xq, return_std=True)
        if nu == 2.0:
            np.testing.assert_array_equal(mu, mu64)
            np.testing.assert_array_equal(sd, sd64)
            continue
        assert np.any(mu != mu64)  # the split form ran
        assert gp.pred_stats_["redone_float64"] < 100
        em, es = _errors(mu, sd, mu64, sd64)
        assert em.max() <= MEAN_TOL_MAX and np.median(em) <= MEAN_TOL_MEDIAN, (em.max(), np.median(em))
        assert es.max() <= SD_TOL_MAX, es.max()
