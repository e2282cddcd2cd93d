"""The float32 Matern forms of the split kernels (sv_matern_eval, which = 2:
the correlation deficit D = 1 - M, which = 3: g = M'/r) against 40-digit
values (tests/golden/matern_f32.npz, made by make_matern_f32.py with mpmath)
at float32 r: the closed forms (nu = 0.5, 1.5, 2.5) and the float32 table of
a fixed general nu (8-term Chebyshev series on half-octave intervals of
c = sqrt(2 nu) r, the deficit from the series of K_nu with the leading 1 of
M taken out below the octave 2^esw at or above sqrt(2 max(nu - 1, 1))).  Bounds, in float32 ulp relative: 8 for D; for
g, 8 + 2c, as e^-c at the float32 c = fl(fl(sqrt(2 nu)) r) carries the two
roundings of c times c (wherever g is a normal float32; the table's end,
c >= 64, gives D = 1 and g = 0, below 1e-20 there).  Measured on a GB300:
D within 4.9 ulp (closed forms) and 4.7 ulp (table); g within 3.7 ulp for
c < 2."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "matern_f32.npz")
ULP = 2.0 ** -24


def _golden():
    z = np.load(GOLDEN)
    return z, [float(v) for v in z["nus"]]


def test_golden_against_scipy():
    """The fixture itself against scipy's kv in float64, where 1 - M keeps
    its digits (D >= 1e-3), g is far from underflow and the float64 product
    of c^nu and K_nu neither overflows nor underflows."""
    from scipy.special import gammaln, kv
    z, nus = _golden()
    for nu in nus:
        r, D, g = z["r_%g" % nu], z["D_%g" % nu], z["g_%g" % nu]
        c = np.sqrt(2.0 * nu) * r
        with np.errstate(all="ignore"):
            pre = np.exp((1.0 - nu) * np.log(2.0) - gammaln(nu) + nu * np.log(c))
            M = pre * kv(nu, c)
            gs = -(2.0 * nu / c) * pre * kv(nu - 1.0, c)
        fin = np.isfinite(M) & np.isfinite(gs)
        ok = fin & (D >= 1e-3)
        assert ok.sum() >= 40
        np.testing.assert_allclose(1.0 - M[ok], D[ok], rtol=1e-12, atol=1e-13)
        ok = fin & (np.abs(g) > 1e-200)
        np.testing.assert_allclose(gs[ok], g[ok], rtol=1e-10)


@pytest.mark.gpu
def test_float32_forms_against_golden():
    from pyscaledvecchia_gb300._covariance import _elementwise
    z, nus = _golden()
    worst = {}
    for nu in nus:
        general = 0 if nu in (0.5, 1.5, 2.5) else 1
        r, D, g = z["r_%g" % nu], z["D_%g" % nu], z["g_%g" % nu]
        Dd = _elementwise(r, nu, 2, general)
        gd = _elementwise(r, nu, 3, general)
        assert np.all(Dd == Dd.astype(np.float32))  # float32 values
        eD = np.abs(Dd - D) / np.abs(D) / ULP
        assert eD.max() <= 8.0, (nu, float(eD.max()), float(r[np.argmax(eD)]))
        cc = np.sqrt(2.0 * nu) * r
        normal = (np.abs(g) > 1e-37) & ((cc < 64.0) if general else True)
        c = cc[normal]
        eg = np.abs(gd[normal] - g[normal]) / np.abs(g[normal]) / ULP
        assert np.all(eg <= 8.0 + 2.0 * c), (nu, float((eg / (8.0 + 2.0 * c)).max()))
        assert np.all(np.abs(gd[~normal]) <= 1e-20)
        small = c < 2.0
        worst[nu] = (float(eD.max()), float(eg[small].max()),
                     float((eg / np.maximum(c, 1.0)).max()))
    print("worst ulp (D, g at c < 2, g / max(c, 1)):", worst)


@pytest.mark.gpu
@pytest.mark.parametrize("nu", [2.0, 1.0005, 9.3])
def test_no_table_near_integers(nu):
    """No float32 table within 1e-3 of an integer (the series cancels) or
    above nu = 8 (eight terms no longer reach float32 accuracy): the call is
    refused (the likelihood runs such a nu in float64)."""
    from pyscaledvecchia_gb300._covariance import _elementwise
    with pytest.raises(ValueError):
        _elementwise(np.array([0.5]), nu, 2, 1)


@pytest.mark.gpu
def test_float32_dnu_against_golden():
    """dM/dnu of an estimated nu (which = 4): the float32 table of the
    reference's central difference against 40-digit values.  It changes sign
    as c grows, so the error is measured against the local scale: the
    largest |dM/dnu| at the golden points with c within a factor 2; bound 16
    float32 ulp of that scale (the table's end, c >= 64, gives 0)."""
    from pyscaledvecchia_gb300._covariance import _elementwise
    z, nus = _golden()
    worst = {}
    for nu in nus:
        if nu in (0.5, 1.5, 2.5):
            continue
        r, dn = z["r_%g" % nu], z["dnu_%g" % nu]
        if abs(nu - 1e-3 - round(nu - 1e-3)) < 1e-3 or abs(nu + 1e-3 - round(nu + 1e-3)) < 1e-3:
            with pytest.raises(ValueError):  # nu +- h within 1e-3 of an integer: no table
                _elementwise(r, nu, 4, 1)
            continue
        dd = _elementwise(r, nu, 4, 1)
        c = np.sqrt(2.0 * nu) * r
        scale = np.array([np.abs(dn[(c >= ci / 2) & (c <= ci * 2)]).max() for ci in c])
        inside = c < 64.0
        e = np.abs(dd - dn)[inside] / scale[inside] / ULP
        assert e.max() <= 16.0, (nu, float(e.max()), float(c[inside][np.argmax(e)]))
        assert np.all(np.abs(dd[~inside]) <= 1e-20)
        worst[nu] = float(e.max())
    print("worst dnu error in ulp of the local scale:", worst)
