"""Generate tests/golden/matern_f32.npz: the correlation deficit
D(r) = 1 - M_nu(r) and g(r) = M_nu'(r)/r (the quantities the split kernels
assemble in float32) to 40 digits with mpmath, at float32-representable r,
for the closed forms and for general smoothness values.  M_nu is the
reference's Matern (_matern_general.py:92-116):
  M(r) = 2^(1-nu)/Gamma(nu) c^nu K_nu(c),  c = sqrt(2 nu) r,
  g(r) = -(2 nu / c) 2^(1-nu)/Gamma(nu) c^nu K_{nu-1}(c).
For the general values also dM/dnu as the reference's central difference
(M_{nu+h}(r) - M_{nu-h}(r)) / 2h, h = 1e-3 (_matern_general.py:170-176),
what the split kernels assemble an estimated nu's row with.
Run from the repository root: python tests/golden/make_matern_f32.py"""
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 40
NUS = (0.5, 1.5, 2.5, 0.3, 0.8, 1.75, 3.2, 1.0015, 5.4, 7.9)


def deficit_and_g(r, nu):
    r = mp.mpf(float(r))
    nu = mp.mpf(nu)
    c = mp.sqrt(2 * nu) * r
    pre = 2 ** (1 - nu) / mp.gamma(nu) * c ** nu
    M = pre * mp.besselk(nu, c)
    g = -(2 * nu / c) * pre * mp.besselk(nu - 1, c)
    return float(1 - M), float(g)


def matern_M(r, nu):
    r = mp.mpf(float(r))
    nu = mp.mpf(nu)
    c = mp.sqrt(2 * nu) * r
    return 2 ** (1 - nu) / mp.gamma(nu) * c ** nu * mp.besselk(nu, c)


def dnu(r, nu, h=1e-3):
    return float((matern_M(r, nu + mp.mpf(h)) - matern_M(r, nu - mp.mpf(h))) / (2 * mp.mpf(h)))


def main():
    out = {}
    for nu in NUS:
        s2n = np.sqrt(2.0 * nu)
        # c from 2e-7 sqrt(2 nu) to 80: every octave of the float32 table and
        # beyond its end (c >= 64)
        c = np.geomspace(2e-7 * s2n, 80.0, 160)
        r = (c / s2n).astype(np.float32).astype(np.float64)
        vals = np.array([deficit_and_g(x, nu) for x in r])
        out["r_%g" % nu] = r
        out["D_%g" % nu] = vals[:, 0]
        out["g_%g" % nu] = vals[:, 1]
        if nu not in (0.5, 1.5, 2.5):
            out["dnu_%g" % nu] = np.array([dnu(x, nu) for x in r])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "matern_f32.npz")
    np.savez_compressed(path, nus=np.array(NUS), **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
