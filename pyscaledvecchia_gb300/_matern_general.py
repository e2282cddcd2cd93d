"""General-smoothness Matern correlation on the GPU.

Drop-in counterpart of the reference's ``scaled_vecchia._matern_general``
(src/scaled_vecchia/_matern_general.py):

  M_nu(r) = 2^(1-nu) / Gamma(nu) * c^nu * K_nu(c),   c = sqrt(2 nu) r,
  g(r)    = M_nu'(r) / r  via d/dz[z^nu K_nu(z)] = -z^nu K_{nu-1}(z),

with r floored at 1e-7 (M = 1, g = 0 below the floor), and the central
difference in nu (step 1e-3) for the estimated-smoothness derivative row
(_matern_general.py:87-179).  K_nu is the library's own device evaluation
(Temme's series / Steed's continued fraction with upward recurrence) in
place of scipy.special.kv.
"""
from __future__ import annotations

import numpy as np

from ._covariance import _block_cov_device, _elementwise

_R_FLOOR = 1e-7


def _matern_corr_general(r: np.ndarray, nu: float) -> np.ndarray:
    """M_nu(r) = 2^(1-nu)/Gamma(nu) * c^nu * K_nu(c), c = sqrt(2 nu) r."""
    return _elementwise(r, float(nu), 0, 1)


def _matern_g_general(r: np.ndarray, nu: float) -> np.ndarray:
    """g(r) = M_nu'(r) / r (0 below the r floor, where it is never used)."""
    return _elementwise(r, float(nu), 1, 1)


def _block_cov_general(Xb, ranges, variance, nugget, nu, derivs=True,
                       nug_mask=None, estimate_nu=False, nu_fd_h=1e-3):
    """Like ``_covariance._block_cov`` for a general (possibly estimated) nu.

    With ``estimate_nu`` the derivative rows are
    [log sigma^2, log lambda_1..d, log nu, log tau].
    """
    return _block_cov_device(Xb, ranges, variance, nugget, float(nu), derivs, nug_mask,
                             general=True, estimate_nu=estimate_nu, nu_fd_h=nu_fd_h)
