"""pyscaledvecchia_gb300 -- the scaled Vecchia GP hot path on GB300 (sm_103a).

A from-scratch GPU implementation of the method of

    Katzfuss, M., Guinness, J., & Lawrence, E. (2020/2022).
    "Scaled Vecchia approximation for fast computer-model emulation."

with the public interface of the reference package ``scaled_vecchia``
(jdtuck/pyscaledvecchia)::

    from pyscaledvecchia_gb300 import ScaledVecchiaGP
    gp = ScaledVecchiaGP(m_est=30, m_pred=140, nu=2.5).fit(X_train, y_train)
    mean, sd = gp.predict(X_test, return_std=True)
    draws    = gp.sample_joint(X_path, n_sim=100)

Exact maximin ordering, nearest-neighbour conditioning sets, the block
likelihood/score/Fisher evaluation, prediction and joint sampling run in
hand-written CUDA kernels behind the C ABI of include/svgpu.h.  A CUDA device
is required; there is no CPU fallback.
"""

from .gp import ScaledVecchiaGP
from .likelihood import vecchia_profile_loglik
from .ordering import find_ordered_nn, maximin_order

__all__ = [
    "ScaledVecchiaGP",
    "maximin_order",
    "find_ordered_nn",
    "vecchia_profile_loglik",
]

__version__ = "0.1.0"
