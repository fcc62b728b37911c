"""Energy derivatives and reweighting sensitivities (no counterpart in the
reference, which has no derivatives).

``cg_gradient`` returns, per replica, dE/dr for every bead and 14 energy terms
T (see ``include/chromo_gb300.h``).  The derivatives with respect to the
parameters theta = (chi, mu_0, mu_1, eps_00, eps_11, eps_01) are linear in T:

* dE/dchi   = T[0]  (chi (V / V_bead) vf^2 summed over unsaturated voxels);
* dE/dmu_b  = -f_b T[10 + b], the binding term -mu_b f_b sum_i s_ib with
  f_b = mu_adjust_factor for mu_b <= 0 and 2 - mu_adjust_factor otherwise
  (chromo/polymers.pyx:1522-1537);
* dE/deps_bb = 1/2 v_int,b v_bin T[1 + b] + (1 - v_int,b / v_bin) T[7 + b],
  from field_prefactor = 1/2 eps v_int v_bin and intranucleosome =
  eps (1 - v_int / v_bin) (chromo/fields.pyx:687-712);
* dE/deps_01 = v_int,0 v_bin T[4], the cross-talk prefactor stored on binder 0.

Observables used for reweighting are linear in T too: the mean occupancy of
binder b, T[10 + b] / N, and the variance over voxels of the bead density,
T[13] / G minus a constant.  With running sums of T and T T^T over sampled
configurations (``cg_sample_terms``), d<O>/dtheta = -Cov(O, dE/dtheta)
(energies in kT) follows for any such O and theta.
"""
from typing import Sequence

import numpy as np

THETA_NAMES = ("chi", "mu_0", "mu_1", "eps_00", "eps_11", "eps_01")
N_TERMS = 14


def theta_coefficients(mu: Sequence[float], mu_adjust_factor: float,
                       interaction_volume: Sequence[float], vol_bin: float) -> np.ndarray:
    """C [6, 14] with dE/dtheta = C @ T for one replica."""
    C = np.zeros((6, N_TERMS))
    C[0, 0] = 1.0
    for b in range(min(2, len(mu))):
        f = mu_adjust_factor if mu[b] <= 0 else 2.0 - mu_adjust_factor
        C[1 + b, 10 + b] = -f
    for b in range(min(2, len(interaction_volume))):
        v = float(interaction_volume[b])
        C[3 + b, 1 + b] = 0.5 * v * vol_bin
        C[3 + b, 7 + b] = 1.0 - v / vol_bin
    if len(interaction_volume) >= 2:
        C[5, 4] = float(interaction_volume[0]) * vol_bin
    return C


def observable_coefficients(n_beads: int, n_vox: int, n_binders: int) -> np.ndarray:
    """O [n_binders + 1, 14]: mean occupancy of each binder, then the
    variance of the bead density over voxels (up to a constant)."""
    O = np.zeros((n_binders + 1, N_TERMS))
    for b in range(n_binders):
        O[b, 10 + b] = 1.0 / n_beads
    O[n_binders, 13] = 1.0 / n_vox
    return O


def terms_covariance(sum_t: np.ndarray, sum_tt: np.ndarray, count: float) -> np.ndarray:
    """Cov(T) [14, 14] from the running sums of one replica."""
    if count < 2:
        raise ValueError("need at least two samples")
    m = sum_t / count
    return sum_tt / count - np.outer(m, m)


def reweighting_sensitivity(sum_t, sum_tt, count, obs_coef, theta_coef) -> np.ndarray:
    """d<O>/dtheta = -Cov(O, dE/dtheta) = -O Cov(T) C^T  [n_obs, 6]."""
    cov = terms_covariance(np.asarray(sum_t), np.asarray(sum_tt), float(count))
    return -np.asarray(obs_coef) @ cov @ np.asarray(theta_coef).T
