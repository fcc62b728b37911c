"""Host-side precompute of the energy parameters the kernels read.

* ``dss_parameters``: SSWLC elastic parameters per bond, interpolated from the
  dssWLC table as in ``SSWLC._find_parameters`` (chromo/polymers.pyx:1545-1601).
* ``binding_free_energy_table``: -ln of the single-site binding partition
  function for every (binder, marked tails, bound tails), the expression of
  ``bead_binding_dE`` (chromo/polymers.pyx:1494-1517), tabulated once so the
  kernel does a lookup instead of scipy ``comb`` + numpy per bead.
* ``field_prefactors``: oligomerisation, intranucleosome and cross-talk
  prefactors of ``init_field_energy_prefactors`` (chromo/fields.pyx:687-712).
"""
from pathlib import Path

import numpy as np
from scipy.special import comb

from ._native import MAX_BINDERS, MAX_MARK

_TABLE = None


def dss_table() -> np.ndarray:
    global _TABLE
    if _TABLE is None:
        _TABLE = np.loadtxt(Path(__file__).resolve().parent / "data" / "dssWLCparams")
    return _TABLE


def dss_parameters(bead_length, lp):
    """(delta, eps_bend, gamma, eps_par, eps_perp, eta) per bond."""
    t = dss_table()
    bl = np.asarray(bead_length, dtype=np.float64)
    # element-wise the same arithmetic as one np.interp call per bond
    delta = bl / lp
    eb = np.interp(delta, t[:, 0], t[:, 1]) / delta
    g = np.interp(delta, t[:, 0], t[:, 2]) * delta * lp
    ep = np.interp(delta, t[:, 0], t[:, 3]) / (delta * lp ** 2)
    epp = np.interp(delta, t[:, 0], t[:, 4]) / (delta * lp ** 2)
    eta = np.interp(delta, t[:, 0], t[:, 5]) / lp
    return delta, eb, g, ep, epp, eta


def binding_free_energy_table(sites, e_mod, e_nomod):
    """[MAX_BINDERS, MAX_MARK+1, MAX_MARK+1] table of -ln(site partition function)."""
    f = np.zeros((MAX_BINDERS, MAX_MARK + 1, MAX_MARK + 1))
    for b in range(len(sites)):
        Nn = int(sites[b])
        for Nm in range(MAX_MARK + 1):
            for s in range(MAX_MARK + 1):
                i = np.arange(s + 1)
                with np.errstate(divide="ignore"):
                    f[b, Nm, s] = -np.log(np.sum(
                        comb(Nm, i) * comb(Nn - Nm, s - i)
                        * np.exp(-(i * e_mod[b] + (s - i) * e_nomod[b]))))
    return f


def field_prefactors(interaction_energy, interaction_volume, cross_talk, names, vol_bin):
    """(pref[nb], intra[nb], xpref[nb, nb]) with cross_talk[i] a dict name -> energy."""
    nb = len(names)
    pref = np.zeros(nb)
    intra = np.zeros(nb)
    xpref = np.zeros((nb, nb))
    for i in range(nb):
        pref[i] = 0.5 * interaction_energy[i] * interaction_volume[i] * vol_bin
        intra[i] = interaction_energy[i] * (1 - interaction_volume[i] / vol_bin)
        for j, other in enumerate(names):
            if other in cross_talk[i]:
                xpref[i, j] = cross_talk[i][other] * interaction_volume[i] * vol_bin
    return pref, intra, xpref
