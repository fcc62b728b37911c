"""Builders of the C-ABI parameter structs from plain arrays."""
import numpy as np

from . import _native as nat
from .energetics import binding_free_energy_table

MOVE_KIND = {n: i for i, n in enumerate(nat.MOVE_NAMES)}


def field_params(*, field_kind, confine_kind=0, confine_length=0.0, nxyz=(1, 1, 1),
                 widths=(1.0, 1.0, 1.0), n_binders=1, chi=0.0, vf_limit=0.5, bead_vol=1.0,
                 pref=(), intra=(), xpref=None, fast_field=0, n_points=1000):
    fp = nat.FieldParams()
    fp.fast_field, fp.n_points = int(bool(fast_field)), int(n_points)
    fp.field_kind, fp.confine_kind, fp.confine_length = int(field_kind), int(confine_kind), float(confine_length)
    fp.nx, fp.ny, fp.nz = (int(v) for v in nxyz)
    fp.n_binders = int(n_binders)
    fp.x_width, fp.y_width, fp.z_width = (float(w) for w in widths)
    fp.chi, fp.vf_limit, fp.bead_vol = float(chi), float(vf_limit), float(bead_vol)
    for b in range(len(pref)):
        fp.pref[b] = float(pref[b])
        fp.intra[b] = float(intra[b])
    if xpref is not None:
        xp = np.asarray(xpref, dtype=np.float64)
        for b in range(xp.shape[0]):
            for c in range(xp.shape[1]):
                fp.xpref[b * nat.MAX_BINDERS + c] = float(xp[b, c])
    return fp


def binding_params(*, sites, e_mod, e_nomod, mu, mu_adjust_factor=1.0, max_binders=-1):
    bp = nat.BindingParams()
    nb = len(sites)
    bp.n_binders = nb
    bp.max_binders = int(max_binders)
    table = binding_free_energy_table(list(sites), list(e_mod), list(e_nomod))
    for b in range(nb):
        bp.sites[b] = int(sites[b])
        bp.mu[b] = float(mu[b])
    bp.mu_adjust_factor = float(mu_adjust_factor)
    flat = table.reshape(-1)
    for i in range(len(flat)):
        bp.bind_f[i] = float(flat[i])
    return bp


def move_ctl(move_name, *, amp_move, amp_bead, num_per_cycle=1, simple=True, bead_bounds=(0, 0),
             move_bounds=(0.0, 0.0), move_on=1, acc_rate=0.0, alpha=2 / 21, num_attempt=0,
             num_success=0):
    c = nat.MoveCtl()
    c.move_kind = MOVE_KIND[move_name]
    c.ctrl_kind = 1 if simple else 0
    c.num_per_cycle = int(num_per_cycle)
    c.move_on = int(move_on)
    c.amp_move = float(amp_move)
    c.amp_bead = int(amp_bead)
    c.bead_lo, c.bead_hi = (float(x) for x in bead_bounds)
    c.move_lo, c.move_hi = (float(x) for x in move_bounds)
    c.acc_rate, c.alpha = float(acc_rate), float(alpha)
    c.num_attempt, c.num_success = int(num_attempt), int(num_success)
    return c


def bonds_array(eps_bend, gamma, eps_par, eps_perp, eta):
    return np.ascontiguousarray(np.stack([eps_bend, gamma, eps_par, eps_perp, eta], axis=1))
