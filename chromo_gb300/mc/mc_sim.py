"""``mc_sim`` on the GPU (chromo/mc/mc_sim.pyx:26-103, mc_step :106-182).

Same signature and loop as the reference: ``num_mc_steps`` steps, each
cycling the controllers in order, each controller attempting
``num_per_cycle`` moves on the polymer and then updating its amplitudes.  The
whole loop runs in one kernel launch; the polymer's arrays, the field's
density and the controllers' amplitudes, counters and acceptance rates are
copied back when it returns.

Randomness: the reference draws from libc ``rand()`` (never seeded) and from
numpy seeded with ``random_seed``.  Here both streams are counter-based
Philox4x32-10 keyed by ``random_seed``, so a run is reproducible from its
seed.  ``mc_sim_audit`` instead takes the two streams as arrays, which is how
this loop is checked move by move against the reference.

One polymer per call: the reference's field supports one polymer in
practice (chromo/fields.pyx:53-54); for many independent chains use
``chromo_gb300.batched.ReplicaBatch``.
"""
import itertools

import numpy as np

from .. import _native as nat
from ..device import binding_params, field_params
from ..fields import FieldBase, NullField, UniformDensityField

_CONFINE = {"": 0, "Spherical": 1, "Cubical": 2}
POSITION_PRECISION = "fp32"  # "fp32" (GPU storage) or "fp64" (the reference's storage)


def set_position_precision(p: str):
    """Store positions in "fp32" (default, FP32 arithmetic) or "fp64" (FP64
    arithmetic, the reference's numerics move for move)."""
    global POSITION_PRECISION
    if p not in ("fp32", "fp64"):
        raise ValueError("precision must be 'fp32' or 'fp64'")
    POSITION_PRECISION = p


def _field_kind(poly, field):
    if field is None or not isinstance(field, FieldBase) or poly not in field:
        return 0
    return 2 if isinstance(field, UniformDensityField) else 1


def _grid_dims(field):
    if isinstance(field, UniformDensityField):
        return [field.nx, field.ny, field.nz]
    return [1, 1, 1]


def _ctl_struct(ctrl):
    mv = ctrl.move
    c = nat.MoveCtl()
    c.move_kind = nat.MOVE_NAMES.index(mv.name)
    c.ctrl_kind = getattr(ctrl, "kind", 0)
    c.num_per_cycle = int(mv.num_per_cycle)
    c.move_on = int(mv.move_on)
    c.amp_move = float(mv.amp_move)
    c.amp_bead = int(mv.amp_bead)
    c.bead_lo, c.bead_hi = (float(x) for x in ctrl.bead_amp_bounds)
    c.move_lo, c.move_hi = (float(x) for x in ctrl.move_amp_bounds)
    c.acc_rate = float(mv.acceptance_tracker.acceptance_rate)
    c.alpha = float(mv.acceptance_tracker.alpha)
    c.num_attempt = int(mv.num_attempt)
    c.num_success = int(mv.num_success)
    return c


def _bounds(ctrls):
    seg, tan = 2, 1
    for ctrl in ctrls:
        top = max(float(ctrl.move.amp_bead),
                  float(ctrl.bead_amp_bounds[1]) if getattr(ctrl, "kind", 0) == 1 else 0.0)
        if ctrl.move.name == "tangent_rotation":
            tan = max(tan, int(np.ceil(top)))
        else:
            seg = max(seg, int(np.ceil(top)) + 2)
    return seg, tan


def _binding_struct(poly):
    binders = poly.beads[0].binders
    return binding_params(
        sites=[b.sites_per_bead for b in binders], e_mod=[b.bind_energy_mod for b in binders],
        e_nomod=[b.bind_energy_no_mod for b in binders],
        mu=[b.chemical_potential for b in binders],
        mu_adjust_factor=float(getattr(poly, "mu_adjust_factor", 1.0)),
        max_binders=int(poly.max_binders))


def _field_struct(poly, field):
    kind = _field_kind(poly, field)
    nb = poly.num_binders
    if kind == 2:
        pref, intra, xpref = field.prefactor_arrays()
        return field_params(
            field_kind=2, confine_kind=_CONFINE[field.confine_type],
            confine_length=field.confine_length, nxyz=(field.nx, field.ny, field.nz),
            widths=(field.x_width, field.y_width, field.z_width), n_binders=nb, chi=field.chi,
            vf_limit=field.vf_limit, bead_vol=poly.beads[0].vol, pref=pref, intra=intra,
            xpref=xpref, fast_field=field.fast_field, n_points=field.n_points)
    if kind == 1:
        return field_params(field_kind=1, confine_kind=_CONFINE[field.confine_type],
                            confine_length=field.confine_length, n_binders=nb)
    return field_params(field_kind=0, n_binders=nb)


def _device(poly, field, ctrls=(), precision=None):
    """A one-replica Sim holding ``poly`` in ``field``."""
    precision = precision or POSITION_PRECISION
    if poly.num_binders > nat.MAX_BINDERS:
        raise NotImplementedError(f"at most {nat.MAX_BINDERS} binder types")
    seg, tan = _bounds(ctrls)
    nonuni = isinstance(field, UniformDensityField) and not field.uniform_access
    sim = nat.Sim([poly.num_beads], [_grid_dims(field)], poly.num_binders,
                  pos_fp64=(precision == "fp64"), max_segment=seg, max_tangent=tan,
                  nonuniform_access=nonuni)
    sim.set_chain(0, r=poly.r, t3=poly.t3, t2=poly.t2, states=poly.states,
                  marks=poly.chemical_mods, bonds=poly.bond_parameters())
    if hasattr(poly, "twist_parameters"):  # SSTWLC
        sim.set_twist(0, *poly.twist_parameters())
    sim.set_field(0, _field_struct(poly, field),
                  access_vol=field.access_vols if nonuni else None)
    sim.set_binding(0, _binding_struct(poly))
    if ctrls:
        sim.set_controllers(0, [_ctl_struct(c) for c in ctrls])
    if _field_kind(poly, field) == 2:
        sim.deposit(0)
    return sim


def _pull(sim, poly, field, ctrls):
    r, t3, t2, st = sim.get_chain(0)
    poly.r[:] = r
    poly.t3[:] = t3
    poly.t2[:] = t2
    poly.states[:] = st
    poly.r_trial[:] = r
    poly.t3_trial[:] = t3
    poly.t2_trial[:] = t2
    poly.states_trial[:] = st
    if _field_kind(poly, field) == 2:
        field._density_fx = sim.density(0)
    if ctrls:
        for ctrl, c in zip(ctrls, sim.get_controllers(0, len(ctrls))):
            mv = ctrl.move
            mv.amp_move = c.amp_move
            mv.amp_bead = int(c.amp_bead)
            mv.num_attempt = int(c.num_attempt)
            mv.num_success = int(c.num_success)
            mv.acceptance_tracker.acceptance_rate = c.acc_rate


def _check(polymers, field):
    polymers = list(polymers)
    if len(polymers) != 1:
        raise NotImplementedError("mc_sim runs one polymer per field; use "
                                  "chromo_gb300.batched.ReplicaBatch for many chains")
    if isinstance(field, UniformDensityField) and len(field.polymers) > 1:
        raise NotImplementedError("a UniformDensityField holding several polymers is not supported")
    return polymers[0]


def mc_sim(polymers, readerproteins, num_mc_steps, mc_move_controllers, field,
           mu_adjust_factor, random_seed):
    """Perform ``num_mc_steps`` Monte Carlo steps (chromo/mc/mc_sim.pyx:26-103)."""
    poly = _check(polymers, field)
    num_mc_steps = int(num_mc_steps)
    if num_mc_steps < 0:
        raise ValueError("num_mc_steps must be non-negative")
    poly.mu_adjust_factor = float(mu_adjust_factor)
    ctrls = list(mc_move_controllers)
    if not ctrls or num_mc_steps == 0:
        return
    sim = _device(poly, field, ctrls)
    try:
        sim.run(num_mc_steps, int(random_seed))
        sim.sync()
        _pull(sim, poly, field, ctrls)
    finally:
        sim.close()


class ResidentChain:
    """One polymer kept on the device across successive runs.

    ``polymer_in_field`` (chromo/mc/__init__.py:36-161) calls ``mc_sim`` once
    per snapshot, and each call would upload the chain, its field and its
    controllers and read them back.  Here the device state stays resident
    between runs: ``run`` continues the same simulation (its move counter keeps
    counting, so every run draws fresh random streams whatever its seed), then
    refreshes the polymer, the field's density and the controllers on the host
    as ``mc_sim`` does.  A changed ``mu_adjust_factor`` is uploaded before the
    run it applies to."""

    def __init__(self, polymers, field, mc_move_controllers):
        self.poly = _check(polymers, field)
        self.field = field
        self.ctrls = list(mc_move_controllers)
        self.maf = float(getattr(self.poly, "mu_adjust_factor", 1.0))
        self.sim = _device(self.poly, field, self.ctrls) if self.ctrls else None

    def run(self, num_mc_steps, mu_adjust_factor, random_seed):
        num_mc_steps = int(num_mc_steps)
        if num_mc_steps < 0:
            raise ValueError("num_mc_steps must be non-negative")
        self.poly.mu_adjust_factor = float(mu_adjust_factor)
        if self.sim is None or num_mc_steps == 0:
            return
        if self.poly.mu_adjust_factor != self.maf:
            self.sim.set_binding(0, _binding_struct(self.poly))
            self.maf = self.poly.mu_adjust_factor
        self.sim.run(num_mc_steps, int(random_seed))
        self.sim.sync()
        _pull(self.sim, self.poly, self.field, self.ctrls)

    def close(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None


_STEP_SEEDS = itertools.count(0x5EED000000000000)


def mc_step(adaptible_move, poly, readerproteins, field, active_field=1, update_distances=0,
            random_seed=None):
    """One attempted move of ``adaptible_move`` on ``poly`` (chromo/mc/mc_sim.pyx:106-182):
    proposal at the move's current amplitudes, polymer dE plus the field dE when
    ``active_field`` is set and ``poly`` is in ``field`` (not for tangent rotations),
    Metropolis decision and commit, on the GPU; the move's attempt and success counters and
    acceptance tracker are updated, its amplitudes are not (that is ``mc_sim``'s
    controller step).

    ``update_distances`` only concerns polymers that track pairwise distances (the steric
    chromatin model, not on this path) and must be 0.  The random stream is Philox keyed by
    ``random_seed``; by default each call takes the next seed of a per-process sequence,
    so that successive calls draw fresh streams (the reference draws from libc ``rand()``).
    """
    if update_distances:
        raise NotImplementedError("pairwise-distance updates (steric chromatin) are not on this path")
    from .mc_controller import NoControl
    amp_bead, amp_move = int(adaptible_move.amp_bead), float(adaptible_move.amp_move)
    ctrl = NoControl(adaptible_move, (amp_bead, amp_bead), (amp_move, amp_move))
    seed = next(_STEP_SEEDS) if random_seed is None else int(random_seed)
    saved = adaptible_move.num_per_cycle
    adaptible_move.num_per_cycle = 1
    try:
        mc_sim([poly], readerproteins, 1, [ctrl], field if active_field else None,
               float(getattr(poly, "mu_adjust_factor", 1.0)), seed)
    finally:
        adaptible_move.num_per_cycle = saved


def mc_sim_audit(polymers, readerproteins, num_mc_steps, mc_move_controllers, field,
                 mu_adjust_factor, draws, binding_draws, precision=None):
    """``mc_sim`` with explicit random streams, returning a record per attempted
    move (kind, n_inds, ind0, indf, dE_poly, dE_field, accepted, n_draws).

    ``draws``: values in [0, 2^31 - 1] consumed where the reference calls
    libc ``rand()``; ``binding_draws``: new binding states consumed where it
    calls ``np.random.randint(0, sites + 1)``."""
    poly = _check(polymers, field)
    poly.mu_adjust_factor = float(mu_adjust_factor)
    ctrls = list(mc_move_controllers)
    sim = _device(poly, field, ctrls, precision=precision)
    try:
        recs, du, bu = sim.run_audit(0, int(num_mc_steps), draws, binding_draws,
                                     max_records=int(num_mc_steps) * sum(
                                         int(c.move.num_per_cycle) for c in ctrls) + 8)
        _pull(sim, poly, field, ctrls)
    finally:
        sim.close()
    return recs, du, bu


def _energies_of(poly, field=None):
    """(elastic, binding, field-consistent, 0) energies of ``poly`` in FP64 on the GPU."""
    # a one-off evaluation: positions stay in FP64, as on the host
    if field is None:
        sim = _device(poly, NullField([]), precision="fp64")
    else:
        sim = _device(poly, field, precision="fp64")
    try:
        return sim.energy(0)
    finally:
        sim.close()


def _deposit_field(field):
    if not field.polymers:
        field._density_fx = np.zeros((field.n_bins, field.num_binders + 1), dtype=np.int64)
        return
    if len(field.polymers) > 1:
        raise NotImplementedError("a UniformDensityField holding several polymers is not supported")
    poly = field.polymers[0]
    sim = _device(poly, field)
    try:
        field._density_fx = sim.density(0)
    finally:
        sim.close()
