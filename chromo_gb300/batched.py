"""Many independent chains on one GPU, each in its own field.

The reference runs ``mc_sim`` on one polymer in one field
(chromo/mc/mc_sim.pyx:26-103, chromo/fields.pyx:53-54).  ``ReplicaBatch``
holds R such simulations resident on the device at once: replica r is the
chain ``polymers[r]`` in ``fields[r]`` with its own move controllers, binder
chemical potentials and chi.  One kernel launch advances every replica
(one CTA per replica); ``run_exchange`` alternates MC rounds with replica
exchange, which swaps chi between neighbouring rungs of ladders of
replicas (accept with probability min(1, exp((chi_a - chi_b)(S_a - S_b))),
S the chi-free part of the field energy), all under one CUDA graph.

``energy_drift`` compares the FP64 energies recomputed from the resident
state with the running sum of accepted dE.  Away from rounding it is zero,
except for one reference rule kept for parity: tangent_rotation evaluates
each rotated bead with its neighbours' current tangents
(chromo/polymers.pyx:1074-1080), so when two adjacent beads rotate in the
same move the summed dE is not the energy change.  Moves whose dE carries a
1e25 / 1e99 penalty are left out of the running sum (one would absorb every
later dE in FP64); a replica whose baseline or current energy carries a
penalty has no measurable drift and reports NaN.
"""
from typing import List, Optional, Sequence

import numpy as np

from . import _native as nat
from .derivatives import observable_coefficients, reweighting_sensitivity, theta_coefficients
from .fields import NullField, UniformDensityField
from .mc import get_amplitude_bounds
from .mc.mc_controller import SimpleControl, all_moves
from .mc.mc_sim import (_binding_struct, _bounds, _ctl_struct, _field_kind, _field_struct,
                        _grid_dims)


# energies at or above this carry the 1e25 max_binders or 1e99 field penalty
PENALTY_FLOOR = 1e20


def _drift(E, E0, run):
    """(E - E0) - run, NaN where E or E0 carries a penalty."""
    d = (E - E0) - run
    return np.where((np.abs(E) < PENALTY_FLOOR) & (np.abs(E0) < PENALTY_FLOOR), d, np.nan)


class EnergyDriftError(RuntimeError):
    """The recomputed energy left the running sum of dE by more than the tolerance."""


class ReplicaBatch:
    """R chains, each in its own field, resident on the GPU.

    ``polymers``: Chromatin / SSWLC chains, all with the same binder types;
    ``fields``: one UniformDensityField or NullField per chain, holding only
    that chain; ``controllers``: one list of move controllers per chain
    (default: ``all_moves`` with SimpleControl and the chain's own
    amplitude bounds, as ``chromo.mc.polymer_in_field`` sets up);
    ``precision``: "fp32" (default) or "fp64" position storage;
    ``warps_per_block`` / ``lanes_per_move``: the kernel's launch shape (0:
    chosen by the library); ``autotune=True`` times the candidate shapes on
    scratch copies of this batch first (``chromo_gb300.autotune``) and uses
    the fastest (results cached per problem)."""

    def __init__(self, polymers: Sequence, fields: Sequence, controllers: Optional[List[list]] = None,
                 *, precision: str = "fp32", warps_per_block: int = 0, lanes_per_move: int = 0,
                 autotune: bool = False):
        self.polymers = list(polymers)
        self.fields = list(fields)
        R = len(self.polymers)
        if R < 1 or len(self.fields) != R:
            raise ValueError("one field per polymer, at least one polymer")
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        nb = {p.num_binders for p in self.polymers}
        if len(nb) != 1:
            raise ValueError("every polymer must carry the same number of binder types")
        nb = nb.pop()
        if nb > nat.MAX_BINDERS:
            raise NotImplementedError(f"at most {nat.MAX_BINDERS} binder types")
        for p, f in zip(self.polymers, self.fields):
            if not isinstance(f, (UniformDensityField, NullField)):
                raise TypeError("fields must be UniformDensityField or NullField")
            if isinstance(f, UniformDensityField) and (len(f.polymers) != 1 or f.polymers[0] is not p):
                raise ValueError("each UniformDensityField must hold exactly its own polymer")
        if controllers is None:
            controllers = []
            for p in self.polymers:
                bead, move = get_amplitude_bounds([p])
                controllers.append(all_moves("", bead.bounds, move.bounds, SimpleControl))
        if len(controllers) != R:
            raise ValueError("one controller list per polymer")
        self.controllers = [list(c) for c in controllers]
        seg, tan = 2, 1
        for ctrls in self.controllers:
            s, t = _bounds(ctrls)
            seg, tan = max(seg, s), max(tan, t)
        self._nb, self._seg, self._tan = nb, seg, tan
        self._fp64 = precision == "fp64"
        self._nonuni = any(isinstance(f, UniformDensityField) and not f.uniform_access for f in self.fields)
        self.tuning = None
        if autotune:
            from . import autotune as at
            (warps_per_block, lanes_per_move), self.tuning = at.tune(
                self._make_sim, [p.num_beads for p in self.polymers],
                [_grid_dims(f) for f in self.fields], nb, self._fp64)
        self.sim = self._make_sim(warps_per_block, lanes_per_move)
        self.rebaseline()

    def _make_sim(self, warps_per_block: int, lanes_per_move: int) -> "nat.Sim":
        """A resident simulation of this batch's chains, fields and controllers."""
        sim = nat.Sim([p.num_beads for p in self.polymers], [_grid_dims(f) for f in self.fields],
                      self._nb, pos_fp64=self._fp64, max_segment=self._seg, max_tangent=self._tan,
                      warps_per_block=warps_per_block, nonuniform_access=self._nonuni,
                      lanes_per_move=lanes_per_move)
        for r, (p, f, ctrls) in enumerate(zip(self.polymers, self.fields, self.controllers)):
            sim.set_chain(r, r=p.r, t3=p.t3, t2=p.t2, states=p.states, marks=p.chemical_mods,
                          bonds=p.bond_parameters())
            if hasattr(p, "twist_parameters"):  # SSTWLC
                sim.set_twist(r, *p.twist_parameters())
            uni = isinstance(f, UniformDensityField)
            sim.set_field(r, _field_struct(p, f), access_vol=f.access_vols if (self._nonuni and uni) else None)
            sim.set_binding(r, _binding_struct(p))
            sim.set_controllers(r, [_ctl_struct(c) for c in ctrls])
        sim.deposit(-1)
        return sim

    # ------------------------------------------------------------------ running
    @property
    def n_replicas(self) -> int:
        return self.sim.R

    def run(self, num_mc_steps: int, random_seed: int, stream=None):
        """``mc_sim`` on every replica at once (returns once enqueued; ``sync``)."""
        if int(num_mc_steps) < 0:
            raise ValueError("num_mc_steps must be non-negative")
        if int(num_mc_steps):
            self.sim.run(int(num_mc_steps), int(random_seed), stream)

    def run_exchange(self, n_rounds: int, steps_per_round: int, n_rungs: int, random_seed: int,
                     stream=None, mu_rungs: int = 0, mu_binder: int = 0):
        """``n_rounds`` of (``steps_per_round`` MC steps, one exchange) under a
        CUDA graph.  Ladders are n_rungs consecutive replicas; with
        ``mu_rungs`` > 1 replicas form grids of mu_rungs x n_rungs and the
        chemical potential of binder ``mu_binder`` is also exchanged between
        neighbouring mu rungs.  The swaps change energies outside of any move,
        so the drift baseline is reset."""
        self.sim.set_mu_ladder(int(mu_rungs), int(mu_binder))
        self.sim.run_batched(int(n_rounds), int(steps_per_round), int(n_rungs), int(random_seed), stream)
        self.sim.sync(stream)
        self.rebaseline()

    def exchange(self, n_rungs: int, round_: int, random_seed: int, stream=None):
        """One exchange round (rung pairs of parity ``round_ % 2``)."""
        self.sim.exchange(int(n_rungs), int(round_), int(random_seed), stream)
        self.sim.sync(stream)
        self.rebaseline()

    def sync(self, stream=None):
        """Wait for the enqueued work; device-side errors raise here."""
        self.sim.sync(stream)

    # ----------------------------------------------------------------- energies
    def energies(self) -> np.ndarray:
        """[R, 5] FP64: elastic, binding, field, running sum of accepted dE, chi-free S."""
        return self.sim.energies()

    def rebaseline(self):
        """Take the current energies as the reference point of ``energy_drift``."""
        e = self.sim.energies()
        self._E0 = e[:, 0] + e[:, 1] + e[:, 2]
        self.sim.reset_running_energy()

    def energy_drift(self) -> np.ndarray:
        """Per replica: (E_now - E_baseline) - (sum of accepted dE since then);
        NaN where either energy carries a penalty (|E| >= PENALTY_FLOOR)."""
        e = self.sim.energies()
        return _drift(e[:, 0] + e[:, 1] + e[:, 2], self._E0, e[:, 3])

    def check_drift(self, rel_tol: float = 1e-6):
        """Raise EnergyDriftError if |drift| > rel_tol * max(1, |E|) for any
        replica whose energies carry no penalty."""
        e = self.sim.energies()
        E = e[:, 0] + e[:, 1] + e[:, 2]
        drift = _drift(E, self._E0, e[:, 3])
        bad = np.nonzero(np.abs(drift) > rel_tol * np.maximum(1.0, np.abs(E)))[0]
        if len(bad):
            raise EnergyDriftError(f"energy drift above {rel_tol:g} on replicas {bad.tolist()[:8]}: "
                                   f"{drift[bad][:8].tolist()}")
        return drift

    @property
    def chi(self) -> np.ndarray:
        return self.sim.chi()

    def mu(self, binder: int = 0) -> np.ndarray:
        """Chemical potential of ``binder`` on every replica (moved by mu-ladder exchange)."""
        return self.sim.mu(binder)

    # ---------------------------------------------------------- derivatives
    def _theta_coef(self, r, mus=None):
        p, f = self.polymers[r], self.fields[r]
        binders = p.beads[0].binders
        vol_bin = f.vol_bin if isinstance(f, UniformDensityField) else 1.0
        mu = [b.chemical_potential for b in binders] if mus is None else [m[r] for m in mus]
        return theta_coefficients(mu, float(getattr(p, "mu_adjust_factor", 1.0)),
                                  [b.interaction_volume for b in binders], vol_bin)

    def _device_mus(self):
        return [self.sim.mu(b) for b in range(self.polymers[0].num_binders)]

    def gradient(self):
        """Per replica: dE/dr [N_r, 3] (FP32) and dE/d(chi, mu_0, mu_1, eps_00,
        eps_11, eps_01) [6] (FP64) of the energy ``energies`` sums."""
        g, T = self.sim.gradient()
        per, off = [], 0
        for p in self.polymers:
            per.append(g[off:off + p.num_beads])
            off += p.num_beads
        mus = self._device_mus()
        theta = np.stack([self._theta_coef(r, mus) @ T[r] for r in range(self.n_replicas)])
        return per, theta

    def sample(self, n_samples: int, steps_between: int, random_seed: int, stream=None):
        """``n_samples`` times: ``steps_between`` MC steps, then add every
        replica's energy terms to the running sums on the device."""
        for k in range(int(n_samples)):
            if steps_between:
                self.sim.run(int(steps_between), int(random_seed) + k, stream)
            self.sim.sample_terms(stream)
        self.sim.sync(stream)

    def sensitivities(self, reset: bool = False) -> np.ndarray:
        """[R, n_binders + 1, 6]: d<O>/dtheta for O = mean occupancy of each
        binder and the variance of the bead density over voxels, by
        reweighting the sampled configurations (-Cov(O, dE/dtheta))."""
        sum_t, sum_tt, count = self.sim.samples(reset)
        mus = self._device_mus()
        out = []
        for r, (p, f) in enumerate(zip(self.polymers, self.fields)):
            n_vox = f.n_bins if isinstance(f, UniformDensityField) else 1
            O = observable_coefficients(p.num_beads, n_vox, p.num_binders)
            out.append(reweighting_sensitivity(sum_t[r], sum_tt[r], count[r], O, self._theta_coef(r, mus)))
        return np.stack(out)

    # ------------------------------------------------------------ read back
    def push(self):
        """Upload the host objects' positions, tangents and binding states (all
        replicas in one call) and rebuild the densities."""
        self.sim.set_chains([dict(r=p.r, t3=p.t3, t2=p.t2, states=p.states) for p in self.polymers])
        self.sim.deposit(-1)
        self.rebaseline()

    def pull(self):
        """Copy positions, tangents, binding states, densities, chi and controller
        state back into the host objects."""
        chi = self.sim.chi()
        chains = self.sim.get_chains()
        for r, (p, f, ctrls) in enumerate(zip(self.polymers, self.fields, self.controllers)):
            rr, t3, t2, st = chains[r]
            p.r[:] = rr
            p.t3[:] = t3
            p.t2[:] = t2
            p.states[:] = st
            p.r_trial[:] = rr
            p.t3_trial[:] = t3
            p.t2_trial[:] = t2
            p.states_trial[:] = st
            if _field_kind(p, f) == 2:
                f._density_fx = self.sim.density(r)
                f.chi = float(chi[r])
            for ctrl, c in zip(ctrls, self.sim.get_controllers(r, len(ctrls))):
                mv = ctrl.move
                mv.amp_move = c.amp_move
                mv.amp_bead = int(c.amp_bead)
                mv.num_attempt = int(c.num_attempt)
                mv.num_success = int(c.num_success)
                mv.acceptance_tracker.acceptance_rate = c.acc_rate

    # ------------------------------------------------------------ checkpoint
    def save_checkpoint(self, path):
        """Write the batch's whole device state (chains, grids, controllers,
        chi / mu slots, every replica's move counter and running dE, exchange
        round and swap counts) to ``path`` (a .npy byte image).  A batch built
        from the same polymers, fields and controllers that loads it continues
        bit for bit as this one would, given the same seeds."""
        np.save(path, self.sim.save_state(), allow_pickle=False)

    def load_checkpoint(self, path):
        """Restore a ``save_checkpoint`` image and refresh the host objects."""
        self.sim.load_state(np.load(path, allow_pickle=False))
        self.pull()
        e = self.sim.energies()
        self._E0 = e[:, 0] + e[:, 1] + e[:, 2] - e[:, 3]  # the baseline the saved running sum had

    def close(self):
        self.sim.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
