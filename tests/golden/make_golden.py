"""Generate golden vectors for the MC inner loop from the reference itself.

Run here (the container that mounts the reference), after
``python oracle/build_reference.py``::

    python tests/golden/make_golden.py

For each seeded case this script

1. builds the polymer, binders and field through the reference's own API
   (``Chromatin.gaussian_walk_polymer``, ``make_binder_collection``,
   ``UniformDensityField`` / ``NullField``);
2. seeds libc ``rand()`` with ``srand(seed)`` (the reference never seeds it,
   ``chromo/mc/mc_sim.pyx:52-56``) and numpy with ``np.random.seed``;
3. runs a per-move audit loop that is ``mc_sim``/``mc_step``
   (``chromo/mc/mc_sim.pyx:88-182``) line for line, built from the
   reference's move functions, ``MCAdapter.accept/reject`` and the ``cdef``
   energy methods reached through ``oracle/ref_shim.pyx``, recording every
   attempted move's polymer dE, field dE and decision;
4. runs the reference's own ``mc_sim`` from the same start with the same
   seeds and asserts it ends in exactly the same state as the audit loop;
5. stores inputs, the consumed ``rand()`` values, the consumed binding-state
   draws, the per-move records and the final state in ``<case>.npz``.

The stored streams let the CPU oracle and the GPU audit mode replay the very
same trajectory without the reference present.
"""
import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "oracle" / "ref_stubs"), str(ROOT / "oracle" / "_ref")]

import chromo.binders as cb  # noqa: E402
import chromo.mc as cmc  # noqa: E402
import chromo.mc.mc_controller as ctl  # noqa: E402
import chromo.mc.move_funcs as mf  # noqa: E402
from chromo.fields import NullField, UniformDensityField  # noqa: E402
from chromo.mc.mc_sim import mc_sim  # noqa: E402
from chromo.polymers import SSTWLC, Chromatin  # noqa: E402
import ref_shim  # noqa: E402

LIBC = ctypes.CDLL(None)
LIBC.rand.restype = ctypes.c_int
RAND_MAX = 2147483647
OUT = Path(__file__).resolve().parent
MOVES = ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]


def markov_marks(rng, n, run_length):
    """3-state Markov mark track on {0,1,2}: stay with prob 1-1/run_length,
    otherwise jump uniformly to one of the other two states."""
    out = np.empty(n, dtype=np.int64)
    s = rng.integers(0, 3)
    for i in range(n):
        out[i] = s
        if rng.random() < 1.0 / run_length:
            s = (s + rng.integers(1, 3)) % 3
    return out


def reset_presets():
    for name, mu in (("HP1", -1.0), ("PRC1", -1.0)):
        b = cb.get_by_name(name)
        b.chemical_potential = mu
        b.interaction_energy = -4.0
        b.cross_talk_interaction_energy = {"PRC1": 0} if name == "HP1" else {"HP1": 0}


CASES = {
    # one binder, periodic box, all moves with SimpleControl (the plain config, scaled down)
    "one_binder": dict(n=200, nbins=10, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0,
                       steps=4, moves="all", seed=11, run=20),
    # two binders with cross talk stored on HP1 (the batched config's binder set)
    "two_binders": dict(n=200, nbins=8, vox=40.0, binders=[("HP1", -0.5, -4.0, {"PRC1": 1.0}),
                                                           ("PRC1", -0.3, -3.0, {})],
                        chi=1.5, steps=4, moves="all", seed=12, run=50),
    # dense small box with a low volume-fraction limit: exercises the 1e99 branch
    "vf_limit": dict(n=300, nbins=5, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0,
                     vf_limit=0.03, steps=2, moves="all", seed=13, run=20),
    # positive chemical potential, annealing factor, and a cap on bound binders
    "anneal_maxb": dict(n=200, nbins=6, vox=40.0, binders=[("HP1", 0.3, -4.0, {}),
                                                           ("PRC1", -0.6, -3.0, {"HP1": 0.5})],
                        chi=0.8, steps=4, moves="all", seed=14, run=10, mu_adjust_factor=0.7,
                        max_binders=2),
    # null field with a spherical confinement (confinement dE only)
    "null_spherical": dict(n=200, binders=[("HP1", -0.4, -4.0, {})], null_field=True,
                           confine=("Spherical", 400.0), steps=4, moves="all", seed=15, run=20),
    # spherical confinement of a density field with accessible volumes computed
    # for the voxels the sphere cuts (assume_fully_accessible=0)
    "sphere_access": dict(n=120, nbins=16, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0,
                          confine=("Spherical", 300.0), access=True, steps=4, moves="all", seed=17,
                          run=20),
    # fast_field: per-move density changes from 64 sub-bins per voxel and axis
    # (the reference's tables), full deposits exact; two binders with cross talk
    "fast_field": dict(n=200, nbins=8, vox=40.0, binders=[("HP1", -0.5, -4.0, {"PRC1": 1.0}),
                                                          ("PRC1", -0.3, -3.0, {})],
                       chi=1.2, fast=64, steps=4, moves="all", seed=18, run=30),
    # twist: an SSTWLC chain (twist persistence length 100 nm), whose bond energy
    # adds the twist term of the t2 / t3 frames (chromo/polymers.pyx:1889-2320)
    "twist": dict(n=200, nbins=8, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0, lt=100.0,
                  steps=4, moves="all", seed=19, run=20),
    # large amplitudes without adaptation: long segments, many tangent beads
    "big_amps": dict(n=160, nbins=8, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0,
                     steps=30, moves="big", seed=16, run=20),
}


def build_case(cfg):
    reset_presets()
    rng = np.random.default_rng(cfg["seed"])
    n = cfg["n"]
    names = [b[0] for b in cfg["binders"]]
    for name, mu, eps, cross in cfg["binders"]:
        b = cb.get_by_name(name)
        b.chemical_potential = mu
        b.interaction_energy = eps
        b.cross_talk_interaction_energy = dict(cross)
    binders = cb.make_binder_collection([cb.get_by_name(nm) for nm in names])
    marks = np.stack([markov_marks(rng, n, cfg["run"]) for _ in names], axis=1)
    states = rng.integers(0, 3, size=marks.shape).astype(np.int64) if cfg.get("random_states") \
        else np.zeros_like(marks)
    np.random.seed(cfg["seed"])
    kw = dict(states=states, binder_names=np.array(names), chemical_mods=marks,
              chemical_mod_names=np.array([f"m{i}" for i in range(len(names))]),
              max_binders=cfg.get("max_binders", -1))
    if cfg.get("lt"):
        p = SSTWLC.gaussian_walk_polymer("p", n, np.full(n - 1, 16.5), lp=53.0, lt=cfg["lt"], **kw)
    else:
        p = Chromatin.gaussian_walk_polymer("p", n, np.full(n - 1, 16.5), **kw)
    return p, binders, marks, states


def make_field(cfg, p, binders):
    if cfg.get("null_field"):
        ct, cl = cfg["confine"]
        return NullField([p], confine_type=ct, confine_length=cl)
    w = cfg["nbins"] * cfg["vox"]
    ct, cl = cfg.get("confine", ("", 0.0))
    return UniformDensityField([p], binders, w, cfg["nbins"], w, cfg["nbins"], w, cfg["nbins"],
                               confine_type=ct, confine_length=cl, chi=cfg["chi"],
                               assume_fully_accessible=0 if cfg.get("access") else 1,
                               vf_limit=cfg.get("vf_limit", 0.5),
                               fast_field=1 if cfg.get("fast") else 0,
                               n_points=cfg.get("fast", 1000))


def make_controllers(cfg, p):
    bab, mab = cmc.get_amplitude_bounds([p])
    if cfg["moves"] == "all":
        return ctl.all_moves("/tmp/golden_logs", bab.bounds, mab.bounds, ctl.SimpleControl)
    big_bead = {"crank_shaft": (100, 150), "end_pivot": (60, 80), "slide": (100, 150),
                "tangent_rotation": (25, 40), "change_binding_state": (6, 8)}
    big_move = {"crank_shaft": (0.8 * np.pi, 1.0 * np.pi), "end_pivot": (0.8 * np.pi, 1.0 * np.pi),
                "slide": (8.0, 10.0), "tangent_rotation": (0.5 * np.pi, 1.0 * np.pi),
                "change_binding_state": (0, 0)}
    cs = ctl.specific_moves([getattr(mf, m) for m in MOVES], "/tmp/golden_logs",
                            big_bead, big_move, ctl.NoControl)
    return cs


def clone(p, cfg):
    names = list(np.asarray(p.binder_names))
    kw = dict(bead_length=np.asarray(p.bead_length).copy(), t3=np.asarray(p.t3).copy(),
              t2=np.asarray(p.t2).copy(), states=np.asarray(p.states).copy(),
              binder_names=np.array(names), chemical_mods=np.asarray(p.chemical_mods).copy(),
              chemical_mod_names=np.asarray(p.chemical_mod_names), max_binders=cfg.get("max_binders", -1))
    if cfg.get("lt"):
        return SSTWLC("p", np.asarray(p.r).copy(), lp=53.0, lt=cfg["lt"], **kw)
    return Chromatin("p", np.asarray(p.r).copy(), **kw)


def audit_loop(p, field, ctrls, steps, mu_adjust_factor):
    """mc_sim.pyx:88-103 + mc_step :106-182, with every move recorded."""
    recs = []
    for _ in range(steps):
        for c in ctrls:
            mv = c.move
            if mv.move_on == 1:
                for _ in range(mv.num_per_cycle):
                    p.mu_adjust_factor = mu_adjust_factor
                    check_field = (p in field) and mv.name != "tangent_rotation"
                    mv.num_attempt += 1
                    inds = np.asarray(mv.move_func(polymer=p, amp_move=mv.amp_move,
                                                   amp_bead=mv.amp_bead)).astype(np.int64)
                    n = len(inds)
                    kind = MOVES.index(mv.name)
                    if n == 0:
                        recs.append((kind, 0, -1, -1, 0.0, 0.0, -1))
                        continue
                    dEp = ref_shim.poly_dE(p, mv.name, inds)
                    dEf = 0.0
                    if check_field:
                        dEf = ref_shim.field_dE(field, p, inds, mv.name == "change_binding_state")
                    dE = 0.0
                    dE += dEp
                    dE += dEf
                    with np.errstate(over="ignore"):
                        exp_dE = np.exp(-dE)
                    u = LIBC.rand() / RAND_MAX
                    acc = u < exp_dE
                    if acc:
                        mv.accept(p, dE, inds, n, False, False, False)
                        if check_field:
                            ref_shim.field_accept(field)
                    else:
                        mv.reject(p, dE, inds, n, False, False, False)
                    recs.append((kind, n, int(inds[0]), int(inds[-1]) + 1, dEp, dEf, int(acc)))
            c.update_amplitudes()
    return recs


def consumed(stream, extra):
    """Index in ``stream`` of the first value not consumed, given the next few
    values drawn after the run."""
    k = len(extra)
    for i in range(len(stream) - k):
        if stream[i] == extra[0] and np.array_equal(stream[i:i + k], extra):
            return i
    raise RuntimeError("consumed-draw search failed; enlarge the stream")


def density_of(field):
    return np.asarray(field.density).copy() if isinstance(field, UniformDensityField) else np.zeros((0, 0))


def run_case(name, cfg):
    p, binders, marks, states0 = build_case(cfg)
    init = dict(r=np.asarray(p.r).copy(), t3=np.asarray(p.t3).copy(), t2=np.asarray(p.t2).copy(),
                states=np.asarray(p.states).copy(), marks=np.asarray(p.chemical_mods).copy())
    field = make_field(cfg, p, binders)
    ctrls = make_controllers(cfg, p)
    ctl0 = [(c.move.amp_move, c.move.amp_bead, c.move.num_per_cycle,
             1 if isinstance(c, ctl.SimpleControl) else 0,
             c.bead_amp_bounds[0], c.bead_amp_bounds[1],
             c.move_amp_bounds[0], c.move_amp_bounds[1]) for c in ctrls]
    maf = cfg.get("mu_adjust_factor", 1.0)
    seed = cfg["seed"] * 1000 + 7
    nseed = cfg["seed"] * 1000 + 9
    LIBC.srand(seed)
    stream = np.array([LIBC.rand() for _ in range(400000)], dtype=np.uint32)
    bs_rng = np.random.RandomState(nseed)
    bstream = np.array([bs_rng.randint(0, 3) for _ in range(50000)], dtype=np.int64)
    # audit loop
    LIBC.srand(seed)
    np.random.seed(nseed)
    recs = audit_loop(p, field, ctrls, cfg["steps"], maf)
    nxt = np.array([LIBC.rand() for _ in range(6)], dtype=np.uint32)
    n_draws = consumed(stream, nxt)
    n_bind = int(sum(r[1] for r in recs if r[0] == 4))
    # the reference's own mc_sim from the same start and seeds
    p2 = clone(build_case(cfg)[0], cfg)
    for k, v in init.items():
        if k in ("r", "t3", "t2"):
            getattr(p2, k)[:, :] = v
    field2 = make_field(cfg, p2, binders)
    ctrls2 = make_controllers(cfg, p2)
    LIBC.srand(seed)
    mc_sim([p2], binders, cfg["steps"], ctrls2, field2, maf, nseed)
    for a in ("r", "t3", "t2", "states"):
        assert np.array_equal(np.asarray(getattr(p, a)), np.asarray(getattr(p2, a))), (name, a)
    assert np.array_equal(density_of(field), density_of(field2)), name
    for c1, c2 in zip(ctrls, ctrls2):
        assert (c1.move.amp_move, c1.move.amp_bead, c1.move.num_attempt, c1.move.num_success) == \
               (c2.move.amp_move, c2.move.amp_bead, c2.move.num_attempt, c2.move.num_success), name
    rec = np.array(recs, dtype=[("kind", np.int32), ("n_inds", np.int32), ("ind0", np.int32),
                                ("indf", np.int32), ("dE_poly", np.float64),
                                ("dE_field", np.float64), ("accepted", np.int32)])
    bl = cb.make_binder_collection  # noqa: F841  (kept for readers of the recipe)
    binder_rows = [cb.get_by_name(b[0]) for b in cfg["binders"]]
    uniform = isinstance(field, UniformDensityField)
    out = dict(
        n_steps=cfg["steps"], mu_adjust_factor=maf, max_binders=cfg.get("max_binders", -1),
        bead_length=np.asarray(p.bead_length).copy(), lp=53.0, bead_rad=5.0,
        eps_bend=np.asarray(p.eps_bend), gamma=np.asarray(p.gamma), eps_par=np.asarray(p.eps_par),
        eps_perp=np.asarray(p.eps_perp), eta=np.asarray(p.eta),
        binder_names=np.array([b[0] for b in cfg["binders"]]),
        sites=np.array([b.sites_per_bead for b in binder_rows]),
        e_mod=np.array([b.bind_energy_mod for b in binder_rows]),
        e_nomod=np.array([b.bind_energy_no_mod for b in binder_rows]),
        mu=np.array([b.chemical_potential for b in binder_rows]),
        interaction_energy=np.array([b.interaction_energy for b in binder_rows]),
        interaction_radius=np.array([b.interaction_radius for b in binder_rows]),
        cross=np.array([[b.cross_talk_interaction_energy.get(o[0], np.nan) for o in cfg["binders"]]
                        for b in binder_rows]),
        field_kind=2 if uniform else 1,
        confine_kind={"": 0, "Spherical": 1, "Cubical": 2}[field.confine_type],
        confine_length=field.confine_length,
        nxyz=np.array([field.nx, field.ny, field.nz]) if uniform else np.array([1, 1, 1]),
        widths=np.array([field.x_width, field.y_width, field.z_width]) if uniform else np.ones(3),
        chi=field.chi if uniform else 0.0, vf_limit=field.vf_limit if uniform else 0.5,
        pref=np.array([r["field_energy_prefactor"] for r in field.binder_dict]) if uniform else np.zeros(len(binder_rows)),
        intra=np.array([r["interaction_energy_intranucleosome"] for r in field.binder_dict]) if uniform else np.zeros(len(binder_rows)),
        xpref=np.array([[r["cross_talk_field_energy_prefactor"][o["name"]] for o in field.binder_dict]
                        for r in field.binder_dict]) if uniform else np.zeros((len(binder_rows),) * 2),
        ctl0=np.array(ctl0, dtype=np.float64),
        ctl_final=np.array([(c.move.amp_move, c.move.amp_bead, c.move.num_attempt, c.move.num_success,
                             c.move.acceptance_tracker.acceptance_rate) for c in ctrls]),
        draws=stream[:n_draws], bstates=bstream[:n_bind].astype(np.int8),
        records=rec,
        r0=init["r"], t30=init["t3"], t20=init["t2"], states0=init["states"], marks=init["marks"],
        r1=np.asarray(p.r).copy(), t31=np.asarray(p.t3).copy(), t21=np.asarray(p.t2).copy(),
        states1=np.asarray(p.states).copy(), density1=density_of(field),
        density0=None if not uniform else None,
        E_elastic1=p.compute_E(),
        access_vols=(np.array([field.access_vols[i] for i in range(field.n_bins)])
                     if uniform and cfg.get("access") else None),
        fast_n=field.n_points if uniform and cfg.get("fast") else None,
        lt=cfg.get("lt"), eps_twist=np.asarray(p.eps_twist).copy() if cfg.get("lt") else None,
        omega0=(np.asarray(p.bead_length) * (2 * np.pi / 10.5) / 0.332) if cfg.get("lt") else None,
    )
    out = {k: v for k, v in out.items() if v is not None}
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(f"{name}: {len(rec)} moves, {n_draws} draws, {n_bind} binding draws, "
          f"accepted {int((rec['accepted'] == 1).sum())}")


if __name__ == "__main__":
    todo = sys.argv[1:] or list(CASES)
    for nm in todo:
        run_case(nm, CASES[nm])
