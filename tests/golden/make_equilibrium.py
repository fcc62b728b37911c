"""Equilibrium statistics of the reference's own ``mc_sim``, for the long-run
statistical check of the GPU path (tests/test_gpu_equilibrium.py).

Run here (the container that mounts the reference), after
``python oracle/build_reference.py``::

    python tests/golden/make_equilibrium.py [one_binder|two_binders]

Each case is one small system run RUNS times.  one_binder: a 100-bead
Chromatin chain (16.5 nm spacing, lp 53 nm) with one binder (HP1 preset,
mu = -0.4, eps = -4) in a periodic 240 nm box of 6^3 voxels, chi = 1, all
five moves under SimpleControl.  two_binders: the same chain with two binders
(HP1: mu = -0.5, eps = -4, cross talk +1 with PRC1; PRC1: mu = -0.3,
eps = -3), chi = 1.5.  sphere_confined: a 100-bead chain (HP1 as in
one_binder, chi = 1) confined to a sphere of radius 100 nm (Spherical
confinement) centred in a 320 nm box of 8^3 voxels, with the accessible
volumes of the voxels the sphere cuts (assume_fully_accessible=0), started
from a seeded walk inside the sphere.  twist: the one_binder system as an
SSTWLC chain (twist persistence length 100 nm).  Each system is run RUNS times
from the same seeded start with independent random streams (libc ``srand``
and numpy seeds per run; ``mc_sim`` reseeds numpy on every call, so every call
gets its own seed).  After BURN MC steps, SAMPLES snapshots are taken every
EVERY steps and the per-run time averages of these observables are stored:

* R2: squared end-to-end distance (unwrapped positions), nm^2;
* Rg2: squared radius of gyration, nm^2;
* occupancy: mean binding state / sites per bead, per binder;
* five fractions of voxels whose bead count (density times the voxel's
  accessible volume) is
  below 0.05, in [0.05, 0.25), [0.25, 0.5), [0.5, 1), or 1 and above (the
  first bin is open below: the reference's FP64 density of an emptied voxel
  is often a rounding residue slightly below zero, the GPU's integer grid an
  exact zero);
* mean squared bead count per voxel.

The GPU test runs many replicas of the same start for the same steps and
compares the means within 3 combined standard errors.
"""
import ctypes
import multiprocessing as mp
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]

CASES = {
    "one_binder": dict(n=100, nbins=6, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0,
                       moves="all", seed=21, run=20),
    "two_binders": dict(n=100, nbins=6, vox=40.0, binders=[("HP1", -0.5, -4.0, {"PRC1": 1.0}),
                                                           ("PRC1", -0.3, -3.0, {})],
                        chi=1.5, moves="all", seed=22, run=20),
    "sphere_confined": dict(n=100, nbins=8, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0,
                            confine=("Spherical", 100.0), access=True, moves="all", seed=23, run=20),
    # the twisted chain's extension relaxes slowly and its per-run averages
    # scatter widely: four times the runs
    "twist": dict(n=100, nbins=6, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0, lt=100.0,
                  moves="all", seed=24, run=20, runs=64),
}
RUNS, BURN, SAMPLES, EVERY = 16, 1500, 300, 20
BINS = np.array([-np.inf, 0.05, 0.25, 0.5, 1.0, np.inf])
VOX = ["vox_0_0.05", "vox_0.05_0.25", "vox_0.25_0.5", "vox_0.5_1", "vox_1_inf"]


def obs_names(binder_names):
    occ = ["occupancy"] if len(binder_names) == 1 else [f"occupancy_{b}" for b in binder_names]
    return ["R2", "Rg2"] + occ + VOX + ["count2"]


def observables(r, states, counts, sites):
    """The observables of one snapshot (shared with the GPU test): R2, Rg2, the
    occupancy of each binder, the voxel bead-count histogram, its second moment."""
    r = np.asarray(r, dtype=np.float64)
    d = r[-1] - r[0]
    rc = r - r.mean(axis=0)
    hist = np.histogram(counts, bins=BINS)[0] / len(counts)
    occ = [np.mean(states[:, b]) / sites[b] for b in range(states.shape[1])]
    return np.concatenate([[d @ d, (rc * rc).sum(axis=1).mean()], occ, hist, [np.mean(counts ** 2)]])


def _setup():
    sys.path[:0] = [str(HERE), str(ROOT / "oracle" / "ref_stubs"), str(ROOT / "oracle" / "_ref"), str(ROOT)]
    import make_golden as mg  # noqa: E402  (the reference drivers of the golden cases)
    return mg


def build(cfg, mg):
    """The case's polymer, binders, field and controllers; a confined case
    starts from a seeded walk inside its sphere (unit steps redrawn while they
    would leave it) instead of the free Gaussian walk."""
    p, binders, marks, states0 = mg.build_case(cfg)
    if cfg.get("confine"):
        from chromo_gb300 import synthetic as syn
        from chromo.polymers import Chromatin
        rng = np.random.default_rng(cfg["seed"])
        r = syn.confined_walks(rng, 1, cfg["n"], 16.5, 0.95 * cfg["confine"][1])[0]
        t3, t2 = syn.tangents_from_coordinates(r)
        names = [b[0] for b in cfg["binders"]]
        p = Chromatin("p", r, bead_length=np.full(cfg["n"] - 1, 16.5), t3=t3, t2=t2, states=states0,
                      binder_names=np.array(names), chemical_mods=marks,
                      chemical_mod_names=np.array([f"m{i}" for i in range(len(names))]))
    field = mg.make_field(cfg, p, binders)
    ctrls = mg.make_controllers(cfg, p)
    return p, binders, field, ctrls, states0


def bead_counts(field):
    """Bead count per voxel: density times the voxel's accessible volume."""
    access = np.array([field.access_vols[i] for i in range(field.nx * field.ny * field.nz)])
    return np.asarray(field.density)[:, 0] * access


def one_run(args):
    name, k = args
    cfg = CASES[name]
    mg = _setup()
    from chromo.mc.mc_sim import mc_sim
    p, binders, field, ctrls, _ = build(cfg, mg)
    sites = [mg.cb.get_by_name(b[0]).sites_per_bead for b in cfg["binders"]]
    libc = ctypes.CDLL(None)
    libc.srand(7919 * (k + 1))
    seed = 100000 * (k + 1)
    mc_sim([p], binders, BURN, ctrls, field, 1.0, seed)
    obs = []
    for s in range(SAMPLES):
        mc_sim([p], binders, EVERY, ctrls, field, 1.0, seed + 1 + s)
        obs.append(observables(p.r, np.asarray(p.states), bead_counts(field), sites))
    return np.mean(obs, axis=0)


def main(name):
    cfg = CASES[name]
    out = HERE / "stats" / f"eq_{name}.npz"
    mg = _setup()
    p, binders, field, ctrls, states0 = build(cfg, mg)
    ctl0 = [(c.move.amp_move, c.move.amp_bead, c.move.num_per_cycle, 1,
             c.bead_amp_bounds[0], c.bead_amp_bounds[1], c.move_amp_bounds[0], c.move_amp_bounds[1])
            for c in ctrls]
    rows = field.binder_dict
    objs = [mg.cb.get_by_name(b[0]) for b in cfg["binders"]]
    names = [b[0] for b in cfg["binders"]]
    n_runs = cfg.get("runs", RUNS)
    with mp.get_context("spawn").Pool(min(n_runs, mp.cpu_count())) as pool:
        runs = np.array(pool.map(one_run, [(name, k) for k in range(n_runs)]))
    out.parent.mkdir(exist_ok=True)
    np.savez_compressed(
        out, obs_names=np.array(obs_names(names)), runs=runs, burn=BURN, samples=SAMPLES, every=EVERY,
        r0=np.asarray(p.r).copy(), t30=np.asarray(p.t3).copy(), t20=np.asarray(p.t2).copy(),
        states0=np.asarray(p.states).copy(), marks=np.asarray(p.chemical_mods).copy(),
        eps_bend=np.asarray(p.eps_bend), gamma=np.asarray(p.gamma), eps_par=np.asarray(p.eps_par),
        eps_perp=np.asarray(p.eps_perp), eta=np.asarray(p.eta),
        sites=np.array([o.sites_per_bead for o in objs]), e_mod=np.array([o.bind_energy_mod for o in objs]),
        e_nomod=np.array([o.bind_energy_no_mod for o in objs]),
        mu=np.array([o.chemical_potential for o in objs]),
        nxyz=np.array([field.nx, field.ny, field.nz]),
        widths=np.array([field.x_width, field.y_width, field.z_width]), chi=field.chi,
        vf_limit=field.vf_limit, bead_rad=5.0,
        pref=np.array([r["field_energy_prefactor"] for r in rows]),
        intra=np.array([r["interaction_energy_intranucleosome"] for r in rows]),
        xpref=np.array([[r["cross_talk_field_energy_prefactor"][o["name"]] for o in rows] for r in rows]),
        ctl0=np.array(ctl0, dtype=np.float64),
        confine_kind={"": 0, "Spherical": 1, "Cubical": 2}[field.confine_type],
        confine_length=float(field.confine_length),
        access_vol=np.array([field.access_vols[i] for i in range(field.nx * field.ny * field.nz)]),
        **({"eps_twist": np.asarray(p.eps_twist).copy(),
            "omega0": np.asarray(p.bead_length) * (2 * np.pi / 10.5) / 0.332} if cfg.get("lt") else {}))
    m, se = runs.mean(axis=0), runs.std(axis=0, ddof=1) / np.sqrt(n_runs)
    for nm, a, b_ in zip(obs_names(names), m, se):
        print(f"{nm:>20}: {a:.6g} +- {b_:.3g}")


if __name__ == "__main__":
    for nm in sys.argv[1:] or list(CASES):
        main(nm)
