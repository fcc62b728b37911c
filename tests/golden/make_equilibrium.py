"""Equilibrium statistics of the reference's own ``mc_sim``, for the long-run
statistical check of the GPU path (tests/test_gpu_equilibrium.py).

Run here (the container that mounts the reference), after
``python oracle/build_reference.py``::

    python tests/golden/make_equilibrium.py

One small system -- a 100-bead Chromatin chain (16.5 nm spacing, lp 53 nm)
with one binder (HP1 preset, mu = -0.4, eps = -4) in a periodic 240 nm box of
6^3 voxels, chi = 1, all five moves under SimpleControl -- is run RUNS times
from the same seeded start with independent random streams (libc ``srand``
and numpy seeds per run; ``mc_sim`` reseeds numpy on every call, so every call
gets its own seed).  After BURN MC steps, SAMPLES snapshots are taken every
EVERY steps and the per-run time averages of these observables are stored:

* R2: squared end-to-end distance (unwrapped positions), nm^2;
* Rg2: squared radius of gyration, nm^2;
* occupancy: mean binding state / sites per bead;
* five fractions of voxels whose bead count (density times voxel volume) is
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
OUT = HERE / "stats" / "eq_one_binder.npz"

CFG = dict(n=100, nbins=6, vox=40.0, binders=[("HP1", -0.4, -4.0, {})], chi=1.0, moves="all",
           seed=21, run=20)
RUNS, BURN, SAMPLES, EVERY = 16, 1500, 300, 20
BINS = np.array([-np.inf, 0.05, 0.25, 0.5, 1.0, np.inf])
OBS = ["R2", "Rg2", "occupancy", "vox_0_0.05", "vox_0.05_0.25", "vox_0.25_0.5", "vox_0.5_1",
       "vox_1_inf", "count2"]


def observables(r, states, counts, sites):
    """The observables of one snapshot (shared with the GPU test)."""
    r = np.asarray(r, dtype=np.float64)
    d = r[-1] - r[0]
    rc = r - r.mean(axis=0)
    hist = np.histogram(counts, bins=BINS)[0] / len(counts)
    return np.concatenate([[d @ d, (rc * rc).sum(axis=1).mean(), np.mean(states[:, 0]) / sites],
                           hist, [np.mean(counts ** 2)]])


def _setup():
    sys.path[:0] = [str(HERE), str(ROOT / "oracle" / "ref_stubs"), str(ROOT / "oracle" / "_ref")]
    import make_golden as mg  # noqa: E402  (the reference drivers of the golden cases)
    return mg


def one_run(k):
    mg = _setup()
    from chromo.mc.mc_sim import mc_sim
    p, binders, marks, _ = mg.build_case(CFG)
    field = mg.make_field(CFG, p, binders)
    ctrls = mg.make_controllers(CFG, p)
    libc = ctypes.CDLL(None)
    libc.srand(7919 * (k + 1))
    seed = 100000 * (k + 1)
    mc_sim([p], binders, BURN, ctrls, field, 1.0, seed)
    vol = field.x_width * field.y_width * field.z_width / (field.nx * field.ny * field.nz)
    obs = []
    for s in range(SAMPLES):
        mc_sim([p], binders, EVERY, ctrls, field, 1.0, seed + 1 + s)
        counts = np.asarray(field.density)[:, 0] * vol
        obs.append(observables(p.r, np.asarray(p.states), counts, 2))
    return np.mean(obs, axis=0)


def main():
    mg = _setup()
    p, binders, marks, states0 = mg.build_case(CFG)
    field = mg.make_field(CFG, p, binders)
    ctrls = mg.make_controllers(CFG, p)
    ctl0 = [(c.move.amp_move, c.move.amp_bead, c.move.num_per_cycle, 1,
             c.bead_amp_bounds[0], c.bead_amp_bounds[1], c.move_amp_bounds[0], c.move_amp_bounds[1])
            for c in ctrls]
    row = field.binder_dict[0]
    hp1 = mg.cb.get_by_name("HP1")
    with mp.get_context("spawn").Pool(min(RUNS, mp.cpu_count())) as pool:
        runs = np.array(pool.map(one_run, range(RUNS)))
    OUT.parent.mkdir(exist_ok=True)
    np.savez_compressed(
        OUT, obs_names=np.array(OBS), runs=runs, burn=BURN, samples=SAMPLES, every=EVERY,
        r0=np.asarray(p.r).copy(), t30=np.asarray(p.t3).copy(), t20=np.asarray(p.t2).copy(),
        states0=np.asarray(p.states).copy(), marks=np.asarray(p.chemical_mods).copy(),
        eps_bend=np.asarray(p.eps_bend), gamma=np.asarray(p.gamma), eps_par=np.asarray(p.eps_par),
        eps_perp=np.asarray(p.eps_perp), eta=np.asarray(p.eta),
        sites=np.array([hp1.sites_per_bead]), e_mod=np.array([hp1.bind_energy_mod]),
        e_nomod=np.array([hp1.bind_energy_no_mod]), mu=np.array([hp1.chemical_potential]),
        nxyz=np.array([field.nx, field.ny, field.nz]),
        widths=np.array([field.x_width, field.y_width, field.z_width]), chi=field.chi,
        vf_limit=field.vf_limit, bead_rad=5.0,
        pref=np.array([row["field_energy_prefactor"]]),
        intra=np.array([row["interaction_energy_intranucleosome"]]),
        xpref=np.array([[row["cross_talk_field_energy_prefactor"][row["name"]]]]),
        ctl0=np.array(ctl0, dtype=np.float64))
    m, se = runs.mean(axis=0), runs.std(axis=0, ddof=1) / np.sqrt(RUNS)
    for name, a, b_ in zip(OBS, m, se):
        print(f"{name:>14}: {a:.6g} +- {b_:.3g}")


if __name__ == "__main__":
    main()
