"""Long runs reproduce the reference's equilibrium statistics.

The fixtures ``tests/golden/stats/eq_<case>.npz`` (written by
``tests/golden/make_equilibrium.py`` from the reference's own ``mc_sim``)
hold the per-run time averages of independent reference runs from one seeded
start: a 100-bead chain in a periodic 6^3-voxel box with one binder
(one_binder) or with two binders and cross talk (two_binders), or confined to
a 100 nm sphere in an 8^3-voxel box with the accessible volumes of the voxels
the sphere cuts (sphere_confined; bead counts per voxel are density times
accessible volume on both sides), or the one-binder system as a twistable
SSTWLC chain (twist; 64 reference runs, 256 replicas).  Here 64
replicas of the same start run on the GPU (FP32 storage, independent Philox
streams) for the same burn-in and sampling schedule -- all but the first at
the launch shape of the batched benchmark, 6 warps x 32 lanes per replica --
and every observable (squared end-to-end distance and radius of gyration,
each binder's occupancy, the histogram of bead counts per voxel and its
second moment) must agree with the reference's mean within 3 combined
standard errors (the per-run and per-replica time averages are independent
samples).  The Markov chains differ only in their random streams (libc
rand() against Philox), so this is the distributional check of the whole
move set, the field, cross talk and the controllers over ~1e8 moves.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
STATS = Path(__file__).resolve().parent / "golden" / "stats"
BINS = np.array([-np.inf, 0.05, 0.25, 0.5, 1.0, np.inf])
MOVE_NAMES = ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]


def observables(r, states, counts, sites):
    """The observables of one snapshot, as the fixture generator computes them."""
    d = r[-1] - r[0]
    rc = r - r.mean(axis=0)
    hist = np.histogram(counts, bins=BINS)[0] / len(counts)
    occ = [np.mean(states[:, b]) / sites[b] for b in range(states.shape[1])]
    return np.concatenate([[d @ d, (rc * rc).sum(axis=1).mean()], occ, hist, [np.mean(counts ** 2)]])


def _replicas(g, R, shape=(0, 0)):
    from chromo_gb300 import _native as nat
    from chromo_gb300.device import binding_params, bonds_array, field_params, move_ctl
    n = len(g["r0"])
    nb = len(g["sites"])
    ctl0 = g["ctl0"]
    max_seg = int(max(max(row[1], row[5]) for k, row in enumerate(ctl0) if k != 3)) + 2
    confined = "access_vol" in g and int(g["confine_kind"]) != 0
    sim = nat.Sim([n] * R, [list(g["nxyz"])] * R, nb, max_segment=max_seg,
                  max_tangent=int(max(ctl0[3][1], ctl0[3][5])), warps_per_block=shape[0],
                  lanes_per_move=shape[1], nonuniform_access=confined)
    bonds = bonds_array(g["eps_bend"], g["gamma"], g["eps_par"], g["eps_perp"], g["eta"])
    fp = field_params(field_kind=2, nxyz=g["nxyz"], widths=g["widths"], n_binders=nb,
                      chi=float(g["chi"]), vf_limit=float(g["vf_limit"]),
                      bead_vol=4.0 / 3.0 * np.pi * float(g["bead_rad"]) ** 3, pref=g["pref"],
                      intra=g["intra"], xpref=g["xpref"],
                      confine_kind=int(g["confine_kind"]) if confined else 0,
                      confine_length=float(g["confine_length"]) if confined else 0.0)
    bp = binding_params(sites=g["sites"], e_mod=g["e_mod"], e_nomod=g["e_nomod"], mu=g["mu"],
                        mu_adjust_factor=1.0)
    ctls = [move_ctl(MOVE_NAMES[k], amp_move=row[0], amp_bead=int(row[1]), num_per_cycle=int(row[2]),
                     simple=True, bead_bounds=(row[4], row[5]), move_bounds=(row[6], row[7]))
            for k, row in enumerate(ctl0)]
    for rep in range(R):
        sim.set_chain(rep, r=g["r0"], t3=g["t30"], t2=g["t20"], states=g["states0"], marks=g["marks"],
                      bonds=bonds)
        sim.set_field(rep, fp, access_vol=g["access_vol"] if confined else None)
        if "eps_twist" in g:  # SSTWLC
            sim.set_twist(rep, g["eps_twist"], g["omega0"])
        sim.set_binding(rep, bp)
        sim.set_controllers(rep, ctls)
    sim.deposit(-1)
    return sim


@pytest.mark.parametrize("case,shape", [("one_binder", (0, 0)), ("two_binders", (6, 32)),
                                        ("sphere_confined", (6, 32)), ("twist", (6, 32))])
def test_equilibrium_statistics_match_reference(case, shape):
    fixture = STATS / f"eq_{case}.npz"
    if not fixture.exists():
        pytest.skip("equilibrium fixture not generated")
    with np.load(fixture, allow_pickle=False) as z:
        g = {k: z[k] for k in z.files}
    # the twisted chain's extension scatters widely between runs: more replicas
    R, seed = (256 if case == "twist" else 64), 20261203
    sim = _replicas(g, R, shape)
    sites = [int(x) for x in g["sites"]]
    sim.run(int(g["burn"]), seed)
    acc = np.zeros((R, len(g["obs_names"])))
    for _ in range(int(g["samples"])):
        sim.run(int(g["every"]), seed)
        sim.sync()
        chains = sim.get_chains()
        for rep in range(R):
            counts = sim.density(rep)[:, 0] * 2.0 ** -40
            acc[rep] += observables(chains[rep][0], chains[rep][3], counts, sites)
    gpu = acc / int(g["samples"])
    ref = g["runs"]
    m_ref, se_ref = ref.mean(0), ref.std(0, ddof=1) / np.sqrt(len(ref))
    m_gpu, se_gpu = gpu.mean(0), gpu.std(0, ddof=1) / np.sqrt(R)
    z = (m_gpu - m_ref) / np.sqrt(se_ref ** 2 + se_gpu ** 2)
    report = "\n".join(f"{n:>14}: ref {a:.5g} +- {sa:.2g}  gpu {b:.5g} +- {sb:.2g}  z {zz:+.2f}"
                       for n, a, sa, b, sb, zz in zip(g["obs_names"], m_ref, se_ref, m_gpu, se_gpu, z))
    print(report)
    assert np.all(np.abs(z) <= 3.0), report
