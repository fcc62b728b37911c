"""Golden vectors for the steric clash energy, from the reference itself.

Run here (the container that mounts the reference), after
``python oracle/build_reference.py``::

    python tests/golden/make_sterics.py

Seeded chains of 60 and 400 beads (random walks of 9 nm steps, so that
beads come within the excluded distance) are built as the reference's
``DetailedChromatinWithSterics`` (chromo/polymers.pyx:2738-2938); its
``eval_E_steric_clashes`` gives the clash energy of the configuration, and
for seeded segment moves (rigid displacements and rotations of [ind0, indf))
``get_delta_distances`` + ``eval_delta_steric_clashes`` give each move's
clash-energy change from the same start.  Inputs and outputs are stored in
``tests/golden/sterics/vectors.npz``.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "oracle" / "ref_stubs"), str(ROOT / "oracle" / "_ref")]

import chromo.polymers as cp  # noqa: E402
from chromo.util.poly_paths import estimate_tangents_from_coordinates  # noqa: E402

OUT = Path(__file__).resolve().parent / "sterics" / "vectors.npz"


def chain(rng, n, step=9.0):
    d = rng.standard_normal((n - 1, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return np.vstack([np.zeros(3), np.cumsum(d * step, axis=0)])


def main():
    rng = np.random.default_rng(20261206)
    out = {}
    for c, n in enumerate((60, 400)):
        r = chain(rng, n)
        t3, t2 = estimate_tangents_from_coordinates(r)
        p = cp.DetailedChromatinWithSterics(
            "s", r, bp_wrap=147.0, bead_length=np.full(n - 1, 9.0), lp=53.0, lt=100.0, t3=t3, t2=t2,
            states=np.zeros((n, 1), dtype=int), binder_names=np.array(["HP1"]),
            chemical_mods=np.zeros((n, 1), dtype=int), chemical_mod_names=np.array(["m"]))
        out[f"r{c}"] = r
        out[f"excluded{c}"] = p.excluded_distance
        out[f"E{c}"] = p.eval_E_steric_clashes()
        moves, trials, dEs = [], [], []
        for k in range(40):
            ind0 = int(rng.integers(0, n - 1))
            indf = int(min(n, ind0 + rng.integers(1, 25)))
            seg = np.asarray(p.r)[ind0:indf].copy()
            if k % 2:
                seg = seg + rng.normal(scale=4.0, size=3)
            else:
                a = rng.normal(size=3)
                a /= np.linalg.norm(a)
                th = rng.uniform(-1.0, 1.0)
                K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
                R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
                c0 = seg[0]
                seg = (seg - c0) @ R.T + c0
            rt = np.asarray(p.r_trial)
            rt[ind0:indf] = seg
            p.get_delta_distances(ind0, indf)
            dEs.append(p.eval_delta_steric_clashes(ind0, indf))
            rt[ind0:indf] = np.asarray(p.r)[ind0:indf]
            p.get_delta_distances(ind0, indf)
            moves.append((ind0, indf))
            trials.append(np.vstack([seg, np.zeros((24 - len(seg), 3))]))
        out[f"moves{c}"] = np.array(moves, dtype=np.int64)
        out[f"trials{c}"] = np.array(trials)
        out[f"dE{c}"] = np.array(dEs)
        print(f"chain {c}: {n} beads, E = {out[f'E{c}']:.6g}, "
              f"{int(np.sum(np.abs(out[f'dE{c}']) > 0))} of 40 moves change the clash energy")
    OUT.parent.mkdir(exist_ok=True)
    np.savez_compressed(OUT, **out)


if __name__ == "__main__":
    main()
