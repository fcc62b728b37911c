"""Known-answer vectors for the move geometry, from the reference's own functions.

Run here (the container that mounts the reference), after
``python oracle/build_reference.py``::

    python tests/golden/make_kat.py

The reference's tests check its rotation and translation matrices and the
bead transform of each move type (tests/test_linalg.py:12-65,
tests/test_moves.py:16-282) on hand-made cases.  This script runs the same
reference functions -- ``return_arbitrary_axis_rotation`` and
``generate_translation_mat`` (chromo/util/linalg.pyx:62-200) and
``transform_r_t3_t2`` (chromo/mc/move_funcs.pyx:121-154) -- on the kinds of
case those tests use (quarter and eighth turns about coordinate axes through
the origin) and on seeded general ones, and stores inputs and outputs in
``tests/golden/kat/geometry.npz``.  ``tests/golden/kat/deposit.npz`` holds
the reference field's densities of bead pairs placed on voxel and box faces,
at corners and outside the box (the periodic wrap its tests/test_fields.py:
62-96 checks through neighbour indexing).
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "oracle" / "ref_stubs"), str(ROOT / "oracle" / "_ref")]

import chromo.binders as cb  # noqa: E402
import chromo.mc.move_funcs as mv  # noqa: E402
from chromo.fields import UniformDensityField  # noqa: E402
import chromo.polymers as poly  # noqa: E402
import chromo.util.linalg as la  # noqa: E402

OUT = Path(__file__).resolve().parent / "kat"


def main():
    rng = np.random.default_rng(20261205)
    axes = [np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0])]
    points = [np.zeros(3)] * 3
    angles = [np.pi / 4, -np.pi / 2, np.pi / 2]
    for _ in range(6):
        a = rng.standard_normal(3)
        axes.append(a / np.linalg.norm(a))
        points.append(rng.uniform(-50.0, 50.0, 3))
        angles.append(rng.uniform(-np.pi, np.pi))
    rot = np.stack([la.return_arbitrary_axis_rotation(a, p, t) for a, p, t in zip(axes, points, angles)])

    deltas = rng.uniform(-5.0, 5.0, (3, 3))
    trans = []
    for d in deltas:
        obj = poly.TransformedObject()
        la.generate_translation_mat(np.ascontiguousarray(d), obj)
        trans.append(np.asarray(obj.transformation_mat).copy())

    n = 10
    r = np.cumsum(rng.standard_normal((n, 3)) * 10.0, axis=0)
    t3 = rng.standard_normal((n, 3))
    t3 /= np.linalg.norm(t3, axis=1)[:, None]
    t2 = np.cross(t3, np.array([1.0, 0.0, 0.0]))
    t2 /= np.linalg.norm(t2, axis=1)[:, None]
    inds = np.arange(2, 8)
    mats = list(rot) + trans
    out_r, out_t3, out_t2 = [], [], []
    for M in mats:
        p = poly.Chromatin("kat", r.copy(), bead_length=np.full(n - 1, 16.5), t3=t3.copy(), t2=t2.copy())
        p.transformation_mat = np.ascontiguousarray(M)
        mv.transform_r_t3_t2(p, inds, len(inds))
        out_r.append(np.asarray(p.r_trial)[inds].copy())
        out_t3.append(np.asarray(p.t3_trial)[inds].copy())
        out_t2.append(np.asarray(p.t2_trial)[inds].copy())
    # periodic trilinear deposition (the wrap the reference's
    # tests/test_fields.py:62-96 checks through neighbour indexing): pairs of
    # beads at the centre, on voxel and box faces, at corners and outside the
    # box, in a 5^3 grid of 40 nm voxels
    pairs = np.array([
        [[0.0, 0.0, 0.0], [-100.0, -100.0, -100.0]],
        [[99.9, 99.9, 99.9], [-120.0, 0.0, 0.0]],
        [[250.0, -300.0, 42.0], [-80.0, 80.0, -80.0]],
        [[-20.0, 0.0, 20.0], [60.0, -60.0, 100.0]],
        [[-100.0, 100.0, 0.0], [1e-9, -1e-9, 39.999]]])
    binders = cb.make_binder_collection([cb.get_by_name("HP1")])
    dens = []
    for k, pair in enumerate(pairs):
        states = np.array([[1], [2]]) if k % 2 else np.array([[2], [0]])
        pp = poly.Chromatin("dep", pair.copy(), bead_length=np.array([16.5]), states=states,
                            binder_names=np.array(["HP1"]), chemical_mods=np.zeros((2, 1), int),
                            chemical_mod_names=np.array(["H3K9me3"]))
        f = UniformDensityField([pp], binders, 200.0, 5, 200.0, 5, 200.0, 5)
        dens.append(np.asarray(f.density).copy())
    OUT.mkdir(exist_ok=True)
    np.savez_compressed(OUT / "deposit.npz", pairs=pairs, density=np.stack(dens))
    np.savez_compressed(OUT / "geometry.npz", axes=np.stack(axes), points=np.stack(points),
                        angles=np.array(angles), rot=rot, deltas=deltas, trans=np.stack(trans),
                        r=r, t3=t3, t2=t2, inds=inds, out_r=np.stack(out_r),
                        out_t3=np.stack(out_t3), out_t2=np.stack(out_t2))
    print("wrote", OUT / "geometry.npz")


if __name__ == "__main__":
    main()
