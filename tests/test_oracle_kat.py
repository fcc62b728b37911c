"""The oracle's move geometry against the reference's own functions.

``tests/golden/make_kat.py`` recorded the reference's rotation matrices
(``return_arbitrary_axis_rotation``), translation matrices
(``generate_translation_mat``) and bead transforms (``transform_r_t3_t2``)
on quarter and eighth turns about coordinate axes -- the cases of the
reference's tests/test_linalg.py and tests/test_moves.py -- and on seeded
general rotations.  The oracle's restatements must give the same bits, and
the axis-aligned cases must also have the analytic values those tests check.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc

FIX = Path(__file__).resolve().parent / "golden" / "kat" / "geometry.npz"


@pytest.fixture(scope="module")
def g():
    with np.load(FIX, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def test_rotation_matrices_match_reference(g):
    for a, p, t, ref in zip(g["axes"], g["points"], g["angles"], g["rot"]):
        M = orc.axis_rotation(a, p, t)
        np.testing.assert_array_equal(M, ref[:3, :])
        np.testing.assert_array_equal(ref[3], [0.0, 0.0, 0.0, 1.0])


def test_axis_aligned_rotations_are_the_analytic_ones(g):
    c45 = np.cos(np.pi / 4)
    expect = [np.array([[c45, -c45, 0, 0], [c45, c45, 0, 0], [0, 0, 1, 0]]),    # 45 deg about z
              np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, -1, 0, 0]]),          # -90 deg about x
              np.array([[0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]])]          # 90 deg about y
    for j, e in enumerate(expect):
        np.testing.assert_allclose(orc.axis_rotation(g["axes"][j], g["points"][j], g["angles"][j]), e,
                                   atol=1e-15)


def _system(g):
    n = len(g["r"])
    z = np.zeros(n - 1)
    return orc.OracleSystem(
        r=g["r"], t3=g["t3"], t2=g["t2"], states=np.zeros((n, 1), np.int64),
        marks=np.zeros((n, 1), np.int64), eps_bend=z, gamma=z, eps_par=z, eps_perp=z, eta=z,
        sites=np.array([2]), e_mod=np.array([0.0]), e_nomod=np.array([0.0]), mu=np.array([0.0]),
        mu_adjust_factor=1.0, max_binders=-1, field_kind=0, confine_kind=0, confine_length=0.0,
        nxyz=(1, 1, 1), widths=(1.0, 1.0, 1.0), access_vol=None, chi=0.0, vf_limit=0.5,
        bead_vol=1.0, pref=np.zeros(1), intra=np.zeros(1), xpref=np.zeros(1), pos="f64",
        fixed_density=0)


def test_bead_transforms_match_reference(g):
    s = _system(g)
    mats = list(g["rot"]) + list(g["trans"])
    for j, M in enumerate(mats):
        for k, i in enumerate(g["inds"]):
            r, t3, t2 = s.transform(i, M[:3, :])
            np.testing.assert_array_equal(r, g["out_r"][j][k])
            np.testing.assert_array_equal(t3, g["out_t3"][j][k])
            np.testing.assert_array_equal(t2, g["out_t2"][j][k])


def test_translations_move_positions_only(g):
    s = _system(g)
    for d, T in zip(g["deltas"], g["trans"]):
        np.testing.assert_array_equal(T[:3, :3], np.eye(3))
        np.testing.assert_array_equal(T[:3, 3], d)
        r, t3, t2 = s.transform(g["inds"][0], T[:3, :])
        np.testing.assert_allclose(r, g["r"][g["inds"][0]] + d, rtol=0, atol=1e-12)
        np.testing.assert_array_equal(t3, g["t3"][g["inds"][0]])
        np.testing.assert_array_equal(t2, g["t2"][g["inds"][0]])


def test_periodic_deposition_matches_reference():
    """Trilinear deposition with periodic wrap: bead pairs at the centre, on
    voxel and box faces, at corners and outside the box, in a 5^3 grid of
    40 nm voxels; the oracle's FP64 density equals the reference field's."""
    with np.load(FIX.parent / "deposit.npz", allow_pickle=False) as z:
        pairs, dens = z["pairs"], z["density"]
    for k, (pair, ref) in enumerate(zip(pairs, dens)):
        states = np.array([[1], [2]]) if k % 2 else np.array([[2], [0]])
        s = orc.OracleSystem(
            r=pair, t3=np.tile([1.0, 0.0, 0.0], (2, 1)), t2=np.tile([0.0, 1.0, 0.0], (2, 1)),
            states=states, marks=np.zeros((2, 1), np.int64), eps_bend=np.zeros(1),
            gamma=np.zeros(1), eps_par=np.zeros(1), eps_perp=np.zeros(1), eta=np.zeros(1),
            sites=np.array([2]), e_mod=np.array([0.0]), e_nomod=np.array([0.0]),
            mu=np.array([0.0]), mu_adjust_factor=1.0, max_binders=-1, field_kind=2,
            confine_kind=0, confine_length=0.0, nxyz=(5, 5, 5), widths=(200.0, 200.0, 200.0),
            access_vol=None, chi=1.0, vf_limit=0.5, bead_vol=4.0 / 3.0 * np.pi * 125.0,
            pref=np.zeros(1), intra=np.zeros(1), xpref=np.zeros(1), pos="f64", fixed_density=0)
        s.deposit_all()
        np.testing.assert_array_equal(s.density, ref, err_msg=f"pair {k}")
