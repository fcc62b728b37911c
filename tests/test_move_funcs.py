"""Calling the move functions directly (chromo/mc/move_funcs.pyx:39-820).

``chromo_gb300.mc.move_funcs`` proposals made on the host the reference's
way -- ``move(polymer, amp_move, amp_bead) -> inds``, trial arrays written in
place -- checked against:

* the reference's transform known answers (tests/golden/kat/geometry.npz,
  recorded by tests/golden/make_kat.py from the reference's
  return_arbitrary_axis_rotation / generate_translation_mat /
  transform_r_t3_t2, the cases of the reference's tests/test_moves.py and
  tests/test_linalg.py): within 1e-12 (Rodrigues' formula here, the
  reference's expanded one there);
* the reference's own trajectories: fed the rand() values and binding states
  the reference consumed in the golden cases, every move of the first MC
  step selects the same beads (a move that took a different number of draws
  would shift every later move's selection);
* the geometry of each move (rigid-body rotations and translations, unit
  tangents, states within range).
"""
from pathlib import Path

import numpy as np
import pytest

from golden_cases import CASES, MOVE_NAMES, load
from chromo_gb300.mc import move_funcs as mv
from chromo_gb300.util import linalg as la

FIX = Path(__file__).resolve().parent / "golden" / "kat" / "geometry.npz"


class _Poly:
    """The attributes a move function reads and writes."""

    def __init__(self, r, t3, t2, states, binder_names):
        self.r, self.t3, self.t2 = (np.array(a, dtype=float) for a in (r, t3, t2))
        self.states = np.array(states, dtype=np.int64)
        self.num_beads, self.num_binders = self.states.shape
        self.binder_names = np.asarray(binder_names)
        self.transformation_mat = np.identity(4)


@pytest.fixture(scope="module")
def kat():
    with np.load(FIX, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(autouse=True)
def _default_source():
    yield
    la.set_random_source()


def test_rotation_and_translation_matrices_match_reference(kat):
    for a, p, t, ref in zip(kat["axes"], kat["points"], kat["angles"], kat["rot"]):
        np.testing.assert_allclose(la.return_arbitrary_axis_rotation(a, p, t), ref, rtol=0, atol=1e-12)
    for d, ref in zip(kat["deltas"], kat["trans"]):
        p = _Poly(np.zeros((2, 3)), np.zeros((2, 3)), np.zeros((2, 3)), np.zeros((2, 1)), ["HP1"])
        la.generate_translation_mat(d, p)
        np.testing.assert_array_equal(p.transformation_mat, ref)


def test_transform_r_t3_t2_matches_reference(kat):
    mats = list(kat["rot"]) + list(kat["trans"])
    for j, M in enumerate(mats):
        p = _Poly(kat["r"], kat["t3"], kat["t2"], np.zeros((len(kat["r"]), 1)), ["HP1"])
        p.transformation_mat = M
        inds = kat["inds"]
        mv.transform_r_t3_t2(p, inds, len(inds))
        for name in ("r", "t3", "t2"):
            np.testing.assert_allclose(getattr(p, name + "_trial")[inds], kat[f"out_{name}"][j],
                                       rtol=0, atol=1e-12, err_msg=f"{name} {j}")


@pytest.mark.parametrize("name", CASES)
def test_first_step_selects_the_reference_beads(name):
    """Fed the reference's consumed draws, each move of the first MC step (all
    at the initial amplitudes; every step when the amplitudes are fixed) picks
    the reference's beads."""
    g = load(name)
    draws, bstates, pos = g["draws"].astype(np.int64), g["bstates"].astype(np.int64), [0, 0]

    def rand():
        pos[0] += 1
        return int(draws[pos[0] - 1])

    def state(n_tails):
        pos[1] += 1
        return int(bstates[pos[1] - 1])

    la.set_random_source(rand, state)
    names = [str(x) for x in g["binder_names"]] if "binder_names" in g else ["HP1"]
    p = _Poly(g["r0"], g["t30"], g["t20"], g["states0"], names)
    recs = g["records"]
    fixed = not np.any(g["ctl0"][:, 3])  # NoControl: every step at the initial amplitudes
    k = 0
    for ci, row in [(ci, row) for _ in range(int(g["n_steps"]) if fixed else 1)
                    for ci, row in enumerate(g["ctl0"])]:
        amp_move, amp_bead, npc = row[0], int(row[1]), int(row[2])
        for _ in range(npc):
            rec = recs[k]
            assert rec["kind"] == ci
            inds = getattr(mv, MOVE_NAMES[ci])(p, amp_move, amp_bead)
            assert len(inds) == rec["n_inds"], (k, len(inds), rec)
            if len(inds):
                assert inds[0] == rec["ind0"], (k, inds[:3], rec)
                if ci != 3:
                    assert inds[-1] + 1 == rec["indf"], (k, inds[-3:], rec)
            # the reference's Metropolis draw; a wrong draw count in any move
            # would shift every later move's draws and selections
            pos[0] += 1 if rec["accepted"] >= 0 else 0
            k += 1
    assert k >= min(100, len(recs))


def _chain(n=60, seed=4):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n - 1, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    r = np.vstack([np.zeros(3), np.cumsum(d * 16.5, axis=0)])
    from chromo_gb300.synthetic import tangents_from_coordinates
    t3, t2 = tangents_from_coordinates(r)
    return _Poly(r, t3, t2, rng.integers(0, 3, size=(n, 2)), ["HP1", "PRC1"])


def _pairwise(x):
    return np.linalg.norm(x[:, None, :] - x[None, :, :], axis=2)


@pytest.mark.parametrize("move", ["crank_shaft", "end_pivot"])
def test_rotations_are_rigid(move):
    la.srand(11)
    p = _chain()
    for _ in range(50):
        inds = getattr(mv, move)(p, 0.25 * np.pi, 20)
        assert np.all(np.diff(inds) == 1) and 1 <= len(inds) <= p.num_beads
        np.testing.assert_allclose(_pairwise(p.r_trial[inds]), _pairwise(p.r[inds]), atol=1e-9)
        np.testing.assert_allclose(np.linalg.norm(p.t3_trial[inds], axis=1), 1.0, atol=1e-12)
        np.testing.assert_allclose(np.sum(p.t3_trial[inds] * p.t2_trial[inds], axis=1),
                                   np.sum(p.t3[inds] * p.t2[inds], axis=1), atol=1e-12)
        R = p.transformation_mat[:3, :3]
        np.testing.assert_allclose(R @ R.T, np.identity(3), atol=1e-12)


def test_slide_translates_positions_only():
    la.srand(12)
    p = _chain()
    for _ in range(50):
        inds = mv.slide(p, 5.0, 20)
        shift = p.r_trial[inds] - p.r[inds]
        np.testing.assert_allclose(shift, np.broadcast_to(shift[0], shift.shape), atol=1e-12)
        assert np.linalg.norm(shift[0]) <= 5.0 + 1e-12
        np.testing.assert_array_equal(p.t3_trial[inds], p.t3[inds])


def test_tangent_rotation_keeps_positions_and_frames():
    la.srand(13)
    p = _chain()
    for _ in range(50):
        inds = mv.tangent_rotation(p, 0.2 * np.pi, 10)
        assert len(set(inds.tolist())) == len(inds) <= 10
        np.testing.assert_array_equal(p.r_trial[inds], p.r[inds])
        np.testing.assert_allclose(np.linalg.norm(p.t3_trial[inds], axis=1), 1.0, atol=1e-12)


def test_binding_move_draws_states_in_range():
    la.srand(14)
    np.random.seed(14)
    p = _chain()
    seen = set()
    for _ in range(100):
        p.states_trial = p.states.copy()
        inds = mv.change_binding_state(p, 0.0, 5)
        changed = np.nonzero(np.any(p.states_trial != p.states, axis=1))[0]
        assert set(changed.tolist()) <= set(inds.tolist())
        cols = np.nonzero(np.any(p.states_trial != p.states, axis=0))[0]
        assert len(cols) <= 1
        seen.update(p.states_trial[inds].ravel().tolist())
    assert seen == {0, 1, 2}
