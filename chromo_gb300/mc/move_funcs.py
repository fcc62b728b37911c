"""The five MC moves (chromo/mc/move_funcs.pyx:39-820).

Each move is an object that names a move kind for ``MCAdapter`` and the
controllers (``kind`` is the kernel's move code; ``__name__`` the reference
function name) and that can also be called the reference's way,
``move(polymer, amp_move, amp_bead) -> inds``: it draws a proposal from libc
``rand()`` (binding states from numpy's global generator), stores the
polymer's ``transformation_mat``, ``last_amp_move`` and ``last_amp_bead``,
writes the proposal into the polymer's ``r_trial`` / ``t3_trial`` /
``t2_trial`` (or ``states_trial``) and returns the moved beads' indices.

That direct call is a host-side utility on the polymer's host arrays.  The
MC loop (``chromo_gb300.mc.mc_sim``) never calls it: the GPU kernel draws
and applies the same five proposals itself, on its own random streams.
"""
import numpy as np

from ..util import bead_selection as beads
from ..util import linalg as la
from ..util.linalg import RAND_MAX, rand


def _trial_arrays(polymer):
    for name in ("r", "t3", "t2", "states"):
        cur = np.asarray(getattr(polymer, name))
        trial = getattr(polymer, name + "_trial", None)
        if trial is None or np.shape(trial) != cur.shape:
            setattr(polymer, name + "_trial", cur.copy())


def transform_r_t3_t2(polymer, inds, n_inds):
    """Apply ``polymer.transformation_mat`` to the beads `inds` (the first
    `n_inds`): r' = R r + T, t' = R t, written to the trial arrays
    (move_funcs.pyx:121-154)."""
    _trial_arrays(polymer)
    m = np.asarray(polymer.transformation_mat, dtype=float)
    idx = np.asarray(inds, dtype=np.int64)[:int(n_inds)]
    R, T = m[:3, :3], m[:3, 3]
    polymer.r_trial[idx] = np.asarray(polymer.r)[idx] @ R.T + T
    polymer.t3_trial[idx] = np.asarray(polymer.t3)[idx] @ R.T
    polymer.t2_trial[idx] = np.asarray(polymer.t2)[idx] @ R.T


def _random_angle(amp_move):
    return amp_move * (rand() / RAND_MAX - 0.5)


def _crank_axis_and_fulcrum(r, ind0, indf, n):
    """Rotation axis (unit, or a random direction when the two axis beads
    nearly coincide) and fulcrum of a crank-shaft move on beads [ind0, indf)
    (move_funcs.pyx:157-280): the axis joins the beads just outside the
    segment, or the segment's own end beads where it reaches a chain end."""
    if indf - 1 == ind0 == 0:
        a, b = indf, ind0
    elif indf - 1 == ind0 == n - 1:
        a, b = ind0, ind0 - 1
    elif ind0 == 0 and indf == n:
        a, b = indf - 1, ind0
    elif ind0 == 0:
        a, b = indf, ind0
    elif indf == n:
        a, b = indf - 1, ind0 - 1
    else:
        a, b = indf, ind0 - 1
    d = r[a] - r[b]
    mag = np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2)
    axis = la.uniform_sample_unit_sphere() if mag < 1e-5 else d * (1.0 / mag)
    if ind0 == 0 and indf != n:
        pivot = indf
    elif ind0 != 0 and indf == n:
        pivot = ind0 - 1
    elif ind0 == 0 and indf == n:
        pivot = ind0
    else:
        pivot = ind0 - 1
    return axis, r[pivot].copy()


class MoveFunction:
    """One move kind; calling it proposes a move on a polymer's host arrays."""

    def __init__(self, name, kind, propose):
        self.__name__ = name
        self.kind = kind
        self._propose = propose

    def __call__(self, polymer, amp_move, amp_bead):
        _trial_arrays(polymer)
        return self._propose(polymer, float(amp_move), int(amp_bead))

    def __repr__(self):
        return f"<move {self.__name__}>"


def _crank_shaft(polymer, amp_move, amp_bead):
    """Rotate a segment about the axis through its outer neighbours
    (move_funcs.pyx:39-101)."""
    n = polymer.num_beads
    ang = _random_angle(amp_move)
    b0 = int(rand() / RAND_MAX * n)
    b1 = max(beads.from_point(amp_bead, n, b0), 1)
    ind0, indf = beads.check_bead_bounds(b0, b1, n)
    inds = np.arange(ind0, indf)
    polymer.last_amp_bead, polymer.last_amp_move = len(inds), ang
    axis, fulcrum = _crank_axis_and_fulcrum(np.asarray(polymer.r), ind0, indf, n)
    la.arbitrary_axis_rotation(axis, fulcrum, ang, polymer)
    transform_r_t3_t2(polymer, inds, len(inds))
    return inds


def _end_pivot(polymer, amp_move, amp_bead):
    """Rotate one end of the chain about a random axis through the bead next
    to it (move_funcs.pyx:285-398)."""
    n = polymer.num_beads
    ang = _random_angle(amp_move)
    left = rand() % 2 == 1
    if left:
        ind0, indf = 0, beads.from_left(amp_bead, n) + 1
    else:
        ind0, indf = beads.from_right(amp_bead, n), n
    inds = np.arange(ind0, indf)
    axis = la.uniform_sample_unit_sphere()
    polymer.last_amp_bead, polymer.last_amp_move = len(inds), ang
    if ind0 == 0 and indf != n:
        pivot = indf
    elif ind0 != 0 and indf == n:
        pivot = ind0 - 1
    elif ind0 == 0 and indf == n and left:
        pivot = indf - 1
    else:
        pivot = ind0
    la.arbitrary_axis_rotation(axis, np.asarray(polymer.r)[pivot].copy(), ang, polymer)
    transform_r_t3_t2(polymer, inds, len(inds))
    return inds


def _slide(polymer, amp_move, amp_bead):
    """Translate a segment by a random vector of length up to amp_move
    (move_funcs.pyx:403-465); tangents unchanged."""
    n = polymer.num_beads
    amp = amp_move * (rand() / RAND_MAX)
    delta = la.uniform_sample_unit_sphere() * amp
    la.generate_translation_mat(delta, polymer)
    b0 = rand() % n
    ind0, indf = beads.check_bead_bounds(b0, beads.from_point(amp_bead, n, b0), n)
    inds = np.arange(ind0, indf)
    polymer.last_amp_bead, polymer.last_amp_move = len(inds), amp
    polymer.r_trial[inds] = np.asarray(polymer.r)[inds] + delta
    polymer.t3_trial[inds] = np.asarray(polymer.t3)[inds]
    polymer.t2_trial[inds] = np.asarray(polymer.t2)[inds]
    return inds


def _tangent_rotation(polymer, amp_move, amp_bead):
    """Rotate the tangents of rand() % amp_bead + 1 distinct random beads, each
    about its own random axis by one common angle (move_funcs.pyx:470-582)."""
    n = polymer.num_beads
    ang = _random_angle(amp_move)
    k = rand() % amp_bead + 1
    picked, inds = set(), []
    while len(inds) < k:
        i = rand() % n
        if i not in picked:
            picked.add(i)
            inds.append(i)
    inds = np.array(inds, dtype=np.int64)
    polymer.last_amp_bead, polymer.last_amp_move = k, ang
    for i in inds:
        m = la.rotation_about_axis(la.uniform_sample_unit_sphere(), np.zeros(3), ang)
        R = m[:3, :3]
        polymer.r_trial[i] = np.asarray(polymer.r)[i]
        polymer.t3_trial[i] = R @ np.asarray(polymer.t3)[i]
        polymer.t2_trial[i] = R @ np.asarray(polymer.t2)[i]
    return inds


def _change_binding_state(polymer, amp_move, amp_bead):
    """Give a random binder's state on a segment new values, each drawn
    uniformly from 0..sites_per_bead (move_funcs.pyx:717-820)."""
    from .. import binders as cb
    n = polymer.num_beads
    b = rand() % polymer.num_binders
    sites = cb.get_by_name(str(polymer.binder_names[b])).sites_per_bead
    b0 = rand() % n
    ind0, indf = beads.check_bead_bounds(b0, beads.from_point(amp_bead, n, b0), n)
    inds = np.arange(ind0, indf)
    polymer.last_amp_bead, polymer.last_amp_move = len(inds), float(sites)
    for i in inds:
        polymer.states_trial[i, b] = la.new_state(sites)
    return inds


crank_shaft = MoveFunction("crank_shaft", 0, _crank_shaft)
end_pivot = MoveFunction("end_pivot", 1, _end_pivot)
slide = MoveFunction("slide", 2, _slide)
tangent_rotation = MoveFunction("tangent_rotation", 3, _tangent_rotation)
change_binding_state = MoveFunction("change_binding_state", 4, _change_binding_state)
move_list = [crank_shaft, end_pivot, slide, tangent_rotation, change_binding_state]
