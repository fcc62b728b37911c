"""The benchmark workloads, built straight into a resident ``Sim``.

Sizes follow the benchmark configurations of this path:

* ``small``   one chain of 1,000 beads in a 1,200 nm box, 30^3 grid of 40 nm
              voxels, one binder (mu = -0.4, eps = -4, chi = 1), marks with
              mean run length 20, FP64 positions; the five moves as
              ``specific_moves`` (one attempt of each kind per MC step,
              chromo/mc/mc_controller.py:374-421) under SimpleControl.
* ``plain``   one chain of 10,000 beads, 60^3 grid of 40 nm voxels, one binder
              (mu = -0.4, eps = -4, chi = 1), marks with mean run length 50.
* ``batched`` 256 chains with lengths log-uniform in [2,000, 20,000], each with
              its own 40^3 grid, two binders (eps_AA = -4, eps_BB = -3,
              eps_AB = +1 stored on A; mu_A, mu_B ~ U[-1, 0] per replica),
              chi ladder of 16 rungs in [0.5, 2.0] (16 ladders of 16 rungs).
* ``diff``    64 chains of 5,000 beads, 40^3 grids, binders as ``batched``
              (the batched + differentiation configuration; no exchange).
* ``profile`` 256 chains of 5,000 beads: the CTA shape of ``batched`` with
              fixed lengths, a bounded case for profilers.
* ``sphere``  256 chains of 5,000 beads, each confined to a sphere of radius
              700 nm inside its 40^3 grid (Spherical confinement, per-voxel
              accessible volumes at the surface), binders and chi ladder as
              ``batched``.
* ``large``   32 chains of 100,000 beads, 100^3 grids, chi ladder of 8 rungs
              times a sweep of 4 mu_A values (one grid of 4 x 8 parameter slots:
              chi exchanged along rows, mu_A along columns).

Chains are seeded Gaussian walks (16.5 nm spacing, lp = 53 nm) and every
replica runs all five moves under SimpleControl with the reference's
amplitude bounds and cycle counts (chromo/mc/__init__.py:295-332,
chromo/mc/mc_controller.py:216-266).
"""
import functools
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import _native as nat
from . import synthetic as syn
from .device import binding_params, bonds_array, field_params, move_ctl
from .energetics import dss_parameters, field_prefactors

BASE_SEED = 20261203
BEAD_SPACING = 16.5
LP = 53.0
BEAD_RAD = 5.0
VOXEL = 40.0
HP1_E_MOD, HP1_E_NOMOD, SITES, R_INT = -0.01, 1.52, 2, 3.0
NUM_PER_CYCLE = {"crank_shaft": 30, "end_pivot": 1, "slide": 60, "tangent_rotation": 60,
                 "change_binding_state": 10}


def amplitude_bounds(n_beads, min_spacing=BEAD_SPACING):
    """get_amplitude_bounds (chromo/mc/__init__.py:295-332)."""
    N = n_beads
    bead = {"crank_shaft": (min(30, N), min(150, N)), "slide": (min(10, N), min(150, N)),
            "end_pivot": (min(50, N / 4), min(150, int(N / 2))), "tangent_rotation": (1, N),
            "change_binding_state": (1, 1)}
    move = {"crank_shaft": (0.1 * np.pi, 0.25 * np.pi),
            "slide": (0.2 * min_spacing, 0.3 * min_spacing),
            "end_pivot": (0.2 * np.pi, 0.25 * np.pi),
            "tangent_rotation": (0.05 * np.pi, 0.2 * np.pi), "change_binding_state": (0, 0)}
    return bead, move


ONE_PER_CYCLE = {m: 1 for m in NUM_PER_CYCLE}  # specific_moves: num_per_cycle = 1


def all_moves_ctl(n_beads, cycle=None):
    """all_moves(..., SimpleControl) as device controllers (``cycle``: the
    attempts per controller cycle, NUM_PER_CYCLE by default; ONE_PER_CYCLE
    gives specific_moves(all five moves, ..., SimpleControl))."""
    cycle = cycle or NUM_PER_CYCLE
    bead, move = amplitude_bounds(n_beads)
    return [move_ctl(m, amp_move=move[m][0], amp_bead=int(bead[m][0]),
                     num_per_cycle=cycle[m], simple=True, bead_bounds=bead[m],
                     move_bounds=move[m]) for m in nat.MOVE_NAMES]


@dataclass
class Workload:
    name: str
    lengths: np.ndarray
    nbins: int
    n_binders: int
    mu: np.ndarray               # [R, nb]
    chi: np.ndarray              # [R]
    eps: List[float]
    cross: List[dict]
    run_length: int
    n_rungs: int
    seed: int
    steps_per_round: int = 62    # ~1e4 attempted moves per replica per exchange round
    mu_rungs: int = 0            # > 1: grids of mu_rungs x n_rungs, mu_A exchanged along mu rungs
    sphere_radius: float = 0.0   # > 0: Spherical confinement with accessible volumes
    cycle: dict = None           # attempts per controller cycle (None: NUM_PER_CYCLE)
    pos_fp64: bool = False       # FP64 positions (the CPU-runnable configuration)
    replicas: int = field(init=False)

    def __post_init__(self):
        self.replicas = len(self.lengths)

    @property
    def moves_per_step(self):
        return int(sum((self.cycle or NUM_PER_CYCLE).values()))


def make_workload(name: str, seed_offset: int = 0) -> Workload:
    if name == "plain":
        return Workload("plain", np.array([10000]), 60, 1, np.array([[-0.4]]), np.array([1.0]),
                        [-4.0], [{}], 50, 0, BASE_SEED + 1 + seed_offset)
    if name == "small":  # the CPU-runnable plain configuration
        return Workload("small", np.array([1000]), 30, 1, np.array([[-0.4]]), np.array([1.0]),
                        [-4.0], [{}], 20, 0, BASE_SEED + seed_offset, cycle=dict(ONE_PER_CYCLE),
                        pos_fp64=True)
    rng = np.random.default_rng(BASE_SEED + 2 + seed_offset)
    if name == "batched":
        R, rungs = 256, 16
        lengths = syn.log_uniform_lengths(rng, R, 2000, 20000)
        mu = rng.uniform(-1.0, 0.0, size=(R, 2))
        chi = np.tile(np.linspace(0.5, 2.0, rungs), R // rungs)
        return Workload("batched", lengths, 40, 2, mu, chi, [-4.0, -3.0], [{"PRC1": 1.0}, {}],
                        50, rungs, BASE_SEED + 2 + seed_offset)
    if name == "diff":  # batched + differentiation: 64 chains of 5,000 beads, no exchange
        R = 64
        mu = rng.uniform(-1.0, 0.0, size=(R, 2))
        chi = np.full(R, 1.0)
        return Workload("diff", np.full(R, 5000), 40, 2, mu, chi, [-4.0, -3.0],
                        [{"PRC1": 1.0}, {}], 50, 0, BASE_SEED + 3 + seed_offset)
    if name == "profile":  # fixed-length chains for profilers; the same CTA shape as "batched"
        R = 256
        mu = rng.uniform(-1.0, 0.0, size=(R, 2))
        chi = np.tile(np.linspace(0.5, 2.0, 16), R // 16)
        return Workload("profile", np.full(R, 5000), 40, 2, mu, chi, [-4.0, -3.0],
                        [{"PRC1": 1.0}, {}], 50, 16, BASE_SEED + 3 + seed_offset)
    if name == "sphere":
        R = 256
        mu = rng.uniform(-1.0, 0.0, size=(R, 2))
        chi = np.tile(np.linspace(0.5, 2.0, 16), R // 16)
        return Workload("sphere", np.full(R, 5000), 40, 2, mu, chi, [-4.0, -3.0],
                        [{"PRC1": 1.0}, {}], 50, 16, BASE_SEED + 5 + seed_offset,
                        sphere_radius=700.0)
    if name == "large":
        R, rungs = 32, 8
        mu_a = np.repeat([-1.0, -2.0 / 3.0, -1.0 / 3.0, 0.0], rungs)
        mu = np.stack([mu_a, rng.uniform(-1.0, 0.0, size=R)], axis=1)
        chi = np.tile(np.linspace(0.5, 2.0, rungs), R // rungs)
        return Workload("large", np.full(R, 100000), 100, 2, mu, chi, [-4.0, -3.0],
                        [{"PRC1": 1.0}, {}], 50, rungs, BASE_SEED + 4 + seed_offset, mu_rungs=4)
    raise ValueError(f"unknown workload {name}")


@dataclass
class ChainState:
    r: np.ndarray
    t3: np.ndarray
    t2: np.ndarray
    states: np.ndarray
    marks: np.ndarray


def make_chains(w: Workload) -> List[ChainState]:
    rng = np.random.default_rng(w.seed)
    out = []
    walks = None
    if w.sphere_radius > 0:  # equal lengths: all chains walked together
        walks = syn.confined_walks(rng, w.replicas, int(w.lengths[0]), BEAD_SPACING, w.sphere_radius)
    for j, n in enumerate(w.lengths):
        n = int(n)
        r = walks[j] if walks is not None else syn.gaussian_walk(rng, n, BEAD_SPACING)
        t3, t2 = syn.tangents_from_coordinates(r)
        marks = np.stack([syn.markov_marks(rng, n, w.run_length) for _ in range(w.n_binders)], 1)
        out.append(ChainState(r, t3, t2, np.zeros((n, w.n_binders), np.int64), marks))
    return out


@functools.lru_cache(maxsize=4)
def _sphere_volumes(nbins, radius):
    """Accessible volumes of a sphere of `radius` centred in an nbins^3 grid of
    VOXEL-sized voxels (computed once per grid; every replica shares them)."""
    from .fields import spherical_accessible_volumes
    width = nbins * VOXEL
    v = spherical_accessible_volumes(nbins, nbins, nbins, VOXEL, VOXEL, VOXEL, radius,
                                     width ** 3 / nbins ** 3)
    v.setflags(write=False)
    return v


def binder_names(nb):
    return ["HP1", "PRC1", "B3"][:nb]


def build_sim(w: Workload, chains=None, pos_fp64=None, warps_per_block=0, lanes_per_move=0) -> nat.Sim:
    chains = chains if chains is not None else make_chains(w)
    pos_fp64 = w.pos_fp64 if pos_fp64 is None else pos_fp64
    R, nb = w.replicas, w.n_binders
    confined = w.sphere_radius > 0
    sim = nat.Sim(w.lengths, [[w.nbins] * 3] * R, nb, pos_fp64=pos_fp64, max_segment=152,
                  max_tangent=int(max(w.lengths)), warps_per_block=warps_per_block,
                  lanes_per_move=lanes_per_move, nonuniform_access=confined)
    width = w.nbins * VOXEL
    access = _sphere_volumes(w.nbins, w.sphere_radius) if confined else None
    vint = 4.0 / 3.0 * np.pi * R_INT ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint] * nb, w.cross, binder_names(nb), VOXEL ** 3)
    bead_vol = 4.0 / 3.0 * np.pi * BEAD_RAD ** 3
    for rep in range(R):
        c = chains[rep]
        n = int(w.lengths[rep])
        _, eb, g, ep, epp, eta = dss_parameters(np.full(n - 1, BEAD_SPACING), LP)
        sim.set_chain(rep, r=c.r, t3=c.t3, t2=c.t2, states=c.states, marks=c.marks,
                      bonds=bonds_array(eb, g, ep, epp, eta))
        sim.set_field(rep, field_params(field_kind=2, nxyz=(w.nbins,) * 3, widths=(width,) * 3,
                                        n_binders=nb, chi=float(w.chi[rep]), vf_limit=0.5,
                                        bead_vol=bead_vol, pref=pref, intra=intra, xpref=xpref,
                                        confine_kind=1 if confined else 0,
                                        confine_length=w.sphere_radius),
                      access_vol=access)
        sim.set_binding(rep, binding_params(sites=[SITES] * nb, e_mod=[HP1_E_MOD] * nb,
                                            e_nomod=[HP1_E_NOMOD] * nb, mu=list(w.mu[rep]),
                                            mu_adjust_factor=1.0))
        sim.set_controllers(rep, all_moves_ctl(n, w.cycle))
    sim.deposit(-1)
    return sim


def algorithmic_bytes(tally: np.ndarray, n_binders: int, pos_bytes: int = 12) -> float:
    """Bytes a move must move at minimum, summed over a tally [R, 5, 6].

    Per attempted move of m beads touching U voxels:
      m * (pos_bytes * k_pos + n_bind)   read the moved beads' vectors and states
      + 2 * 2 * pos_bytes + 2 * 20       the two boundary neighbours' r, t3 and two
                                         bonds' five parameters (per rotated bead
                                         for tangent_rotation)
      + U * (1 + nb) * 8                 read the touched voxels (binder columns
                                         only, U * nb * 8, for binding moves; none
                                         for tangent_rotation)
      + accepted: write back m * pos_bytes * k_pos and the touched voxels.
    k_pos = 3 (crank_shaft, end_pivot: r, t3, t2), 1 (slide: r), 2 (tangent:
    t3, t2), 0 (binding; marks are read too).
    """
    t = tally.reshape(-1, 5, 6).sum(0).astype(np.float64)
    nb = n_binders
    kpos = [3, 3, 1, 2, 0]
    total = 0.0
    for k in range(5):
        att, acc, m, U, m_acc, U_acc = t[k]
        n_bind = nb * (2 if k == 4 else 1)
        b = m * (pos_bytes * kpos[k] + n_bind)
        if k == 3:
            b += m * (2 * 2 * pos_bytes + 2 * 20)
            vox_cols = 0
        else:
            b += att * (2 * 2 * pos_bytes + 2 * 20) if k != 4 else 0
            vox_cols = nb if k == 4 else 1 + nb
        b += U * vox_cols * 8
        b += m_acc * pos_bytes * kpos[k] + U_acc * vox_cols * 8
        if k == 4:
            b += m_acc * nb
        total += b
    return total


def move_stats(tally: np.ndarray) -> dict:
    """Per move kind, from a tally [R, 5, 6]: the share of the attempted
    moves, the acceptance rate, and the mean beads and touched voxels of an
    attempted move."""
    t = tally.reshape(-1, 5, 6).sum(0).astype(np.float64)
    total = max(1.0, float(t[:, 0].sum()))
    out = {}
    for k, name in enumerate(nat.MOVE_NAMES):
        att = max(1.0, t[k, 0])
        out[name] = {"share": round(t[k, 0] / total, 4), "acceptance": round(t[k, 1] / att, 4),
                     "mean_beads": round(t[k, 2] / att, 2), "mean_voxels": round(t[k, 3] / att, 2)}
    return out
