"""Coarse-graining and refinement of a chromatin fiber (chromo/util/rediscretize.py).

The reference's two-step workflow: equilibrate a coarse chain, each of whose
beads stands for ``cg_factor`` beads of the fine chain (placed at its
segment's centroid, pulled towards the origin by cg_factor^(1/3), in a field
shrunk by the same factor), then rebuild the fine chain from it (free walks
off the two ends, Brownian bridges between consecutive coarse beads, the same
for the orientations), grow the field back and re-equilibrate the binding
states with binding moves.

Design.  Segments are handled as arrays: a segment table (start, stop) drives
every per-segment reduction, and the majority states come from one count
matrix per column.  Two steps stay sequential because floating point makes
their order part of the result: the Brownian-bridge recurrence, and the
confinement kernels, which are applied one violating bead after the other
(their windows overlap).  Random numbers come from numpy's global generator
in the reference's order -- one block of normals per bridge or walk, one
``choice`` per coarse bead and column -- so a seeded call returns the
reference's arrays bit for bit (checked against vectors the reference
produced).  The deprecated ``*_old`` variants of the reference are not
restated.  The binding re-equilibration of ``refine_chromatin`` runs
through this package's ``mc_sim`` (binding moves on the GPU, Philox streams
keyed by ``random_seed``) where the reference calls ``mc_step`` with libc
``rand()``.
"""
import warnings
from typing import Dict, List, Optional, Tuple

import numpy as np

from ..fields import UniformDensityField
from ..polymers import Chromatin, gaussian_walk

_EX = np.array([1.0, 0.0, 0.0])
_EY = np.array([0.0, 1.0, 0.0])
_FIELD_KEYS = ("nx", "ny", "nz", "x_width", "y_width", "z_width", "confine_type", "confine_length",
               "chi", "assume_fully_accessible", "vf_limit", "fast_field", "n_points")


# ------------------------------------------------------------------ segments

def get_cg_bead_intervals(num_beads: int, cg_factor: float) -> Dict[int, Tuple[int, int]]:
    """Bead range [lo, hi) of the fine chain behind each coarse bead
    (chromo/util/rediscretize.py:24-54): full segments of ``cg_factor`` beads,
    then the remainder, whose range reaches one bead past the chain's end (as
    in the reference; slicing clips it)."""
    n_full = int(np.floor(num_beads / cg_factor))
    table = {i: (i * cg_factor, (i + 1) * cg_factor) for i in range(n_full)}
    rest = num_beads - n_full * cg_factor
    if rest > 0:
        lo = n_full * cg_factor
        table[n_full] = (lo, lo + rest + 1)
    return table


def _segments(intervals: Dict[int, Tuple[int, int]]) -> List[slice]:
    return [slice(int(intervals[i][0]), int(intervals[i][1])) for i in range(len(intervals))]


def get_avg_in_intervals(r: np.ndarray, intervals: Dict[int, Tuple[int, int]]) -> np.ndarray:
    """Centroid of the rows of each segment (chromo/util/rediscretize.py:57-84)."""
    return np.array([r[s].mean(axis=0) for s in _segments(intervals)], dtype=float).reshape(-1, 3)


def _normalised(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=1)[:, None]


def _perpendicular(t3: np.ndarray) -> np.ndarray:
    """Unit t3 x e_x per row (t3 x e_y for a row equal to e_x)."""
    t2 = np.cross(t3, _EX)
    on_x = np.all(t3 == _EX, axis=1)
    if on_x.any():
        t2[on_x] = np.cross(t3[on_x], _EY)
    return _normalised(t2)


def get_orientations_in_intervals(t3: np.ndarray, intervals: Dict[int, Tuple[int, int]]
                                  ) -> Tuple[np.ndarray, np.ndarray]:
    """Unit mean t3 of each segment and a perpendicular t2
    (chromo/util/rediscretize.py:87-122)."""
    t3_cg = _normalised(get_avg_in_intervals(t3, intervals))
    return t3_cg, _perpendicular(t3_cg)


def get_majority_state_in_interval(states: np.ndarray, intervals: Dict[int, Tuple[int, int]]
                                   ) -> np.ndarray:
    """Most frequent value of each column over each segment, the smallest value
    on a tie (chromo/util/rediscretize.py:125-160)."""
    segs = _segments(intervals)
    owner = np.concatenate([np.full(len(states[s]), k) for k, s in enumerate(segs)]).astype(np.int64)
    rows = np.concatenate([np.arange(len(states))[s] for s in segs]).astype(np.int64)
    out = np.zeros((len(segs), states.shape[1]), dtype=int)
    for col in range(states.shape[1]):
        vals = states[rows, col].astype(np.int64)
        counts = np.zeros((len(segs), int(vals.max(initial=0)) + 1), dtype=np.int64)
        np.add.at(counts, (owner, vals), 1)
        out[:, col] = counts.argmax(axis=1)
    return out


def get_random_state_in_interval(states: np.ndarray, intervals: Dict[int, Tuple[int, int]]
                                 ) -> np.ndarray:
    """A value drawn uniformly (``np.random.choice``) from each column over each
    segment of more than one bead, coarse bead by coarse bead
    (chromo/util/rediscretize.py:163-196)."""
    out = np.zeros((len(intervals), states.shape[1]), dtype=int)
    for k, (lo, hi) in ((k, intervals[k]) for k in range(len(intervals))):
        seg = states[int(lo):int(hi)]
        out[k] = [np.random.choice(seg[:, c]) if hi - lo > 1 else seg[0, c]
                  for c in range(states.shape[1])]
    return out


# ------------------------------------------------------------------ fields and binders

def _field_dict(udf) -> Dict:
    return {k: getattr(udf, k) for k in _FIELD_KEYS}


def get_cg_binders(binders_refined, cg_factor: float):
    """Binders of the coarse chain (chromo/util/rediscretize.py:364-398): the
    reference scales energies, radii, volumes and cross talk by one, so the
    table is copied unchanged."""
    return binders_refined.copy()


def refine_binders(binders_cg, cg_factor: float):
    """Binders of the refined chain (chromo/util/rediscretize.py:958-991): a
    copy of the table, unchanged."""
    return binders_cg.copy()


def _resized_field(d: Dict, dims, widths, confine_length: float, polymers, binders
                   ) -> UniformDensityField:
    return UniformDensityField(
        polymers=polymers, binders=binders, x_width=widths[0], nx=dims[0], y_width=widths[1],
        ny=dims[1], z_width=widths[2], nz=dims[2], confine_type=d["confine_type"],
        confine_length=confine_length, chi=d["chi"], assume_fully_accessible=d["assume_fully_accessible"],
        vf_limit=d["vf_limit"], fast_field=d["fast_field"], n_points=d["n_points"])


def get_cg_udf(udf_refined_dict: Dict, binders_refined, cg_factor: float,
               polymers_cg: List[Chromatin]) -> UniformDensityField:
    """Field of the coarse chain (chromo/util/rediscretize.py:199-272): voxel
    counts divided by cg_factor^(1/3) (at least two per side; one buffer voxel
    more when confined) at the original voxel size, confinement radius divided
    by cg_factor^(1/3).  ``udf_refined_dict`` may also be a field."""
    d = udf_refined_dict if isinstance(udf_refined_dict, dict) else _field_dict(udf_refined_dict)
    s = cg_factor ** (1 / 3)
    old = [d["nx"], d["ny"], d["nz"]]
    dims = [int(round(n / s)) for n in old]
    if min(dims) < 2:
        raise ValueError(f"Coarse-graining factor {cg_factor} is not supported by the field.")
    if d["confine_type"] != "":
        dims = [n + 1 for n in dims]
    widths = [n * d[w] / o for n, w, o in zip(dims, ("x_width", "y_width", "z_width"), old)]
    return _resized_field(d, dims, widths, d["confine_length"] / s, polymers_cg,
                          get_cg_binders(binders_refined, cg_factor))


def refine_udf(udf_cg: UniformDensityField, binders_cg, cg_factor: float,
               polymers_refined: List[Chromatin]) -> UniformDensityField:
    """Field of the refined chain (chromo/util/rediscretize.py:845-900): voxel
    counts times cg_factor^(1/3) (one buffer voxel more when confined) at the
    coarse field's voxel size, confinement radius times cg_factor^(1/3)."""
    s = cg_factor ** (1 / 3)
    dims = [int(round(n * s)) for n in (udf_cg.nx, udf_cg.ny, udf_cg.nz)]
    if udf_cg.confine_type != "":
        dims = [n + 1 for n in dims]
    widths = [n * dv for n, dv in zip(dims, (udf_cg.dx, udf_cg.dy, udf_cg.dz))]
    return _resized_field(_field_dict(udf_cg), dims, widths, udf_cg.confine_length * s,
                          polymers_refined, refine_binders(binders_cg, cg_factor))


# ------------------------------------------------------------------ coarse chain

def get_cg_chromatin(polymer: Chromatin, cg_factor: float, name_cg: Optional[str] = "Chr_CG",
                     random_states: Optional[bool] = False) -> Chromatin:
    """Coarse chain (chromo/util/rediscretize.py:401-471): segment centroids
    pulled inward by cg_factor^(1/3), unit mean orientations, majority binding
    states, majority (or randomly drawn) chemical modifications, and the fine
    chain's first bond length for every coarse bond."""
    seg = get_cg_bead_intervals(polymer.num_beads, cg_factor)
    t3, t2 = get_orientations_in_intervals(polymer.t3, seg)
    pick = get_random_state_in_interval if random_states else get_majority_state_in_interval
    r = get_avg_in_intervals(polymer.r, seg) / cg_factor ** (1 / 3)
    return Chromatin(name=name_cg, r=r, bead_length=np.full(len(r) - 1, float(polymer.bead_length[0])),
                     bead_rad=polymer.bead_rad, t3=t3, t2=t2,
                     states=get_majority_state_in_interval(polymer.states, seg),
                     binder_names=polymer.binder_names, chemical_mods=pick(polymer.chemical_mods, seg),
                     chemical_mod_names=polymer.chemical_mod_names, log_path=polymer.log_path,
                     max_binders=polymer.max_binders)


# ------------------------------------------------------------------ refinement

def get_refined_intervals(cg_r: np.ndarray, num_beads_cg: int, num_beads_refined: int
                          ) -> Tuple[Dict[int, int], Dict[int, Tuple[np.ndarray, np.ndarray]]]:
    """Fine beads of each coarse segment and the segment's end points, NaN at
    a free end (chromo/util/rediscretize.py:537-583).  The n - 1 coarse bonds
    each get the same number of fine beads; the first and last coarse beads
    start free half-segments, and the remainder of the division is a free
    segment after the last coarse bead."""
    free = np.full(3, np.nan)
    bonds = num_beads_cg - 1
    size = num_beads_refined // bonds
    head = size // 2
    steps = {0: head}
    steps.update({i: size for i in range(1, bonds)})
    steps[bonds] = size - head - 1
    ends = {0: (free, cg_r[0, :])}
    ends.update({i: (cg_r[i - 1, :], cg_r[i, :]) for i in range(1, num_beads_cg)})
    rest = num_beads_refined % bonds
    if rest > 0:
        steps[num_beads_cg] = rest
        ends[num_beads_cg] = (cg_r[num_beads_cg - 1, :], np.full(3, np.nan))
    return steps, ends


def brownian_bridge(N: int, p0: np.ndarray, p1: np.ndarray,
                    avg_step_target: Optional[float] = None) -> np.ndarray:
    """N + 1 points from p0 to p1 (chromo/util/rediscretize.py:586-685).

    The straight path from p0 to p1 plus a Brownian bridge: with n = N + 1
    points and dt = 1 / N, the deviation obeys b[k+1] = b[k] (1 - dt / (1 -
    k dt)) + sqrt(dt) xi_k for the N - 1 interior points (xi drawn as one
    block of normals) and returns to zero at p1.  With a target mean step the
    deviations are first scaled by |p1 - p0| and then rescaled so that the
    mean step is the target (or the straight step, if the target is shorter;
    a warning says so)."""
    if N == 1:
        return np.array([p0, p1])
    n = N + 1
    dt = 1.0 / (n - 1)
    kicks = np.random.randn(n - 2, 3) * np.sqrt(dt)
    decay = 1 - dt / (1 - np.arange(n - 2) * dt)
    dev = np.zeros((n, 3))
    for k in range(n - 2):
        dev[k + 1, :] = dev[k, :] * decay[k] + kicks[k]
    straight = np.linspace(p0, p1, n)
    span = np.linalg.norm(p1 - p0)
    if avg_step_target is None:
        return straight + dev
    dev *= span
    straight_step = span / (n - 1)
    mean_step = np.sum(np.linalg.norm(np.diff(straight + dev, axis=0), axis=1)) / (n - 1)
    if avg_step_target < straight_step:
        warnings.warn(f"a mean step of {avg_step_target} cannot join the points; "
                      f"using the straight-line step {straight_step}")
        mean_step = straight_step
    shrink = (mean_step / straight_step) / (avg_step_target / straight_step)
    return straight + dev / shrink


def gaussian_walk_from_point(start, N, step_size):
    """A random walk of N steps of the given sizes from ``start`` (N + 1 points)
    (chromo/util/rediscretize.py:688-705)."""
    return gaussian_walk(N, step_size) + start


def enforce_spherical_confinement(r: np.ndarray, rad: float) -> np.ndarray:
    """Pull every bead found outside the sphere of radius ``rad`` -- and its
    three neighbours on each side, with weights 0.95 at the bead to 0.98 three
    away -- towards the origin by its excess factor |r| / rad; in place
    (chromo/util/rediscretize.py:708-753).  Violators are found on the input
    and their windows applied in bead order (windows near the chain ends are
    clipped)."""
    weights = np.array([0.98, 0.97, 0.96, 0.95, 0.96, 0.97, 0.98])
    dist = np.array([np.linalg.norm(p) for p in r])
    n = len(r)
    for i in np.nonzero(dist > rad)[0]:
        lo, hi = max(0, i - 3), min(n, i + 4)
        w = weights[lo - (i - 3):hi - (i - 3)] * (1 / (dist[i] / rad))
        r[lo:hi, :] = r[lo:hi, :] * w[:, None]
    return r


def get_refined_path(cg_r: np.ndarray, num_beads_refined: int,
                     bead_spacing: Optional[float] = np.pi) -> np.ndarray:
    """Fine path through the coarse points (chromo/util/rediscretize.py:756-807):
    a walk off the first coarse point reversed to end there, Brownian bridges
    between consecutive coarse points (each without its end point), and a walk
    off the last coarse point for the remainder beads."""
    steps, ends = get_refined_intervals(cg_r, len(cg_r), num_beads_refined)
    tail = len(cg_r)
    pieces = []
    for k in sorted(steps):
        m = steps[k]
        p0, p1 = ends[k]
        if k == 0:
            pieces.append(gaussian_walk_from_point(p1, m, np.full(m, bead_spacing))[::-1][:m])
        elif k == tail:
            pieces.append(gaussian_walk_from_point(p0, m, np.full(m, bead_spacing)))
        else:
            pieces.append(brownian_bridge(m, np.asarray(p0), np.asarray(p1),
                                          avg_step_target=bead_spacing)[:m])
    return np.vstack(pieces)


def get_refined_orientations(t3_cg: np.ndarray, num_beads_refined: int
                             ) -> Tuple[np.ndarray, np.ndarray]:
    """t3 refined as a path through the coarse t3 (spacing pi), made unit, and
    a perpendicular t2 (chromo/util/rediscretize.py:810-842)."""
    t3 = _normalised(get_refined_path(t3_cg, num_beads_refined))
    return t3, _perpendicular(t3)


def refine_chromatin(polymer_cg: Chromatin, num_beads_refined: int, bead_spacing: float,
                     chemical_mods: np.ndarray, udf_cg: UniformDensityField,
                     binding_equilibration: Optional[int] = 0, name_refine: Optional[str] = "Chr",
                     output_dir: Optional[str] = ".", random_seed: int = 0
                     ) -> Tuple[Chromatin, UniformDensityField]:
    """Fine chain and field from a coarse chain (chromo/util/rediscretize.py:994-1107).

    The coarse path is refined at the bead spacing shrunk by the linear scale
    s = (N_fine / N_cg)^(1/3) and the result stretched by s; orientations are
    refined as a path; binders start unbound with the given chemical
    modifications; the field grows by s; beads are pulled inside a spherical
    confinement; then ``binding_equilibration`` binding moves are attempted
    (one per MC step of this package's ``mc_sim`` on the GPU, no amplitude
    control, seeded by ``random_seed``)."""
    n_cg = len(polymer_cg.r)
    s = (num_beads_refined / n_cg) ** (1 / 3)
    r = get_refined_path(polymer_cg.r, num_beads_refined, bead_spacing / s) * s
    t3, t2 = get_refined_orientations(polymer_cg.t3, num_beads_refined)
    polymer = Chromatin(name=name_refine, r=r, bead_length=np.full(len(r) - 1, float(bead_spacing)),
                        bead_rad=polymer_cg.bead_rad, t3=t3, t2=t2,
                        states=np.zeros((num_beads_refined, chemical_mods.shape[1]), dtype=int),
                        binder_names=polymer_cg.binder_names, chemical_mods=chemical_mods,
                        chemical_mod_names=polymer_cg.chemical_mod_names,
                        max_binders=polymer_cg.max_binders)
    udf = refine_udf(udf_cg, udf_cg.binders, num_beads_refined / n_cg, [polymer])
    if udf.confine_type == "Spherical":
        polymer.r = enforce_spherical_confinement(polymer.r, udf.confine_length)
    if binding_equilibration > 0:
        from ..mc import mc_sim
        from ..mc import move_funcs as mv
        from ..mc.mc_controller import NoControl, specific_move
        moves = specific_move(mv.change_binding_state, log_dir=output_dir,
                              bead_amp_bounds={"change_binding_state": (1, 1)},
                              move_amp_bounds={"change_binding_state": (1, 1)},
                              controller=NoControl)
        mc_sim([polymer], udf.binders, int(binding_equilibration), moves, udf, 1.0, random_seed)
    return polymer, udf


__all__ = ["get_cg_bead_intervals", "get_avg_in_intervals", "get_orientations_in_intervals",
           "get_majority_state_in_interval", "get_random_state_in_interval", "get_cg_udf",
           "get_cg_binders", "get_cg_chromatin", "get_refined_intervals", "brownian_bridge",
           "gaussian_walk_from_point", "enforce_spherical_confinement", "get_refined_path",
           "get_refined_orientations", "refine_udf", "refine_binders", "refine_chromatin"]
