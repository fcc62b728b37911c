"""Coarse-graining and refinement of a chromatin fiber (chromo/util/rediscretize.py).

The two-step workflow of the reference: equilibrate a coarse-grained chain
(each bead standing for ``cg_factor`` beads of the fine chain, placed at the
centroid of its segment and moved radially inward by ``cg_factor^(1/3)``, in
a field whose box shrinks by the same factor), then rebuild the fine chain
from it: Gaussian random walks off the two free ends, Brownian bridges
between consecutive coarse beads, orientations refined the same way, the
field grown back, and binding states re-equilibrated by binding moves.

The functions keep the reference's names, arguments and results, and draw
from numpy's global generator in the reference's order, so a seeded call
returns the reference's arrays.  The deprecated ``*_old`` variants of the
reference are not restated.  The binding re-equilibration of
``refine_chromatin`` runs through this package's ``mc_sim`` (binding moves
on the GPU, Philox random streams keyed by ``random_seed``) where the
reference calls ``mc_step`` with libc ``rand()``.
"""
from typing import Dict, List, Optional, Tuple

import numpy as np

from ..fields import UniformDensityField
from ..polymers import Chromatin, gaussian_walk


def get_cg_bead_intervals(num_beads: int, cg_factor: float) -> Dict[int, Tuple[int, int]]:
    """Bead intervals [lo, hi) of the fine chain behind each coarse bead
    (chromo/util/rediscretize.py:24-54).  A partial last interval extends one
    bead past the chain's end, as in the reference (slicing clips it)."""
    cg_beads = num_beads / cg_factor
    num_intervals = int(np.floor(cg_beads))
    left_over_beads = num_beads - (num_intervals * cg_factor)
    intervals = {i: (i * cg_factor, (i + 1) * cg_factor) for i in range(num_intervals)}
    if left_over_beads > 0:
        intervals[num_intervals] = (intervals[num_intervals - 1][1],
                                    intervals[num_intervals - 1][1] + left_over_beads + 1)
    return intervals


def get_avg_in_intervals(r: np.ndarray, intervals: Dict[int, Tuple[int, int]]) -> np.ndarray:
    """Centroid of each interval's rows (chromo/util/rediscretize.py:57-84)."""
    out = np.zeros((len(intervals), 3), dtype=float)
    for ind, (lo, hi) in intervals.items():
        out[ind, :] = np.average(r[lo:hi], axis=0)
    return out


def _unit_t2(t3: np.ndarray) -> np.ndarray:
    """t2 = t3 x e_x normalised (t3 x e_y where t3 equals e_x)."""
    t2 = np.zeros(t3.shape)
    ex, ey = np.array([1, 0, 0]), np.array([0, 1, 0])
    for i in range(t3.shape[0]):
        t2[i] = np.cross(t3[i], ex) if not np.all(np.equal(t3[i], ex)) else np.cross(t3[i], ey)
    mags = np.linalg.norm(t2, axis=1)
    for i in range(t2.shape[0]):
        t2[i] /= mags[i]
    return t2


def get_orientations_in_intervals(t3: np.ndarray, intervals: Dict[int, Tuple[int, int]]
                                  ) -> Tuple[np.ndarray, np.ndarray]:
    """Normalised mean t3 of each interval and a perpendicular t2
    (chromo/util/rediscretize.py:87-122)."""
    t3_cg = get_avg_in_intervals(t3, intervals)
    mags = np.linalg.norm(t3_cg, axis=1)
    for i in range(t3_cg.shape[0]):
        t3_cg[i] /= mags[i]
    return t3_cg, _unit_t2(t3_cg)


def get_majority_state_in_interval(states: np.ndarray, intervals: Dict[int, Tuple[int, int]]
                                   ) -> np.ndarray:
    """Most common state of each column over each interval, the smallest on a
    tie (chromo/util/rediscretize.py:125-160)."""
    out = np.zeros((len(intervals), states.shape[1]), dtype=int)
    for ind, (lo, hi) in intervals.items():
        seg = states[lo:hi]
        for i in range(states.shape[1]):
            out[ind, i] = np.argmax(np.bincount(seg[:, i])) if hi - lo > 1 else seg[0, i]
    return out


def get_random_state_in_interval(states: np.ndarray, intervals: Dict[int, Tuple[int, int]]
                                 ) -> np.ndarray:
    """A state drawn (np.random.choice) from each column over each interval
    (chromo/util/rediscretize.py:163-196)."""
    out = np.zeros((len(intervals), states.shape[1]), dtype=int)
    for ind, (lo, hi) in intervals.items():
        seg = states[lo:hi]
        for i in range(states.shape[1]):
            out[ind, i] = np.random.choice(seg[:, i]) if hi - lo > 1 else seg[0, i]
    return out


def _field_dict(udf) -> Dict:
    return {k: getattr(udf, k) for k in ("nx", "ny", "nz", "x_width", "y_width", "z_width",
                                          "confine_type", "confine_length", "chi",
                                          "assume_fully_accessible", "vf_limit", "fast_field",
                                          "n_points")}


def get_cg_binders(binders_refined, cg_factor: float):
    """Binders of the coarse-grained chain (chromo/util/rediscretize.py:364-398):
    a copy of the table with every property kept (the reference scales
    interaction energy, radius, volume and cross talk by 1)."""
    return binders_refined.copy()


def refine_binders(binders_cg, cg_factor: float):
    """Binders of the refined chain (chromo/util/rediscretize.py:958-991): a
    copy of the table with every property kept."""
    return binders_cg.copy()


def get_cg_udf(udf_refined_dict: Dict, binders_refined, cg_factor: float,
               polymers_cg: List[Chromatin]) -> UniformDensityField:
    """Field of the coarse-grained chain (chromo/util/rediscretize.py:199-272):
    voxels per side divided by cg_factor^(1/3) (at least two; one buffer voxel
    more when confined), the same voxel size, confinement radius divided by
    cg_factor^(1/3).  ``udf_refined_dict`` may also be a field."""
    d = udf_refined_dict if isinstance(udf_refined_dict, dict) else _field_dict(udf_refined_dict)
    s = cg_factor ** (1 / 3)
    nx, ny, nz = (int(round(d[k] / s)) for k in ("nx", "ny", "nz"))
    if nx < 2 or ny < 2 or nz < 2:
        raise ValueError(f"Coarse-graining factor {cg_factor} is not supported by the field.")
    if d["confine_type"] != "":
        nx, ny, nz = nx + 1, ny + 1, nz + 1
    return UniformDensityField(
        polymers=polymers_cg, binders=get_cg_binders(binders_refined, cg_factor),
        x_width=nx * d["x_width"] / d["nx"], nx=nx, y_width=ny * d["y_width"] / d["ny"], ny=ny,
        z_width=nz * d["z_width"] / d["nz"], nz=nz, confine_type=d["confine_type"],
        confine_length=d["confine_length"] / s, chi=d["chi"],
        assume_fully_accessible=d["assume_fully_accessible"], vf_limit=d["vf_limit"],
        fast_field=d["fast_field"], n_points=d["n_points"])


def get_cg_chromatin(polymer: Chromatin, cg_factor: float, name_cg: Optional[str] = "Chr_CG",
                     random_states: Optional[bool] = False) -> Chromatin:
    """Coarse-grained chain (chromo/util/rediscretize.py:401-471): segment
    centroids scaled inward by cg_factor^(1/3), mean orientations, majority
    binding states and majority (or random) chemical modifications, the first
    bond length for every coarse bond."""
    intervals = get_cg_bead_intervals(polymer.num_beads, cg_factor)
    r_cg = get_avg_in_intervals(polymer.r, intervals)
    t3_cg, t2_cg = get_orientations_in_intervals(polymer.t3, intervals)
    states_cg = get_majority_state_in_interval(polymer.states, intervals)
    if random_states:
        mods_cg = get_random_state_in_interval(polymer.chemical_mods, intervals)
    else:
        mods_cg = get_majority_state_in_interval(polymer.chemical_mods, intervals)
    bead_length_cg = np.ones(len(r_cg) - 1) * polymer.bead_length[0]
    r_cg /= cg_factor ** (1 / 3)
    return Chromatin(name=name_cg, r=r_cg, bead_length=bead_length_cg, bead_rad=polymer.bead_rad,
                     t3=t3_cg, t2=t2_cg, states=states_cg, binder_names=polymer.binder_names,
                     chemical_mods=mods_cg, chemical_mod_names=polymer.chemical_mod_names,
                     log_path=polymer.log_path, max_binders=polymer.max_binders)


def get_refined_intervals(cg_r: np.ndarray, num_beads_cg: int, num_beads_refined: int
                          ) -> Tuple[Dict[int, int], Dict[int, Tuple[np.ndarray, np.ndarray]]]:
    """Fine beads per coarse segment and each segment's fixed end points (NaN
    for a free end) (chromo/util/rediscretize.py:537-583)."""
    seg_size = int(np.floor(num_beads_refined / (num_beads_cg - 1)))
    seg_half_1 = int(np.floor(seg_size / 2))
    seg_half_2 = seg_size - seg_half_1
    left_over = num_beads_refined % (num_beads_cg - 1)
    num_steps = {0: seg_half_1}
    for i in range(1, num_beads_cg - 1):
        num_steps[i] = seg_size
    num_steps[num_beads_cg - 1] = seg_half_2 - 1
    nan3 = np.asarray([np.nan, np.nan, np.nan])
    start_end = {0: (nan3, cg_r[0, :])}
    for i in range(1, num_beads_cg):
        start_end[i] = (cg_r[i - 1, :], cg_r[i, :])
    if left_over > 0:
        num_steps[num_beads_cg] = left_over
        start_end[num_beads_cg] = (cg_r[num_beads_cg - 1, :], np.asarray([np.nan, np.nan, np.nan]))
    return num_steps, start_end


def brownian_bridge(N: int, p0: np.ndarray, p1: np.ndarray,
                    avg_step_target: Optional[float] = None) -> np.ndarray:
    """N + 1 points from p0 to p1: a Brownian bridge (one np.random.randn(3)
    per interior point) added to the straight path, its deviations scaled so
    that the mean step approaches ``avg_step_target`` (at least the straight
    path's step) (chromo/util/rediscretize.py:586-685)."""
    if N == 1:
        return np.array([p0, p1])
    N += 1
    dt = 1.0 / (N - 1)
    dt_sqrt = np.sqrt(dt)
    B = np.empty((N, 3), dtype=float)
    B[0] = 0
    for n in range(N - 2):
        t = n * dt
        xi = np.random.randn(3) * dt_sqrt
        B[n + 1, :] = B[n, :] * (1 - dt / (1 - t)) + xi
    B[N - 1, :] = np.array([0, 0, 0])
    direct_length = np.linalg.norm(p1 - p0)
    direct_step = direct_length / (N - 1)
    direct_path = np.linspace(p0, p1, N)
    if avg_step_target is not None:
        B *= direct_length
    path = direct_path + B
    avg_step = np.sum(np.linalg.norm(np.diff(path, axis=0), axis=1)) / (N - 1)
    if avg_step_target is not None:
        if avg_step_target < direct_step:
            print(f"Points cannot be connected with steps of {avg_step_target}.")
            print(f"The minimum step size required is {direct_step}.")
            print(f"The bead spacing will be adjusted to {direct_step}.")
            avg_step = direct_step
        actual_to_direct = avg_step / direct_step
        target_to_direct = avg_step_target / direct_step
        path = direct_path + (B / (actual_to_direct / target_to_direct))
    return path


def gaussian_walk_from_point(start, N, step_size):
    """Gaussian random walk of N steps from ``start`` (N + 1 points)
    (chromo/util/rediscretize.py:688-705)."""
    return gaussian_walk(N, step_size) + start


def enforce_spherical_confinement(r: np.ndarray, rad: float) -> np.ndarray:
    """Pull beads outside a sphere of radius ``rad`` (and their three
    neighbours on each side, by a 7-point kernel) inward by their excess
    factor, in place (chromo/util/rediscretize.py:708-753)."""
    kernel = np.array([0.98, 0.97, 0.96, 0.95, 0.96, 0.97, 0.98])
    num_r = len(r)
    num_r_m4 = num_r - 4
    violators, factors = [], []
    for i in range(num_r):
        dist = np.linalg.norm(r[i])
        if dist > rad:
            violators.append(i)
            factors.append(dist / rad)
    for ind, fac in zip(violators, factors):
        if 3 <= ind <= num_r_m4:
            for j in range(3):
                r[ind - 3:ind + 4, j] = np.multiply(r[ind - 3:ind + 4, j], kernel * (1 / fac))
        elif ind < 3:
            for j in range(3):
                r[:ind + 4, j] = np.multiply(r[:ind + 4, j], kernel[3 - ind:] * (1 / fac))
        elif ind > num_r_m4:
            for j in range(3):
                r[ind - 3:, j] = np.multiply(r[ind - 3:, j], kernel[:num_r_m4 - ind] * (1 / fac))
    return r


def get_refined_path(cg_r: np.ndarray, num_beads_refined: int,
                     bead_spacing: Optional[float] = np.pi) -> np.ndarray:
    """Fine path through the coarse points: reversed Gaussian walk off the
    first point, Brownian bridges between consecutive points, a Gaussian walk
    off the last point for the left-over beads
    (chromo/util/rediscretize.py:756-807)."""
    num_beads_cg = len(cg_r)
    num_steps, start_end = get_refined_intervals(cg_r, num_beads_cg, num_beads_refined)
    segs = []
    for ind, (p0, p1) in start_end.items():
        n = num_steps[ind]
        if ind == 0:
            seg = np.flip(gaussian_walk_from_point(p1, n, np.array([bead_spacing] * n)), axis=0)[:n]
        elif ind == num_beads_cg:
            seg = gaussian_walk_from_point(p0, n, np.array([bead_spacing] * n))
        else:
            seg = brownian_bridge(n, np.asarray(p0), np.asarray(p1), avg_step_target=bead_spacing)[:n]
        segs.append(seg)
    return np.vstack(segs)


def get_refined_orientations(t3_cg: np.ndarray, num_beads_refined: int
                             ) -> Tuple[np.ndarray, np.ndarray]:
    """t3 refined as a path through the coarse t3 (spacing pi), normalised,
    and a perpendicular t2 (chromo/util/rediscretize.py:810-842)."""
    t3 = get_refined_path(t3_cg, num_beads_refined)
    mags = np.linalg.norm(t3, axis=1)
    for i in range(t3.shape[0]):
        t3[i] /= mags[i]
    return t3, _unit_t2(t3)


def refine_udf(udf_cg: UniformDensityField, binders_cg, cg_factor: float,
               polymers_refined: List[Chromatin]) -> UniformDensityField:
    """Field of the refined chain (chromo/util/rediscretize.py:845-900):
    voxels per side times cg_factor^(1/3) (one buffer voxel more when
    confined), the same voxel size, confinement radius times cg_factor^(1/3)."""
    s = cg_factor ** (1 / 3)
    nx, ny, nz = (int(round(n * s)) for n in (udf_cg.nx, udf_cg.ny, udf_cg.nz))
    if udf_cg.confine_type != "":
        nx, ny, nz = nx + 1, ny + 1, nz + 1
    return UniformDensityField(
        polymers=polymers_refined, binders=refine_binders(binders_cg, cg_factor),
        x_width=nx * udf_cg.dx, nx=nx, y_width=ny * udf_cg.dy, ny=ny, z_width=nz * udf_cg.dz,
        nz=nz, confine_type=udf_cg.confine_type, confine_length=udf_cg.confine_length * s,
        chi=udf_cg.chi, assume_fully_accessible=udf_cg.assume_fully_accessible,
        vf_limit=udf_cg.vf_limit, fast_field=udf_cg.fast_field, n_points=udf_cg.n_points)


def refine_chromatin(polymer_cg: Chromatin, num_beads_refined: int, bead_spacing: float,
                     chemical_mods: np.ndarray, udf_cg: UniformDensityField,
                     binding_equilibration: Optional[int] = 0, name_refine: Optional[str] = "Chr",
                     output_dir: Optional[str] = ".", random_seed: int = 0
                     ) -> Tuple[Chromatin, UniformDensityField]:
    """Fine chain and field from a coarse-grained chain
    (chromo/util/rediscretize.py:994-1107): refined path (bead spacing scaled
    inward by (N_fine / N_cg)^(1/3), then the path scaled outward by the same
    factor), refined orientations, unbound binders, the given chemical
    modifications, the grown field, spherical confinement enforced, then
    ``binding_equilibration`` binding-move attempts (one per MC step of this
    package's ``mc_sim`` on the GPU, no amplitude control, seeded by
    ``random_seed``)."""
    num_beads_cg = len(polymer_cg.r)
    scaling = (num_beads_refined / num_beads_cg) ** (1 / 3)
    spacing_in = np.ones(num_beads_cg - 1) * bead_spacing / scaling
    r = get_refined_path(polymer_cg.r, num_beads_refined, spacing_in[0])
    t3, t2 = get_refined_orientations(polymer_cg.t3, num_beads_refined)
    states = np.zeros((num_beads_refined, chemical_mods.shape[1]), dtype=int)
    r *= scaling
    polymer = Chromatin(name=name_refine, r=r, bead_length=np.ones(len(r) - 1) * bead_spacing,
                        bead_rad=polymer_cg.bead_rad, t3=t3, t2=t2, states=states,
                        binder_names=polymer_cg.binder_names, chemical_mods=chemical_mods,
                        chemical_mod_names=polymer_cg.chemical_mod_names,
                        max_binders=polymer_cg.max_binders)
    udf = refine_udf(udf_cg, udf_cg.binders, num_beads_refined / num_beads_cg, [polymer])
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
