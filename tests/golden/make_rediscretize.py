"""Golden vectors for the coarse-grain / refine workflow, from the reference.

Run here (the container that mounts the reference), after
``python oracle/build_reference.py``::

    python tests/golden/make_rediscretize.py

Seeded inputs go through the reference's own ``chromo.util.rediscretize``
functions (``get_cg_bead_intervals`` ... ``refine_chromatin``), each random
call seeded with ``np.random.seed`` right before it; inputs and outputs are
stored in ``tests/golden/rediscretize/vectors.npz`` (a subfolder, so the MC
golden-case loader does not pick it up).
"""
import contextlib
import io
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "oracle" / "ref_stubs"), str(ROOT / "oracle" / "_ref")]

import chromo.binders as cb  # noqa: E402
import chromo.util.rediscretize as rd  # noqa: E402
from chromo.fields import UniformDensityField  # noqa: E402
from chromo.polymers import Chromatin  # noqa: E402

OUT = Path(__file__).resolve().parent / "rediscretize"
INTERVAL_CASES = [(10, 3), (12, 4), (100, 7), (50, 5), (61, 6)]


def chain(rng, n, step=16.5):
    """Seeded random walk of unit steps times `step`, tangents from neighbours."""
    d = rng.standard_normal((n - 1, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    r = np.vstack([np.zeros(3), np.cumsum(d * step, axis=0)])
    t3 = np.gradient(r, axis=0)
    t3 /= np.linalg.norm(t3, axis=1)[:, None]
    t2 = np.cross(t3, np.array([1.0, 0.0, 0.0]))
    t2 /= np.linalg.norm(t2, axis=1)[:, None]
    return r, t3, t2


def quiet(f, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return f(*a, **k)


def main():
    rng = np.random.default_rng(20261204)
    out = {}
    for j, (n, f) in enumerate(INTERVAL_CASES):
        iv = rd.get_cg_bead_intervals(n, f)
        out[f"iv{j}"] = np.array([iv[i] for i in range(len(iv))], dtype=np.int64)

    n, f = 61, 6
    r, t3, t2 = chain(rng, n)
    states = rng.integers(0, 3, size=(n, 2)).astype(np.int64)
    mods = rng.integers(0, 3, size=(n, 2)).astype(np.int64)
    out.update(r=r, t3=t3, t2=t2, states=states, mods=mods)
    iv = rd.get_cg_bead_intervals(n, f)
    out["avg_r"] = rd.get_avg_in_intervals(r, iv)
    out["ori_t3"], out["ori_t2"] = rd.get_orientations_in_intervals(t3, iv)
    out["maj_states"] = rd.get_majority_state_in_interval(states, iv)
    np.random.seed(5)
    out["rand_mods"] = rd.get_random_state_in_interval(mods, iv)

    cg_r = out["avg_r"]
    m = len(cg_r)
    for j, nref in enumerate((61, 64, 23)):
        steps, se = rd.get_refined_intervals(cg_r, m, nref)
        out[f"ri_steps{j}"] = np.array([steps[i] for i in range(len(steps))], dtype=np.int64)
        out[f"ri_se{j}"] = np.array([np.concatenate([se[i][0], se[i][1]]) for i in range(len(se))])

    bb = [(4, np.zeros(3), np.ones(3), 1.0), (1, np.zeros(3), np.ones(3), 2.0),
          (7, np.array([1.0, -2.0, 0.5]), np.array([30.0, 4.0, -9.0]), 16.5),
          (9, np.zeros(3), np.array([50.0, 0.0, 0.0]), 1.0),  # target below the straight step
          (6, np.zeros(3), np.array([3.0, 4.0, 0.0]), None)]
    for j, (N, p0, p1, tgt) in enumerate(bb):
        np.random.seed(100 + j)
        out[f"bb{j}"] = quiet(rd.brownian_bridge, N, p0, p1, avg_step_target=tgt)

    np.random.seed(11)
    out["path"] = quiet(rd.get_refined_path, cg_r, 64, 16.5)
    np.random.seed(12)
    out["ref_t3"], out["ref_t2"] = quiet(rd.get_refined_orientations, out["ori_t3"], 64)

    rs = r * 0.2
    rs[[0, 2, 30, 58, 60]] *= 4.0  # violators at both ends and in the middle
    out["sph_in"] = rs.copy()
    out["sph_out"] = rd.enforce_spherical_confinement(rs.copy(), 100.0)

    # chromatin-level functions
    names = ["HP1", "PRC1"]
    binders = cb.make_binder_collection([cb.get_by_name(nm) for nm in names])
    p = Chromatin("p", r.copy(), bead_length=np.full(n - 1, 16.5), t3=t3.copy(), t2=t2.copy(),
                  states=states.copy(), binder_names=np.array(names), chemical_mods=mods.copy(),
                  chemical_mod_names=np.array(["H3K9me3", "H3K27me3"]))
    pcg = rd.get_cg_chromatin(p, f, name_cg="cg")
    for k in ("r", "t3", "t2", "states", "chemical_mods", "bead_length"):
        out[f"cg_{k}"] = np.asarray(getattr(pcg, k)).copy()
    np.random.seed(13)
    pcg_rand = rd.get_cg_chromatin(p, f, random_states=True)
    out["cgr_chemical_mods"] = np.asarray(pcg_rand.chemical_mods).copy()
    for j, (ct, cl) in enumerate((("", 0.0), ("Spherical", 400.0))):
        udf = UniformDensityField([p], binders, 800.0, 20, 800.0, 20, 800.0, 20,
                                  confine_type=ct, confine_length=cl, chi=1.0)
        d = {k: getattr(udf, k) for k in ("nx", "ny", "nz", "x_width", "y_width", "z_width",
                                          "confine_type", "confine_length", "chi",
                                          "assume_fully_accessible", "vf_limit", "fast_field",
                                          "n_points")}
        ucg = rd.get_cg_udf(d, binders, f, [pcg])
        out[f"udf_cg{j}"] = np.array([ucg.nx, ucg.ny, ucg.nz, ucg.x_width, ucg.y_width,
                                      ucg.z_width, ucg.confine_length])
        np.random.seed(14 + j)
        pref, uref = quiet(rd.refine_chromatin, pcg, 64, 16.5, np.vstack([mods, mods])[:64], ucg)
        out[f"rc_r{j}"] = np.asarray(pref.r).copy()
        out[f"rc_t3{j}"] = np.asarray(pref.t3).copy()
        out[f"rc_t2{j}"] = np.asarray(pref.t2).copy()
        out[f"rc_udf{j}"] = np.array([uref.nx, uref.ny, uref.nz, uref.x_width, uref.y_width,
                                      uref.z_width, uref.confine_length])
    OUT.mkdir(exist_ok=True)
    np.savez_compressed(OUT / "vectors.npz", **out)
    print("wrote", OUT / "vectors.npz", len(out), "arrays")


if __name__ == "__main__":
    main()
