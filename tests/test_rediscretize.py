"""Coarse-grain / refine workflow against the reference's own outputs.

``tests/golden/make_rediscretize.py`` ran the reference's
``chromo.util.rediscretize`` on seeded inputs; here the same inputs and the
same numpy seeds go through ``chromo_gb300.util.rediscretize`` and every
array must come out identical (the workflow is host-side numpy; no GPU).
"""
import contextlib
import io
from pathlib import Path

import numpy as np
import pytest

import chromo_gb300.binders as cb
from chromo_gb300.fields import UniformDensityField
from chromo_gb300.polymers import Chromatin
from chromo_gb300.util import rediscretize as rd

FIX = Path(__file__).resolve().parent / "golden" / "rediscretize" / "vectors.npz"
INTERVAL_CASES = [(10, 3), (12, 4), (100, 7), (50, 5), (61, 6)]


@pytest.fixture(scope="module")
def g():
    with np.load(FIX, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def quiet(f, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return f(*a, **k)


def test_bead_intervals(g):
    for j, (n, f) in enumerate(INTERVAL_CASES):
        iv = rd.get_cg_bead_intervals(n, f)
        np.testing.assert_array_equal(np.array([iv[i] for i in range(len(iv))]), g[f"iv{j}"])


def test_segment_averages_orientations_and_states(g):
    iv = rd.get_cg_bead_intervals(61, 6)
    np.testing.assert_array_equal(rd.get_avg_in_intervals(g["r"], iv), g["avg_r"])
    t3, t2 = rd.get_orientations_in_intervals(g["t3"], iv)
    np.testing.assert_array_equal(t3, g["ori_t3"])
    np.testing.assert_array_equal(t2, g["ori_t2"])
    np.testing.assert_array_equal(rd.get_majority_state_in_interval(g["states"], iv), g["maj_states"])
    np.random.seed(5)
    np.testing.assert_array_equal(rd.get_random_state_in_interval(g["mods"], iv), g["rand_mods"])


def test_refined_intervals(g):
    cg_r = g["avg_r"]
    for j, nref in enumerate((61, 64, 23)):
        steps, se = rd.get_refined_intervals(cg_r, len(cg_r), nref)
        np.testing.assert_array_equal(np.array([steps[i] for i in range(len(steps))]), g[f"ri_steps{j}"])
        got = np.array([np.concatenate([se[i][0], se[i][1]]) for i in range(len(se))])
        np.testing.assert_array_equal(got, g[f"ri_se{j}"])


def test_brownian_bridges(g):
    bb = [(4, np.zeros(3), np.ones(3), 1.0), (1, np.zeros(3), np.ones(3), 2.0),
          (7, np.array([1.0, -2.0, 0.5]), np.array([30.0, 4.0, -9.0]), 16.5),
          (9, np.zeros(3), np.array([50.0, 0.0, 0.0]), 1.0),
          (6, np.zeros(3), np.array([3.0, 4.0, 0.0]), None)]
    for j, (N, p0, p1, tgt) in enumerate(bb):
        np.random.seed(100 + j)
        np.testing.assert_array_equal(quiet(rd.brownian_bridge, N, p0, p1, avg_step_target=tgt),
                                      g[f"bb{j}"])


def test_refined_path_and_orientations(g):
    np.random.seed(11)
    np.testing.assert_array_equal(quiet(rd.get_refined_path, g["avg_r"], 64, 16.5), g["path"])
    np.random.seed(12)
    t3, t2 = quiet(rd.get_refined_orientations, g["ori_t3"], 64)
    np.testing.assert_array_equal(t3, g["ref_t3"])
    np.testing.assert_array_equal(t2, g["ref_t2"])


def test_spherical_confinement_enforcement(g):
    np.testing.assert_array_equal(rd.enforce_spherical_confinement(g["sph_in"].copy(), 100.0),
                                  g["sph_out"])


def _chromatin(g):
    names = ["HP1", "PRC1"]
    binders = cb.make_binder_collection([cb.get_by_name(nm) for nm in names])
    p = Chromatin("p", g["r"].copy(), bead_length=np.full(len(g["r"]) - 1, 16.5),
                  t3=g["t3"].copy(), t2=g["t2"].copy(), states=g["states"].copy(),
                  binder_names=np.array(names), chemical_mods=g["mods"].copy(),
                  chemical_mod_names=np.array(["H3K9me3", "H3K27me3"]))
    return p, binders


def test_coarse_grained_chromatin(g):
    p, _ = _chromatin(g)
    pcg = rd.get_cg_chromatin(p, 6, name_cg="cg")
    for k in ("r", "t3", "t2", "states", "chemical_mods", "bead_length"):
        np.testing.assert_array_equal(np.asarray(getattr(pcg, k)), g[f"cg_{k}"], err_msg=k)
    np.random.seed(13)
    pr = rd.get_cg_chromatin(p, 6, random_states=True)
    np.testing.assert_array_equal(pr.chemical_mods, g["cgr_chemical_mods"])


@pytest.mark.parametrize("j,ct,cl", [(0, "", 0.0), (1, "Spherical", 400.0)])
def test_coarse_grained_field_and_refinement(g, j, ct, cl):
    p, binders = _chromatin(g)
    pcg = rd.get_cg_chromatin(p, 6, name_cg="cg")
    udf = UniformDensityField([p], binders, 800.0, 20, 800.0, 20, 800.0, 20, confine_type=ct,
                              confine_length=cl, chi=1.0)
    ucg = rd.get_cg_udf(rd._field_dict(udf), binders, 6, [pcg])
    np.testing.assert_array_equal(
        np.array([ucg.nx, ucg.ny, ucg.nz, ucg.x_width, ucg.y_width, ucg.z_width, ucg.confine_length]),
        g[f"udf_cg{j}"])
    np.random.seed(14 + j)
    mods = np.vstack([g["mods"], g["mods"]])[:64]
    pref, uref = quiet(rd.refine_chromatin, pcg, 64, 16.5, mods, ucg)
    np.testing.assert_array_equal(pref.r, g[f"rc_r{j}"])
    np.testing.assert_array_equal(pref.t3, g[f"rc_t3{j}"])
    np.testing.assert_array_equal(pref.t2, g[f"rc_t2{j}"])
    np.testing.assert_array_equal(
        np.array([uref.nx, uref.ny, uref.nz, uref.x_width, uref.y_width, uref.z_width,
                  uref.confine_length]), g[f"rc_udf{j}"])
    assert np.all(pref.states == 0) and pref.num_beads == 64


def test_cg_factor_too_large_is_refused():
    with pytest.raises(ValueError):
        rd.get_cg_udf({"nx": 3, "ny": 3, "nz": 3, "x_width": 3.0, "y_width": 3.0, "z_width": 3.0,
                       "confine_type": "", "confine_length": 0.0, "chi": 1.0,
                       "assume_fully_accessible": 1, "vf_limit": 0.5, "fast_field": 0,
                       "n_points": 1000}, None, 64, [])


@pytest.mark.gpu
def test_refinement_re_equilibrates_binding_on_the_gpu(g):
    """Binding re-equilibration of the refined chain runs binding moves through
    mc_sim on the GPU: states stay within 0..sites, some beads get bound (the
    binders' chemical potential favours binding on marked beads), and the
    positions are untouched (up to their FP32 storage on the device)."""
    p, binders = _chromatin(g)
    pcg = rd.get_cg_chromatin(p, 6, name_cg="cg")
    udf = UniformDensityField([p], binders, 800.0, 20, 800.0, 20, 800.0, 20, chi=1.0)
    ucg = rd.get_cg_udf(rd._field_dict(udf), binders, 6, [pcg])
    np.random.seed(21)
    mods = np.vstack([g["mods"], g["mods"]])[:64]
    ref0, _ = quiet(rd.refine_chromatin, pcg, 64, 16.5, mods, ucg)
    np.random.seed(21)
    ref1, _ = quiet(rd.refine_chromatin, pcg, 64, 16.5, mods, ucg, binding_equilibration=400,
                    random_seed=3)
    np.testing.assert_array_equal(ref1.r, ref0.r.astype(np.float32))
    sites = [cb.get_by_name(nm).sites_per_bead for nm in ("HP1", "PRC1")]
    assert np.all(ref1.states >= 0) and np.all(ref1.states <= np.array(sites))
    assert ref1.states.sum() > 0
