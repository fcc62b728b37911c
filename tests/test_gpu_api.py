"""The drop-in Python API (chromo_gb300.polymers / fields / mc) on the GPU.

Written like the reference's own usage: build a Chromatin chain, binders and a
UniformDensityField through the same constructors, make controllers with
``all_moves``, and call ``mc_sim``.
"""
import numpy as np
import pytest

import chromo_gb300.binders as cb
from chromo_gb300.fields import NullField, UniformDensityField
from chromo_gb300.mc import get_amplitude_bounds, mc_sim, mc_sim_audit
from chromo_gb300.mc.mc_controller import NoControl, SimpleControl, all_moves, specific_moves
import chromo_gb300.mc.move_funcs as mf
from golden_cases import CASES, MOVE_NAMES, load
from test_api_host import _poly_from_golden

pytestmark = pytest.mark.gpu


def _setup(g):
    p, binders = _poly_from_golden(g)
    if int(g["field_kind"]) == 2:
        n = [int(x) for x in g["nxyz"]]
        w = [float(x) for x in g["widths"]]
        ct = {0: "", 1: "Spherical", 2: "Cubical"}[int(g["confine_kind"])]
        f = UniformDensityField([p], binders, w[0], n[0], w[1], n[1], w[2], n[2],
                                confine_type=ct, confine_length=float(g["confine_length"]),
                                chi=float(g["chi"]), vf_limit=float(g["vf_limit"]),
                                assume_fully_accessible=0 if "access_vols" in g else 1,
                                fast_field=1 if "fast_n" in g else 0,
                                n_points=int(g.get("fast_n", 1000)))
    else:
        ct = {1: "Spherical", 2: "Cubical"}[int(g["confine_kind"])]
        f = NullField([p], confine_type=ct, confine_length=float(g["confine_length"]))
    bab, mab = get_amplitude_bounds([p])
    ctl0 = g["ctl0"]
    if all(int(r[3]) == 1 for r in ctl0):
        ctrls = all_moves("/tmp/logs", bab.bounds, mab.bounds, SimpleControl)
    else:
        bead = {MOVE_NAMES[k]: (r[4], r[5]) for k, r in enumerate(ctl0)}
        move = {MOVE_NAMES[k]: (r[6], r[7]) for k, r in enumerate(ctl0)}
        ctrls = specific_moves([getattr(mf, m) for m in MOVE_NAMES], "/tmp/logs", bead, move,
                               NoControl)
    for c, row in zip(ctrls, ctl0):
        assert c.move.amp_bead == int(row[1]) and c.move.amp_move == pytest.approx(row[0])
    return p, binders, f, ctrls


@pytest.mark.parametrize("name", [c for c in CASES if c != "vf_limit"])
def test_mc_sim_audit_reproduces_reference(name):
    """Through the public API with FP64 positions, the same random streams give
    the reference's per-move records, final chain and move amplitudes."""
    g = load(name)
    p, binders, f, ctrls = _setup(g)
    recs, du, bu = mc_sim_audit([p], binders, int(g["n_steps"]), ctrls, f,
                                float(g["mu_adjust_factor"]), g["draws"], g["bstates"],
                                precision="fp64")
    ref = g["records"]
    np.testing.assert_array_equal(recs["accepted"], ref["accepted"])
    np.testing.assert_array_equal(recs["n_inds"], ref["n_inds"])
    dE, dEr = recs["dE_poly"] + recs["dE_field"], ref["dE_poly"] + ref["dE_field"]
    assert np.all(np.abs(dE - dEr) <= 1e-9 * np.maximum(1, np.abs(dEr)))
    np.testing.assert_allclose(p.r, g["r1"], rtol=0, atol=1e-9)
    np.testing.assert_array_equal(p.states, g["states1"])
    for c, row in zip(ctrls, g["ctl_final"]):
        assert c.move.amp_bead == int(row[1])
        assert c.move.amp_move == pytest.approx(row[0], rel=1e-12)
        assert c.move.num_attempt == int(row[2]) and c.move.num_success == int(row[3])
        assert c.move.acceptance_tracker.acceptance_rate == pytest.approx(row[4], rel=1e-12)
    if int(g["field_kind"]) == 2:
        np.testing.assert_allclose(f.density, g["density1"], rtol=1e-9, atol=1e-15)


def test_mc_sim_philox_runs_and_keeps_grid_consistent():
    np.random.seed(3)
    hp1 = cb.get_by_name("HP1")
    hp1.chemical_potential, hp1.interaction_energy = -0.4, -4.0
    hp1.cross_talk_interaction_energy = {}
    binders = cb.make_binder_collection([hp1])
    n = 1000
    marks = np.random.randint(0, 3, (n, 1))
    p = Chromatin_gw(n, marks)
    f = UniformDensityField([p], binders, 1200.0, 30, 1200.0, 30, 1200.0, 30, chi=1.0)
    bab, mab = get_amplitude_bounds([p])
    ctrls = all_moves("/tmp/logs", bab.bounds, mab.bounds, SimpleControl)
    r0 = p.r.copy()
    mc_sim([p], binders, 20, ctrls, f, 1.0, 12345)
    att = [c.move.num_attempt for c in ctrls]
    assert att == [20 * k for k in (30, 1, 60, 60, 10)]
    assert 0 < sum(c.move.num_success for c in ctrls) < sum(att)
    assert not np.array_equal(p.r, r0)
    inc = f.density_fixed_point.copy()
    f._density_fx = None  # recompute from the final positions
    np.testing.assert_array_equal(f.density_fixed_point, inc)
    # the same seed reproduces the same trajectory
    q = Chromatin_gw(n, marks, seed=None, r=r0)
    g2 = UniformDensityField([q], binders, 1200.0, 30, 1200.0, 30, 1200.0, 30, chi=1.0)
    c2 = all_moves("/tmp/logs", bab.bounds, mab.bounds, SimpleControl)
    mc_sim([q], binders, 20, c2, g2, 1.0, 12345)
    np.testing.assert_array_equal(q.r, p.r)
    np.testing.assert_array_equal(q.states, p.states)


def Chromatin_gw(n, marks, seed=7, r=None):
    from chromo_gb300.polymers import Chromatin, estimate_tangents_from_coordinates, gaussian_walk
    if r is None:
        np.random.seed(seed)
        r = gaussian_walk(n - 1, np.full(n - 1, 16.5))
    t3, t2 = estimate_tangents_from_coordinates(r)
    return Chromatin("p", r.copy(), bead_length=np.full(n - 1, 16.5), t3=t3, t2=t2,
                     states=np.zeros((n, 1), dtype=int), binder_names=np.array(["HP1"]),
                     chemical_mods=marks, chemical_mod_names=np.array(["H3K9me3"]))


@pytest.mark.parametrize("name", CASES)
def test_compute_E_matches_reference(name):
    g = load(name)
    p, _ = _poly_from_golden(g, state="1")
    assert p.compute_E() == pytest.approx(float(g["E_elastic1"]), rel=1e-12)
