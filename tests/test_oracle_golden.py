"""The CPU oracle replays the reference's own trajectories bit for bit.

The golden cases (tests/golden/*.npz, written by tests/golden/make_golden.py
from the reference's ``mc_sim``) store the libc ``rand()`` values and numpy
binding-state draws the reference consumed.  Fed the same streams, the oracle
must reproduce every attempted move's polymer dE, field dE and decision, and
the final positions, binding states, density grid and move amplitudes.
"""
import numpy as np
import pytest

from golden_cases import CASES, load, oracle_ctls, oracle_system


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference(name):
    g = load(name)
    s = oracle_system(g, pos="f64", fixed_density=0)
    if int(g["field_kind"]) == 2:
        s.deposit_all()
        # field construction deposits every bead (chromo/fields.pyx:2041)
    ctls = oracle_ctls(g)
    recs = s.mc_sim(ctls, int(g["n_steps"]), g["draws"], g["bstates"].astype(np.int64))
    ref = g["records"]
    assert len(recs) == len(ref)
    for f in ("kind", "n_inds", "accepted"):
        np.testing.assert_array_equal(recs[f], ref[f])
    if "eps_twist" in g:
        # the twist angle's dot products go through numpy's BLAS in the
        # reference, whose summation order is unspecified: last-bit differences
        np.testing.assert_allclose(recs["dE_poly"], ref["dE_poly"], rtol=1e-9, atol=1e-12)
    else:
        np.testing.assert_array_equal(recs["dE_poly"], ref["dE_poly"])
    np.testing.assert_array_equal(recs["dE_field"], ref["dE_field"])
    np.testing.assert_array_equal(s.r, g["r1"])
    np.testing.assert_array_equal(s.t3, g["t31"])
    np.testing.assert_array_equal(s.t2, g["t21"])
    np.testing.assert_array_equal(s.states, g["states1"])
    if int(g["field_kind"]) == 2:
        np.testing.assert_array_equal(s.density, g["density1"])
    final = np.array([(c.amp_move, c.amp_bead, c.num_attempt, c.num_success, c.acc_rate)
                      for c in ctls])
    np.testing.assert_array_equal(final, g["ctl_final"])
    assert s.draw_pos == len(g["draws"])
    assert s.bstate_pos == len(g["bstates"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_elastic_energy_matches_reference(name):
    g = load(name)
    s = oracle_system(g, pos="f64", fixed_density=0, state="1")
    e_el, _, _ = s.energies()
    assert e_el == pytest.approx(float(g["E_elastic1"]), rel=1e-12)


@pytest.mark.parametrize("name", [c for c in CASES if c != "null_spherical"])
def test_oracle_fixed_point_tracks_fp64(name):
    """The fixed-point density mode (the GPU's storage) gives the same
    decisions and dE within 1e-9 on the reference's trajectory."""
    g = load(name)
    if name == "vf_limit":
        pytest.skip("above vf_limit the reference's dE is 1e99-scale cancellation noise")
    s = oracle_system(g, pos="f64", fixed_density=1)
    s.deposit_all()
    recs = s.mc_sim(oracle_ctls(g), int(g["n_steps"]), g["draws"], g["bstates"].astype(np.int64))
    ref = g["records"]
    np.testing.assert_array_equal(recs["accepted"], ref["accepted"])
    dE = recs["dE_poly"] + recs["dE_field"]
    dE_ref = ref["dE_poly"] + ref["dE_field"]
    assert np.all(np.abs(dE - dE_ref) <= 1e-9 * np.maximum(1, np.abs(dE_ref)))
