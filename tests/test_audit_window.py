"""A 1e4-move audit window on the 10,000-bead plain configuration.

The plain GPU-scale configuration (one chain of 10,000 beads, 60^3 grid of
40 nm voxels, one binder, all five moves under SimpleControl) is run for 63
MC steps (10,143 attempted moves) from shared supplied random streams by
the GPU audit kernel and by the oracle, the C restatement of the reference's
loop that is pinned bit for bit to the reference on the golden cases:

* FP64 storage: every move's polymer and field dE within 1e-9 relative, the
  same decisions, and the same final chain, controllers and density grid;
* FP32 storage (the production arithmetic): every move's dE within
  1e-5 * max(1, |dE|) of the oracle's FP64 evaluation of the same proposal,
  decisions identical outside the tie band |dE + ln u| <= 1e-5 max(1, |dE|),
  and, if no tie flips a decision, the same final state bit for bit.

The streams are seeded numpy draws in the role of libc rand() (31-bit) and
of numpy's binding-state draws; nothing here needs the reference itself.
"""
import numpy as np
import pytest

from golden_cases import MOVE_NAMES, gpu_sim, oracle_ctls, oracle_system

pytestmark = pytest.mark.gpu
N_STEPS = 63


def window_case(seed=20261204):
    """The plain 10,000-bead configuration as a golden-case dictionary."""
    from chromo_gb300 import workloads as wl
    from chromo_gb300.energetics import dss_parameters, field_prefactors
    w = wl.make_workload("plain")
    c = wl.make_chains(w)[0]
    n, nb = int(w.lengths[0]), w.n_binders
    rng = np.random.default_rng(seed)
    states = rng.integers(0, 3, size=(n, nb)).astype(np.int64)
    _, eb, gam, ep, epp, eta = dss_parameters(np.full(n - 1, wl.BEAD_SPACING), wl.LP)
    vint = 4.0 / 3.0 * np.pi * wl.R_INT ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint] * nb, w.cross, wl.binder_names(nb), wl.VOXEL ** 3)
    bead, move = wl.amplitude_bounds(n)
    ctl0 = np.array([(move[m][0], bead[m][0], wl.NUM_PER_CYCLE[m], 1, bead[m][0], bead[m][1],
                      move[m][0], move[m][1]) for m in MOVE_NAMES], dtype=np.float64)
    width = w.nbins * wl.VOXEL
    g = dict(r0=c.r, t30=c.t3, t20=c.t2, states0=states, marks=c.marks, eps_bend=eb, gamma=gam,
             eps_par=ep, eps_perp=epp, eta=eta, sites=np.array([wl.SITES] * nb),
             e_mod=np.array([wl.HP1_E_MOD] * nb), e_nomod=np.array([wl.HP1_E_NOMOD] * nb),
             mu=np.asarray(w.mu[0]), mu_adjust_factor=1.0, max_binders=-1, field_kind=2,
             confine_kind=0, confine_length=0.0, nxyz=np.array([w.nbins] * 3),
             widths=np.array([width] * 3), chi=float(w.chi[0]), vf_limit=0.5, bead_rad=wl.BEAD_RAD,
             pref=np.asarray(pref), intra=np.asarray(intra), xpref=np.asarray(xpref), ctl0=ctl0,
             n_steps=N_STEPS)
    draws = (rng.integers(0, 2 ** 31 - 1, size=600000, dtype=np.int64)).astype(np.uint32)
    bstates = rng.integers(0, 3, size=100000).astype(np.int8)
    return g, draws, bstates


def _dE(recs):
    return recs["dE_poly"] + recs["dE_field"]


def test_fp64_window_matches_oracle_exactly():
    g, draws, bstates = window_case()
    o = oracle_system(g, pos="f64", fixed_density=0)
    o.deposit_all()
    orecs = o.mc_sim(oracle_ctls(g), N_STEPS, draws, bstates.astype(np.int64))
    sim = gpu_sim(g, pos_fp64=True)
    recs, du, bu = sim.run_audit(0, N_STEPS, draws, bstates, max_records=len(orecs) + 8)
    assert len(recs) == len(orecs) >= 10000
    for f in ("kind", "n_inds", "ind0", "indf", "accepted"):
        np.testing.assert_array_equal(recs[f], orecs[f])
    ok = recs["accepted"] >= 0
    a, b = _dE(recs)[ok], _dE(orecs)[ok]
    assert np.all(np.abs(a - b) <= 1e-9 * np.maximum(1.0, np.abs(b)))
    assert du == o.draw_pos and bu == o.bstate_pos
    r, t3, _, st = sim.get_chain(0)
    np.testing.assert_allclose(r, o.r, rtol=0, atol=1e-9)
    np.testing.assert_allclose(t3, o.t3, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(st, o.states)


def test_fp32_window_within_tolerance_of_fp64_oracle():
    g, draws, bstates = window_case()
    o = oracle_system(g, pos="f32", fixed_density=1)
    o.deposit_all()
    orecs = o.mc_sim(oracle_ctls(g), N_STEPS, draws, bstates.astype(np.int64))
    sim = gpu_sim(g, pos_fp64=False)
    recs, du, bu = sim.run_audit(0, N_STEPS, draws, bstates, max_records=len(orecs) + 8)
    n = min(len(recs), len(orecs))
    assert len(orecs) >= 10000
    end = np.cumsum(orecs["n_draws"][:n].astype(np.int64))
    u = draws[np.maximum(end - 1, 0)].astype(np.float64) / 2147483647.0
    dEo = _dE(orecs)[:n]
    with np.errstate(divide="ignore"):
        tie = np.abs(dEo + np.log(u)) <= 1e-5 * np.maximum(1.0, np.abs(dEo))
    flips = np.nonzero(recs["accepted"][:n] != orecs["accepted"][:n])[0]
    stop = flips[0] if len(flips) else n
    if len(flips):
        assert tie[stop], f"decision differs outside the tie band at move {stop}"
    for f in ("kind", "n_inds", "ind0", "indf"):
        np.testing.assert_array_equal(recs[f][:stop + 1], orecs[f][:stop + 1])
    ok = recs["accepted"][:stop] >= 0
    err = np.abs(_dE(recs)[:stop][ok] - dEo[:stop][ok]) / np.maximum(1.0, np.abs(dEo[:stop][ok]))
    print(f"FP32 window: {stop} moves compared, worst relative dE error {err.max():.3e}, "
          f"{int(tie[:n].sum())} moves in the tie band")
    assert err.max() <= 1e-5
    if not len(flips):
        assert len(recs) == len(orecs) and du == o.draw_pos and bu == o.bstate_pos
        r, t3, _, st = sim.get_chain(0)
        np.testing.assert_array_equal(r.astype(np.float32), o.r)
        np.testing.assert_array_equal(t3.astype(np.float32), o.t3)
        np.testing.assert_array_equal(st, o.states)
        np.testing.assert_array_equal(sim.density(0), o.density_fx)
