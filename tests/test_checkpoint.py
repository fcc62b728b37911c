"""Exact resume of batched runs from a device-state checkpoint.

The reference resumes from a polymer CSV snapshot with fresh random streams
(chromo/mc/__init__.py:167-227), so a resumed run is a different Markov
chain.  ``cg_save_state`` / ``cg_load_state`` (``ReplicaBatch.save_checkpoint``
/ ``load_checkpoint``) keep everything a continued run depends on -- chains,
grids, controllers, every replica's chi and mu slot, its move counter (the
index of its Philox sub-streams) and running dE, the exchange round counter
and swap counts -- so a run split at a checkpoint ends bit for bit where the
uninterrupted run ends.  The layout check refuses an image of another batch.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim():
    from chromo_gb300 import workloads as wl
    R = 16
    rng = np.random.default_rng(9)
    mu = rng.uniform(-1.0, 0.0, size=(R, 2))
    mu[:, 0] = np.tile(np.repeat([-1.0, -0.2], 4), R // 8)
    w = wl.Workload("ckpt", np.full(R, 1200), 12, 2, mu, np.tile(np.linspace(0.5, 2.0, 4), R // 4),
                    [-4.0, -3.0], [{"PRC1": 1.0}, {}], 50, 4, wl.BASE_SEED + 41, steps_per_round=8,
                    mu_rungs=2)
    sim = wl.build_sim(w)
    sim.set_mu_ladder(2, 0)
    return w, sim


def _snapshot(sim, w):
    chains = sim.get_chains()
    return dict(chains=chains, grids=[sim.density(r) for r in range(w.replicas)],
                chi=sim.chi(), mu=sim.mu(0), swaps=sim.swap_counts(),
                ctl=[[(c.amp_move, c.amp_bead, c.acc_rate, c.num_attempt, c.num_success)
                      for c in sim.get_controllers(r)] for r in range(w.replicas)],
                energies=sim.energies())


def _assert_same(a, b):
    for (ra, ta, ua, sa), (rb, tb, ub, sb) in zip(a["chains"], b["chains"]):
        np.testing.assert_array_equal(ra, rb)
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(sa, sb)
    for ga, gb in zip(a["grids"], b["grids"]):
        np.testing.assert_array_equal(ga, gb)
    np.testing.assert_array_equal(a["chi"], b["chi"])
    np.testing.assert_array_equal(a["mu"], b["mu"])
    for k in a["swaps"]:
        np.testing.assert_array_equal(a["swaps"][k], b["swaps"][k])
    assert a["ctl"] == b["ctl"]
    np.testing.assert_array_equal(a["energies"], b["energies"])


def test_split_run_resumes_bit_for_bit(tmp_path):
    w, sim = _sim()
    try:
        for _ in range(3):
            sim.run_batched(1, w.steps_per_round, w.n_rungs, 77)
        sim.sync()
        image = sim.save_state()
        for _ in range(4):
            sim.run_batched(1, w.steps_per_round, w.n_rungs, 77)
        sim.sync()
        straight = _snapshot(sim, w)
    finally:
        sim.close()
    w, sim2 = _sim()
    try:
        path = tmp_path / "state.npy"
        np.save(path, image)
        sim2.load_state(np.load(path))
        for _ in range(4):
            sim2.run_batched(1, w.steps_per_round, w.n_rungs, 77)
        sim2.sync()
        resumed = _snapshot(sim2, w)
    finally:
        sim2.close()
    _assert_same(straight, resumed)
    assert straight["swaps"]["chi_swaps"].sum() > 0 and straight["swaps"]["mu_swaps"].sum() > 0


def test_image_of_another_layout_is_refused():
    from chromo_gb300 import _native as nat
    from chromo_gb300 import workloads as wl
    w, sim = _sim()
    try:
        image = sim.save_state()
    finally:
        sim.close()
    other = wl.build_sim(wl.Workload("other", np.full(8, 1200), 12, 2, np.zeros((8, 2)), np.ones(8),
                                     [-4.0, -3.0], [{}, {}], 50, 0, wl.BASE_SEED + 42))
    try:
        with pytest.raises(nat.CgError) as ei:
            other.load_state(image)
        assert ei.value.code == -1 and "layout" in str(ei.value)
    finally:
        other.close()
