"""The on-device FP64 drift guard of the batched rounds (cg_set_drift_guard).

Every k-th round recomputes each replica's full FP64 energy on the device and
compares its change with the running sum of accepted dE plus the energy
change of the replica's accepted chi / mu swaps.

* Accounting: with FP64 storage and no tangent-rotation moves (whose summed
  dE is not the energy change for adjacent beads, chromo/polymers.pyx:
  1074-1080) the two agree to rounding, through chi swaps along ladders and
  mu swaps along a mu ladder, so the guard's measured drift is below
  1e-9 * |E| and it never trips.
* Failure detection: a replica whose uploaded chain is corrupted on the host
  (one bead moved 60 nm and the grid not rebuilt) trips the guard at the
  next check: the round's cg_sync returns CG_ERR_DRIFT, that replica's drift
  is large and the others' stay small.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _guarded_sim(pos_fp64, mu_rungs=0):
    from chromo_gb300 import workloads as wl
    R = 16
    rng = np.random.default_rng(41)
    chi = np.tile(np.linspace(0.5, 2.0, 4), R // 4)
    mu = rng.uniform(-1.0, 0.0, size=(R, 2))
    if mu_rungs:  # slots [grid][mu rung][chi rung]
        mu[:, 0] = np.tile(np.repeat(np.linspace(-1.0, 0.0, mu_rungs), 4), R // (4 * mu_rungs))
    w = wl.Workload("guard", np.full(R, 1500), 16, 2, mu, chi, [-4.0, -3.0], [{"PRC1": 1.0}, {}], 50, 4,
                    wl.BASE_SEED + 21, steps_per_round=10, mu_rungs=mu_rungs)
    sim = wl.build_sim(w, pos_fp64=pos_fp64)
    if mu_rungs:
        sim.set_mu_ladder(mu_rungs, 0)
    return w, sim


def _no_tangent(sim, w):
    for r in range(w.replicas):
        ctl = sim.get_controllers(r)
        ctl[3].move_on = 0
        sim.set_controllers(r, ctl)


@pytest.mark.parametrize("mu_rungs", [0, 2])
def test_guard_accounting_is_exact_without_tangent_rotation(mu_rungs):
    w, sim = _guarded_sim(pos_fp64=True, mu_rungs=mu_rungs)
    try:
        _no_tangent(sim, w)
        sim.set_drift_guard(2, tol_abs=1e-6, tol_rel=1e-9)
        for _ in range(8):
            sim.run_batched(1, w.steps_per_round, w.n_rungs, 5)
        sim.sync()
        drift, checks = sim.drift()
        E = sim.energies()[:, :3].sum(1)
        assert checks == 4
        assert np.all(np.abs(drift) <= 1e-9 * np.maximum(1.0, np.abs(E)))
        swaps = sim.swap_counts()
        assert swaps["chi_swaps"].sum() > 0
        if mu_rungs:
            assert swaps["mu_swaps"].sum() > 0
    finally:
        sim.close()


def test_guard_trips_on_corrupted_replica():
    from chromo_gb300 import _native as nat
    w, sim = _guarded_sim(pos_fp64=False)
    try:
        sim.set_drift_guard(1, tol_abs=5.0, tol_rel=1e-3)
        for _ in range(3):
            sim.run_batched(1, w.steps_per_round, w.n_rungs, 7)
        sim.sync()
        drift0, checks0 = sim.drift()
        assert checks0 == 3 and np.all(np.abs(drift0) < 5.0)
        bad = 5
        r, t3, t2, st = sim.get_chain(bad)
        r[700] += np.array([60.0, 0.0, 0.0])  # the grid still holds the old position
        sim.set_chain(bad, r=r)
        sim.run_batched(1, w.steps_per_round, w.n_rungs, 7)
        with pytest.raises(nat.CgError) as ei:
            sim.sync()
        assert ei.value.code == -8
        drift, checks = sim.drift()
        assert checks == 4
        assert abs(drift[bad]) > 100.0
        others = np.delete(np.abs(drift), bad)
        assert np.all(others < 5.0)
    finally:
        sim.close()


def test_running_sum_and_guard_through_penalised_start():
    """Three replicas of the confined workload (5,000 beads in 700 nm spheres)
    whose seeded start puts bead weight into surface voxels of tiny accessible
    volume: their first energies carry 1e99 penalties, and the moves that
    leave those voxels have dE of that size.  Those moves stay out of the
    running sum of dE (in an FP64 sum they would absorb every later dE), so
    once the penalties are gone the running sum follows the energy exactly
    again (FP64 storage, tangent rotation off), and the guard, which skips
    the penalised interval, checks the later ones and never trips."""
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("sphere")
    chains = wl.make_chains(w)
    pick = [196, 211, 214]
    sub = wl.Workload("sphere-subset", w.lengths[pick], w.nbins, w.n_binders, w.mu[pick], w.chi[pick],
                      w.eps, w.cross, w.run_length, 3, w.seed, steps_per_round=20,
                      sphere_radius=w.sphere_radius)
    sim = wl.build_sim(sub, [chains[i] for i in pick], pos_fp64=True)
    try:
        _no_tangent(sim, sub)
        E0 = sim.energies()[:, :3].sum(1)
        assert np.all(np.abs(E0) >= 1e20), "the start must carry the 1e99 penalty"
        sim.set_drift_guard(2, tol_abs=1e-6, tol_rel=1e-9)
        for _ in range(12):
            sim.run_batched(1, sub.steps_per_round, sub.n_rungs, 9)
        sim.sync()
        e1 = sim.energies()
        E1 = e1[:, :3].sum(1)
        assert np.all(np.abs(E1) < 1e20), "the penalties are left within 240 MC steps"
        drift, checks = sim.drift()
        assert checks == 6
        assert np.all(np.abs(drift) <= 1e-9 * np.maximum(1.0, np.abs(E1)))
        # a window without penalties (and without chi swaps, which the
        # running sum of move dE does not see): running-sum change == energy change
        sim.run(2 * sub.steps_per_round, 10)
        sim.sync()
        e2 = sim.energies()
        d = (e2[:, :3].sum(1) - E1) - (e2[:, 3] - e1[:, 3])
        assert np.all(np.abs(d) <= 1e-9 * np.maximum(1.0, np.abs(E1))), d
        assert np.abs(e2[:, 3]).max() < 1e20
    finally:
        sim.close()
