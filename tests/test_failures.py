"""Failure detection, with every failure made on the host.

The reference raises Python exceptions (ValueError from bead selection,
chromo/util/bead_selection.pyx:86-89); here the C ABI returns cg_status codes
that the Python layer raises.  Nothing in this file makes a GPU fault: the
failures are bad host inputs rejected before any upload, a random stream cut
short (the audit kernel bounds every read of it and reports the shortfall),
a window the kernel refuses, and energies from a stand-in object."""
import numpy as np
import pytest

from golden_cases import gpu_sim, load


def test_oracle_reports_a_window_larger_than_the_chain():
    """Planted in the oracle: a bead amplitude above the chain length is the
    reference's ValueError (chromo/util/bead_selection.pyx:86-89)."""
    from golden_cases import oracle_system
    from oracle.oracle import make_ctl
    g = load("one_binder")
    o = oracle_system(g, pos="f64", fixed_density=0)
    if int(g["field_kind"]) == 2:
        o.deposit_all()
    n = int(g["r0"].shape[0])
    ctl = make_ctl("slide", amp_move=1.0, amp_bead=n + 5, num_per_cycle=1, simple=False,
                   bead_bounds=(1, n + 5), move_bounds=(0.5, 1.5))
    with pytest.raises(ValueError):
        o.mc_sim([ctl], 1, g["draws"], g["bstates"].astype(np.int64))


def test_replica_batch_argument_checks_need_no_gpu():
    from chromo_gb300.batched import ReplicaBatch
    with pytest.raises(ValueError):
        ReplicaBatch([], [])
    with pytest.raises(ValueError):
        ReplicaBatch([object()], [object(), object()])


def test_drift_check_raises_on_drift():
    """check_drift against energies from a stand-in for the device handle."""
    from chromo_gb300.batched import EnergyDriftError, ReplicaBatch

    class FakeSim:
        def __init__(self):
            self.e = np.array([[10.0, -2.0, 5.0, 0.0, 1.0], [1.0, 0.0, 0.0, 0.0, 0.0]])

        def energies(self):
            return self.e.copy()

        def reset_running_energy(self):
            self.e[:, 3] = 0.0

    b = ReplicaBatch.__new__(ReplicaBatch)
    b.sim = FakeSim()
    b.rebaseline()
    b.sim.e[0, 0] += 3.0            # energy moved by 3 ...
    b.sim.e[0, 3] += 3.0            # ... and the accepted dE say 3: no drift
    b.sim.e[1, 2] += 0.5            # replica 1 moved by 0.5 with no dE recorded
    np.testing.assert_allclose(b.energy_drift(), [0.0, 0.5])
    with pytest.raises(EnergyDriftError, match=r"replicas \[1\]"):
        b.check_drift(rel_tol=1e-3)
    b.sim.e[1, 3] += 0.5
    b.check_drift(rel_tol=1e-12)


def test_negative_step_count_is_rejected_before_any_device_work():
    from chromo_gb300.mc import mc_sim
    with pytest.raises(ValueError):
        mc_sim([object()], None, -1, [object()], None, 1.0, 0)


@pytest.mark.gpu
def test_non_finite_positions_are_rejected_on_upload():
    from chromo_gb300 import _native as nat
    g = load("one_binder")
    sim = gpu_sim(g, pos_fp64=False)
    try:
        r = g["r0"].copy()
        r[3, 1] = np.nan
        with pytest.raises(nat.CgError) as ei:
            sim.set_chain(0, r=r, t3=g["t30"], t2=g["t20"], states=g["states0"])
        assert ei.value.code == -5
        # the handle stays usable
        sim.run(1, 3)
        sim.sync()
    finally:
        sim.close()


@pytest.mark.gpu
def test_short_random_stream_reports_cg_err_stream():
    from chromo_gb300 import _native as nat
    g = load("one_binder")
    sim = gpu_sim(g, pos_fp64=True)
    try:
        with pytest.raises(nat.CgError) as ei:
            sim.run_audit(0, int(g["n_steps"]), g["draws"][:50], g["bstates"])
        assert ei.value.code == -4
    finally:
        sim.close()


@pytest.mark.gpu
def test_window_larger_than_chain_is_a_value_error():
    """A slide window of 120 beads on a 100-bead chain: the kernel stops with
    CG_ERR_WINDOW, raised as a ValueError like the reference's bead selection."""
    from chromo_gb300 import workloads as wl
    from chromo_gb300.device import move_ctl
    w = wl.Workload("window", np.array([100]), 10, 1, np.array([[-0.4]]), np.array([1.0]),
                    [-4.0], [{}], 20, 0, wl.BASE_SEED + 21)
    sim = wl.build_sim(w)
    try:
        ctl = move_ctl("slide", amp_move=5.0, amp_bead=120, num_per_cycle=1, simple=False,
                       bead_bounds=(1, 120), move_bounds=(1.0, 10.0))
        sim.set_controllers(0, [ctl])
        with pytest.raises(ValueError):
            sim.run(1, 1)
            sim.sync()
    finally:
        sim.close()
