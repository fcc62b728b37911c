"""ReplicaBatch: many chains, each in its own field, through the Python API."""
import numpy as np
import pytest

from chromo_gb300.batched import EnergyDriftError, ReplicaBatch
from golden_cases import load
from test_gpu_api import _setup

pytestmark = pytest.mark.gpu


def _batch(R=4, case="one_binder", precision="fp32", tangent=True, chis=None):
    polys, fields, ctrls = [], [], []
    for r in range(R):
        # a fresh load per chain: polymers keep the arrays they are given (no
        # copy, as in the reference), so chains built from one array would alias
        p, _, f, c = _setup(load(case))
        if chis is not None:
            f.chi = float(chis[r])
        if not tangent:
            for ctl in c:
                if ctl.move.name == "tangent_rotation":
                    ctl.move.move_on = 0
        polys.append(p)
        fields.append(f)
        ctrls.append(c)
    return ReplicaBatch(polys, fields, ctrls, precision=precision), polys, fields, ctrls


def test_run_then_pull_updates_host_objects():
    b, polys, fields, ctrls = _batch()
    with b:
        r0 = [p.r.copy() for p in polys]
        b.run(5, 123)
        b.sync()
        b.pull()
        for r, (p, f, c) in enumerate(zip(polys, fields, ctrls)):
            rr, _, _, st = b.sim.get_chain(r)
            np.testing.assert_array_equal(p.r, rr)
            np.testing.assert_array_equal(p.states, st)
            np.testing.assert_array_equal(f.density_fixed_point, b.sim.density(r))
            assert not np.array_equal(p.r, r0[r])
            assert all(ctl.move.num_attempt > 0 for ctl in c if ctl.move.move_on)
        # replicas share the chain but not the random streams
        assert not np.array_equal(polys[0].r, polys[1].r)


def test_fp64_energy_drift_is_rounding_only_without_tangent_rotation():
    """With FP64 storage and no tangent_rotation (whose reference rule for
    adjacent beads is not an exact energy difference), the running sum of
    accepted dE tracks the recomputed energy to rounding."""
    b, *_ = _batch(precision="fp64", tangent=False)
    with b:
        b.run(20, 7)
        b.sync()
        drift = b.check_drift(rel_tol=1e-9)
        assert np.all(np.isfinite(drift))
        assert np.any(b.energies()[:, 3] != 0.0)


def test_fp32_drift_is_small_and_reported():
    b, *_ = _batch(precision="fp32")
    with b:
        b.run(20, 9)
        b.sync()
        e = b.energies()
        E = e[:, 0] + e[:, 1] + e[:, 2]
        drift = b.energy_drift()
        assert np.all(np.abs(drift) <= 1e-3 * np.maximum(1.0, np.abs(E)))
        if np.any(drift != 0.0):
            with pytest.raises(EnergyDriftError):
                b.check_drift(rel_tol=0.0)


def test_run_exchange_permutes_chi_within_ladders():
    chis = [0.5, 1.0, 1.5, 2.0]
    b, polys, fields, _ = _batch(chis=chis)
    with b:
        np.testing.assert_array_equal(b.chi, chis)
        b.run_exchange(4, 2, 2, 31)
        got = b.chi
        # ladders of two rungs: replicas (0, 1) and (2, 3) can only trade with each other
        assert sorted(got[:2]) == chis[:2] and sorted(got[2:]) == chis[2:]
        b.pull()
        assert [f.chi for f in fields] == list(got)
        assert np.all(np.abs(b.energy_drift()) < 1e-12)  # rebaselined after the swaps


def test_all_replica_transfers_match_per_replica_calls():
    """cg_set_chains / cg_get_chains move the same data as R single-replica calls."""
    b, polys, _, _ = _batch(R=3)
    with b:
        b.run(3, 5)
        b.sync()
        whole = b.sim.get_chains()
        for r in range(3):
            single = b.sim.get_chain(r)
            for x, y in zip(whole[r], single):
                np.testing.assert_array_equal(x, y)
        # push the host chains (the initial state) back and read them again
        b.push()
        again = b.sim.get_chains(out=whole)  # filled in place
        assert again is whole
        for r, p in enumerate(polys):
            np.testing.assert_array_equal(again[r][0], p.r.astype(np.float32).astype(np.float64))
            np.testing.assert_array_equal(again[r][3], p.states)
