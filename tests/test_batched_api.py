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


@pytest.mark.parametrize("fp64", [False, True])
def test_chain_transfers_direct_and_staged_agree(fp64, monkeypatch):
    """cg_set_chains / cg_get_chains read and write the caller's arrays from
    the GPU where it can address pageable host memory, else through a pinned
    staging buffer (CHROMO_GB300_STAGED_HOST_IO=1 forces that path).  Both
    give the same resident state and the same arrays back: every replica, a
    partial upload (None entries keep the resident values), and a rejected
    upload (a NaN coordinate, or a state outside 0..3), which changes
    nothing."""
    from chromo_gb300 import _native as nat
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("batched")
    pick = [0, 5, 77, 200]
    sub = wl.Workload("transfer", w.lengths[pick], w.nbins, w.n_binders, w.mu[pick], w.chi[pick], w.eps,
                      w.cross, w.run_length, 2, w.seed)
    chains = wl.make_chains(w)
    chains = [chains[i] for i in pick]
    rng = np.random.default_rng(3)
    new = [dict(r=c.r + rng.normal(size=c.r.shape), t3=c.t3, t2=c.t2,
                states=rng.integers(0, 3, size=c.states.shape)) for c in chains]
    got = {}
    for mode in ("direct", "staged"):
        if mode == "staged":
            monkeypatch.setenv("CHROMO_GB300_STAGED_HOST_IO", "1")
        sim = wl.build_sim(sub, chains, pos_fp64=fp64)
        try:
            sim.set_chains(new)
            part = [dict(r=new[0]["r"] * 0.5), {}, dict(states=np.zeros_like(new[2]["states"])), {}]
            sim.set_chains(part)
            before = sim.get_chains()
            bad = [dict(r=new[k]["r"].copy()) for k in range(4)]
            bad[3]["r"][17, 2] = np.nan
            with pytest.raises(nat.CgError):
                sim.set_chains(bad)
            bad_states = [{}, dict(states=np.full_like(new[1]["states"], 7)), {}, {}]
            with pytest.raises(nat.CgError):
                sim.set_chains(bad_states)
            after = sim.get_chains()
            for x, y in zip(before, after):
                for a, b in zip(x, y):
                    np.testing.assert_array_equal(a, b)
            got[mode] = after
        finally:
            sim.close()
        monkeypatch.delenv("CHROMO_GB300_STAGED_HOST_IO", raising=False)
    for x, y in zip(got["direct"], got["staged"]):
        for a, b in zip(x, y):
            np.testing.assert_array_equal(a, b)
    # the values are the uploads rounded to the storage type
    cast = np.float64 if fp64 else np.float32
    np.testing.assert_array_equal(got["direct"][0][0], (new[0]["r"] * 0.5).astype(cast).astype(np.float64))
    np.testing.assert_array_equal(got["direct"][1][0], new[1]["r"].astype(cast).astype(np.float64))
    np.testing.assert_array_equal(got["direct"][2][3], 0)
    np.testing.assert_array_equal(got["direct"][3][3], new[3]["states"])
