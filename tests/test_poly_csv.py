"""Polymer snapshots in the reference's CSV format (chromo/polymers.pyx:575-758).

The round trip mirrors the reference's tests/test_components.py:10-20: a
straight Chromatin chain written with ``to_file(None)`` and read back with
``from_file(StringIO(...))`` gives the same snapshot.  The layout checks pin
what pandas' ``DataFrame.to_csv`` writes for the reference's two-level
columns (pandas itself is not installed here, so the exact text is a
restatement: two header lines, index column, shortest round-trip floats)."""
from io import StringIO

import numpy as np
import pytest

from chromo_gb300.polymers import Chromatin


def _straight():
    return Chromatin.straight_line_in_x(
        "Chr-1", np.ascontiguousarray(np.array([1.0] * 9), dtype=np.float64),
        states=np.zeros((10, 1), dtype=int), binder_names=np.array(["HP1"]),
        chemical_mods=np.zeros((10, 1), dtype=int), chemical_mod_names=np.array(["H3K9me3"]))


def test_polymer_saving_round_trip():
    p = _straight()
    q = Chromatin.from_file(StringIO(p.to_file(None)), "Chr-1")
    assert q.to_csv(None) == p.to_csv(None)
    for a in ("r", "t3", "t2", "states", "chemical_mods", "bead_length"):
        np.testing.assert_array_equal(getattr(q, a), getattr(p, a))
    assert list(q.binder_names) == ["HP1"] and list(q.chemical_mod_names) == ["H3K9me3"]
    assert q.max_binders == p.max_binders and q.name == "Chr-1" and q.lp == p.lp


def test_csv_layout():
    text = _straight().to_csv(None)
    lines = text.splitlines()
    assert lines[0] == (",r,r,r,t3,t3,t3,t2,t2,t2,states,chemical_mods,bead_length,"
                        "max_binders,name,lp")
    assert lines[1] == ",x,y,z,x,y,z,x,y,z,HP1,H3K9me3,,,,"
    assert lines[2] == "0,0.0,0.0,0.0,1.0,0.0,0.0,0.0,1.0,0.0,0,0,1.0,-1,Chr-1,53.0"
    assert lines[3] == "1,1.0,0.0,0.0,1.0,0.0,0.0,0.0,1.0,0.0,0,0,1.0,-1,,"
    assert lines[-1] == "9,9.0,0.0,0.0,1.0,0.0,0.0,0.0,1.0,0.0,0,0,0.0,-1,,"
    assert len(lines) == 12


def test_random_chain_round_trip_is_exact(tmp_path):
    rng = np.random.default_rng(4)
    n = 200
    r = np.cumsum(rng.normal(size=(n, 3)) * 9.5, axis=0)
    t3 = rng.normal(size=(n, 3))
    t3 /= np.linalg.norm(t3, axis=1, keepdims=True)
    t2 = np.cross(t3, rng.normal(size=(n, 3)))
    t2 /= np.linalg.norm(t2, axis=1, keepdims=True)
    p = Chromatin("chain", r, bead_length=np.full(n - 1, 16.5), t3=t3, t2=t2,
                  states=rng.integers(0, 3, size=(n, 2)), binder_names=np.array(["HP1", "PRC1"]),
                  chemical_mods=rng.integers(0, 3, size=(n, 2)),
                  chemical_mod_names=np.array(["H3K9me3", "H3K27me3"]), max_binders=3)
    path = tmp_path / "chain-0.csv"
    p.to_csv(str(path))
    q = Chromatin.from_file(str(path))
    assert q.name == "chain-0"
    for a in ("r", "t3", "t2", "states", "chemical_mods", "bead_length"):
        np.testing.assert_array_equal(getattr(q, a), getattr(p, a))
    assert q.max_binders == 3


@pytest.mark.gpu
def test_polymer_in_field_writes_csv_snapshots(tmp_path):
    from chromo_gb300.mc import get_amplitude_bounds, polymer_in_field
    from golden_cases import load
    from test_gpu_api import _setup
    p, binders, f, ctrls = _setup(load("one_binder"))
    bab, mab = get_amplitude_bounds([p])
    snaps = polymer_in_field([p], binders, f, 3, 2, bab, mab, ctrls, random_seed=5,
                             output_dir=tmp_path)
    assert len(snaps) == 2
    for i in range(2):
        q = type(p).from_file(str(tmp_path / f"{p.name}-{i}.csv"))
        np.testing.assert_array_equal(q.r, snaps[i][0]["r"])
        np.testing.assert_array_equal(q.states, snaps[i][0]["states"])
    np.testing.assert_array_equal(q.r, p.r)


@pytest.mark.gpu
def test_polymer_in_field_segments_continue_one_resident_simulation(tmp_path):
    """polymer_in_field runs its segments on one resident simulation: segment i
    is num_save_mc steps with the i-th seed drawn from random_seed and the
    i-th mu_schedule factor, continuing the device state (chains, grid,
    controllers, move counter) of segment i - 1.  The snapshots (and their
    CSV files, written in the background) equal those of the same runs made
    by hand on one Sim."""
    from chromo_gb300.mc import get_amplitude_bounds, polymer_in_field
    from chromo_gb300.mc.mc_sim import _binding_struct, _device
    from golden_cases import load
    from test_gpu_api import _setup

    class Sched:
        @staticmethod
        def function(i, n):
            return 1.0 - 0.2 * i

    g = load("two_binders")
    p, binders, f, ctrls = _setup(g)
    bab, mab = get_amplitude_bounds([p])
    snaps = polymer_in_field([p], binders, f, 4, 3, bab, mab, ctrls, random_seed=9,
                             mu_schedule=Sched, output_dir=tmp_path)
    q, _, f2, ctrls2 = _setup(load("two_binders"))  # fresh arrays: the run above moved p's
    np.random.seed(9)
    sim = _device(q, f2, ctrls2)
    try:
        for i in range(3):
            seed = np.random.randint(0, 1E9)
            q.mu_adjust_factor = Sched.function(i, 3)
            sim.set_binding(0, _binding_struct(q))
            sim.run(4, seed)
            sim.sync()
            r, t3, t2, st = sim.get_chain(0)
            np.testing.assert_array_equal(snaps[i][0]["r"], r)
            np.testing.assert_array_equal(snaps[i][0]["t3"], t3)
            np.testing.assert_array_equal(snaps[i][0]["states"], st)
            c = type(p).from_file(str(tmp_path / f"{p.name}-{i}.csv"))
            np.testing.assert_array_equal(c.r, r)
        dev = sim.get_controllers(0, len(ctrls))
        for ctrl, d in zip(ctrls, dev):
            assert ctrl.move.amp_bead == int(d.amp_bead) and ctrl.move.num_attempt == int(d.num_attempt)
    finally:
        sim.close()
