"""Launch-shape autotuner: candidate shapes, the per-problem cache, and (on
the GPU) that the tuned shape is the fastest one timed and that a tuned batch
follows exactly the trajectory of an untuned one (every shape gives the
one-move-at-a-time result)."""
import json

import numpy as np
import pytest

from chromo_gb300 import autotune as at


def test_candidates_keep_every_replica_resident():
    wps = {32: 12, 16: 12, 8: 12}
    # 256 replicas on 152 SMs: two CTAs per SM, at most 6 warps each
    c = at.candidates(256, 152, False, wps)
    assert (6, 32) in c and (6, 16) in c and (6, 8) in c
    assert all(w <= 6 and w * 32 // g <= 32 for w, g in c)
    # 32 replicas: one CTA per SM, up to 12 warps (8 with 8 lanes per move: 32 moves in flight)
    c = at.candidates(32, 152, False, wps)
    assert (12, 32) in c and (12, 16) in c and (8, 8) in c and (12, 8) not in c
    # FP64 storage: 32 lanes per move only
    assert {g for _, g in at.candidates(32, 152, True, {32: 12})} == {32}


def test_problem_key_is_stable_and_discriminating():
    k1 = at.problem_key([2000, 5000, 20000], [[40, 40, 40]] * 3, 2, False, 152, "GB300")
    k2 = at.problem_key([2000, 5000, 20000], [[40, 40, 40]] * 3, 2, False, 152, "GB300")
    k3 = at.problem_key([2000, 5000, 20000], [[40, 40, 40]] * 3, 2, True, 152, "GB300")
    assert k1 == k2 and k1 != k3
    assert json.loads(k1)["R"] == 3


def test_cached_shape_is_returned_without_timing(tmp_path, monkeypatch):
    monkeypatch.setenv("CHROMO_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    lengths, grids = [3000] * 4, [[16, 16, 16]] * 4
    key = at.problem_key(lengths, grids, 2, False, 152, "fake")
    (tmp_path / "tune.json").write_text(json.dumps({key: {"shape": [5, 16], "table": {"5x16": 1.0}}}))

    def build(w, g):
        raise AssertionError("a cached problem must not be timed")

    shape, table = at.tune(build, lengths, grids, 2, device=("fake", 152))
    assert shape == (5, 16) and table == {"5x16": 1.0}


@pytest.mark.gpu
def test_tuned_shape_is_fastest_and_trajectory_is_unchanged(tmp_path, monkeypatch):
    monkeypatch.setenv("CHROMO_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("batched")
    rng = np.random.default_rng(3)
    w.lengths = np.full(8, 2500)
    w.replicas = 8
    w.nbins = 16
    w.mu = rng.uniform(-1, 0, size=(8, 2))
    w.chi = np.linspace(0.5, 2.0, 8)
    chains = wl.make_chains(w)
    build = lambda W, G: wl.build_sim(w, chains, warps_per_block=W, lanes_per_move=G)
    shapes = [(2, 32), (4, 32), (4, 16)]
    shape, table = at.tune(build, w.lengths, [[16] * 3] * 8, 2, shapes=shapes, steps=2, warmup=1)
    assert set(table) == {"2x32", "4x32", "4x16"}
    assert table[f"{shape[0]}x{shape[1]}"] == max(table.values())
    out = []
    for W, G in [shape, (1, 32)]:
        sim = build(W, G)
        sim.run(3, 11)
        sim.sync()
        out.append([sim.get_chain(r)[0] for r in range(8)])
        sim.close()
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)
