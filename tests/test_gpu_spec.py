"""Several moves in flight per replica give exactly the sequential result.

The production kernel evaluates up to W moves of a cycle at once and commits
the longest prefix free of conflicts with earlier accepted moves.  With each
move's random numbers drawn from its own sub-stream, the outcome must equal
that of W = 1 (one move at a time) bit for bit: positions, binding states,
the fixed-point grid, controller amplitudes, counters and tallies.
"""
import numpy as np
import pytest

from chromo_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _small(nrep=6, n=1500, nbins=12, nb=2):
    w = wl.make_workload("batched")
    rng = np.random.default_rng(5)
    w.lengths = np.full(nrep, n)
    w.replicas = nrep
    w.nbins = nbins
    w.mu = rng.uniform(-1, 0, size=(nrep, nb))
    w.chi = np.linspace(0.5, 2.0, nrep)
    w.n_binders = nb
    w.eps = [-4.0, -3.0][:nb]
    w.cross = [{"PRC1": 1.0}, {}][:nb]
    return w


SHAPES_FP32 = [(1, 32), (2, 32), (4, 32), (8, 32), (1, 16), (3, 16), (6, 16), (1, 8), (4, 8), (8, 8)]
SHAPES_FP64 = [(1, 32), (2, 32), (4, 32), (8, 32)]


@pytest.mark.parametrize("fp64", [False, True])
def test_moves_in_flight_equal_sequential(fp64):
    """Every launch shape (W warps of 32 / G moves each, up to 32 moves in
    flight) against one move at a time (W = 1, G = 32)."""
    w = _small()
    chains = wl.make_chains(w)
    out = {}
    shapes = SHAPES_FP64 if fp64 else SHAPES_FP32
    for W, G in shapes:
        sim = wl.build_sim(w, chains, pos_fp64=fp64, warps_per_block=W, lanes_per_move=G)
        assert sim.launch_shape()[:3] == (W, G, W * 32 // G)
        sim.run(6, 99)
        sim.sync()
        out[(W, G)] = ([sim.get_chain(r) for r in range(w.replicas)],
                  [sim.density(r) for r in range(w.replicas)],
                  [[(c.amp_move, c.amp_bead, c.num_attempt, c.num_success, c.acc_rate)
                    for c in sim.get_controllers(r)] for r in range(w.replicas)],
                  np.stack([sim.tally(r) for r in range(w.replicas)]))
        sim.close()
    base = out[(1, 32)]
    for shape in shapes[1:]:
        chains_w, dens_w, ctl_w, tal_w = out[shape]
        for r in range(w.replicas):
            for a, b in zip(base[0][r], chains_w[r]):
                np.testing.assert_array_equal(a, b)
            np.testing.assert_array_equal(base[1][r], dens_w[r])
            assert base[2][r] == ctl_w[r]
        np.testing.assert_array_equal(base[3], tal_w)


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_grid_consistent_after_parallel_run(lanes):
    w = _small(nrep=4, n=3000, nbins=16)
    sim = wl.build_sim(w, warps_per_block=8, lanes_per_move=lanes)
    sim.run(10, 3)
    sim.sync()
    inc = [sim.density(r) for r in range(w.replicas)]
    sim.deposit(-1)
    for r in range(w.replicas):
        np.testing.assert_array_equal(sim.density(r), inc[r])


def test_smaller_layout_does_not_break_a_live_simulation():
    """The MC kernel's dynamic shared-memory limit is a per-kernel attribute
    shared by every simulation in the process: creating a simulation with a
    smaller CTA layout (one warp) must leave a live one with a larger layout
    (twelve warps) able to launch."""
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("plain")
    chains = wl.make_chains(w)
    big = wl.build_sim(w, chains, warps_per_block=12)
    small = wl.build_sim(w, chains, warps_per_block=1)
    try:
        small.run(1, 3)
        big.run(1, 3)
        big.sync()
        small.sync()
        assert big.tally(0)[:, 0].sum() > 0
    finally:
        small.close()
        big.close()
