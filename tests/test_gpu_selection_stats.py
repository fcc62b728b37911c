"""Statistics of the production kernel's bead selection and state draws.

The reference's bead-selection tests are statistical
(tests/test_bead_selection.py:213-313: selections from the left, the right
and a point follow the capped exponential rule).  Here the same rules,
driven by the production kernel's Philox streams, are tested through its
per-move log on a 20,000-bead chain at fixed amplitudes (NoControl):

* end pivot: the end segment's length r (from_left of a window of 150 beads,
  chromo/util/bead_selection.pyx:19-90) follows the exact law of
  r = floor(-log10(u + 1e-5) * 0.45 w + 1.0001), redrawn while r > w;
* slide: the segment length |b1 - b0| of from_point (:115-154) follows the
  same law, for segments clear of the chain ends (weighted by the number of
  start beads that keep them clear);
* tangent rotation: the number of rotated beads is uniform on 1..amp_bead
  (move_funcs.pyx:496-512) and every bead is equally likely to be picked.

(New binding states are checked draw for draw against the oracle's Philox
replay in tests/test_gpu_spec_oracle.py.)

Each is a chi-square test at p > 1e-4 over 1e5 moves (the Philox streams
are fixed, so the outcome is deterministic).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
N, W, SEED = 20000, 150, 424242


def capped_law(w):
    """P(r = k), k = 0..w, of floor(-log10(u + 1e-5) 0.45 w + 1.0001) given r <= w."""
    k = np.arange(w + 2, dtype=np.float64)
    # r >= k  <=>  u <= 10^(-(k - 1.0001) / (0.45 w)) - 1e-5
    upper = np.clip(10.0 ** (-(k - 1.0001) / (0.45 * w)) - 1e-5, 0.0, 1.0)
    p = upper[:-1] - upper[1:]
    return p / p.sum()


def chi2_p(obs, expect):
    from scipy.stats import chisquare
    keep = expect * obs.sum() >= 5
    o = np.append(obs[keep], obs[~keep].sum())
    e = np.append(expect[keep], expect[~keep].sum()) * obs.sum()
    if e[-1] == 0:
        o, e = o[:-1], e[:-1]
    return chisquare(o, e * o.sum() / e.sum()).pvalue


def _chain_sim(kind, amp_bead, npc, amp_move):
    from chromo_gb300 import workloads as wl
    from chromo_gb300.device import move_ctl
    w = wl.Workload("sel", np.array([N]), 40, 1, np.array([[-0.4]]), np.array([1.0]), [-4.0], [{}], 50, 0,
                    wl.BASE_SEED + 31)
    sim = wl.build_sim(w)
    bead, move = wl.amplitude_bounds(N)
    ctls = []
    for m in ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]:
        c = move_ctl(m, amp_move=amp_move if m == kind else move[m][0],
                     amp_bead=amp_bead if m == kind else int(bead[m][0]),
                     num_per_cycle=npc if m == kind else 1, simple=False, bead_bounds=bead[m],
                     move_bounds=move[m])
        c.move_on = 1 if m == kind else 0
        ctls.append(c)
    sim.set_controllers(0, ctls)
    return sim


def _log(kind, amp_bead, amp_move, moves=100000, npc=1000):
    sim = _chain_sim(kind, amp_bead, npc, amp_move)
    try:
        log = sim.run_logged(moves // npc, SEED, moves + 10)[0]
    finally:
        sim.close()
    assert len(log) == moves
    return log


def test_end_pivot_segment_lengths_follow_capped_exponential():
    log = _log("end_pivot", W, 0.05)
    r = np.where(log["ind0"] == 0, log["indf"] - 1, N - log["ind0"])
    assert r.min() >= 0 and r.max() <= W
    p = chi2_p(np.bincount(r, minlength=W + 1).astype(float), capped_law(W))
    left = np.mean(log["ind0"] == 0)
    assert abs(left - 0.5) < 4 * 0.5 / np.sqrt(len(log))
    assert p > 1e-4, p


def test_slide_segment_lengths_follow_capped_exponential():
    log = _log("slide", W, 1.0)
    keep = (log["ind0"] >= W) & (log["indf"] <= N - W)
    n = (log["indf"] - log["ind0"])[keep]
    law = capped_law(W)
    # from_point: length r >= 1 (r = 0 gives b1 = b0, one bead); a segment of
    # length r stays clear of both ends for N - 2W - r + 1 start beads
    lengths = np.arange(W + 1)
    expect = law * (N - 2 * W - lengths + 1)
    expect[1] += expect[0]  # r = 0 and r = 1 both give one bead
    expect[0] = 0
    obs = np.bincount(n, minlength=W + 1).astype(float)
    p = chi2_p(obs[1:], expect[1:] / expect.sum())
    assert p > 1e-4, p


def test_tangent_rotation_counts_and_beads_are_uniform():
    amp = 40
    log = _log("tangent_rotation", amp, 0.01, moves=100000)
    counts = np.bincount(log["n_inds"], minlength=amp + 1)[1:]
    p = chi2_p(counts.astype(float), np.full(amp, 1.0 / amp))
    assert p > 1e-4, p
    # the first picked bead of each move (ind0) is uniform over the chain
    hist = np.bincount(log["ind0"] * 20 // N, minlength=20).astype(float)
    p2 = chi2_p(hist, np.full(20, 1 / 20))
    assert p2 > 1e-4, p2
