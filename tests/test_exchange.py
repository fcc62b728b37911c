"""Replica exchange along chi ladders (new here: the reference runs one chain
per simulation).

The device's swap decisions are checked against a host restatement of the
rule: rungs (2i + p, 2i + 1 + p) of each ladder, p = round % 2, swap their chi
iff u < exp((chi_a - chi_b) (S_a - S_b)), with S_r = sum_v (V / V_bead) vf^2
from replica r's fixed-point grid and u = (x >> 1) / (2^31 - 1), x the first
word of Philox4x32-10 at counter (round, rung, 0x3C6EF372) under the seed's
key.  The host Philox is pinned to the published known-answer vectors."""
import numpy as np
import pytest

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    """Philox4x32 with 10 rounds (Salmon et al., SC'11)."""
    c = [int(x) & MASK for x in ctr]
    k = [int(x) & MASK for x in key]
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k[0], p1 & MASK, (p0 >> 32) ^ c[3] ^ k[1], p0 & MASK]
        k = [(k[0] + W0) & MASK, (k[1] + W1) & MASK]
    return c


def test_philox_known_answers():
    """Known-answer vectors published with the Random123 library."""
    assert philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox4x32_10([MASK] * 4, [MASK] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                         [0xA4093822, 0x299F31D0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def exchange_uniform(seed, round_, rung):
    o = philox4x32_10([round_ & MASK, (round_ >> 32) & MASK, rung, 0x3C6EF372],
                      [(seed & MASK) ^ 0xA4093822, (seed >> 32) & MASK])
    return (o[0] >> 1) / 2147483647.0


def chi_free_sum(grid, vol_bin, bead_vol, vf_limit=0.5):
    """S = sum of (V / Vb) vf^2 over the voxels at or below vf_limit: the part of
    the field energy that chi multiplies (a voxel above the limit costs 1e99 vf,
    chromo/fields.pyx:1832-1840, whatever chi is)."""
    vf = (grid[:, 0].astype(np.float64) * 2.0 ** -40) / vol_bin * bead_vol
    keep = ~(vf > vf_limit)
    return float(np.sum((vol_bin / bead_vol) * vf[keep] * vf[keep]))


def expected_exchange(chi, S, rep_of_rung, n_rungs, round_, seed, tie=1e-9):
    """One exchange round on the host; returns (chi, rep_of_rung, n_swaps, ties)."""
    chi, ror = chi.copy(), rep_of_rung.copy()
    parity = round_ & 1
    swaps = ties = 0
    for ladder in range(len(chi) // n_rungs):
        for pair in range(n_rungs // 2):
            if 2 * pair + 1 + parity >= n_rungs:
                continue
            ra = ladder * n_rungs + 2 * pair + parity
            ia, ib = ror[ra], ror[ra + 1]
            x = (chi[ia] - chi[ib]) * (S[ia] - S[ib])
            u = exchange_uniform(seed, round_, ra)
            ties += abs(u - np.exp(x)) < tie
            if u < np.exp(x):
                chi[ia], chi[ib] = chi[ib], chi[ia]
                ror[ra], ror[ra + 1] = ib, ia
                swaps += 1
    return chi, ror, swaps, ties


def _small_ladder_sim(chi=None):
    from chromo_gb300 import workloads as wl
    R = 8
    rng = np.random.default_rng(5)
    w = wl.Workload("exchange", np.full(R, 400), 10, 2, rng.uniform(-1, 0, size=(R, 2)),
                    np.zeros(R) if chi is None else chi, [-4.0, -3.0], [{"PRC1": 1.0}, {}], 50, 4,
                    wl.BASE_SEED + 11)
    return w, wl.build_sim(w)


def _chi_sums(sim, w):
    from chromo_gb300 import workloads as wl
    vol_bin = wl.VOXEL ** 3
    bead_vol = 4.0 / 3.0 * np.pi * wl.BEAD_RAD ** 3
    return np.array([chi_free_sum(sim.density(r), vol_bin, bead_vol) for r in range(w.replicas)])


@pytest.mark.gpu
def test_exchange_rounds_match_host_rule():
    pytest.importorskip("torch")
    w, sim = _small_ladder_sim()
    S0 = _chi_sums(sim, w)
    sim.close()
    # a ladder spacing that makes |(chi_a - chi_b)(S_a - S_b)| of order one
    spread = max(float(np.std(S0)), 1e-12)
    chi = np.tile(np.arange(4) / spread, 2)
    w, sim = _small_ladder_sim(chi)
    try:
        seed = 0x1234_5678_9ABC
        ror = np.arange(w.replicas)
        cur = sim.chi()
        np.testing.assert_array_equal(cur, chi)
        total = 0
        for rnd in range(8):
            sim.run(2, 100 + rnd)
            S = _chi_sums(sim, w)
            want, ror, swaps, ties = expected_exchange(cur, S, ror, 4, rnd, seed)
            sim.exchange(4, rnd, seed)
            got = sim.chi()
            if not ties:
                np.testing.assert_array_equal(got, want)
            cur = got
            total += swaps
        assert 0 < total < 8 * 6, "the rule should both accept and reject some swaps here"
    finally:
        sim.close()


@pytest.mark.gpu
def test_batched_rounds_exchange_after_mc():
    """cg_run_batched: MC then exchange per round, the round number taken from a
    device counter starting at 0; the chi-free sums are those of the grids
    left by the MC kernel."""
    pytest.importorskip("torch")
    w, sim = _small_ladder_sim()
    S0 = _chi_sums(sim, w)
    sim.close()
    chi = np.tile(np.arange(4) / max(float(np.std(S0)), 1e-12), 2)
    w, sim = _small_ladder_sim(chi)
    try:
        seed = 77
        ror = np.arange(w.replicas)
        cur = sim.chi()
        for rnd in range(4):
            sim.run_batched(1, 2, 4, seed)
            sim.sync()
            S = _chi_sums(sim, w)
            want, ror, _, ties = expected_exchange(cur, S, ror, 4, rnd, seed)
            got = sim.chi()
            if not ties:
                np.testing.assert_array_equal(got, want)
            cur = got
    finally:
        sim.close()


def mu_uniform(seed, round_, slot):
    o = philox4x32_10([round_ & MASK, (round_ >> 32) & MASK, slot, 0x5BE0CD19],
                      [(seed & MASK) ^ 0xA4093822, (seed >> 32) & MASK])
    return (o[0] >> 1) / 2147483647.0


def expected_mu_exchange(mu, nbound, ror, n_chi, n_mu, round_, seed, f=1.0, tie=1e-9):
    """The mu pass of one exchange round on the host: slots of each grid are
    (mu rung m, chi rung c) -> (grid * n_mu + m) * n_chi + c; pairs (2i+p,
    2i+1+p) of mu rungs at equal chi rung swap mu iff u < exp(-dE), dE the
    change of sum_r -m(mu_r) N_r, m(mu) = mu (2 - f) for mu > 0 else mu f."""
    mu, ror = mu.copy(), ror.copy()
    parity = round_ & 1
    swaps = ties = 0
    eff = lambda x: x * (2 - f) if x > 0 else x * f
    for grid in range(len(mu) // (n_chi * n_mu)):
        for c in range(n_chi):
            for pair in range(n_mu // 2):
                m = 2 * pair + parity
                if m + 1 >= n_mu:
                    continue
                sa = (grid * n_mu + m) * n_chi + c
                sb = sa + n_chi
                ia, ib = ror[sa], ror[sb]
                na, nb = nbound[ia], nbound[ib]
                dE = eff(mu[ia]) * na + eff(mu[ib]) * nb - eff(mu[ib]) * na - eff(mu[ia]) * nb
                u = mu_uniform(seed, round_, sa)
                ties += abs(u - np.exp(-dE)) < tie
                if u < np.exp(-dE):
                    mu[ia], mu[ib] = mu[ib], mu[ia]
                    ror[sa], ror[sb] = ib, ia
                    swaps += 1
    return mu, ror, swaps, ties


@pytest.mark.gpu
def test_mu_ladder_rounds_match_host_rule():
    """Two-dimensional ladder: 8 replicas as one grid of 4 mu rungs x 2 chi
    rungs; each round swaps chi along the rows, then mu of binder 0 along the
    columns, both against the host restatement of the rules."""
    pytest.importorskip("torch")
    from chromo_gb300 import workloads as wl
    R, n_chi, n_mu = 8, 2, 4
    rng = np.random.default_rng(9)
    mu = np.stack([np.repeat([-0.5, -0.45, -0.4, -0.35], n_chi), rng.uniform(-1, 0, size=R)], axis=1)
    w = wl.Workload("mu_ladder", np.full(R, 400), 10, 2, mu, np.tile([0.8, 1.2], n_mu),
                    [-4.0, -3.0], [{"PRC1": 1.0}, {}], 50, n_chi, wl.BASE_SEED + 12)
    sim = wl.build_sim(w)
    try:
        sim.set_mu_ladder(n_mu, 0)
        seed = 0xBEEF_0001
        ror = np.arange(R)
        chi, cur_mu = sim.chi(), sim.mu(0)
        np.testing.assert_array_equal(cur_mu, mu[:, 0])
        mu_total = 0
        for rnd in range(10):
            sim.run(2, 300 + rnd)
            sim.sync()
            S = _chi_sums(sim, w)
            nbound = np.array([sim.get_chain(r)[3][:, 0].sum() for r in range(R)], dtype=np.float64)
            want_chi, ror, _, ties_c = expected_exchange(chi, S, ror, n_chi, rnd, seed)
            want_mu, ror, swaps, ties_m = expected_mu_exchange(cur_mu, nbound, ror, n_chi, n_mu, rnd, seed)
            sim.exchange(n_chi, rnd, seed)
            sim.sync()
            chi, cur_mu = sim.chi(), sim.mu(0)
            if not (ties_c or ties_m):
                np.testing.assert_array_equal(chi, want_chi)
                np.testing.assert_array_equal(cur_mu, want_mu)
            mu_total += swaps
        # the other binder's mu never moves
        np.testing.assert_array_equal(sim.mu(1), mu[:, 1])
        counts = sim.swap_counts()
        assert int(counts["mu_swaps"].sum()) == mu_total
        assert 0 < mu_total < int(counts["mu_attempts"].sum())
    finally:
        sim.close()


@pytest.mark.gpu
def test_exchange_with_voxel_above_vf_limit():
    """One replica holds a voxel above vf_limit (half its chain packed into one
    voxel).  That voxel's 1e99 vf does not depend on chi, so the true energy
    change of a chi swap is -(chi_a - chi_b)(S_a - S_b) with S over the voxels
    at or below the limit only: the device's S equals that host sum, differs
    from the sum over all voxels, and every swap decision follows it."""
    pytest.importorskip("torch")
    from chromo_gb300 import workloads as wl
    w, sim = _small_ladder_sim()
    S0 = _chi_sums(sim, w)
    sim.close()
    chi = np.tile(np.arange(4) / max(float(np.std(S0)), 1e-12), 2)
    w, sim = _small_ladder_sim(chi)
    try:
        r, t3, t2, st = sim.get_chain(0)
        rng = np.random.default_rng(3)
        r[:200] = 20.0 + rng.uniform(-2.0, 2.0, size=(200, 3))  # 200 beads inside one 40 nm voxel
        sim.set_chain(0, r=r)
        sim.deposit(-1)
        vol_bin, bead_vol = wl.VOXEL ** 3, 4.0 / 3.0 * np.pi * wl.BEAD_RAD ** 3
        g0 = sim.density(0)
        vf = (g0[:, 0].astype(np.float64) * 2.0 ** -40) / vol_bin * bead_vol
        assert vf.max() > 0.5
        S = _chi_sums(sim, w)
        S_all0 = float(np.sum((vol_bin / bead_vol) * vf * vf))
        assert S_all0 > S[0] * 1.5, "the over-limit voxel must matter to the test"
        dev = sim.energies()[:, 4]
        np.testing.assert_allclose(dev, S, rtol=1e-12)
        seed, ror, cur = 4242, np.arange(w.replicas), sim.chi()
        for rnd in range(6):
            S = _chi_sums(sim, w)
            want, ror, _, ties = expected_exchange(cur, S, ror, 4, rnd, seed)
            sim.exchange(4, rnd, seed)
            got = sim.chi()
            if not ties:
                np.testing.assert_array_equal(got, want)
            cur = got
    finally:
        sim.close()
