"""The oracle's Philox mode: the random numbers of the GPU production kernel.

The production kernel gives every attempted move t of replica `rep` its own
sub-streams (chromo_gb300/csrc/cg_spec.cuh, MoveRng): draw j is word j & 3 of
Philox4x32-10 at counter (j >> 2, t_lo, t_hi, 0x2545F491) under key
(seed_lo ^ rep * 0x85EBCA6B, seed_hi ^ 0x1B873593), shifted right by one (a
31-bit value in the role of libc rand()); binding state k is
umulhi(word at (k >> 2, t_lo, t_hi, 0x7F4A7C15) under key ^ (0x68E31DA4,
0xB5297A4D), sites + 1), in the role of np.random.randint(0, sites + 1).

Pinned here on the CPU: the oracle's Philox block against the published
Random123 known-answer vectors, and its Philox-mode replay against a replay of
the same streams written out by a Python restatement (the supplied-stream mode
that the golden cases pin to the reference).  The GPU side is compared with
the oracle in tests/test_gpu_spec_oracle.py.
"""
import numpy as np
import pytest

from golden_cases import load, oracle_ctls, oracle_system
from oracle import oracle as orc

MASK = 0xFFFFFFFF
M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85


def philox(ctr, key):
    c = [int(x) & MASK for x in ctr]
    k = [int(x) & MASK for x in key]
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k[0], p1 & MASK, (p0 >> 32) ^ c[3] ^ k[1], p0 & MASK]
        k = [(k[0] + W0) & MASK, (k[1] + W1) & MASK]
    return c


def keys(seed, rep):
    key = [(seed & MASK) ^ ((rep * 0x85EBCA6B) & MASK), ((seed >> 32) & MASK) ^ 0x1B873593]
    return key, [key[0] ^ 0x68E31DA4, key[1] ^ 0xB5297A4D]


def move_draws(seed, rep, t, n):
    key, _ = keys(seed, rep)
    out = []
    for j in range(n):
        out.append(philox([j >> 2, t & MASK, t >> 32, 0x2545F491], key)[j & 3] >> 1)
    return out


def move_states(seed, rep, t, n, sites):
    _, keyb = keys(seed, rep)
    return [(philox([k >> 2, t & MASK, t >> 32, 0x7F4A7C15], keyb)[k & 3] * (sites + 1)) >> 32
            for k in range(n)]


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_oracle_philox_known_answers(tag):
    """Known-answer vectors published with the Random123 library."""
    assert orc.philox4x32_10([0, 0, 0, 0], [0, 0], tag) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox4x32_10([MASK] * 4, [MASK] * 2, tag) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
                             tag) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("name", ["two_binders", "anneal_maxb", "null_spherical"])
def test_philox_mode_equals_supplied_streams(name):
    """Philox mode == the supplied-stream mode fed the same numbers, move by
    move (the streams written out per move from the records' draw counts)."""
    g = load(name)
    seed, rep, steps = 0x1234ABCD9876, 3, 6
    o = oracle_system(g, pos="f32", fixed_density=1)
    if int(g["field_kind"]) == 2:
        o.deposit_all()
    recs, t_end, ties = o.mc_sim_philox(oracle_ctls(g), steps, seed, rep, 1000)
    assert ties == 0 and t_end == 1000 + len(recs)
    sites = int(g["sites"].max())
    draws, bstates = [], []
    for k, r in enumerate(recs):
        draws += move_draws(seed, rep, 1000 + k, int(r["n_draws"]))
        if r["kind"] == 4:
            assert np.all(g["sites"] == sites)
            bstates += move_states(seed, rep, 1000 + k, int(r["n_inds"]), sites)
    o2 = oracle_system(g, pos="f32", fixed_density=1)
    if int(g["field_kind"]) == 2:
        o2.deposit_all()
    recs2 = o2.mc_sim(oracle_ctls(g), steps, np.array(draws, dtype=np.uint32),
                      np.array(bstates + [0], dtype=np.int64))
    np.testing.assert_array_equal(recs2, recs)
    np.testing.assert_array_equal(o2.r, o.r)
    np.testing.assert_array_equal(o2.states, o.states)
    np.testing.assert_array_equal(o2.density_fx, o.density_fx)


def test_following_changes_only_tie_band_decisions():
    """Decisions of a followed run replace the oracle's own only inside the tie
    band: following the flipped decisions of the oracle's own run changes none
    of the moves clear of it."""
    g = load("one_binder")
    o = oracle_system(g, pos="f32", fixed_density=1)
    o.deposit_all()
    recs, _, _ = o.mc_sim_philox(oracle_ctls(g), 5, 99, 0, 0)
    flipped = np.where(recs["accepted"] >= 0, 1 - recs["accepted"], -1).astype(np.int8)
    o2 = oracle_system(g, pos="f32", fixed_density=1)
    o2.deposit_all()
    recs2, _, ties = o2.mc_sim_philox(oracle_ctls(g), 5, 99, 0, 0, follow=flipped)
    u = np.array([move_draws(99, 0, k, int(r["n_draws"]))[-1] for k, r in enumerate(recs)
                  if r["accepted"] >= 0]) / 2147483647.0
    dE = (recs["dE_poly"] + recs["dE_field"])[recs["accepted"] >= 0]
    with np.errstate(divide="ignore"):
        band = np.abs(dE + np.log(u)) <= 1e-5 * np.maximum(1.0, np.abs(dE))
    assert ties == int(band.sum())
    if ties == 0:
        np.testing.assert_array_equal(recs2, recs)
