"""Seeded synthetic inputs with the shapes of the benchmark workloads.

There is no public dataset for this path; chains are Gaussian random walks
with fixed bead spacing (``gaussian_walk``, chromo/util/poly_paths.py:269-295)
with tangents estimated from the coordinates
(``estimate_tangents_from_coordinates``, :506-545), and mark tracks are
3-state Markov chains on {0, 1, 2}.
"""
import numpy as np


def gaussian_walk(rng, n_beads, step=16.5):
    steps = rng.standard_normal((n_beads - 1, 3))
    steps /= np.linalg.norm(steps, axis=1)[:, None]
    r = np.zeros((n_beads, 3))
    r[1:] = np.cumsum(steps * step, axis=0)
    return r


def confined_walks(rng, n_chains, n_beads, step, radius):
    """`n_chains` walks of unit steps times `step` from the origin that stay
    inside a sphere of `radius`: a step that would leave it is drawn again
    (the rule of confined_gaussian_walk, chromo/util/poly_paths.py:298-336),
    all chains advanced together.  Returns [n_chains, n_beads, 3]."""
    r = np.zeros((n_chains, n_beads, 3))
    for i in range(1, n_beads):
        todo = np.arange(n_chains)
        while len(todo):
            d = rng.standard_normal((len(todo), 3))
            p = r[todo, i - 1] + d / np.linalg.norm(d, axis=1)[:, None] * step
            ok = (p * p).sum(axis=1) <= radius * radius
            r[todo[ok], i] = p[ok]
            todo = todo[~ok]
    return r


def tangents_from_coordinates(r):
    n = r.shape[0]
    t3 = np.zeros((n, 3))
    d = r[1] - r[0]
    t3[0] = d / np.linalg.norm(d)
    d = r[n - 1] - r[n - 2]
    t3[n - 1] = d / np.linalg.norm(d)
    d = r[2:] - r[:-2]
    t3[1:-1] = d / np.linalg.norm(d, axis=1)[:, None]
    t2 = np.cross(t3, np.array([1.0, 0.0, 0.0]))
    bad = np.all(t2 == 0, axis=1)
    if bad.any():
        t2[bad] = np.cross(t3[bad], np.array([0.0, 1.0, 0.0]))
    t2 /= np.linalg.norm(t2, axis=1)[:, None]
    return t3, t2


def markov_marks(rng, n, run_length):
    """Stay with probability 1 - 1/run_length, else jump to one of the other two states."""
    u = rng.random(n)
    jump = rng.integers(1, 3, size=n)
    out = np.empty(n, dtype=np.int64)
    s = int(rng.integers(0, 3))
    for i in range(n):
        out[i] = s
        if u[i] < 1.0 / run_length:
            s = (s + int(jump[i])) % 3
    return out


def log_uniform_lengths(rng, n, lo, hi):
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), size=n))).astype(np.int64)
