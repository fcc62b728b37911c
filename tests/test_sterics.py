"""Steric clash energy of the detailed chromatin model (chromo/polymers.pyx:2738-2938).

The oracle's restatement against vectors of the reference's own
``DetailedChromatinWithSterics`` (tests/golden/make_sterics.py): the clash
energy of two seeded chains and the clash-energy change of 40 seeded segment
moves on each, within 1e-12 relative (the reference sums the same terms in
the same order; the values reach 1e17 for nearly coincident beads).  The GPU
kernels are checked against the oracle in the gpu-marked tests below.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc

FIX = Path(__file__).resolve().parent / "golden" / "sterics" / "vectors.npz"


@pytest.fixture(scope="module")
def g():
    with np.load(FIX, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("c", [0, 1])
def test_oracle_steric_energy_and_moves_match_reference(g, c):
    r, e = g[f"r{c}"], float(g[f"excluded{c}"])
    assert orc.steric_energy(r, e) == pytest.approx(float(g[f"E{c}"]), rel=1e-12)
    for (ind0, indf), trial, want in zip(g[f"moves{c}"], g[f"trials{c}"], g[f"dE{c}"]):
        got = orc.steric_delta(r, trial[:indf - ind0], ind0, indf, e)
        assert got == pytest.approx(want, rel=1e-12, abs=1e-9), (ind0, indf)


def _moved_term_magnitude(r, seg, ind0, indf, e, V0=1.0):
    """Sum of the (non-negative) clash terms, current and trial, of the pairs
    a move of beads [ind0, indf) to `seg` changes."""
    rt = r.copy()
    rt[ind0:indf] = seg
    total = 0.0
    for pos in (r, rt):
        d = np.linalg.norm(pos[ind0:indf, None, :] - pos[None, :, :], axis=2)
        i = np.arange(ind0, indf)[:, None]
        j = np.arange(len(r))[None, :]
        keep = ~((j >= i) & (j >= ind0) & (j < indf)) & (d < e)
        f = e / np.where(keep, d, e)
        total += float(np.sum(np.where(keep, V0 * (f ** 12 - 2 * f ** 6 + 1), 0.0)))
    return total


@pytest.mark.gpu
@pytest.mark.parametrize("c", [0, 1])
def test_gpu_steric_kernels_match_oracle(g, c):
    """cg_steric_energy / cg_steric_delta on the device against the oracle.

    The device sums the same non-negative clash terms in another order (rows
    in parallel, each pair's trial-minus-current difference first) with the
    device's pow, so a move's dE agrees to 1e-12 of the magnitude of the terms
    it sums (terms reach 1e17 for nearly coincident beads, where the
    difference itself can be O(1))."""
    from chromo_gb300 import _native as nat
    r, e = g[f"r{c}"], float(g[f"excluded{c}"])
    n = len(r)
    sim = nat.Sim([n], [[4, 4, 4]], 1, pos_fp64=True)
    try:
        sim.set_chain(0, r=r, t3=np.tile([1.0, 0, 0], (n, 1)), t2=np.tile([0, 1.0, 0], (n, 1)))
        assert sim.steric_energy(0, e) == pytest.approx(orc.steric_energy(r, e), rel=1e-12)
        for (ind0, indf), trial in zip(g[f"moves{c}"], g[f"trials{c}"]):
            seg = trial[:indf - ind0]
            want = orc.steric_delta(r, seg, ind0, indf, e)
            scale = _moved_term_magnitude(r, seg, ind0, indf, e)
            got = sim.steric_delta(0, ind0, indf, seg, e)
            assert abs(got - want) <= 1e-12 * scale + 1e-9, (ind0, indf, got, want, scale)
    finally:
        sim.close()
