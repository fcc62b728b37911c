"""Bead selection of the MC moves (chromo/util/bead_selection.pyx:19-192).

Host-side helpers for calling a move function directly; the MC loop selects
beads inside the GPU kernel with the same rule.  A segment end is drawn at a
distance r = floor(-log10(u + 1e-5) * window * 0.45 + 1.0001) from a start
bead (u = rand() / RAND_MAX), drawn again while r exceeds the cap.
"""
import numpy as np

from .linalg import RAND_MAX, rand


def capped_exponential(window: int, cap: int) -> int:
    """A draw of the distance rule above, at most `cap` (bead_selection.pyx:19-66)."""
    while True:
        r = int(-np.log10(rand() / RAND_MAX + 0.00001) * window * 0.45 + 1.0001)
        if r <= cap:
            return r


def from_left(window: int, N_beads: int) -> int:
    """Distance from the left end of a chain of N_beads (bead_selection.pyx:69-90)."""
    if window > N_beads:
        raise ValueError("Bead selection window size must be less than polymer length")
    return capped_exponential(window, window)


def from_right(window: int, N_beads: int) -> int:
    """Index measured from the right end (bead_selection.pyx:93-112)."""
    return N_beads - from_left(window, N_beads)


def from_point(window: int, N_beads: int, ind0: int) -> int:
    """The other end of a segment starting at ind0, to the left or the right
    with equal odds, within `window` and the chain (bead_selection.pyx:115-154)."""
    if window > N_beads:
        raise ValueError("Bead selection window size must be less than polymer length")
    if window < 1:
        return ind0
    if rand() % 2 == 0:
        reach = max(1, min(window, ind0))
        return from_right(reach, max(ind0, 1))
    reach = max(1, min(window, N_beads - ind0))
    return from_left(reach, max(N_beads - ind0, 1)) + ind0


def check_bead_bounds(bound_0: int, bound_1: int, num_beads: int):
    """(ind0, indf) of the segment between two drawn ends, clipped to the chain
    and at least one bead long (bead_selection.pyx:157-192)."""
    b0 = min(max(bound_0, 0), num_beads)
    if bound_1 > num_beads:
        return b0, num_beads
    if bound_1 < 0:
        return 0, b0 + 1
    if b0 == bound_1:
        return b0, b0 + 1
    return min(b0, bound_1), max(b0, bound_1)
