"""MC move adapters (chromo/mc/moves.pyx:58-369)."""
import numpy as np

from ..util import mc_stat
from .move_funcs import (change_binding_state, crank_shaft, end_pivot, move_list, slide,
                         tangent_rotation)


class MCAdapter:
    """Move amplitudes and acceptance bookkeeping of one move kind
    (chromo/mc/moves.pyx:58-129)."""

    def __init__(self, log_dir: str, log_file_prefix: str, move_func, moves_in_average: float = 20,
                 init_amp_bead: int = 100, init_amp_move: float = 0.05):
        self.name = move_func.__name__
        self.move_func = move_func
        self.amp_move = float(init_amp_move)
        self.num_per_cycle = 1
        self.amp_bead = int(init_amp_bead)
        self.num_attempt = 0
        self.num_success = 0
        self.move_on = 1
        self.last_amp_move = 0
        self.last_amp_bead = 0
        self.acceptance_tracker = mc_stat.AcceptanceTracker(log_dir, log_file_prefix,
                                                            moves_in_average)

    def __str__(self):
        return f"MCAdapter<{self.name}>"

    def to_file(self, path):
        pass


class Bounds:
    """Named amplitude bounds (chromo/mc/moves.pyx:302-340)."""

    def __init__(self, name: str, bounds: dict):
        self.name = name
        self.bounds = bounds

    def to_file(self, path):
        pass


def all_moves(log_dir: str):
    return [MCAdapter(log_dir + "/" + m.__name__, "", m) for m in move_list]
