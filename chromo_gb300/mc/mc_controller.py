"""Move amplitude controllers (chromo/mc/mc_controller.py).

``SimpleControl``'s update rule (:126-189) runs on the GPU at the end of each
controller's cycle; ``update_amplitudes`` here applies the same rule on the
host for callers that drive it themselves.
"""
from typing import Callable, Dict, List, Optional, Tuple

from . import moves as mv
from . import move_funcs as mf


class Controller:
    kind = 0

    def __init__(self, mc_adapter, bead_amp_bounds: Tuple[int, int],
                 move_amp_bounds: Tuple[float, float]):
        if bead_amp_bounds[0] > bead_amp_bounds[1]:
            raise ValueError("Lower bead amplitude bound must be less than upper bead amplitude bound")
        if move_amp_bounds[0] > move_amp_bounds[1]:
            raise ValueError("Lower move amplitude bound must be less than upper move amplitude bound")
        self.move = mc_adapter
        self.bead_amp_bounds = bead_amp_bounds
        self.move_amp_bounds = move_amp_bounds

    def update_amplitudes(self):
        pass


class NoControl(Controller):
    kind = 0


class SimpleControl(Controller):
    kind = 1

    def __init__(self, mc_adapter, bead_amp_bounds, move_amp_bounds):
        super().__init__(mc_adapter, bead_amp_bounds, move_amp_bounds)
        self.name = "SimpleController"

    def to_file(self, path):
        pass

    def update_amplitudes(self, setpoint_acceptance=0.5, move_adjust_factor=0.95, num_delta_beads=1):
        self.update_move_amplitude(setpoint_acceptance, move_adjust_factor, num_delta_beads)

    def update_move_amplitude(self, setpoint_acceptance=0.5, move_adjust_factor=0.95,
                              num_delta_beads=1):
        acceptance = self.move.acceptance_tracker.acceptance_rate
        if acceptance < setpoint_acceptance:
            prop = self.move.amp_move * move_adjust_factor
            if prop > self.move_amp_bounds[0]:
                self.move.amp_move = prop
            else:
                self.move.amp_bead = max(self.bead_amp_bounds[0],
                                         self.update_bead_amplitude(False, num_delta_beads))
        elif acceptance > setpoint_acceptance:
            prop = self.move.amp_move / move_adjust_factor
            if prop < self.move_amp_bounds[1]:
                self.move.amp_move = prop
            else:
                self.move.amp_bead = min(self.bead_amp_bounds[1],
                                         self.update_bead_amplitude(True, num_delta_beads))

    def update_bead_amplitude(self, increase: bool, num_delta_beads: Optional[int] = 1):
        if increase:
            self.move.amp_move = self.move_amp_bounds[0]
            return self.move.amp_bead + num_delta_beads
        self.move.amp_move = self.move_amp_bounds[1]
        return self.move.amp_bead - num_delta_beads


def _controllers(moves, log_dir, bead_amp_bounds, move_amp_bounds, controller):
    return [controller(
        mv.MCAdapter(str(log_dir) + "/acceptance_trackers", m.__name__ + "_snap_", m,
                     moves_in_average=20, init_amp_bead=bead_amp_bounds[m.__name__][0],
                     init_amp_move=move_amp_bounds[m.__name__][0]),
        bead_amp_bounds=bead_amp_bounds[m.__name__], move_amp_bounds=move_amp_bounds[m.__name__])
        for m in moves]


def all_moves(log_dir: str, bead_amp_bounds: Dict[str, Tuple[float, float]],
              move_amp_bounds: Dict[str, Tuple[float, float]],
              controller=NoControl) -> List[Controller]:
    """Controllers for the five moves with num_per_cycle 30/1/60/60/10
    (chromo/mc/mc_controller.py:216-266)."""
    cs = _controllers([mf.crank_shaft, mf.end_pivot, mf.slide, mf.tangent_rotation,
                       mf.change_binding_state], log_dir, bead_amp_bounds, move_amp_bounds,
                      controller)
    for c, n in zip(cs, (30, 1, 60, 60, 10)):
        c.move.num_per_cycle = n
    return cs


def all_moves_except_binding_state(log_dir, bead_amp_bounds, move_amp_bounds, controller=NoControl):
    cs = _controllers([mf.crank_shaft, mf.end_pivot, mf.slide, mf.tangent_rotation], log_dir,
                      bead_amp_bounds, move_amp_bounds, controller)
    for c in cs:
        c.move.num_per_cycle = 5
    return cs


def specific_move(move_fxn, log_dir, bead_amp_bounds, move_amp_bounds, controller=NoControl):
    cs = _controllers([move_fxn], log_dir, bead_amp_bounds, move_amp_bounds, controller)
    cs[0].move.num_per_cycle = 1
    return cs


def specific_moves(move_fxns: List[Callable], log_dir, bead_amp_bounds, move_amp_bounds,
                   controller=NoControl):
    cs = _controllers(move_fxns, log_dir, bead_amp_bounds, move_amp_bounds, controller)
    for c in cs:
        c.move.num_per_cycle = 1
    return cs


def only_binding_move(log_dir, bead_amp_bounds, move_amp_bounds, controller=NoControl):
    cs = _controllers([mf.change_binding_state], log_dir, bead_amp_bounds, move_amp_bounds,
                      controller)
    cs[0].move.num_per_cycle = 5
    return cs
