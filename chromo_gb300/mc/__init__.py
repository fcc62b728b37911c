"""Monte Carlo driver API (chromo/mc/__init__.py).

``mc_sim`` runs on the GPU; ``get_amplitude_bounds`` and ``polymer_in_field``
mirror the reference's host-side orchestration (snapshots are kept in memory
and, with an output directory, written in the reference's polymer CSV
format).
"""
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import numpy as np

from .mc_controller import Controller, SimpleControl, all_moves
from .mc_sim import mc_sim, mc_sim_audit, mc_step, set_position_precision
from .moves import Bounds


def get_amplitude_bounds(polymers) -> Tuple[Bounds, Bounds]:
    """Bead-selection and move-amplitude bounds (chromo/mc/__init__.py:295-332)."""
    poly_len = np.min([p.r.shape[0] for p in polymers])
    min_spacing = np.min([np.min(p.bead_length) for p in polymers])
    bead = Bounds("bead_amp_bounds", {
        "crank_shaft": (min(30, poly_len), min(150, poly_len)),
        "slide": (min(10, poly_len), min(150, poly_len)),
        "end_pivot": (min(50, poly_len / 4), min(150, int(poly_len / 2))),
        "tangent_rotation": (1, poly_len),
        "change_binding_state": (1, 1)})
    move = Bounds("move_amp_bounds", {
        "crank_shaft": (0.1 * np.pi, 0.25 * np.pi),
        "slide": (0.2 * min_spacing, 0.3 * min_spacing),
        "end_pivot": (0.2 * np.pi, 0.25 * np.pi),
        "tangent_rotation": (0.05 * np.pi, 0.2 * np.pi),
        "change_binding_state": (0, 0)})
    return bead, move


def polymer_in_field(polymers, binders, field, num_save_mc, num_saves, bead_amp_bounds,
                     move_amp_bounds, mc_move_controllers: Optional[List[Controller]] = None,
                     random_seed: Optional[int] = 0, mu_schedule=None, output_dir=None, **kwargs):
    """Run ``num_saves`` rounds of ``num_save_mc`` MC steps, keeping a snapshot of
    every polymer after each round (chromo/mc/__init__.py:36-161).  With an
    ``output_dir`` each snapshot is also written as ``<name>-<i>.csv`` in the
    reference's polymer CSV format (``PolymerBase.to_csv``)."""
    np.random.seed(random_seed)
    if mc_move_controllers is None:
        mc_move_controllers = all_moves(str(output_dir or "."), bead_amp_bounds.bounds,
                                        move_amp_bounds.bounds, SimpleControl)
    snapshots = []
    for mc_count in range(num_saves):
        mu_adjust_factor = mu_schedule.function(mc_count, num_saves) if mu_schedule is not None else 1
        inner_seed = np.random.randint(0, 1E9)
        mc_sim(polymers, binders, num_save_mc, mc_move_controllers, field, mu_adjust_factor,
               inner_seed)
        snap = [dict(r=p.r.copy(), t3=p.t3.copy(), t2=p.t2.copy(), states=p.states.copy())
                for p in polymers]
        snapshots.append(snap)
        if output_dir is not None:
            for p in polymers:
                p.to_csv(str(Path(output_dir) / f"{p.name}-{mc_count}.csv"))
    return snapshots
