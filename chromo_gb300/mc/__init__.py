"""Monte Carlo driver API (chromo/mc/__init__.py).

``mc_sim`` runs on the GPU; ``get_amplitude_bounds`` and ``polymer_in_field``
mirror the reference's host-side orchestration (snapshots are kept in memory
and, with an output directory, written in the reference's polymer CSV
format while the device runs the next segment).
"""
import copy
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import numpy as np

from .mc_controller import Controller, SimpleControl, all_moves
from .mc_sim import ResidentChain, mc_sim, mc_sim_audit, mc_step, set_position_precision
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


class _SnapshotWriter:
    """Writes snapshot CSVs on one background thread, one snapshot at a time:
    the write of snapshot k runs while the device runs segment k + 1.  An
    error of a write is raised at the next ``submit`` or at ``close``."""

    def __init__(self):
        self.pool = ThreadPoolExecutor(max_workers=1, thread_name_prefix="snapshot-csv")
        self.pending = None

    def _wait(self):
        if self.pending is not None:
            fut, self.pending = self.pending, None
            fut.result()

    def submit(self, jobs):
        """jobs: [(frozen polymer, path)] of one snapshot."""
        self._wait()
        self.pending = self.pool.submit(lambda: [q.to_csv(path) for q, path in jobs])

    def close(self):
        try:
            self._wait()
        finally:
            self.pool.shutdown(wait=True)


def _frozen(poly, snap):
    """A copy of ``poly`` holding the snapshot's arrays (what ``to_csv`` writes),
    so that the next segment can update ``poly`` while the copy is written."""
    q = copy.copy(poly)
    for k, v in snap.items():
        setattr(q, k, v)
    return q


def polymer_in_field(polymers, binders, field, num_save_mc, num_saves, bead_amp_bounds,
                     move_amp_bounds, mc_move_controllers: Optional[List[Controller]] = None,
                     random_seed: Optional[int] = 0, mu_schedule=None, output_dir=None,
                     start_index: int = 0, **kwargs):
    """Run ``num_saves`` segments of ``num_save_mc`` MC steps, keeping a snapshot of
    every polymer after each segment (chromo/mc/__init__.py:36-161).  With an
    ``output_dir`` each snapshot is also written as ``<name>-<i>.csv`` in the
    reference's polymer CSV format (``PolymerBase.to_csv``), i counting from
    ``start_index`` (a resumed run continues the numbering).

    The polymer stays resident on the device for the whole run
    (``ResidentChain``): segment i runs ``num_save_mc`` steps with the i-th seed
    drawn from ``random_seed`` (as the reference draws one per ``mc_sim``
    call) and the i-th ``mu_schedule`` factor; its snapshot is copied to the
    host and written by a background thread while segment i + 1 runs."""
    np.random.seed(random_seed)
    if mc_move_controllers is None:
        mc_move_controllers = all_moves(str(output_dir or "."), bead_amp_bounds.bounds,
                                        move_amp_bounds.bounds, SimpleControl)
    snapshots = []
    chain = ResidentChain(polymers, field, mc_move_controllers)
    writer = _SnapshotWriter() if output_dir is not None else None
    try:
        for mc_count in range(start_index, start_index + num_saves):
            mu_adjust_factor = (mu_schedule.function(mc_count - start_index, num_saves)
                                if mu_schedule is not None else 1)
            inner_seed = np.random.randint(0, 1E9)
            chain.run(num_save_mc, mu_adjust_factor, inner_seed)
            snap = [dict(r=p.r.copy(), t3=p.t3.copy(), t2=p.t2.copy(), states=p.states.copy())
                    for p in polymers]
            snapshots.append(snap)
            if writer is not None:
                writer.submit([(_frozen(p, s), str(Path(output_dir) / f"{p.name}-{mc_count}.csv"))
                               for p, s in zip(polymers, snap)])
    finally:
        chain.close()
        if writer is not None:
            writer.close()
    return snapshots


def latest_snapshots(output_dir) -> Dict[str, Tuple[int, Path]]:
    """The latest ``<name>-<i>.csv`` snapshot of every polymer in ``output_dir``:
    {name: (i, path)} (the role of get_latest_configuration and
    find_polymers_in_output_dir, chromo/util/poly_stat.py:184-259, for the flat
    layout ``polymer_in_field`` writes)."""
    out: Dict[str, Tuple[int, Path]] = {}
    for path in Path(output_dir).glob("*-*.csv"):
        name, _, idx = path.stem.rpartition("-")
        if not name or not idx.isdigit():
            continue
        i = int(idx)
        if name not in out or i > out[name][0]:
            out[name] = (i, path)
    return out


def continue_polymer_in_field_simulation(polymer_class, binders, field, output_dir, num_save_mc,
                                         num_saves, mc_move_controllers: Optional[List[Controller]] = None,
                                         random_seed: Optional[int] = 0):
    """Continue a ``polymer_in_field`` run from the latest snapshot of each
    polymer in ``output_dir`` (chromo/mc/__init__.py:167-227): the polymers are
    read back with ``polymer_class.from_file``, placed in ``field``, and run for
    ``num_saves`` more snapshots, numbered after the latest.  Returns the new
    snapshots, as ``polymer_in_field``."""
    latest = latest_snapshots(output_dir)
    if not latest:
        raise FileNotFoundError(f"no <name>-<i>.csv snapshot in {output_dir}")
    names = sorted(latest)
    polymers = [polymer_class.from_file(str(latest[n][1]), n) for n in names]
    field.polymers = polymers
    field.n_polymers = len(polymers)
    if hasattr(field, "_density_fx"):
        field._density_fx = None  # the density of the loaded polymers is deposited anew
    bead_amp_bounds, move_amp_bounds = get_amplitude_bounds(polymers)
    return polymer_in_field(polymers, binders, field, num_save_mc, num_saves, bead_amp_bounds,
                            move_amp_bounds, mc_move_controllers, random_seed=random_seed,
                            output_dir=output_dir,
                            start_index=max(latest[n][0] for n in names) + 1)
