"""Autotuner of the MC kernel's launch shape.

The production kernel runs one CTA per replica with two shape parameters:
W, the warps of a replica's CTA, and G, the lanes that evaluate one move (8,
16 or 32; FP64 storage only has 32), so W * 32 / G moves of a replica are in
flight at once.  Which shape is fastest depends on how many replicas share an
SM (register residency), on chain lengths and move sizes (conflicts between
moves in flight, divergence between the moves sharing a warp), on the grid
and the binder count, so it is measured rather than modelled:

    shape, table = tune(build, n_beads, grid_dims, n_binders)

``build(W, G)`` returns a fresh ``_native.Sim`` of the problem to tune (the
same chains, fields and controllers as the real run).  Every candidate shape
gets a scratch simulation, ``warmup`` untimed MC steps and ``steps`` timed
ones (CUDA events on the launching stream); the fastest attempted-moves/s
wins.  Results are kept per problem in a JSON cache
(``CHROMO_GB300_TUNE_CACHE``, default ``~/.cache/chromo_gb300/autotune.json``)
so a problem is tuned once per GPU model.

The reference has no counterpart: its loop runs one move at a time on one
core (chromo/mc/mc_sim.pyx:88-182).
"""
import json
import math
import os
from pathlib import Path
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as nat

Shape = Tuple[int, int]  # (warps per replica CTA, lanes per move)
MAX_WARPS = 12
MAX_IN_FLIGHT = 32


def cache_path() -> Path:
    p = os.environ.get("CHROMO_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "chromo_gb300" / "autotune.json"


def problem_key(n_beads: Sequence[int], grid_dims: Sequence, n_binders: int, pos_fp64: bool,
                n_sm: int, device_name: str, extra: str = "") -> str:
    """Signature of a tuning problem: device, replica count, chain-length
    quantiles, distinct grids, binders and storage precision."""
    lengths = np.asarray(n_beads, dtype=np.int64)
    q = [int(np.quantile(lengths, f)) for f in (0.0, 0.5, 1.0)]
    grids = sorted({tuple(int(x) for x in g) for g in np.asarray(grid_dims).reshape(-1, 3)})
    return json.dumps({"device": device_name, "sm": int(n_sm), "R": int(len(lengths)), "len_q": q,
                       "grids": grids[:4], "n_grids": len(grids), "nb": int(n_binders),
                       "fp64": bool(pos_fp64), "extra": extra}, sort_keys=True)


def candidates(n_replicas: int, n_sm: int, pos_fp64: bool, warps_per_sm: Dict[int, int]) -> List[Shape]:
    """Shapes worth timing: for each G, the W that keep every replica's CTA
    resident at once (ceil(R / SMs) CTAs per SM within the register file) --
    the largest such W and a few below it -- with at most 32 moves in flight.
    When every replica has an SM to itself, a few small W at 32 lanes too: a
    chain whose controller cycles hold few moves (one with specific_moves)
    has few moves to put in flight, and fewer warps then shorten each
    batch's barriers."""
    ctas = max(1, math.ceil(n_replicas / max(1, n_sm)))
    out = []
    for G in ((32,) if pos_fp64 else (32, 16, 8)):
        wmax = min(MAX_WARPS, MAX_IN_FLIGHT * G // 32, max(1, warps_per_sm[G] // ctas))
        ws = {wmax, wmax - 1, wmax - 2, (wmax + 1) // 2}
        if G == 32 and n_replicas <= n_sm:
            ws |= {w for w in (1, 2, 4) if w <= wmax}
        out += [(w, G) for w in sorted(ws - {0}, reverse=True) if w >= 1]
    return out


def _time_shape(build: Callable[[int, int], "nat.Sim"], shape: Shape, steps: int, warmup: int,
                seed: int) -> float:
    import torch
    sim = build(*shape)
    try:
        stream = torch.cuda.current_stream()
        sh = stream.cuda_stream
        if warmup:
            sim.run(warmup, seed, sh)
        sim.sync(sh)
        sim.reset_tally()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(steps, seed + 1, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        sim.sync(sh)
        attempts = float(sum(sim.tally(r)[:, 0].sum() for r in range(sim.R)))
        return attempts / (e0.elapsed_time(e1) / 1000.0)
    finally:
        sim.close()


def tune(build: Callable[[int, int], "nat.Sim"], n_beads: Sequence[int], grid_dims: Sequence,
         n_binders: int, pos_fp64: bool = False, steps: int = 8, warmup: int = 2, seed: int = 7,
         shapes: Optional[Sequence[Shape]] = None, use_cache: bool = True,
         extra_key: str = "", device: Optional[Tuple[str, int]] = None) -> Tuple[Shape, Dict[str, float]]:
    """Time every candidate shape on scratch simulations from ``build`` and
    return (fastest shape, {"WxG": moves/s}).  A cached result for the same
    problem key is returned without timing when ``use_cache``.  ``device`` =
    (name, SM count) of the GPU (default: the current CUDA device)."""
    if device is None:
        import torch
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        device = (props.name, props.multi_processor_count)
    name, n_sm = device
    key = problem_key(n_beads, grid_dims, n_binders, pos_fp64, n_sm, name, extra_key)
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
        hit = cache.get(key)
        if hit:
            return (int(hit["shape"][0]), int(hit["shape"][1])), hit["table"]
    if shapes is None:
        wps = {G: nat.mc_warps_per_sm(pos_fp64, G) for G in ((32,) if pos_fp64 else (32, 16, 8))}
        shapes = candidates(len(n_beads), n_sm, pos_fp64, wps)
    table = {}
    for shape in shapes:
        table[f"{shape[0]}x{shape[1]}"] = _time_shape(build, shape, steps, warmup, seed)
    best = max(table, key=table.get)
    shape = tuple(int(x) for x in best.split("x"))
    if use_cache:
        cache[key] = {"shape": list(shape), "table": table}
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            tmp = path.with_suffix(".tmp")
            tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
            os.replace(tmp, path)
        except OSError:
            pass
    return shape, table
