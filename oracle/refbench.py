"""Time the reference's own CPU implementation of the MC inner loop.

TEST / BASELINE INFRASTRUCTURE ONLY (used by bench.py's reference arm and CPU
baseline).  The reference (chromo, Python + Cython) is run from the build in
``oracle/_ref``: on a host where only the Cython-generated C++ is present (the
x86 shared objects are not usable on another architecture) the C++ is
compiled here with g++, which needs the Python and numpy headers but not
Cython.  Workers are started with the ``spawn`` method, each runs whole
replicas of the benchmark workload through the reference's ``mc_sim`` for a
time budget, and the aggregate rate is sum(attempted moves) / wall time.
If the reference cannot be built, the C restatement (``chromo_oracle.c``)
is timed instead and reported as kind "port".

The timed window is matched to the GPU's: before timing, every sampled
replica is brought to the state after ``settle_steps`` MC steps (the GPU
benchmark's settle phase, after which the move controllers' bead amplitudes
sit at their bounds) by the C restatement, and the reference then starts from
that chain and those controller amplitudes and acceptance rates.
"""
import multiprocessing as mp
import os
import subprocess
import sys
import sysconfig
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF = HERE / "_ref"
MODULES = ["chromo/mc/move_funcs", "chromo/polymers", "chromo/fields", "chromo/binders",
           "chromo/util/bead_selection", "chromo/util/linalg", "chromo/mc/mc_sim",
           "chromo/mc/moves", "ref_shim"]


def ensure_reference_built():
    """(ok, reason).  Compiles oracle/_ref's generated C++ for this host if needed."""
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    if not (REF / "chromo" / "polymers.cpp").exists():
        return False, "reference build (oracle/_ref) absent"
    try:
        import numpy as np
        inc = [sysconfig.get_paths()["include"], np.get_include(), str(REF)]
    except Exception as e:  # pragma: no cover
        return False, f"numpy headers unavailable: {e}"
    if not Path(inc[0], "Python.h").exists():
        return False, "Python.h not found"
    jobs = []
    for m in MODULES:
        cpp, so = REF / f"{m}.cpp", REF / f"{m}{ext}"
        if so.exists() and so.stat().st_mtime >= cpp.stat().st_mtime:
            continue
        jobs.append(subprocess.Popen(["g++", "-O2", "-shared", "-fPIC", "-w", "-o", str(so), str(cpp)]
                                     + [f"-I{p}" for p in inc]))
    if any(j.wait() != 0 for j in jobs):
        return False, "g++ failed on the reference's generated C++"
    return True, ""


def _ref_path():
    for p in (str(REF), str(HERE / "ref_stubs"), str(ROOT)):
        if p not in sys.path:
            sys.path.insert(0, p)


def _settled(w, rep, chain, settle_steps, seed):
    """Replica `rep` after `settle_steps` MC steps of the C restatement (its
    own libc rand() draws): (chain with the settled r, t3, t2, states;
    [(amp_move, amp_bead, acc_rate) per controller]; the oracle system and its
    controllers, for the port worker)."""
    import copy
    import ctypes
    import numpy as np
    from oracle.oracle import OracleSystem, make_ctl
    from chromo_gb300.energetics import dss_parameters, field_prefactors
    from chromo_gb300.workloads import (BEAD_RAD, BEAD_SPACING, HP1_E_MOD, HP1_E_NOMOD, LP,
                                        NUM_PER_CYCLE, R_INT, SITES, VOXEL, amplitude_bounds,
                                        binder_names)
    n = len(chain.r)
    _, eb, g, ep, epp, eta = dss_parameters(np.full(n - 1, BEAD_SPACING), LP)
    nb = w.n_binders
    vint = 4.0 / 3.0 * np.pi * R_INT ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint] * nb, w.cross, binder_names(nb), VOXEL ** 3)
    width = w.nbins * VOXEL
    confine = {}
    if getattr(w, "sphere_radius", 0) > 0:  # spherical confinement with accessible volumes
        from chromo_gb300.workloads import _sphere_volumes
        confine = dict(confine_kind=1, confine_length=float(w.sphere_radius),
                       access_vol=_sphere_volumes(w.nbins, float(w.sphere_radius)))
    o = OracleSystem(r=chain.r, t3=chain.t3, t2=chain.t2, states=chain.states, marks=chain.marks,
                     eps_bend=eb, gamma=g, eps_par=ep, eps_perp=epp, eta=eta, sites=[SITES] * nb,
                     e_mod=[HP1_E_MOD] * nb, e_nomod=[HP1_E_NOMOD] * nb, mu=w.mu[rep],
                     nxyz=(w.nbins,) * 3, widths=(width,) * 3, chi=float(w.chi[rep]),
                     bead_vol=4.0 / 3.0 * np.pi * BEAD_RAD ** 3, pref=pref, intra=intra,
                     xpref=xpref, pos="f64", fixed_density=0, **confine)
    o.deposit_all()
    bead, move = amplitude_bounds(n)
    cycle = w.cycle or NUM_PER_CYCLE
    ctls = [make_ctl(m, amp_move=move[m][0], amp_bead=int(bead[m][0]),
                     num_per_cycle=cycle[m], bead_bounds=bead[m], move_bounds=move[m])
            for m in ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]]
    if settle_steps:
        ctypes.CDLL(None).srand(seed)
        o.mc_sim(ctls, settle_steps, None, None, max_records=0)
    c = copy.copy(chain)
    c.r, c.t3, c.t2 = o.r.copy(), o.t3.copy(), o.t2.copy()
    c.states = o.states.copy()
    amps = [(float(k.amp_move), int(k.amp_bead), float(k.acc_rate)) for k in ctls]
    return c, amps, (o, ctls)


def _build_reference_replica(w, rep, chain, amps=None):
    import numpy as np
    import chromo.binders as cb
    import chromo.mc as cmc
    from chromo.fields import UniformDensityField
    from chromo.mc.mc_controller import SimpleControl, all_moves
    from chromo.polymers import Chromatin
    from chromo_gb300.workloads import BEAD_SPACING, VOXEL, binder_names
    names = binder_names(w.n_binders)
    for b, nm in enumerate(names):
        obj = cb.get_by_name(nm) if nm in ("HP1", "PRC1") else None
        obj.chemical_potential = float(w.mu[rep][b])
        obj.interaction_energy = float(w.eps[b])
        obj.cross_talk_interaction_energy = dict(w.cross[b])
    binders = cb.make_binder_collection([cb.get_by_name(nm) for nm in names])
    n = len(chain.r)
    p = Chromatin(f"r{rep}", chain.r.copy(), bead_length=np.full(n - 1, BEAD_SPACING),
                  t3=chain.t3.copy(), t2=chain.t2.copy(), states=chain.states.copy(),
                  binder_names=np.array(names), chemical_mods=chain.marks.copy(),
                  chemical_mod_names=np.array([f"m{b}" for b in range(len(names))]))
    width = w.nbins * VOXEL
    confine = {}
    if getattr(w, "sphere_radius", 0) > 0:  # spherical confinement with accessible volumes
        confine = dict(confine_type="Spherical", confine_length=float(w.sphere_radius),
                       assume_fully_accessible=0)
    f = UniformDensityField([p], binders, width, w.nbins, width, w.nbins, width, w.nbins,
                            chi=float(w.chi[rep]), **confine)
    bab, mab = cmc.get_amplitude_bounds([p])
    if w.cycle:  # one attempt of each move per MC step: the reference's specific_moves
        import chromo.mc.moves as mv
        from chromo.mc.mc_controller import specific_moves
        ctrls = specific_moves([mv.crank_shaft, mv.end_pivot, mv.slide, mv.tangent_rotation,
                                mv.change_binding_state], "/tmp/chromo_refbench_logs", bab.bounds,
                               mab.bounds, SimpleControl)
    else:
        ctrls = all_moves("/tmp/chromo_refbench_logs", bab.bounds, mab.bounds, SimpleControl)
    for c, a in zip(ctrls, amps or []):  # the settled amplitudes and acceptance rates
        c.move.amp_move, c.move.amp_bead = a[0], a[1]
        c.move.acceptance_tracker.acceptance_rate = a[2]
    return p, binders, f, ctrls


def _ref_worker(args):
    wname, reps, budget, seed, settle_steps = args
    _ref_path()
    import ctypes
    from chromo.mc.mc_sim import mc_sim
    from chromo_gb300.workloads import make_chains, make_workload
    w = make_workload(wname)
    chains = make_chains(w)
    built = []
    for r in reps:
        c, amps, _ = _settled(w, r, chains[r], settle_steps, seed + r)
        built.append(_build_reference_replica(w, r, c, amps))
    ctypes.CDLL(None).srand(seed)
    attempts, t0 = 0, time.perf_counter()
    i = 0
    while time.perf_counter() - t0 < budget:
        p, binders, f, ctrls = built[i % len(built)]
        before = sum(c.move.num_attempt for c in ctrls)
        mc_sim([p], binders, 1, ctrls, f, 1.0, seed + i)
        attempts += sum(c.move.num_attempt for c in ctrls) - before
        i += 1
    return attempts, time.perf_counter() - t0


def _port_worker(args):
    wname, reps, budget, seed, settle_steps = args
    for p in (str(ROOT), str(HERE)):
        if p not in sys.path:
            sys.path.insert(0, p)
    from chromo_gb300.workloads import make_chains, make_workload
    w = make_workload(wname)
    chains = make_chains(w)
    systems = [_settled(w, rep, chains[rep], settle_steps, seed + rep)[2] for rep in reps]
    attempts, t0, i = 0, time.perf_counter(), 0
    while time.perf_counter() - t0 < budget:
        o, ctls = systems[i % len(systems)]
        before = sum(c.num_attempt for c in ctls)
        o.mc_sim(ctls, 1, None, None, max_records=0)
        attempts += sum(c.num_attempt for c in ctls) - before
        i += 1
    return attempts, time.perf_counter() - t0


def run(workload="batched", budget=2.0, n_procs=None, prefer="reference", settle_steps=0):
    """Aggregate attempted moves/s of the CPU implementation on this host, from
    the state after `settle_steps` MC steps of every sampled replica.  A
    single-chain workload runs in one process (the reference's mc_sim is
    serial; more processes would run other chains, not this one faster)."""
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    from chromo_gb300.workloads import make_workload
    w = make_workload(workload)
    n_procs = n_procs or os.cpu_count() or 1
    n_procs = max(1, min(n_procs, w.replicas))
    kind, reason = "port", ""
    if prefer == "reference":
        ok, reason = ensure_reference_built()
        kind = "reference" if ok else "port"
    worker = _ref_worker if kind == "reference" else _port_worker
    if w.replicas > 1:
        reps = [list(range(i, w.replicas, n_procs)) for i in range(n_procs)]
    else:
        reps = [[0] for _ in range(n_procs)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(n_procs) as pool:
        res = pool.map(worker, [(workload, reps[i][:2], budget, 1234 + i, settle_steps)
                                for i in range(n_procs)])
    wall = max(r[1] for r in res)
    attempts = sum(r[0] for r in res)
    return {"value": attempts / wall, "unit": "moves/s", "cores": n_procs, "kind": kind,
            "sample": (f"{workload} workload: {n_procs} spawn workers x {budget:.1f} s, each cycling "
                       f"{min(2, len(reps[0]))} of its replicas through mc_sim one step at a time "
                       f"from the state after {settle_steps} settle MC steps; {attempts} attempted moves"),
            "fallback_reason": reason, "elapsed_s": time.perf_counter() - t0}


if __name__ == "__main__":
    import json
    print(json.dumps(run(*(sys.argv[1:2] or ["batched"]), budget=float(sys.argv[2]) if len(sys.argv) > 2 else 2.0)))
