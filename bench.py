#!/usr/bin/env python3
"""Attempted MC moves/s of chromo's inner loop on GB300 (batched vs plain GPU).

One "step" is one replica-exchange round of the batched workload: every
replica (256 chains, 2,000-20,000 beads, own 40^3 grid, two binders) runs 62
MC steps of all five moves (~1e4 attempted moves per replica), then chi is
exchanged along 16-rung ladders.  The round is a captured CUDA graph replayed
K times.  Before the W warm-up rounds, SETTLE_ROUNDS rounds bring the move
controllers to steady state (SimpleControl widens the segments for thousands
of MC steps; the bead amplitudes of crank shaft, end pivot and slide reach
their bounds), so every leg measures the steady state.

``value`` is whole-job attempted moves/s over the K timed rounds with the
state resident in HBM; ``roofline`` is the MC kernel of those same rounds
(CUDA event-record nodes inside the replayed graph: algorithmic bytes per
launch over its device duration, against the measured HBM peak); ``e2e`` is
the same K rounds from the same start state through the C ABI with host
buffers (state uploaded from pinned memory and the snapshot read back every
step); ``plain`` is one 10,000-bead chain on the same kernel (one CTA),
settled the same way; ``cpu_baseline`` is the reference's own CPU code on
this host's cores, started from a state settled for the same number of MC
steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "attempted MC moves/s on 1 GB300 (batched vs plain GPU) at dE err ≤1e-5 vs FP64"
WORKLOAD_DESC = ("batched replicas: 256 chains, lengths log-uniform in [2000, 20000] beads (seeded), "
                 "each in its own periodic 1600 nm box with a 40^3 grid of 40 nm voxels; FP32 "
                 "positions, int64 fixed-point density, FP64 dE; two binders (eps_AA=-4, eps_BB=-3, "
                 "eps_AB=+1, mu ~ U[-1,0]); all five moves with SimpleControl; chi ladder of 16 rungs "
                 "in [0.5, 2.0], exchange every 62 MC steps (~1e4 moves per replica)")


WORKLOAD_DESCS = {
    "batched": WORKLOAD_DESC,
    "large": ("large batched: 32 chains of 100,000 beads, each in its own periodic 4000 nm box with a "
              "100^3 grid of 40 nm voxels; FP32 positions, int64 fixed-point density; two binders; "
              "one grid of 4 mu_A values x 8 chi rungs in [0.5, 2.0], chi and mu_A exchanged every 62 "
              "MC steps (~1e4 moves per replica)"),
    "diff": ("batched + differentiation: 64 chains of 5,000 beads, 40^3 grids (40 nm voxels), two "
             "binders, no exchange; dE/dr and dE/d(chi, mu_A, mu_B, eps_AA, eps_BB, eps_AB) kernels "
             "and 1e6 on-device reweighting samples reported under 'derivatives'"),
    "plain": ("plain single chain: one 10,000-bead chain in a periodic 2400 nm box with a 60^3 grid "
              "of 40 nm voxels, FP32 positions, int64 fixed-point density; one binder (mu = -0.4, "
              "eps = -4, chi = 1), marks with mean run length 50; all five moves with SimpleControl; "
              "1e6 attempted moves per step (10 steps = 1e7 moves)"),
    "small": ("plain CPU-runnable chain: one 1,000-bead chain in a periodic 1200 nm box with a 30^3 grid "
              "of 40 nm voxels, FP64 positions; one binder (mu = -0.4, eps = -4, chi = 1), marks with "
              "mean run length 20; specific_moves (one attempt of each of the five moves per MC "
              "step) with SimpleControl; 1e4 MC steps per step (10 steps = 1e5 attempts per move kind)"),
    "sphere": ("confined batched: 256 chains of 5,000 beads, each confined to a sphere of radius "
               "700 nm inside its 1600 nm box with a 40^3 grid of 40 nm voxels (Spherical "
               "confinement; per-voxel accessible volumes at the surface); two binders; chi ladder "
               "of 16 rungs in [0.5, 2.0], exchange every 62 MC steps (~1e4 moves per replica)"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "large", "diff", "sphere", "plain", "small"],
                    help="batched: 256 replicas (the headline); large: 32 x 100,000 beads with a "
                         "chi x mu ladder; diff: 64 x 5,000 beads plus the derivative kernels and 1e6 "
                         "reweighting samples; sphere: 256 confined chains; plain: one 10,000-bead "
                         "chain, 1e7 moves; small: one 1,000-bead FP64 chain, 1e5 attempts per move kind")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-budget", type=float, default=2.0)
    ap.add_argument("--profile", action="store_true",
                    help="case for ncu: 256 x 5000-bead replicas settled for %d MC launches, then "
                         "1 warm-up + 2 MC launches" % 80)
    return ap.parse_args()


def profile_case(args):
    """A bounded case for profilers: 256 replicas of 5,000 beads each (the
    batched workload's CTA shape), 40^3 grids of 3 int64 columns (393 MB of
    grids: larger than L2, under 1 GB on the device), brought to steady state
    by SETTLE_ROUNDS launches of the MC kernel (62 steps each), then one
    warm-up launch and two launches: a profiler captures MC launch number
    SETTLE_ROUNDS + 2 (-k regex:spec_kernel -s SETTLE_ROUNDS+1 -c 1)."""
    import numpy as np
    import torch
    from chromo_gb300.build import build
    build()
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("profile")
    sim = wl.build_sim(w, warps_per_block=6, lanes_per_move=32)
    sh = torch.cuda.current_stream().cuda_stream
    for k in range(SETTLE_ROUNDS):
        sim.run(w.steps_per_round, 1000 + k, sh)
    sim.run(w.steps_per_round, 1, sh)
    sim.sync(sh)
    sim.reset_tally()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(2):
        sim.run(w.steps_per_round, 2 + i, sh)
    e1.record()
    torch.cuda.synchronize()
    sim.sync(sh)
    tal = np.stack([sim.tally(r) for r in range(w.replicas)])
    moves = float(tal[:, :, 0].sum())
    ms = e0.elapsed_time(e1)
    print(json.dumps({"case": "profile", "replicas": int(w.replicas), "moves": moves, "ms": ms,
                      "moves_per_s": moves / (ms / 1000.0),
                      "algorithmic_bytes": wl.algorithmic_bytes(tal, w.n_binders),
                      "move_stats": wl.move_stats(tal)}), flush=True)


# Exchange rounds (62 MC steps each) run before the warm-up rounds: after
# 4,960 MC steps the bead amplitudes of crank shaft, end pivot and slide sit at
# their bounds (150 beads) and the per-round cost has stopped growing.
SETTLE_ROUNDS = 80
TUNE_WARMUP, TUNE_STEPS = 62, 124  # from the settled state: one round of warm-up, two timed
GUARD_TOL_ABS, GUARD_TOL_REL = 20.0, 1e-3  # drift guard bound per check (kT, relative to |E|)


def settled_state(w, chains, stream, rounds=SETTLE_ROUNDS, sim=None):
    """(chains, controllers per replica) after `rounds` exchange rounds of the
    workload (the default launch shape; untimed)."""
    from chromo_gb300 import workloads as wl
    own = sim is None
    if own:
        sim = wl.build_sim(w, chains)
    for _ in range(rounds):
        sim.run_batched(1, w.steps_per_round, w.n_rungs, 5, stream)
    sim.sync(stream)
    snap = ([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in sim.get_chains()],
            [sim.get_controllers(r) for r in range(w.replicas)])
    if own:
        sim.close()
    return snap


def build_settled(w, chains, snap, **shape):
    """A sim of the workload holding a settled state (chains and controllers)."""
    from chromo_gb300 import workloads as wl
    sim = wl.build_sim(w, chains, **shape)
    sim.set_chains(snap[0])
    for r in range(w.replicas):
        sim.set_controllers(r, snap[1][r])
    sim.deposit(-1)
    return sim


def _tune_child(workload, rank, local):
    """Autotune the launch shape of this rank's workload at steady state
    (fills the cache): every candidate starts from the settled state."""
    import torch
    torch.cuda.set_device(local)
    from chromo_gb300 import autotune
    from chromo_gb300 import workloads as wl
    w = wl.make_workload(workload, seed_offset=rank)
    chains = wl.make_chains(w)
    snap = settled_state(w, chains, torch.cuda.current_stream().cuda_stream)
    autotune.tune(lambda W, G: build_settled(w, chains, snap, warps_per_block=W, lanes_per_move=G),
                  w.lengths, [[w.nbins] * 3] * w.replicas, w.n_binders, steps=TUNE_STEPS,
                  warmup=TUNE_WARMUP, extra_key=workload + "-settled")


def _guard_report(sim, every, moves_per_round):
    """The on-device drift guard's checks (large workload), or None."""
    if not every:
        return None
    import numpy as np
    d, checks = sim.drift()
    return {"every_rounds": every, "moves_per_replica_between_checks": every * moves_per_round,
            "checks": checks, "max_abs_drift_kT": float(np.abs(d).max()),
            "median_abs_drift_kT": float(np.median(np.abs(d))),
            "bound": "%g kT + %g |E|" % (GUARD_TOL_ABS, GUARD_TOL_REL)}


def _at_bound(ctls):
    """Fraction of replicas whose crank-shaft, end-pivot and slide bead
    amplitudes sit at their upper bounds."""
    hit = [all(c[k].amp_bead >= int(c[k].bead_hi) for k in (0, 1, 2)) for c in ctls]
    return sum(hit) / max(1, len(hit))


def derivatives_leg(sim, w, stream):
    """Batched + differentiation: the backward kernels (dE/dr of every bead in
    FP32 and the 14 energy terms per replica, cg_gradient) timed over five
    calls, then 1e6 sampled configurations (every replica sampled after each
    MC step, T and T T^T summed on the device by cg_sample_terms) and the
    reweighting sensitivities d<O>/dtheta = -Cov(O, dE/dtheta) they give."""
    import math
    import numpy as np
    import torch
    from chromo_gb300 import workloads as wl
    from chromo_gb300.derivatives import (THETA_NAMES, observable_coefficients,
                                          reweighting_sensitivity, theta_coefficients)
    sh = stream.cuda_stream
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(5):
        grad, terms = sim.gradient()
    grad_ms = (time.perf_counter() - t0) / 5 * 1e3
    per_rep = int(math.ceil(1e6 / w.replicas))
    sim.samples(reset=True)
    sim.reset_tally()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(per_rep):
        sim.run(1, 7000 + k, sh)
        sim.sample_terms(sh)
    e1.record(stream)
    torch.cuda.synchronize()
    sim.sync(sh)
    ms = e0.elapsed_time(e1)
    sum_t, sum_tt, count = sim.samples()
    moves = float(sum(sim.tally(r)[:, 0].sum() for r in range(sim.R)))
    vint = 4.0 / 3.0 * np.pi * wl.R_INT ** 3
    O = observable_coefficients(int(w.lengths[0]), w.nbins ** 3, w.n_binders)
    sens = np.stack([reweighting_sensitivity(sum_t[r], sum_tt[r], count[r], O,
                                             theta_coefficients(w.mu[r], 1.0, [vint] * w.n_binders,
                                                                wl.VOXEL ** 3))
                     for r in range(sim.R)])
    names = [f"occupancy_{b}" for b in range(w.n_binders)] + ["density_variance"]
    mean = {f"d<{o}>/d{t}": float(sens[:, i, j].mean()) for i, o in enumerate(names)
            for j, t in enumerate(THETA_NAMES) if (o.startswith("occ") and t in ("chi", "mu_0", "mu_1"))
            or (o == "density_variance" and t == "chi")}
    return {"gradient_ms_per_call": grad_ms,
            "gradient": "dE/dr of all %d beads (FP32) + 14 energy terms per replica" % int(w.lengths.sum()),
            "sampled_configurations": int(count.sum()), "sampling_s": ms / 1e3,
            "configurations_per_s": float(count.sum()) / (ms / 1e3),
            "mc_moves_during_sampling": moves,
            "mean_sensitivities_over_replicas": mean}


# MC steps per bench step of the single-chain workloads: ~1e6 attempted moves
# on the 10,000-bead chain (10 steps = the 1e7 moves of that configuration);
# 1e4 MC steps of one attempt per move kind on the 1,000-bead chain (10 steps
# = 1e5 attempts of every move kind)
SINGLE_STEP_MC = {"plain": 6200, "small": 10000}


def single_chain_bench(args, rank, world):
    """One chain on the production kernel (one CTA): the plain configurations.
    W warm-up steps from the seeded start, K timed steps (one MC launch each,
    CUDA events on the launching stream), then the same K steps from the same
    start state through the C ABI with host buffers (upload, re-deposit, run,
    read back every step), and the reference's mc_sim on one host core from
    the state after the same warm-up MC steps (the C restatement advances the
    chain there; the reference then times itself)."""
    import numpy as np
    import torch
    from chromo_gb300.build import build
    build()
    from chromo_gb300 import workloads as wl
    torch.cuda.set_device(0 if world == 1 else rank % max(1, torch.cuda.device_count()))
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    w = wl.make_workload(args.workload, seed_offset=rank)
    step_mc = SINGLE_STEP_MC[args.workload]
    sim = wl.build_sim(w)
    warm = max(args.warmup, 3)
    for k in range(warm):
        sim.run(step_mc, 100 + k, sh)
    sim.sync(sh)
    start_chains = sim.get_chains()
    start_ctl = sim.get_controllers(0)
    sim.close()
    # launch shape from the autotuner, every candidate started from the
    # warmed-up state (untimed; cached per problem)
    from chromo_gb300 import autotune

    def build_at_start(W, G):
        s = wl.build_sim(w, warps_per_block=W, lanes_per_move=G)
        s.set_chains([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in start_chains])
        s.set_controllers(0, start_ctl)
        s.deposit(-1)
        return s

    tune_steps = max(50, step_mc // 20)
    shape, tune_table = autotune.tune(build_at_start, w.lengths, [[w.nbins] * 3], w.n_binders,
                                      pos_fp64=w.pos_fp64, steps=tune_steps, warmup=tune_steps // 5,
                                      extra_key=args.workload + "-warm")
    sim = build_at_start(*shape)
    sim.reset_tally()
    barrier(world)
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(torch.cuda.current_device()) as clocks:
        evs[0].record(stream)
        for k in range(args.steps):
            sim.run(step_mc, 200 + k, sh)
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
    sim.sync(sh)
    barrier(world)
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = evs[0].elapsed_time(evs[-1])
    ms_max = allreduce_max(ms, world)
    tal = sim.tally(0)[None]
    attempts = float(tal[:, :, 0].sum())
    value = allreduce_sum(attempts, world) / (ms_max / 1000.0)
    pos_bytes = 24 if w.pos_fp64 else 12
    peak, peak_kind = load_peaks()
    achieved = wl.algorithmic_bytes(tal, w.n_binders, pos_bytes) / (ms / 1000.0) / 1e9
    # e2e: the same K steps from the same start through the C ABI with host buffers
    sim.set_chains([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in start_chains])
    sim.set_controllers(0, start_ctl)
    spare, other = sim.get_chains(), sim.get_chains()
    inp, t_e2e = start_chains, 0.0
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.set_chains([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in inp])
        sim.deposit(-1)
        sim.run(step_mc, 200 + k, sh)
        sim.sync(sh)
        out = sim.get_chains(out=spare)
        t_e2e += time.perf_counter() - t0
        spare = other if k == 0 else inp
        inp = out
    n = int(w.lengths[0])
    io_bytes = n * ((3 * 24 + 8 * w.n_binders) if sim.direct_transfers() else (3 * (32 if w.pos_fp64 else 16) + 4))
    e2e_value = allreduce_sum(attempts, world) / allreduce_max(t_e2e, world)
    launch = sim.launch_shape()
    sim.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import refbench
        cpu = refbench.run(args.workload, budget=max(args.cpu_budget, 10.0), n_procs=1,
                           settle_steps=warm * step_mc)
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if w.pos_fp64 else "f32",
        "data": "synthetic (seeded Gaussian-walk chain, Markov mark track)",
        "config": {"workload": WORKLOAD_DESCS[args.workload], "replicas": 1, "beads_total": n,
                   "mc_steps_per_step": step_mc, "attempted_moves_per_step": int(attempts / args.steps),
                   "warmup_mc_steps": warm * step_mc,
                   "l2": "single chain: its state (%.1f MB) is L2-resident; nothing is flushed"
                         % ((w.nbins ** 3 * 16 + n * 104) / 1e6),
                   "launch_shape": dict(zip(("warps_per_replica", "lanes_per_move", "moves_in_flight",
                                             "hash_slots"), launch)),
                   "autotune_moves_per_s": {k: round(v) for k, v in tune_table.items()}},
        "rounds": {"step_ms": [round(x, 3) for x in step_ms]},
        "move_stats": wl.move_stats(tal),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "traffic_note": "not captured for the single-chain workloads",
                     "kernel": "spec_kernel<%s,32>" % ("double" if w.pos_fp64 else "float"),
                     "peak_source": peak_kind, "avg_launch_ms": ms / args.steps,
                     "timing": "one MC launch per step, CUDA events on the launching stream"},
        "e2e": {"value": e2e_value, "unit": "moves/s", "h2d_bytes_per_step": io_bytes,
                "d2h_bytes_per_step": io_bytes,
                "path": "C ABI, host-driven steps: cg_set_chains, cg_deposit, cg_run, cg_get_chains"},
        "gpu_launches": args.steps,
        "clocks": clocks.summary(),
    }
    if cpu is not None:
        out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(out), flush=True)


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import statistics
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    from chromo_gb300 import distributed
    return distributed.init("nccl")


def barrier(world):
    from chromo_gb300 import distributed
    distributed.barrier(world)


def allreduce_max(x, world):
    from chromo_gb300 import distributed
    return distributed.allreduce(x, "max", world)


def allreduce_sum(x, world):
    from chromo_gb300 import distributed
    return distributed.allreduce(x, "sum", world)


def reference_arm(args, rank, world):
    if rank != 0:
        return
    from oracle import refbench
    from chromo_gb300.workloads import make_workload
    w = make_workload(args.workload)
    per_step = 1.0
    settle = (max(args.warmup, 3) * SINGLE_STEP_MC[args.workload] if args.workload in SINGLE_STEP_MC
              else SETTLE_ROUNDS * w.steps_per_round)
    res = refbench.run(args.workload, budget=per_step * (args.steps + args.warmup),
                       n_procs=os.cpu_count(), settle_steps=settle)
    out = {
        "impl": "reference", "metric": METRIC, "value": res["value"], "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_DESCS[args.workload],
                   "replicas": int(w.replicas)},
        "cpu_baseline": {"value": res["value"], "unit": "moves/s", "cores": res["cores"],
                         "kind": res["kind"], "sample": res["sample"]},
        "e2e": {"value": res["value"], "unit": "moves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if res.get("fallback_reason"):
        out["cpu_baseline"]["note"] = "reference unavailable (" + res["fallback_reason"] + "); C port timed"
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.profile:
        profile_case(args)
        return
    rank, world, local = dist_init(args)
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload in SINGLE_STEP_MC:
        single_chain_bench(args, rank, world)
        return
    # wall seconds of each untimed setup phase and timed leg, reported with the line
    phases, t_last = {}, [time.perf_counter()]

    def mark(name):
        now = time.perf_counter()
        phases[name] = round(now - t_last[0], 2)
        t_last[0] = now

    import numpy as np
    import torch
    from chromo_gb300.build import build
    build()
    import chromo_gb300._native as nat
    from chromo_gb300 import workloads as wl
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    w = wl.make_workload(args.workload, seed_offset=rank)
    mark("import_and_build")
    chains = wl.make_chains(w)
    mark("make_chains")
    # launch shape (warps per replica, lanes per move) picked by the autotuner
    # on scratch copies of this workload (untimed; cached per problem).  The
    # tuning runs in a child process so that its scratch allocations leave
    # no trace in this process's device memory.
    from chromo_gb300 import autotune
    import multiprocessing as mp
    child = mp.get_context("spawn").Process(target=_tune_child, args=(args.workload, rank, local))
    child.start()
    child.join()
    if child.exitcode != 0:
        print(f"autotune child exited with {child.exitcode}; tuning in this process", file=sys.stderr)
    snap = []

    def build_for_tuning(W, G):  # only when the child left no cached result
        if not snap:
            snap.append(settled_state(w, chains, sh))
        return build_settled(w, chains, snap[0], warps_per_block=W, lanes_per_move=G)

    shape, tune_table = autotune.tune(
        build_for_tuning, w.lengths, [[w.nbins] * 3] * w.replicas, w.n_binders, steps=TUNE_STEPS,
        warmup=TUNE_WARMUP, extra_key=args.workload + "-settled")
    snap.clear()
    mark("autotune")
    sim = wl.build_sim(w, chains, warps_per_block=shape[0], lanes_per_move=shape[1])
    if w.mu_rungs:
        sim.set_mu_ladder(w.mu_rungs, 0)
    steps_round = w.steps_per_round
    moves_round = w.replicas * steps_round * w.moves_per_step
    guard_every, guard = 0, None
    if args.workload == "large":
        # the on-device FP64 full-energy recompute every ~1e5 moves per replica,
        # inside the captured round; the tolerance covers the reference's
        # tangent-rotation rule for adjacent beads (its summed dE is not the
        # energy change) and FP32 rounding
        guard_every = int(np.ceil(1e5 / (steps_round * w.moves_per_step)))
        sim.set_drift_guard(guard_every, tol_abs=GUARD_TOL_ABS, tol_rel=GUARD_TOL_REL)
    warm = max(args.warmup, 3)
    # the MC kernel of every round is timed on the device (event-record nodes
    # in the replayed graph), settle and warm-up rounds included
    sim.set_round_timing(SETTLE_ROUNDS + warm + args.steps)
    mark("build_sim")
    # ---- settle: the controllers reach steady state (graph capture on the first round)
    for _ in range(SETTLE_ROUNDS):
        sim.run_batched(1, steps_round, w.n_rungs, 11 + rank, sh)
    sim.sync(sh)
    settle_ctl = [sim.get_controllers(r) for r in range(w.replicas)]
    mark("settle")
    # ---- warm-up rounds
    for _ in range(warm):
        sim.run_batched(1, steps_round, w.n_rungs, 11 + rank, sh)
    sim.sync(sh)
    sim.reset_tally()
    # the state the timed rounds start from (chains and move controllers),
    # restored for the end-to-end leg so that both legs do the same MC work
    start_chains = sim.get_chains()
    start_ctl = [sim.get_controllers(r) for r in range(w.replicas)]
    # ---- timed rounds
    barrier(world)
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        evs[0].record(stream)
        for k in range(args.steps):
            sim.run_batched(1, steps_round, w.n_rungs, 11 + rank, sh)
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
    sim.sync(sh)
    barrier(world)
    round_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = evs[0].elapsed_time(evs[-1])
    ms_max = allreduce_max(ms, world)
    tal = np.stack([sim.tally(r) for r in range(w.replicas)])
    attempts = float(tal[:, :, 0].sum())
    total_attempts = allreduce_sum(attempts, world)
    value = total_attempts / (ms_max / 1000.0)
    mc_ms_all = sim.round_times()
    settle_mc_ms = mc_ms_all[:SETTLE_ROUNDS]
    mc_ms = mc_ms_all[-args.steps:]
    mark("warmup_and_timed")
    # ---- roofline: the MC kernel of the timed rounds themselves
    avg_launch_s = float(np.mean(mc_ms)) / 1000.0
    bytes_per_launch = wl.algorithmic_bytes(tal, w.n_binders) / args.steps
    peak, peak_kind = load_peaks()
    achieved = bytes_per_launch / avg_launch_s / 1e9
    # DRAM bytes per attempted move of one MC launch of this workload at steady
    # state, from the committed ncu capture, times the moves of one launch
    traffic, traffic_src = None, None
    prof = ROOT / "profiles" / f"spec_kernel_{args.workload}_dram.json"
    if prof.exists():
        d = json.loads(prof.read_text())
        traffic = float(d["dram_bytes_per_attempted_move"]) * attempts / args.steps
        traffic_src = f"profiles/{prof.name}"
    # ---- energy drift: FP64 energies recomputed on the device (cg_energies)
    # around three MC launches (~3e4 moves per replica, no exchange) against
    # the running sum of accepted dE.  Includes the reference's tangent-rotation
    # rule (adjacent rotated beads each see the other's current tangent,
    # chromo/polymers.pyx:1074-1080), so it is not rounding alone.
    en0 = sim.energies(sh)
    for i in range(3):
        sim.run(steps_round, 301 + i, sh)
    sim.sync(sh)
    en1 = sim.energies(sh)
    E0, E1 = en0[:, :3].sum(1), en1[:, :3].sum(1)
    d_true = E1 - E0
    d_run = en1[:, 3] - en0[:, 3]
    # a replica whose energy still carries a 1e99 penalty (a voxel above the
    # volume-fraction limit, or a bead outside the confinement) at either end
    # has no drift measurable in FP64
    soft = (np.abs(E0) < 1e20) & (np.abs(E1) < 1e20)
    drift_abs = np.abs(d_true - d_run)[soft]
    drift = {"max_abs_kT": float(drift_abs.max()), "median_abs_kT": float(np.median(drift_abs)),
             "max_rel_to_energy": float((drift_abs / np.maximum(1.0, np.abs(E1[soft]))).max()),
             "moves_per_replica": int(3 * steps_round * w.moves_per_step),
             "replicas_with_penalised_energy": int((~soft).sum()),
             "how": "FP64 full-energy recompute on the device before and after 3 MC launches "
                    "vs the running sum of accepted dE"}
    mark("energy_drift")
    # ---- e2e through the C ABI with host buffers: the same K rounds from the
    # same start state (chains and controllers).  Every step uploads its input
    # chains from host memory (all replicas: positions, tangents, binding
    # states), rebuilds the densities, runs one exchange round and reads the
    # resulting chains back; the next step's input is that snapshot.
    pos_b = 16
    spare, other = sim.get_chains(), sim.get_chains()  # host snapshot buffers, allocated untimed
    sim.set_chains([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in start_chains])  # pinned staging
    for r in range(w.replicas):
        sim.set_controllers(r, start_ctl[r])
    if guard_every:  # the guard's reference energies belong to the state just uploaded
        guard = _guard_report(sim, guard_every, steps_round * w.moves_per_step)
        sim.set_drift_guard(guard_every, tol_abs=GUARD_TOL_ABS, tol_rel=GUARD_TOL_REL)
    inp = start_chains
    t_e2e = 0.0
    e2e_parts = np.zeros(4)  # seconds in upload, re-deposit, round, read-back
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.set_chains([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in inp])
        t1 = time.perf_counter()
        sim.deposit(-1)  # the densities of the uploaded chains
        t2 = time.perf_counter()
        sim.run_batched(1, steps_round, w.n_rungs, 11 + rank, sh)
        sim.sync(sh)
        t3 = time.perf_counter()
        out = sim.get_chains(out=spare)
        t4 = time.perf_counter()
        t_e2e += t4 - t0
        e2e_parts += (t1 - t0, t2 - t1, t3 - t2, t4 - t3)
        spare = other if k == 0 else inp  # the start snapshot is never overwritten
        inp = out
    nbeads = int(w.lengths.sum())
    direct = sim.direct_transfers()
    # bytes across the host-device link per step: the caller's FP64 arrays and
    # int64 states read (written) by the GPU itself, or the packed FP32
    # 4-vectors and 32-bit state words of the staged path
    h2d = nbeads * ((3 * 24 + 8 * w.n_binders) if direct else (3 * pos_b + 4))
    d2h = h2d
    e2e_value = allreduce_sum(moves_round * args.steps, world) / allreduce_max(t_e2e, world)
    mark("e2e")
    # ---- plain single chain (one CTA) on the same kernel, settled for the
    # same number of MC steps as the batched replicas
    wp = wl.make_workload("plain", seed_offset=rank)
    psim = wl.build_sim(wp)
    psim.run(SETTLE_ROUNDS * steps_round, 5, sh)
    psim.sync(sh)
    p_snap = (psim.get_chains(), [psim.get_controllers(0)])
    psim.reset_tally()
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pe0.record(stream)
    psim.run(300, 6, sh)
    pe1.record(stream)
    torch.cuda.synchronize()
    psim.sync(sh)
    p_att = float(psim.tally(0)[:, 0].sum())
    plain_value = p_att / (pe0.elapsed_time(pe1) / 1000.0)
    psim.close()
    # the same chain with one move in flight (one warp, no speculative
    # batching): the kernel run strictly one move after the other
    ssim = wl.build_sim(wp, warps_per_block=1)
    ssim.set_chains([dict(r=r, t3=t3, t2=t2, states=st) for r, t3, t2, st in p_snap[0]])
    ssim.set_controllers(0, p_snap[1][0])
    ssim.deposit(-1)
    ssim.reset_tally()
    pe0.record(stream)
    ssim.run(100, 6, sh)
    pe1.record(stream)
    torch.cuda.synchronize()
    ssim.sync(sh)
    seq_value = float(ssim.tally(0)[:, 0].sum()) / (pe0.elapsed_time(pe1) / 1000.0)
    ssim.close()
    launches = args.steps * (3 if w.n_rungs else 1)
    mark("plain")
    deriv = derivatives_leg(sim, w, stream) if args.workload == "diff" else None
    mark("derivatives")
    # CPU baseline last (spawned workers), so that the host cores it loads do
    # not share the timed GPU legs' power and memory budget
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import refbench
        cpu = refbench.run(args.workload, budget=args.cpu_budget, n_procs=os.cpu_count(),
                           settle_steps=SETTLE_ROUNDS * steps_round)
    mark("cpu_baseline")
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian-walk chains, Markov mark tracks)",
            "config": {"workload": WORKLOAD_DESCS[args.workload], "replicas": int(w.replicas),
                       "beads_total": nbeads, "mc_steps_per_step": steps_round,
                       "attempted_moves_per_step": int(attempts / args.steps),
                       "l2": "inputs larger than L2 (%.0f MB of grids and chains > 129 MB)"
                             % ((w.replicas * w.nbins ** 3 * 32 + nbeads * 104) / 1e6),
                       "graph": "one exchange round captured in a CUDA graph, replayed per step",
                       "settle": {"rounds": SETTLE_ROUNDS, "mc_steps": SETTLE_ROUNDS * steps_round,
                                  "bead_amplitudes_at_bound": _at_bound(settle_ctl),
                                  "mc_kernel_ms_every_10th_round":
                                      [round(float(x), 2) for x in settle_mc_ms[::10]]},
                       "launch_shape": dict(zip(("warps_per_replica", "lanes_per_move", "moves_in_flight",
                                                 "hash_slots"), sim.launch_shape())),
                       "autotune_moves_per_s": {k: round(v) for k, v in tune_table.items()}},
            "rounds": {"round_ms": [round(x, 3) for x in round_ms],
                       "mc_kernel_ms": [round(float(x), 3) for x in mc_ms]},
            "move_stats": wl.move_stats(tal),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                         # the lean form serves launches without SSTWLC twist
                         "kernel": "spec_kernel<float,%d,true>" % sim.launch_shape()[1],
                         "peak_source": peak_kind, "bytes_per_launch": bytes_per_launch,
                         "avg_launch_ms": avg_launch_s * 1e3, "moves_per_launch": attempts / args.steps,
                         "timing": "the MC kernel of the K timed rounds: CUDA event-record nodes "
                                   "around it inside the replayed graph"},
            "e2e": {"value": e2e_value, "unit": "moves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "path": "C ABI, host-driven rounds: cg_set_chains (the previous round's host "
                            "snapshot, all replicas), cg_deposit, cg_run_batched, cg_get_chains (into "
                            "reused host arrays); transfers: " +
                            ("the GPU reads and writes the pageable FP64 host arrays over NVLink-C2C"
                             if direct else "FP64 -> pinned FP32 staging -> HBM and back"),
                    "ms_per_step": dict(zip(("set_chains", "deposit", "round", "get_chains"),
                                            (round(float(x) * 1e3 / args.steps, 3) for x in e2e_parts)))},
            "plain": {"value": plain_value, "unit": "moves/s",
                      "workload": "one 10,000-bead chain, 60^3 grid, one binder, 300 MC steps after "
                                  "%d settle MC steps" % (SETTLE_ROUNDS * steps_round),
                      "batched_over_plain": value / plain_value,
                      "one_move_in_flight": {"value": seq_value, "unit": "moves/s",
                                             "workload": "the same chain, one warp, 100 MC steps",
                                             "batched_over": value / seq_value}},
            "energy_drift": drift,
            "drift_guard": guard,
            "gpu_launches": launches,
            "clocks": clocks.summary(),
            "phase_seconds": phases,
        }
        if deriv is not None:
            out["derivatives"] = deriv
        if cpu is not None:
            out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
