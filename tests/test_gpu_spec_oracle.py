"""The production MC kernel, move by move, against the oracle.

``spec_kernel`` -- the kernel behind ``cg_run`` / ``cg_run_batched`` and every
throughput number -- runs with its per-move log on (``cg_run_logged``).  The
oracle (the C restatement of the reference's loop, pinned bit for bit to the
reference's own ``mc_sim`` on the golden cases) replays the same attempted
moves from the same Philox sub-streams (``or_mc_sim_philox``) in its
FP32-storage, fixed-point-grid mode and evaluates each move's dE in FP64.  The
contract is the reference's per-move one (chromo/mc/mc_sim.pyx:144-182):

* segment bounds, bead counts and draws consumed per move: identical;
* |dE_gpu - dE_oracle| <= 1e-5 * max(1, |dE_oracle|) for every move;
* decisions identical; inside the tie band |dE + ln u| <= 1e-5 * max(1, |dE|),
  where FP32 arithmetic may legitimately decide the other way, the oracle
  takes the GPU's decision and the test reports how many moves did;
* final chains, binding states, controllers and density grid bit-identical.

Cases: replicas of the batched configuration (two binders with cross talk,
eps_AA = -4, eps_BB = -3, eps_AB = +1 on A; 40^3 grids; chains of 2,000,
5,000 and 20,000 beads) at the production launch shapes (6 warps x 32 lanes,
the autotuner's pick on the 256-replica workload, and 16- and 8-lane shapes),
first under the full move mix, then 10,000 attempts of each move kind with
the kind's cycle lengthened so that its moves are evaluated many at a time;
and every golden case, including the volume-fraction-limit regime, whose
1e99 penalties are summed exactly on both sides.
"""
import numpy as np
import pytest

from golden_cases import CASES, MOVE_NAMES, gpu_sim, load, oracle_ctls, oracle_system

pytestmark = pytest.mark.gpu
TOL = 1e-5
SEED = 0x5EC0A11D
SHAPES = [(6, 32), (4, 16), (2, 8)]  # (warps per replica, lanes per move)
REPLICAS = [245, 1, 77]               # batched replicas of 2,057, 4,991 and 19,763 beads


def _dE(r):
    return r["dE_poly"] + r["dE_field"]


def compare_records(g, o, tol=TOL, label=""):
    """Per-move equality of one replica's GPU log `g` and oracle records `o`."""
    assert len(g) == len(o), (label, len(g), len(o))
    for f in ("kind", "n_inds", "ind0", "indf", "n_draws", "accepted"):
        bad = np.nonzero(g[f] != o[f])[0]
        assert not len(bad), f"{label}: {f} differs first at move {bad[0]}: {g[bad[0]]} vs {o[bad[0]]}"
    ok = o["accepted"] >= 0
    a, b = _dE(g)[ok], _dE(o)[ok]
    err = np.abs(a - b) / np.maximum(1.0, np.abs(b))
    worst = float(err.max()) if len(err) else 0.0
    assert worst <= tol, f"{label}: dE error {worst:.3e} at move {np.nonzero(ok)[0][np.argmax(err)]}"
    return worst


def compare_state(sim, rep, o, ctls_gpu, ctls_o, label=""):
    r, t3, t2, st = sim.get_chain(rep)
    np.testing.assert_array_equal(r.astype(o.r.dtype), o.r, err_msg=label)
    np.testing.assert_array_equal(t3.astype(o.r.dtype), o.t3, err_msg=label)
    np.testing.assert_array_equal(t2.astype(o.r.dtype), o.t2, err_msg=label)
    np.testing.assert_array_equal(st, o.states, err_msg=label)
    np.testing.assert_array_equal(sim.density(rep), o.density_fx, err_msg=label)
    for cg_, co in zip(ctls_gpu, ctls_o):
        for f in ("amp_move", "amp_bead", "acc_rate", "num_attempt", "num_success"):
            assert getattr(cg_, f) == getattr(co, f), (label, f, getattr(cg_, f), getattr(co, f))


# ------------------------------------------------------------ batched replicas

def _batched_subset():
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("batched")
    chains = wl.make_chains(w)
    rng = np.random.default_rng(20261205)
    sub = wl.Workload("batched-subset", w.lengths[REPLICAS], w.nbins, w.n_binders, w.mu[REPLICAS],
                      w.chi[REPLICAS], w.eps, w.cross, w.run_length, 0, w.seed)
    picked = []
    for j in REPLICAS:
        c = chains[j]
        c.states = rng.integers(0, 3, size=c.states.shape).astype(np.int64)
        picked.append(c)
    return sub, picked


def _oracle_for(w, c, rep, pos="f32"):
    """The oracle system holding replica `rep` of workload `w` (chain `c`),
    with the GPU's FP32 storage arithmetic (pos="f32") or FP64 storage."""
    from chromo_gb300 import workloads as wl
    from chromo_gb300.energetics import dss_parameters, field_prefactors
    from oracle.oracle import OracleSystem
    n, nb = int(w.lengths[rep]), w.n_binders
    _, eb, gam, ep, epp, eta = dss_parameters(np.full(n - 1, wl.BEAD_SPACING), wl.LP)
    vint = 4.0 / 3.0 * np.pi * wl.R_INT ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint] * nb, w.cross, wl.binder_names(nb), wl.VOXEL ** 3)
    width = w.nbins * wl.VOXEL
    o = OracleSystem(r=c.r, t3=c.t3, t2=c.t2, states=c.states, marks=c.marks, eps_bend=eb, gamma=gam,
                     eps_par=ep, eps_perp=epp, eta=eta, sites=[wl.SITES] * nb,
                     e_mod=[wl.HP1_E_MOD] * nb, e_nomod=[wl.HP1_E_NOMOD] * nb, mu=w.mu[rep],
                     mu_adjust_factor=1.0, max_binders=-1, field_kind=2, confine_kind=0,
                     nxyz=(w.nbins,) * 3, widths=(width,) * 3, chi=float(w.chi[rep]), vf_limit=0.5,
                     bead_vol=4.0 / 3.0 * np.pi * wl.BEAD_RAD ** 3, pref=np.asarray(pref),
                     intra=np.asarray(intra), xpref=np.asarray(xpref), pos=pos, fixed_density=1)
    o.deposit_all()
    return o


# (name, the only move kind on or None for the full mix, its cycle length, MC
# steps, amplitudes start at the lower or upper bounds): the mix from the start
# amplitudes, the mix from the widest ones (150-bead segments: the steady state
# of the benchmark, with moves too large for shared-memory voxel tables), then
# each kind alone from the widest amplitudes
PHASES = ([("mix", None, None, 40, 0), ("mix-wide", None, None, 40, 1)]
          + [(m, m, 250, 40, 1) for m in MOVE_NAMES])


def controllers(factory, n_beads, only, npc, wide=0):
    """all_moves + SimpleControl at the reference's amplitude bounds
    (chromo/mc/__init__.py:295-332), starting from the lower bounds (or from
    the upper ones with `wide`); with `only`, that kind alone, `npc` moves per
    cycle (the others' amplitudes still updated once per step, as their
    controllers are in the reference's loop)."""
    from chromo_gb300 import workloads as wl
    bead, move = wl.amplitude_bounds(n_beads)
    out = []
    for m in MOVE_NAMES:
        amp_bead = int(bead[m][wide])
        if wide and m == "tangent_rotation":  # up to 200 beads (the bound, N, is never reached)
            amp_bead = min(200, amp_bead)
        c = factory(m, amp_move=move[m][wide], amp_bead=amp_bead,
                    num_per_cycle=npc if only == m else wl.NUM_PER_CYCLE[m], simple=True,
                    bead_bounds=bead[m], move_bounds=move[m])
        if only is not None and m != only:
            c.move_on = 0
        out.append(c)
    return out


def _cap(steps, npc):
    return steps * (npc or 161) + 10


@pytest.fixture(scope="module")
def batched_reference():
    """Runs the bench shape with its move log and checks every phase against
    the oracle (which follows the GPU's decisions in the tie band); returns the
    logs and final state for the other shapes."""
    from chromo_gb300 import workloads as wl
    from chromo_gb300.device import move_ctl
    from oracle.oracle import make_ctl
    w, chains = _batched_subset()
    W, G = SHAPES[0]
    sim = wl.build_sim(w, chains, warps_per_block=W, lanes_per_move=G)
    oracles = [_oracle_for(w, chains[k], k) for k in range(w.replicas)]
    move_pos = [0] * w.replicas
    out = {"phases": [], "ties": 0, "worst": 0.0, "w": w}
    for name, only, npc, steps, wide in PHASES:
        for rep in range(w.replicas):
            sim.set_controllers(rep, controllers(move_ctl, int(w.lengths[rep]), only, npc, wide))
        logs = sim.run_logged(steps, SEED, _cap(steps, npc))
        for rep in range(w.replicas):
            label = f"{name} rep {rep}"
            ctl_o = controllers(make_ctl, int(w.lengths[rep]), only, npc, wide)
            o_rec, move_pos[rep], ties = oracles[rep].mc_sim_philox(
                ctl_o, steps, SEED, rep, move_pos[rep], follow=logs[rep]["accepted"])
            out["ties"] += ties
            out["worst"] = max(out["worst"], compare_records(logs[rep], o_rec, label=label))
            compare_state(sim, rep, oracles[rep], sim.get_controllers(rep), ctl_o, label=label)
        out["phases"].append(logs)
    out["final"] = [sim.get_chain(rep) for rep in range(w.replicas)]
    out["density"] = [sim.density(rep) for rep in range(w.replicas)]
    sim.close()
    return out


def test_batched_replicas_match_oracle_at_bench_shape(batched_reference):
    """6 warps x 32 lanes (the shape the autotuner picks for the 256-replica
    workload): every move of the mixed phase and of 10,000 attempts per move
    kind matches the oracle; state bit-identical after every phase."""
    ref = batched_reference
    kinds = np.zeros(5, dtype=np.int64)
    for logs in ref["phases"]:
        for r in logs:
            kinds += np.bincount(r["kind"], minlength=5)
    print(f"spec kernel vs oracle: {int(kinds.sum())} moves {dict(zip(MOVE_NAMES, kinds.tolist()))}; "
          f"worst relative dE error {ref['worst']:.3e}; {ref['ties']} tie-band decisions followed")
    assert kinds.min() >= 10000 * len(REPLICAS)


@pytest.mark.parametrize("shape", SHAPES[1:])
def test_batched_replicas_same_moves_at_other_shapes(batched_reference, shape):
    """16 and 8 lanes per move: the same per-move log, bit for bit, as the
    bench shape (which the oracle pins), and the same final state and grid."""
    from chromo_gb300 import workloads as wl
    from chromo_gb300.device import move_ctl
    ref = batched_reference
    w = ref["w"]
    _, chains = _batched_subset()
    sim = wl.build_sim(w, chains, warps_per_block=shape[0], lanes_per_move=shape[1])
    for (name, only, npc, steps, wide), want in zip(PHASES, ref["phases"]):
        for rep in range(w.replicas):
            sim.set_controllers(rep, controllers(move_ctl, int(w.lengths[rep]), only, npc, wide))
        logs = sim.run_logged(steps, SEED, _cap(steps, npc))
        for rep in range(w.replicas):
            np.testing.assert_array_equal(logs[rep], want[rep], err_msg=f"{shape} {name} rep {rep}")
    for rep in range(w.replicas):
        for a, b in zip(sim.get_chain(rep), ref["final"][rep]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(sim.density(rep), ref["density"][rep])
    sim.close()


# ------------------------------------------------------------ golden cases

@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("shape", [(0, 0)] + SHAPES)
def test_golden_case_matches_oracle(name, shape):
    """Every golden case (one and two binders, cross talk, annealed positive mu
    with max_binders, the volume-fraction limit, spherical NullField,
    accessible volumes, large amplitudes) for 30 MC steps of Philox-driven
    moves; (0, 0) is the library's default launch shape for one replica."""
    g = load(name)
    W, G = shape
    sim = gpu_sim(g, pos_fp64=False, warps_per_block=W, lanes_per_move=G)
    o = oracle_system(g, pos="f32", fixed_density=1)
    if int(g["field_kind"]) == 2:
        o.deposit_all()
    steps = 30
    cap = steps * int(sum(int(row[2]) for row in g["ctl0"])) + 10
    log = sim.run_logged(steps, SEED + 7, cap)[0]
    ctl_o = oracle_ctls(g)
    orecs, _, ties = o.mc_sim_philox(ctl_o, steps, SEED + 7, 0, 0, follow=log["accepted"])
    worst = compare_records(log, orecs, label=name)
    compare_state(sim, 0, o, sim.get_controllers(0), ctl_o, label=name)
    print(f"{name} {shape}: {len(log)} moves, worst dE error {worst:.3e}, {ties} tie-band")
    sim.close()


def test_vf_limit_decisions_identical_without_following():
    """Above vf_limit the 1e99 penalties are summed exactly on both sides, so
    the decisions there are well defined: the oracle, not following the GPU,
    takes every decision the GPU takes."""
    g = load("vf_limit")
    sim = gpu_sim(g, pos_fp64=False)
    o = oracle_system(g, pos="f32", fixed_density=1)
    o.deposit_all()
    steps = 60
    cap = steps * int(sum(int(row[2]) for row in g["ctl0"])) + 10
    log = sim.run_logged(steps, SEED + 11, cap)[0]
    orecs, _, ties = o.mc_sim_philox(oracle_ctls(g), steps, SEED + 11, 0, 0)
    assert ties == 0
    compare_records(log, orecs, label="vf_limit")
    huge = np.abs(_dE(orecs)) > 1e80
    print(f"vf_limit: {len(log)} moves, {int(huge.sum())} decided by the 1e99 penalty")
    assert huge.any()
    sim.close()


# ------------------------------------------------------------ FP64 storage

def test_small_configuration_fp64_matches_oracle():
    """The CPU-runnable configuration (1,000 beads, 30^3 grid, one binder,
    FP64 storage, specific_moves: one attempt of each move kind per MC step,
    SimpleControl) on the production kernel at the library's launch shape:
    2,000 MC steps (10,000 moves) move by move against the oracle's FP64
    replay of the same Philox sub-streams.  FP64 arithmetic on both sides,
    but not the same library: the rotation angles' sin / cos are CUDA's on
    the GPU and the C library's in the oracle, which differ in the last bit
    now and then, so the chains drift apart at the 1e-12 level.  Checked:
    segments, draws and decisions identical, dE within 1e-9 relative, states
    and controllers identical, positions within 1e-9, grid cells within 16
    fixed-point units (of 2^40 per bead)."""
    from chromo_gb300 import workloads as wl
    from oracle.oracle import make_ctl
    w = wl.make_workload("small")
    chains = wl.make_chains(w)
    sim = wl.build_sim(w, chains)
    assert w.pos_fp64 and sim.pos_fp64
    o = _oracle_for(w, chains[0], 0, pos="f64")
    n = int(w.lengths[0])
    bead, move = wl.amplitude_bounds(n)
    ctl_o = [make_ctl(m, amp_move=move[m][0], amp_bead=int(bead[m][0]), num_per_cycle=1,
                      bead_bounds=bead[m], move_bounds=move[m]) for m in MOVE_NAMES]
    steps = 2000
    log = sim.run_logged(steps, SEED + 13, steps * 5 + 10)[0]
    orecs, _, ties = o.mc_sim_philox(ctl_o, steps, SEED + 13, 0, 0, follow=log["accepted"])
    assert np.all(np.bincount(log["kind"], minlength=5) == steps)
    worst = compare_records(log, orecs, tol=1e-9, label="small fp64")
    r, t3, t2, st = sim.get_chain(0)
    for a, b in ((r, o.r), (t3, o.t3), (t2, o.t2)):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9)
    np.testing.assert_array_equal(st, o.states)
    assert np.abs(sim.density(0) - o.density_fx).max() <= 16
    for cg_, co in zip(sim.get_controllers(0), ctl_o):
        for f in ("amp_move", "amp_bead", "acc_rate", "num_attempt", "num_success"):
            assert getattr(cg_, f) == getattr(co, f), (f, getattr(cg_, f), getattr(co, f))
    print(f"small fp64: {len(log)} moves, worst dE error {worst:.3e}, {ties} tie-band")
    sim.close()
