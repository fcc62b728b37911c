"""Load the golden cases written by ``tests/golden/make_golden.py``."""
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))
MOVE_NAMES = ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]


def load(name):
    with np.load(GOLDEN / f"{name}.npz", allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def oracle_system(g, pos="f64", fixed_density=0, state="0"):
    """Build an ``oracle.OracleSystem`` from a golden case (initial state by default)."""
    from oracle.oracle import OracleSystem
    return OracleSystem(
        r=g["r" + state], t3=g["t3" + state], t2=g["t2" + state],
        states=g["states" + state], marks=g["marks"],
        eps_bend=g["eps_bend"], gamma=g["gamma"], eps_par=g["eps_par"],
        eps_perp=g["eps_perp"], eta=g["eta"], sites=g["sites"], e_mod=g["e_mod"],
        e_nomod=g["e_nomod"], mu=g["mu"], mu_adjust_factor=float(g["mu_adjust_factor"]),
        max_binders=int(g["max_binders"]), field_kind=int(g["field_kind"]),
        confine_kind=int(g["confine_kind"]), confine_length=float(g["confine_length"]),
        nxyz=tuple(int(x) for x in g["nxyz"]), widths=tuple(float(x) for x in g["widths"]),
        access_vol=g.get("access_vols"), chi=float(g["chi"]), vf_limit=float(g["vf_limit"]),
        bead_vol=4.0 / 3.0 * np.pi * float(g["bead_rad"]) ** 3,
        pref=g["pref"], intra=g["intra"], xpref=g["xpref"], pos=pos,
        fixed_density=fixed_density, fast_n=int(g.get("fast_n", 0)),
        eps_twist=g.get("eps_twist"), omega0=g.get("omega0"))


def oracle_ctls(g):
    from oracle.oracle import make_ctl
    out = []
    for k, row in enumerate(g["ctl0"]):
        amp_move, amp_bead, npc, simple, blo, bhi, mlo, mhi = row
        out.append(make_ctl(MOVE_NAMES[k], amp_move=amp_move, amp_bead=int(amp_bead),
                            num_per_cycle=int(npc), simple=bool(simple),
                            bead_bounds=(blo, bhi), move_bounds=(mlo, mhi)))
    return out


def gpu_sim(g, pos_fp64, state="0", warps_per_block=0, lanes_per_move=0):
    """A one-replica ``chromo_gb300._native.Sim`` holding a golden case (at the
    library's default launch shape unless one is given)."""
    from chromo_gb300 import _native as nat
    from chromo_gb300.device import binding_params, bonds_array, field_params, move_ctl
    n, nb = g["states0"].shape
    uniform = int(g["field_kind"]) == 2
    ctl0 = g["ctl0"]
    max_seg = int(max(max(row[1], row[5]) for k, row in enumerate(ctl0) if k != 3)) + 2
    max_tan = int(max(ctl0[3][1], ctl0[3][5]))
    access = g.get("access_vols")
    sim = nat.Sim([n], [list(g["nxyz"])], nb, pos_fp64=pos_fp64, max_segment=max_seg,
                  max_tangent=max_tan, nonuniform_access=access is not None,
                  warps_per_block=warps_per_block, lanes_per_move=lanes_per_move)
    sim.set_chain(0, r=g["r" + state], t3=g["t3" + state], t2=g["t2" + state],
                  states=g["states" + state], marks=g["marks"],
                  bonds=bonds_array(g["eps_bend"], g["gamma"], g["eps_par"], g["eps_perp"], g["eta"]))
    sim.set_field(0, field_params(
        field_kind=int(g["field_kind"]), confine_kind=int(g["confine_kind"]),
        confine_length=float(g["confine_length"]), nxyz=g["nxyz"], widths=g["widths"],
        n_binders=nb, chi=float(g["chi"]), vf_limit=float(g["vf_limit"]),
        bead_vol=4.0 / 3.0 * np.pi * float(g["bead_rad"]) ** 3, pref=g["pref"], intra=g["intra"],
        xpref=g["xpref"], fast_field=int(g.get("fast_n", 0)) > 0,
        n_points=int(g.get("fast_n", 0)) or 1000), access_vol=access)
    sim.set_binding(0, binding_params(sites=g["sites"], e_mod=g["e_mod"], e_nomod=g["e_nomod"],
                                      mu=g["mu"], mu_adjust_factor=float(g["mu_adjust_factor"]),
                                      max_binders=int(g["max_binders"])))
    ctls = []
    for k, row in enumerate(ctl0):
        amp_move, amp_bead, npc, simple, blo, bhi, mlo, mhi = row
        ctls.append(move_ctl(MOVE_NAMES[k], amp_move=amp_move, amp_bead=int(amp_bead),
                             num_per_cycle=int(npc), simple=bool(simple), bead_bounds=(blo, bhi),
                             move_bounds=(mlo, mhi)))
    sim.set_controllers(0, ctls)
    if "eps_twist" in g:
        sim.set_twist(0, g["eps_twist"], g["omega0"])
    if uniform:
        sim.deposit(0)
    return sim
