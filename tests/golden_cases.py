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
        chi=float(g["chi"]), vf_limit=float(g["vf_limit"]),
        bead_vol=4.0 / 3.0 * np.pi * float(g["bead_rad"]) ** 3,
        pref=g["pref"], intra=g["intra"], xpref=g["xpref"], pos=pos,
        fixed_density=fixed_density)


def oracle_ctls(g):
    from oracle.oracle import make_ctl
    out = []
    for k, row in enumerate(g["ctl0"]):
        amp_move, amp_bead, npc, simple, blo, bhi, mlo, mhi = row
        out.append(make_ctl(MOVE_NAMES[k], amp_move=amp_move, amp_bead=int(amp_bead),
                            num_per_cycle=int(npc), simple=bool(simple),
                            bead_bounds=(blo, bhi), move_bounds=(mlo, mhi)))
    return out
