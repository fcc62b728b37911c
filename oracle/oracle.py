"""ctypes wrapper around ``oracle/chromo_oracle.c``.

TEST INFRASTRUCTURE ONLY: the CPU checker for the GPU path.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module; the product package never does.

``build()`` compiles the C restatement twice with gcc (positions stored as
FP64 and as FP32).  ``OracleSystem`` owns numpy arrays for one polymer in one
field and runs ``mc_sim`` on them with caller-supplied random streams.
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
from scipy.special import comb

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "chromo_oracle.c"
MOVE_NAMES = ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]

_P = C.c_void_p
_I = C.c_int64
_D = C.c_double


class _System(C.Structure):
    _fields_ = [
        ("n_beads", _I), ("n_binders", _I),
        ("r", _P), ("t3", _P), ("t2", _P), ("states", _P), ("marks", _P),
        ("eps_bend", _P), ("gamma", _P), ("eps_par", _P), ("eps_perp", _P), ("eta", _P),
        ("bind_f", _P), ("mark_max", _I), ("site_max", _I), ("sites", _P), ("mu", _P),
        ("mu_adjust_factor", _D), ("max_binders", _I),
        ("field_kind", _I), ("confine_kind", _I), ("confine_length", _D),
        ("nx", _I), ("ny", _I), ("nz", _I),
        ("x_width", _D), ("y_width", _D), ("z_width", _D),
        ("access_vol", _P), ("vol_bin", _D), ("chi", _D), ("vf_limit", _D), ("bead_vol", _D),
        ("pref", _P), ("intra", _P), ("xpref", _P),
        ("fixed_density", _I), ("density", _P), ("density_fx", _P),
        ("density_trial", _P), ("dfx", _P), ("slot_of", _P), ("found", _P),
        ("n_found", _I), ("found_cap", _I), ("inds", _P), ("trial", _P),
        ("new_states", _P), ("picked", _P), ("fast_n", _I), ("eps_twist", _P), ("omega0", _P),
    ]


class Ctl(C.Structure):
    """Mirror of one MC move controller (MCAdapter + SimpleControl state)."""
    _fields_ = [
        ("move_kind", _I), ("ctrl_kind", _I), ("num_per_cycle", _I), ("move_on", _I),
        ("amp_move", _D), ("amp_bead", _I),
        ("bead_lo", _D), ("bead_hi", _D), ("move_lo", _D), ("move_hi", _D),
        ("acc_rate", _D), ("alpha", _D), ("num_attempt", _I), ("num_success", _I),
    ]


RECORD_DTYPE = np.dtype([
    ("kind", np.int32), ("n_inds", np.int32), ("ind0", np.int32), ("indf", np.int32),
    ("dE_poly", np.float64), ("dE_field", np.float64),
    ("accepted", np.int32), ("n_draws", np.int32),
])

_libs = {}


def build(force: bool = False) -> None:
    """Compile the oracle for FP64 and FP32 position storage (gcc, no FMA contraction)."""
    BUILD.mkdir(exist_ok=True)
    for tag, pos in (("f64", "double"), ("f32", "float")):
        so = BUILD / f"liboracle_{tag}.so"
        if so.exists() and not force and so.stat().st_mtime > SRC.stat().st_mtime:
            continue
        subprocess.check_call([
            "gcc", "-O2", "-shared", "-fPIC", "-ffp-contract=off", f"-DOR_POS={pos}",
            "-o", str(so), str(SRC), "-lm"])


def lib(tag: str):
    if tag not in _libs:
        build()
        L = C.CDLL(str(BUILD / f"liboracle_{tag}.so"))
        L.or_scratch_init.argtypes = [C.POINTER(_System)]
        L.or_scratch_init.restype = C.c_int
        L.or_scratch_free.argtypes = [C.POINTER(_System)]
        L.or_deposit_all.argtypes = [C.POINTER(_System)]
        for f in ("or_elastic_E", "or_binding_E", "or_field_E"):
            getattr(L, f).argtypes = [C.POINTER(_System)]
            getattr(L, f).restype = C.c_double
        L.or_mc_sim.argtypes = [C.POINTER(_System), C.POINTER(Ctl), _I, _I,
                                _P, _I, C.POINTER(_I), _P, _I, C.POINTER(_I), _P, _I]
        L.or_mc_sim.restype = _I
        L.or_mc_sim_philox.argtypes = [C.POINTER(_System), C.POINTER(Ctl), _I, _I, C.c_uint64, C.c_int32,
                                       C.POINTER(_I), _P, _I, C.POINTER(_I), _P, _I]
        L.or_mc_sim_philox.restype = _I
        L.or_kat_axis_rotation.argtypes = [_P, _P, C.c_double, _P]
        L.or_kat_philox.argtypes = [_P, _P, _P]
        L.or_steric_E.argtypes = [_P, _I, C.c_double, C.c_double]
        L.or_steric_E.restype = C.c_double
        L.or_steric_dE.argtypes = [_P, _P, _I, _I, _I, C.c_double, C.c_double]
        L.or_steric_dE.restype = C.c_double
        L.or_kat_transform.argtypes = [C.POINTER(_System), _I, _P, _P]
        assert L.or_sizeof_system() == C.sizeof(_System)
        assert L.or_sizeof_ctl() == C.sizeof(Ctl)
        assert L.or_sizeof_record() == RECORD_DTYPE.itemsize
        _libs[tag] = L
    return _libs[tag]


def binding_free_energy_table(sites, e_mod, e_nomod, mark_max):
    """-ln of the single-site binding partition function, per binder, mark count
    and bound count; the expression of ``chromo/polymers.pyx:1494-1517``."""
    nb = len(sites)
    site_max = int(max(sites)) if nb else 0
    f = np.zeros((nb, mark_max + 1, site_max + 1))
    for b in range(nb):
        Nn = sites[b]
        for Nm in range(mark_max + 1):
            for s in range(site_max + 1):
                i = np.arange(s + 1)
                with np.errstate(divide="ignore"):
                    f[b, Nm, s] = -np.log(np.sum(
                        comb(Nm, i) * comb(Nn - Nm, s - i)
                        * np.exp(-(i * e_mod[b] + (s - i) * e_nomod[b]))))
    return f


class OracleSystem:
    """One polymer in one field, laid out for the C oracle.

    pos: "f64" (positions stored as FP64) or "f32" (FP32 storage, as on GPU).
    fixed_density: 0 for the reference's FP64 density, 1 for int64 fixed point.
    fast_n: fast_field sub-bins per voxel and axis for the per-move density
    changes (0: exact weights).
    eps_twist, omega0: per-bond twist modulus and natural twist of an SSTWLC
    chain (None: SSWLC).
    """

    def __init__(self, *, r, t3, t2, states, marks, eps_bend, gamma, eps_par, eps_perp,
                 eta, sites, e_mod, e_nomod, mu, mu_adjust_factor=1.0, max_binders=-1,
                 field_kind=2, confine_kind=0, confine_length=0.0,
                 nxyz=(1, 1, 1), widths=(1.0, 1.0, 1.0), access_vol=None, chi=1.0,
                 vf_limit=0.5, bead_vol=4 / 3 * np.pi * 125, pref=(), intra=(), xpref=None,
                 pos="f64", fixed_density=0, fast_n=0, eps_twist=None, omega0=None):
        self.pos = pos
        fdt = np.float64 if pos == "f64" else np.float32
        # private copies: the oracle mutates its state in place
        self.r = np.array(r, dtype=fdt, order="C", copy=True)
        self.t3 = np.array(t3, dtype=fdt, order="C", copy=True)
        self.t2 = np.array(t2, dtype=fdt, order="C", copy=True)
        self.states = np.array(states, dtype=np.int64, order="C", copy=True)
        self.marks = np.array(marks, dtype=np.int64, order="C", copy=True)
        N, nb = self.states.shape
        self.params = [np.ascontiguousarray(x, dtype=np.float64)
                       for x in (eps_bend, gamma, eps_par, eps_perp, eta)]
        self.sites = np.ascontiguousarray(sites, dtype=np.int64)
        self.mu = np.ascontiguousarray(mu, dtype=np.float64)
        mark_max = int(max(int(self.marks.max()) if self.marks.size else 0,
                           int(self.sites.max()) if nb else 0))
        self.bind_f = np.ascontiguousarray(
            binding_free_energy_table(list(self.sites), list(e_mod), list(e_nomod), mark_max))
        self.pref = np.ascontiguousarray(pref if len(pref) else np.zeros(nb), dtype=np.float64)
        self.intra = np.ascontiguousarray(intra if len(intra) else np.zeros(nb), dtype=np.float64)
        self.xpref = np.ascontiguousarray(
            np.zeros((nb, nb)) if xpref is None else xpref, dtype=np.float64)
        nx, ny, nz = (int(v) for v in nxyz)
        G = nx * ny * nz
        self.access_vol = None if access_vol is None else np.ascontiguousarray(access_vol, dtype=np.float64)
        self.density = np.zeros((G, nb + 1))
        self.density_fx = np.zeros((G, nb + 1), dtype=np.int64)
        s = _System()
        s.n_beads, s.n_binders = N, nb
        s.r, s.t3, s.t2 = self.r.ctypes.data, self.t3.ctypes.data, self.t2.ctypes.data
        s.states, s.marks = self.states.ctypes.data, self.marks.ctypes.data
        (s.eps_bend, s.gamma, s.eps_par, s.eps_perp, s.eta) = [p.ctypes.data for p in self.params]
        s.bind_f = self.bind_f.ctypes.data
        s.mark_max, s.site_max = mark_max, self.bind_f.shape[2] - 1
        s.sites, s.mu = self.sites.ctypes.data, self.mu.ctypes.data
        s.mu_adjust_factor, s.max_binders = mu_adjust_factor, max_binders
        s.field_kind, s.confine_kind, s.confine_length = field_kind, confine_kind, confine_length
        s.nx, s.ny, s.nz = nx, ny, nz
        s.x_width, s.y_width, s.z_width = widths
        s.access_vol = None if self.access_vol is None else self.access_vol.ctypes.data
        s.vol_bin = widths[0] * widths[1] * widths[2] / G
        s.chi, s.vf_limit, s.bead_vol = chi, vf_limit, bead_vol
        s.pref, s.intra, s.xpref = self.pref.ctypes.data, self.intra.ctypes.data, self.xpref.ctypes.data
        s.fixed_density = fixed_density
        s.fast_n = int(fast_n) + int(fast_n) % 2
        self.twist = None
        if eps_twist is not None:  # SSTWLC: twist modulus and natural twist per bond
            self.twist = [np.ascontiguousarray(eps_twist, dtype=np.float64),
                          np.ascontiguousarray(omega0, dtype=np.float64)]
            s.eps_twist, s.omega0 = self.twist[0].ctypes.data, self.twist[1].ctypes.data
        s.density, s.density_fx = self.density.ctypes.data, self.density_fx.ctypes.data
        self._s = s
        self._L = lib(pos)
        rc = self._L.or_scratch_init(C.byref(s))
        if rc != 0:
            raise RuntimeError(f"oracle scratch init failed ({rc})")
        self.draw_pos = 0
        self.bstate_pos = 0

    def __del__(self):
        try:
            self._L.or_scratch_free(C.byref(self._s))
        except Exception:
            pass

    @property
    def mu_adjust_factor(self):
        return self._s.mu_adjust_factor

    @mu_adjust_factor.setter
    def mu_adjust_factor(self, v):
        self._s.mu_adjust_factor = v

    def deposit_all(self):
        self._L.or_deposit_all(C.byref(self._s))

    def energies(self):
        """(elastic, binding free energy, dE-consistent field energy)."""
        s = C.byref(self._s)
        return (self._L.or_elastic_E(s), self._L.or_binding_E(s), self._L.or_field_E(s))

    def transform(self, i, M):
        """Bead i moved by the 3 x 4 matrix M (transform_r_t3_t2): (r', t3', t2')."""
        M = np.ascontiguousarray(M, dtype=np.float64).reshape(12)
        out = np.zeros(9)
        self._L.or_kat_transform(C.byref(self._s), int(i), M.ctypes.data, out.ctypes.data)
        return out[:3], out[3:6], out[6:]

    def mc_sim(self, ctls, n_steps, draws, bstates, max_records=None):
        """Run ``mc_sim`` (chromo/mc/mc_sim.pyx:26-103); returns the per-move records."""
        arr = (Ctl * len(ctls))(*ctls)
        internal = draws is None
        draws = np.zeros(1, np.uint32) if internal else np.ascontiguousarray(draws, dtype=np.uint32)
        bstates = np.zeros(1, np.int64) if internal else np.ascontiguousarray(bstates, dtype=np.int64)
        if max_records is None:
            max_records = n_steps * sum(int(c.num_per_cycle) for c in ctls if c.move_on)
        recs = np.zeros(max_records, dtype=RECORD_DTYPE)
        dp, bp = _I(self.draw_pos), _I(self.bstate_pos)
        n = self._L.or_mc_sim(C.byref(self._s), arr, len(ctls), n_steps,
                              None if internal else draws.ctypes.data, len(draws), C.byref(dp),
                              None if internal else bstates.ctypes.data, len(bstates), C.byref(bp),
                              recs.ctypes.data if max_records else None, max_records)
        self.draw_pos, self.bstate_pos = dp.value, bp.value
        for i, c in enumerate(ctls):
            C.memmove(C.byref(c), C.byref(arr[i]), C.sizeof(Ctl))
        if n == -3:  # window larger than the chain: ValueError in the reference
            raise ValueError("bead selection window larger than the polymer "
                             "(chromo/util/bead_selection.pyx:86-89)")
        if n < 0:
            raise RuntimeError(f"oracle mc_sim error {n}")
        return recs[:n]


def _mc_sim_philox(self, ctls, n_steps, seed, rep, move_pos=0, follow=None, max_records=None):
    """``mc_sim`` driven by the GPU production kernel's random numbers: replica
    ``rep`` of a run seeded with ``seed``, from move counter ``move_pos``.
    ``follow`` (the GPU's ``accepted`` per attempted move) settles decisions in
    the tie band |dE + ln u| <= 1e-5 max(1, |dE|).  Returns (records, move
    counter after the run, tie-band decisions taken from ``follow``)."""
    arr = (Ctl * len(ctls))(*ctls)
    if max_records is None:
        max_records = n_steps * sum(int(c.num_per_cycle) for c in ctls if c.move_on)
    recs = np.zeros(max_records, dtype=RECORD_DTYPE)
    fol = None if follow is None else np.ascontiguousarray(follow, dtype=np.int8)
    mp, ties = _I(int(move_pos)), _I(0)
    n = self._L.or_mc_sim_philox(C.byref(self._s), arr, len(ctls), int(n_steps), int(seed) & (2**64 - 1),
                                 int(rep), C.byref(mp), None if fol is None else fol.ctypes.data,
                                 0 if fol is None else len(fol), C.byref(ties),
                                 recs.ctypes.data if max_records else None, max_records)
    for i, c in enumerate(ctls):
        C.memmove(C.byref(c), C.byref(arr[i]), C.sizeof(Ctl))
    if n == -3:
        raise ValueError("bead selection window larger than the polymer "
                         "(chromo/util/bead_selection.pyx:86-89)")
    if n < 0:
        raise RuntimeError(f"oracle mc_sim error {n}")
    return recs[:n], mp.value, ties.value


OracleSystem.mc_sim_philox = _mc_sim_philox


def make_ctl(move_name, *, amp_move, amp_bead, num_per_cycle=1, simple=True,
             bead_bounds=(0, 0), move_bounds=(0.0, 0.0), move_on=1, moves_in_average=20.0):
    c = Ctl()
    c.move_kind = MOVE_NAMES.index(move_name)
    c.ctrl_kind = 1 if simple else 0
    c.num_per_cycle = num_per_cycle
    c.move_on = move_on
    c.amp_move, c.amp_bead = amp_move, amp_bead
    c.bead_lo, c.bead_hi = bead_bounds
    c.move_lo, c.move_hi = move_bounds
    c.acc_rate, c.alpha = 0.0, 2 / (moves_in_average + 1)
    return c


def philox4x32_10(ctr, key, tag="f64"):
    """One Philox4x32-10 block from the oracle (the generator of its Philox
    mode), as four 32-bit words."""
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib(tag).or_kat_philox(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return [int(x) for x in out]


def axis_rotation(axis, point, angle, tag="f64"):
    """The 3 x 4 rotation matrix [R | T] about `axis` through `point`
    (arbitrary_axis_rotation, chromo/util/linalg.pyx:62-143), from the oracle."""
    a = np.ascontiguousarray(axis, dtype=np.float64)
    p = np.ascontiguousarray(point, dtype=np.float64)
    out = np.zeros(12)
    lib(tag).or_kat_axis_rotation(a.ctypes.data, p.ctypes.data, float(angle), out.ctypes.data)
    return out.reshape(3, 4)


def steric_energy(r, excluded_distance, V0=1.0):
    """Clash energy of every bead pair (eval_E_steric_clashes,
    chromo/polymers.pyx:2900-2920), from the oracle."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    return lib("f64").or_steric_E(r.ctypes.data, len(r), float(excluded_distance), float(V0))


def steric_delta(r, r_trial_segment, ind0, indf, excluded_distance, V0=1.0):
    """Clash-energy change of moving beads [ind0, indf) to ``r_trial_segment``
    (get_delta_distances + eval_delta_steric_clashes, :2827-2898)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    t = np.ascontiguousarray(r_trial_segment, dtype=np.float64)
    return lib("f64").or_steric_dE(r.ctypes.data, t.ctypes.data, len(r), int(ind0), int(indf),
                                   float(excluded_distance), float(V0))
