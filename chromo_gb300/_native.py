"""ctypes binding of the C ABI in include/chromo_gb300.h.

The library is loaded from ``chromo_gb300/_lib/libchromo_gb300.so`` (built
in place by ``chromo_gb300.build``).  There is no fallback: if the library or
a GPU is missing, every call raises.
"""
import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libchromo_gb300.so"
MAX_BINDERS = 3
MAX_MARK = 3
MOVE_NAMES = ["crank_shaft", "end_pivot", "slide", "tangent_rotation", "change_binding_state"]

STATUS = {0: "ok", -1: "argument", -2: "cuda", -3: "window", -4: "stream", -5: "nonfinite",
          -6: "spin", -7: "nomem", -8: "drift"}


class CgError(RuntimeError):
    """Error returned by the native library (a cg_status code and message)."""

    def __init__(self, code, msg):
        super().__init__(f"{msg} (cg_status {code}: {STATUS.get(code, '?')})")
        self.code = code


class CgWindowError(CgError, ValueError):
    """Bead selection window larger than the polymer (ValueError in the reference)."""


class MoveCtl(C.Structure):
    _fields_ = [
        ("move_kind", C.c_int64), ("ctrl_kind", C.c_int64), ("num_per_cycle", C.c_int64),
        ("move_on", C.c_int64), ("amp_move", C.c_double), ("amp_bead", C.c_int64),
        ("bead_lo", C.c_double), ("bead_hi", C.c_double), ("move_lo", C.c_double),
        ("move_hi", C.c_double), ("acc_rate", C.c_double), ("alpha", C.c_double),
        ("num_attempt", C.c_int64), ("num_success", C.c_int64),
    ]


RECORD_DTYPE = np.dtype([
    ("kind", np.int32), ("n_inds", np.int32), ("ind0", np.int32), ("indf", np.int32),
    ("dE_poly", np.float64), ("dE_field", np.float64),
    ("accepted", np.int32), ("n_draws", np.int32),
])


class FieldParams(C.Structure):
    _fields_ = [
        ("field_kind", C.c_int32), ("confine_kind", C.c_int32), ("confine_length", C.c_double),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("n_binders", C.c_int32),
        ("x_width", C.c_double), ("y_width", C.c_double), ("z_width", C.c_double),
        ("chi", C.c_double), ("vf_limit", C.c_double), ("bead_vol", C.c_double),
        ("pref", C.c_double * MAX_BINDERS), ("intra", C.c_double * MAX_BINDERS),
        ("xpref", C.c_double * (MAX_BINDERS * MAX_BINDERS)),
        ("fast_field", C.c_int32), ("n_points", C.c_int32),
    ]


class BindingParams(C.Structure):
    _fields_ = [
        ("n_binders", C.c_int32), ("max_binders", C.c_int32),
        ("sites", C.c_int32 * MAX_BINDERS), ("pad", C.c_int32),
        ("mu", C.c_double * MAX_BINDERS), ("mu_adjust_factor", C.c_double),
        ("bind_f", C.c_double * (MAX_BINDERS * (MAX_MARK + 1) * (MAX_MARK + 1))),
    ]


class Config(C.Structure):
    _fields_ = [
        ("n_replicas", C.c_int32), ("pos_fp64", C.c_int32), ("n_binders", C.c_int32),
        ("warps_per_block", C.c_int32), ("n_beads", C.POINTER(C.c_int64)),
        ("grid_dims", C.POINTER(C.c_int32)), ("max_segment", C.c_int64),
        ("max_tangent", C.c_int64), ("nonuniform_access", C.c_int32), ("lanes_per_move", C.c_int32),
    ]


_lib = None
EXPORTS = [
    "cg_create", "cg_destroy", "cg_last_error", "cg_set_chain", "cg_get_chain", "cg_set_field",
    "cg_set_binding", "cg_set_controllers", "cg_get_controllers", "cg_deposit", "cg_get_density",
    "cg_run", "cg_sync", "cg_run_audit", "cg_energy", "cg_reset_running_energy", "cg_get_tally",
    "cg_reset_tally", "cg_exchange", "cg_get_chi", "cg_run_batched", "cg_get_launch_info", "cg_get_transfer_mode",
    "cg_field_energy_static", "cg_energies", "cg_set_chains", "cg_get_chains", "cg_gradient",
    "cg_sample_terms", "cg_get_samples", "cg_get_launch_shape", "cg_mc_warps_per_sm",
    "cg_set_mu_ladder", "cg_get_mu", "cg_get_swap_counts", "cg_run_logged", "cg_set_round_timing",
    "cg_get_round_times", "cg_set_drift_guard", "cg_get_drift", "cg_set_chains_device",
    "cg_deposit_async", "cg_energies_device", "cg_gradient_device", "cg_state_bytes", "cg_save_state",
    "cg_load_state", "cg_set_twist", "cg_steric_energy", "cg_steric_delta",
]
N_TERMS = 14


def lib_path() -> Path:
    return _LIB_PATH


def lib():
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"native library {_LIB_PATH} is missing: run "
                               "`python -m chromo_gb300.build` (needs nvcc)")
        L = C.CDLL(str(_LIB_PATH))
        P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        sig = {
            "cg_create": ([C.POINTER(Config), C.POINTER(P)], C.c_int),
            "cg_destroy": ([P], None),
            "cg_last_error": ([], C.c_char_p),
            "cg_set_chain": ([P, I32, P, P, P, P, P, P], C.c_int),
            "cg_get_chain": ([P, I32, P, P, P, P], C.c_int),
            "cg_set_field": ([P, I32, C.POINTER(FieldParams), P], C.c_int),
            "cg_set_binding": ([P, I32, C.POINTER(BindingParams)], C.c_int),
            "cg_set_controllers": ([P, I32, C.POINTER(MoveCtl), I32], C.c_int),
            "cg_get_controllers": ([P, I32, C.POINTER(MoveCtl), I32], C.c_int),
            "cg_deposit": ([P, I32], C.c_int),
            "cg_get_density": ([P, I32, P], C.c_int),
            "cg_run": ([P, I64, C.c_uint64, P], C.c_int),
            "cg_sync": ([P, P], C.c_int),
            "cg_run_audit": ([P, I32, I64, P, I64, P, I64, P, I64, P, P, P], C.c_int),
            "cg_run_logged": ([P, I64, C.c_uint64, P, I64, P], C.c_int),
            "cg_set_round_timing": ([P, I32], C.c_int),
            "cg_get_round_times": ([P, P, I32, P], C.c_int),
            "cg_set_drift_guard": ([P, I32, D, D], C.c_int),
            "cg_set_chains_device": ([P, P, P, P], C.c_int),
            "cg_deposit_async": ([P, P], C.c_int),
            "cg_energies_device": ([P, P, P], C.c_int),
            "cg_gradient_device": ([P, P, P, P], C.c_int),
            "cg_state_bytes": ([P], C.c_int64),
            "cg_save_state": ([P, P, I64], C.c_int),
            "cg_load_state": ([P, P, I64], C.c_int),
            "cg_set_twist": ([P, I32, P, P], C.c_int),
            "cg_steric_energy": ([P, I32, D, D, P], C.c_int),
            "cg_steric_delta": ([P, I32, I64, I64, P, D, D, P], C.c_int),
            "cg_get_drift": ([P, P, P], C.c_int),
            "cg_energy": ([P, I32, P], C.c_int),
            "cg_reset_running_energy": ([P], C.c_int),
            "cg_get_tally": ([P, I32, P], C.c_int),
            "cg_reset_tally": ([P], C.c_int),
            "cg_exchange": ([P, I32, I64, C.c_uint64, P], C.c_int),
            "cg_get_chi": ([P, P], C.c_int),
            "cg_run_batched": ([P, I64, I64, I32, C.c_uint64, P], C.c_int),
            "cg_get_launch_info": ([P, P, P, P], C.c_int),
            "cg_get_transfer_mode": ([P, P], C.c_int),
            "cg_get_launch_shape": ([P, P, P, P, P], C.c_int),
            "cg_mc_warps_per_sm": ([I32, I32], C.c_int),
            "cg_set_mu_ladder": ([P, I32, I32], C.c_int),
            "cg_get_mu": ([P, I32, P], C.c_int),
            "cg_get_swap_counts": ([P, P, P, P, P], C.c_int),
            "cg_field_energy_static": ([C.POINTER(FieldParams), I64, P, P, P, P, P], C.c_int),
            "cg_energies": ([P, P, P], C.c_int),
            "cg_set_chains": ([P, P, P, P, P], C.c_int),
            "cg_get_chains": ([P, P, P, P, P], C.c_int),
            "cg_gradient": ([P, P, P], C.c_int),
            "cg_sample_terms": ([P, P], C.c_int),
            "cg_get_samples": ([P, P, I32], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def mc_warps_per_sm(pos_fp64: bool, lanes_per_move: int) -> int:
    """Warps of the MC kernel that fit one SM's register file (needs a GPU)."""
    n = lib().cg_mc_warps_per_sm(int(bool(pos_fp64)), int(lanes_per_move))
    if n < 0:
        raise ValueError(f"no MC kernel for lanes_per_move={lanes_per_move} (pos_fp64={pos_fp64})")
    return n


def check(rc):
    if rc != 0:
        msg = lib().cg_last_error().decode()
        if rc == -3:
            raise CgWindowError(rc, msg)
        raise CgError(rc, msg)


def _ptr(a):
    return None if a is None else a.ctypes.data


class Sim:
    """Owner of one cg_sim handle (R replicas resident on the GPU)."""

    def __init__(self, n_beads, grid_dims, n_binders, *, pos_fp64=False, max_segment=152,
                 max_tangent=1, warps_per_block=0, nonuniform_access=False, lanes_per_move=0):
        L = lib()
        self.n_beads = np.ascontiguousarray(n_beads, dtype=np.int64)
        self.grid_dims = np.ascontiguousarray(grid_dims, dtype=np.int32).reshape(-1, 3)
        self.R = len(self.n_beads)
        self.nb = int(n_binders)
        self.pos_fp64 = bool(pos_fp64)
        cfg = Config()
        cfg.n_replicas = self.R
        cfg.pos_fp64 = int(self.pos_fp64)
        cfg.n_binders = self.nb
        cfg.warps_per_block = warps_per_block
        self._nb_buf = self.n_beads
        self._gd_buf = np.ascontiguousarray(self.grid_dims.reshape(-1))
        cfg.n_beads = self._nb_buf.ctypes.data_as(C.POINTER(C.c_int64))
        cfg.grid_dims = self._gd_buf.ctypes.data_as(C.POINTER(C.c_int32))
        cfg.max_segment = int(max_segment)
        cfg.max_tangent = int(max_tangent)
        cfg.nonuniform_access = int(bool(nonuniform_access))
        cfg.lanes_per_move = int(lanes_per_move)
        h = C.c_void_p()
        check(L.cg_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.n_ctl = 5

    def close(self):
        if getattr(self, "h", None):
            lib().cg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_chain(self, rep, r=None, t3=None, t2=None, states=None, marks=None, bonds=None):
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        i64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.int64)
        arrs = [f64(r), f64(t3), f64(t2), i64(states), i64(marks), f64(bonds)]
        check(lib().cg_set_chain(self.h, rep, *[_ptr(a) for a in arrs]))

    def get_chain(self, rep):
        n = int(self.n_beads[rep])
        r, t3, t2 = (np.empty((n, 3)) for _ in range(3))
        st = np.empty((n, self.nb), dtype=np.int64)
        check(lib().cg_get_chain(self.h, rep, _ptr(r), _ptr(t3), _ptr(t2), _ptr(st)))
        return r, t3, t2, st

    def set_chains(self, chains):
        """Upload every replica's chain at once: ``chains[rep]`` is a mapping with
        any of ``r``, ``t3``, ``t2``, ``states`` (missing keys are skipped)."""
        keep = []

        def table(key, dtype, width):
            ptrs = (C.c_void_p * self.R)()
            given = False
            for rep, c in enumerate(chains):
                a = c.get(key)
                if a is None:
                    continue
                a = np.ascontiguousarray(a, dtype=dtype)
                if a.size != int(self.n_beads[rep]) * width:
                    raise ValueError(f"{key} of replica {rep} has the wrong size")
                keep.append(a)
                ptrs[rep] = a.ctypes.data
                given = True
            return ptrs if given else None

        if len(chains) != self.R:
            raise ValueError("one entry per replica")
        check(lib().cg_set_chains(self.h, table("r", np.float64, 3), table("t3", np.float64, 3),
                                  table("t2", np.float64, 3), table("states", np.int64, self.nb)))

    def get_chains(self, out=None):
        """Every replica's (r, t3, t2, states) in one call; ``out`` (the list a
        previous call returned) is filled in place instead of new arrays."""
        if out is None:
            out = [(np.empty((int(n), 3)), np.empty((int(n), 3)), np.empty((int(n), 3)),
                    np.empty((int(n), self.nb), dtype=np.int64)) for n in self.n_beads]
        elif len(out) != self.R or any(
                o[0].shape != (int(n), 3) or o[3].shape != (int(n), self.nb) or o[3].dtype != np.int64
                or not all(a.flags.c_contiguous for a in o) for o, n in zip(out, self.n_beads)):
            raise ValueError("out must be a list of (r, t3, t2, states) arrays as get_chains returns")
        tabs = []
        for k in range(4):
            t = (C.c_void_p * self.R)()
            for rep in range(self.R):
                t[rep] = out[rep][k].ctypes.data
            tabs.append(t)
        check(lib().cg_get_chains(self.h, *tabs))
        return out

    def steric_energy(self, rep, excluded_distance, V0=1.0):
        """Clash energy of replica ``rep``'s resident chain (cg_steric_energy)."""
        out = C.c_double()
        check(lib().cg_steric_energy(self.h, rep, float(excluded_distance), float(V0), C.byref(out)))
        return out.value

    def steric_delta(self, rep, ind0, indf, r_trial, excluded_distance, V0=1.0):
        """Clash-energy change of moving beads [ind0, indf) to ``r_trial``."""
        t = np.ascontiguousarray(r_trial, dtype=np.float64).reshape(-1, 3)
        out = C.c_double()
        check(lib().cg_steric_delta(self.h, rep, int(ind0), int(indf), _ptr(t), float(excluded_distance),
                                    float(V0), C.byref(out)))
        return out.value

    def set_twist(self, rep, eps_twist, omega0):
        """SSTWLC twist of replica ``rep`` (per-bond modulus and natural twist;
        None turns it off)."""
        if eps_twist is None:
            check(lib().cg_set_twist(self.h, rep, None, None))
            return
        e = np.ascontiguousarray(eps_twist, dtype=np.float64)
        w = np.ascontiguousarray(omega0, dtype=np.float64)
        if e.size != int(self.n_beads[rep]) - 1 or w.size != e.size:
            raise ValueError("one twist modulus and natural twist per bond")
        check(lib().cg_set_twist(self.h, rep, _ptr(e), _ptr(w)))

    def set_field(self, rep, fp: FieldParams, access_vol=None):
        av = None if access_vol is None else np.ascontiguousarray(access_vol, dtype=np.float64)
        check(lib().cg_set_field(self.h, rep, C.byref(fp), _ptr(av)))

    def set_binding(self, rep, bp: BindingParams):
        check(lib().cg_set_binding(self.h, rep, C.byref(bp)))

    def set_controllers(self, rep, ctls):
        arr = (MoveCtl * len(ctls))(*ctls)
        check(lib().cg_set_controllers(self.h, rep, arr, len(ctls)))
        self.n_ctl = len(ctls)

    def get_controllers(self, rep, n=None):
        n = n or self.n_ctl
        arr = (MoveCtl * n)()
        check(lib().cg_get_controllers(self.h, rep, arr, n))
        return list(arr)

    def deposit(self, rep=-1):
        check(lib().cg_deposit(self.h, rep))

    def density(self, rep):
        G = int(np.prod(self.grid_dims[rep]))
        g = np.empty((G, self.nb + 1), dtype=np.int64)
        check(lib().cg_get_density(self.h, rep, _ptr(g)))
        return g

    def run(self, n_steps, seed, stream=None):
        check(lib().cg_run(self.h, int(n_steps), int(seed) & (2**64 - 1), stream))

    def sync(self, stream=None):
        check(lib().cg_sync(self.h, stream))

    def run_audit(self, rep, n_steps, draws, bstates, max_records=None):
        draws = np.ascontiguousarray(draws, dtype=np.uint32)
        bstates = np.ascontiguousarray(bstates, dtype=np.int8)
        if max_records is None:
            max_records = n_steps * 200
        recs = np.zeros(max_records, dtype=RECORD_DTYPE)
        nrec, du, bu = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().cg_run_audit(self.h, rep, int(n_steps), _ptr(draws), len(draws), _ptr(bstates),
                                 len(bstates), _ptr(recs), max_records, C.byref(nrec), C.byref(du),
                                 C.byref(bu)))
        return recs[:min(nrec.value, max_records)], du.value, bu.value

    def run_logged(self, n_steps, seed, max_records):
        """``run`` with the production kernel's per-move log: a list with one
        record array per replica (its attempted moves in order, at most
        ``max_records``)."""
        recs = np.zeros((self.R, int(max_records)), dtype=RECORD_DTYPE)
        n = np.zeros(self.R, dtype=np.int64)
        check(lib().cg_run_logged(self.h, int(n_steps), int(seed) & (2**64 - 1), _ptr(recs),
                                  int(max_records), _ptr(n)))
        return [recs[r, :min(int(n[r]), int(max_records))] for r in range(self.R)]

    def energy(self, rep):
        out = np.zeros(4)
        check(lib().cg_energy(self.h, rep, _ptr(out)))
        return out

    def energies(self, stream=None):
        """[R, 5]: elastic, binding, field, running sum of accepted dE, chi-free S."""
        out = np.zeros((self.R, 5))
        check(lib().cg_energies(self.h, _ptr(out), stream))
        return out

    def gradient(self, positions=True, terms=True):
        """(dE/dr [total_beads, 3] FP32 or None, terms [R, 14] or None)."""
        g = np.empty((int(self.n_beads.sum()), 3), dtype=np.float32) if positions else None
        t = np.empty((self.R, N_TERMS)) if terms else None
        check(lib().cg_gradient(self.h, _ptr(g), _ptr(t)))
        return g, t

    def sample_terms(self, stream=None):
        check(lib().cg_sample_terms(self.h, stream))

    def samples(self, reset=False):
        """(sum T [R, 14], sum T T^T [R, 14, 14], count [R])."""
        k = N_TERMS
        out = np.empty((self.R, k + k * k + 1))
        check(lib().cg_get_samples(self.h, _ptr(out), int(bool(reset))))
        return out[:, :k], out[:, k:k + k * k].reshape(self.R, k, k), out[:, -1]

    def reset_running_energy(self):
        check(lib().cg_reset_running_energy(self.h))

    def tally(self, rep):
        out = np.zeros(30, dtype=np.uint64)
        check(lib().cg_get_tally(self.h, rep, _ptr(out)))
        return out.reshape(5, 6)

    def reset_tally(self):
        check(lib().cg_reset_tally(self.h))

    def exchange(self, n_rungs, round_, seed, stream=None):
        check(lib().cg_exchange(self.h, n_rungs, round_, seed, stream))

    def chi(self):
        out = np.zeros(self.R)
        check(lib().cg_get_chi(self.h, _ptr(out)))
        return out

    def set_mu_ladder(self, mu_rungs, binder=0):
        """Exchange mu of ``binder`` between neighbouring mu rungs (0: off)."""
        check(lib().cg_set_mu_ladder(self.h, int(mu_rungs), int(binder)))

    def mu(self, binder=0):
        out = np.zeros(self.R)
        check(lib().cg_get_mu(self.h, int(binder), _ptr(out)))
        return out

    def swap_counts(self):
        """Accepted / attempted chi and mu swaps per lower slot of each pair."""
        arrs = [np.zeros(self.R, dtype=np.uint64) for _ in range(4)]
        check(lib().cg_get_swap_counts(self.h, *[_ptr(a) for a in arrs]))
        return dict(zip(("chi_swaps", "chi_attempts", "mu_swaps", "mu_attempts"), arrs))

    def run_batched(self, n_rounds, n_steps, n_rungs, seed, stream=None):
        check(lib().cg_run_batched(self.h, int(n_rounds), int(n_steps), int(n_rungs),
                                   int(seed) & (2**64 - 1), stream))

    def save_state(self) -> np.ndarray:
        """The whole resident state as a byte image (cg_save_state)."""
        n = lib().cg_state_bytes(self.h)
        if n < 0:
            check(int(n))
        buf = np.empty(int(n), dtype=np.uint8)
        check(lib().cg_save_state(self.h, _ptr(buf), int(n)))
        return buf

    def load_state(self, image: np.ndarray):
        """Restore an image from ``save_state`` of a sim with the same layout."""
        image = np.ascontiguousarray(image, dtype=np.uint8)
        check(lib().cg_load_state(self.h, _ptr(image), int(image.size)))

    def set_drift_guard(self, every_rounds, tol_abs=0.0, tol_rel=0.0):
        """Check every ``every_rounds``-th ``run_batched`` round's recomputed
        FP64 energies against the running sums on the device (0: off)."""
        check(lib().cg_set_drift_guard(self.h, int(every_rounds), float(tol_abs), float(tol_rel)))

    def drift(self):
        """(drift at each replica's last check [R], checks made)."""
        out = np.zeros(self.R)
        n = C.c_int64()
        check(lib().cg_get_drift(self.h, _ptr(out), C.byref(n)))
        return out, n.value

    def set_round_timing(self, capacity):
        """Time the MC kernel of every ``run_batched`` round on the device
        (CUDA events inside the graph), keeping the last ``capacity``."""
        check(lib().cg_set_round_timing(self.h, int(capacity)))

    def round_times(self, max_rounds=1 << 16):
        """MC-kernel milliseconds of the last timed rounds, oldest first."""
        out = np.zeros(int(max_rounds), dtype=np.float32)
        n = C.c_int32()
        check(lib().cg_get_round_times(self.h, _ptr(out), int(max_rounds), C.byref(n)))
        return out[:n.value].astype(np.float64)

    def launch_shape(self):
        """(warps per replica, lanes per move, moves in flight, shared voxel-table slots)."""
        w, g, f, hs = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().cg_get_launch_shape(self.h, C.byref(w), C.byref(g), C.byref(f), C.byref(hs)))
        return w.value, g.value, f.value, hs.value

    def direct_transfers(self) -> bool:
        """Whether set_chains / get_chains read and write the host arrays from
        the GPU (pageable host memory addressable over NVLink-C2C)."""
        d = C.c_int32()
        check(lib().cg_get_transfer_mode(self.h, C.byref(d)))
        return bool(d.value)

    def launch_info(self):
        w, hs, k = C.c_int32(), C.c_int32(), C.c_int64()
        check(lib().cg_get_launch_info(self.h, C.byref(w), C.byref(hs), C.byref(k)))
        return w.value, hs.value, k.value
