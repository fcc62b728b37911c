"""Polymers: the SSWLC chain and its chromatin specialisation (chromo/polymers.pyx).

Constructors, attribute names and array shapes follow the reference
(``PolymerBase`` :65-300, ``SSWLC`` :911-1010, ``Chromatin`` :1821-1887).
Positions ``r``, tangents ``t3``/``t2`` (N x 3, FP64 on the host), binding
``states`` and ``chemical_mods`` (N x n_binders, int) are plain numpy arrays
that ``mc.mc_sim`` uploads to the GPU and refreshes after the run.  The SSWLC
elastic parameters are interpolated from the dssWLC table exactly as in
``SSWLC._find_parameters`` (:1545-1601).

Differences from the reference, by design:

* the trial arrays (``r_trial`` ...) exist for compatibility but are not
  used: proposals live in GPU registers and shared memory;
* ``compute_dE`` is not a Python method here: per-move energies are computed
  inside the GPU kernel (``mc.mc_sim``), and ``compute_E`` runs on the GPU.
"""
from typing import Callable

import numpy as np

from . import binders as _binders
from .energetics import dss_parameters

_empty_2d = np.empty((0, 0))
_mty_2d_int = np.empty((0, 0), dtype=int)
_empty_1d = np.empty((0,))
_empty_1d_str = np.empty((0,), dtype=str)


class TransformedObject:
    """Holder of a 4x4 homogeneous transformation (chromo/polymers.pyx:43-62)."""

    def __init__(self):
        self.transformation_mat = np.identity(4, dtype=np.double)


class GhostBead:
    """A bead whose binders are the named module-level binder objects
    (chromo/beads.py:19-75,97-160)."""

    def __init__(self, id_, r, *, t3=None, t2=None, states=None, binder_names=None, rad=5, **kw):
        self.id = id_
        self.r, self.t3, self.t2, self.states = r, t3, t2, states
        self.binder_names = binder_names
        self.binders = None if binder_names is None else [
            _binders.get_by_name(str(n)) for n in binder_names]
        self.rad = rad
        self.vol = (4 / 3) * np.pi * rad ** 3


class Nucleosome(GhostBead):
    """Chromatin bead with a spherical excluded volume (chromo/beads.py:359-415)."""


class PolymerBase(TransformedObject):
    """State of one polymer (chromo/polymers.pyx:65-300)."""

    def __init__(self, name, r=_empty_2d, *, log_path="", t3=_empty_2d, t2=_empty_2d,
                 bead_length=_empty_1d, lp=0, states=_mty_2d_int, binder_names=_empty_1d,
                 chemical_mods=_mty_2d_int, chemical_mod_names=_empty_1d_str, max_binders=-1):
        super().__init__()
        self.name = name
        self.r = np.ascontiguousarray(r, dtype=np.float64)
        self.t3 = np.ascontiguousarray(t3, dtype=np.float64)
        self.t2 = np.ascontiguousarray(t2, dtype=np.float64)
        self.bead_length = np.atleast_1d(np.asarray(bead_length, dtype=np.float64))
        self.states = np.ascontiguousarray(states, dtype=np.int64)
        self.max_binders = int(max_binders)
        self.binder_names = np.asarray(binder_names)
        self.chemical_mods = np.ascontiguousarray(chemical_mods, dtype=np.int64)
        self.chemical_mod_names = np.asarray(chemical_mod_names)
        self.num_beads = self.r.shape[0]
        self._fill_missing_arguments()
        self.all_inds = np.arange(0, self.num_beads, 1)
        self.num_binders = self.states.shape[1]
        self.n_binders_p1 = self.num_binders + 1
        self.log_path = log_path
        self._check_binders()
        self.lp = lp
        self.mu_adjust_factor = 1.0
        self.last_amp_bead = 0
        self.last_amp_move = 0.0
        self.r_trial = self.r.copy()
        self.t3_trial = self.t3.copy()
        self.t2_trial = self.t2.copy()
        self.states_trial = self.states.copy()

    def _fill_missing_arguments(self):
        n = self.num_beads
        if np.size(self.t3) == 0:
            self.t3 = np.zeros((n, 3))
        if np.size(self.t2) == 0:
            self.t2 = np.zeros((n, 3))
        if np.size(self.states) == 0:
            self.states = np.zeros((n, 1), dtype=np.int64)
        if np.size(self.binder_names) == 0:
            self.binder_names = np.array(["null_reader"])
        if np.size(self.chemical_mods) == 0:
            self.chemical_mods = np.zeros((n, 1), dtype=np.int64)
        if np.size(self.chemical_mod_names) == 0:
            self.chemical_mod_names = np.array(["null_mod"])

    def _check_binders(self):
        # chromo/polymers.pyx:389-409
        if self.states.shape[1] != 0:
            if self.states.shape[1] != len(self.binder_names):
                raise ValueError("Each chemical state must be given a name.")
            if self.states.shape[0] != len(self.r):
                raise ValueError("Initial epigenetic state of wrong length.")

    def is_field_active(self):
        return 1

    def get_num_beads(self):
        return self.r.shape[0]

    def get_num_binders(self):
        return self.states.shape[1]

    def __str__(self):
        return f"Polymer<{self.name}, nbeads={self.num_beads}, nbinder={self.num_binders}>"

    # ---- snapshots in the reference's CSV format (chromo/polymers.pyx:575-758) ----
    def to_csv(self, path=None):
        """Write the snapshot CSV to ``path``; with ``path=None`` return its text."""
        from .util.poly_csv import to_csv_text
        text = to_csv_text(self)
        if path is None:
            return text
        with open(path, "w", newline="") as fh:
            fh.write(text)
        return None

    def to_file(self, path):
        """Synonym of ``to_csv``."""
        return self.to_csv(path)

    @classmethod
    def from_csv(cls, csv_file):
        return cls.from_file(csv_file)

    @classmethod
    def from_file(cls, path, name=None, **kwargs):
        """Construct the polymer stored by ``to_csv`` (a path or a text buffer);
        ``name`` defaults to the file's stem."""
        from .util.poly_csv import polymer_kwargs
        if name is None and isinstance(path, str):
            name = path.split("/")[-1].split(".")[0]
        kw = polymer_kwargs(path, name)
        kw.update(kwargs)
        return cls(**kw)


class SSWLC(PolymerBase):
    """Stretchable, shearable wormlike chain (chromo/polymers.pyx:911-1601)."""

    def __init__(self, name, r, *, bead_length, lp, bead_rad=5, t3=_empty_2d, t2=_empty_2d,
                 states=_mty_2d_int, binder_names=_empty_1d, chemical_mods=_mty_2d_int,
                 chemical_mod_names=_empty_1d, log_path="", max_binders=-1):
        r = np.ascontiguousarray(r, dtype=np.float64)
        bl = np.atleast_1d(np.asarray(bead_length, dtype=np.float64))
        if bl.size == 1 and r.shape[0] > 2:
            bl = np.full(r.shape[0] - 1, float(bl[0]))
        super().__init__(name, r, t3=t3, t2=t2, states=states, binder_names=binder_names,
                         bead_length=bl, lp=lp, log_path=log_path, chemical_mods=chemical_mods,
                         chemical_mod_names=chemical_mod_names, max_binders=max_binders)
        self.bead_rad = bead_rad
        self.construct_beads()
        self._find_parameters(self.bead_length)
        if self.lp == 0:
            raise ValueError("Specify the persistence length in the subclass of Polymer")

    def construct_beads(self):
        self.beads = {i: GhostBead(i, self.r[i], t3=self.t3[i], t2=self.t2[i],
                                   states=self.states[i], binder_names=self.binder_names,
                                   rad=self.bead_rad) for i in range(len(self.r))}

    def _find_parameters(self, bead_length):
        (self.delta, self.eps_bend, self.gamma, self.eps_par, self.eps_perp,
         self.eta) = dss_parameters(bead_length, self.lp)

    def bond_parameters(self):
        """(N-1) x 5 array: eps_bend, gamma, eps_par, eps_perp, eta per bond."""
        return np.ascontiguousarray(np.stack(
            [self.eps_bend, self.gamma, self.eps_par, self.eps_perp, self.eta], axis=1))

    def compute_E(self):
        """Elastic energy of the current configuration, on the GPU in FP64
        (SSWLC.compute_E, chromo/polymers.pyx:1348-1381)."""
        from .mc.mc_sim import _energies_of
        return _energies_of(self)[0]

    def __str__(self):
        return f"Polymer_Class<SSWLC>, {super().__str__()}"

    # ---- initial configurations (chromo/polymers.pyx:1603-1818) ----
    @classmethod
    def straight_line_in_x(cls, name: str, step_sizes: np.ndarray, **kwargs):
        csum = np.cumsum(step_sizes)
        n = len(step_sizes) + 1
        r = np.zeros((n, 3))
        r[1:, 0] = csum
        t3 = np.zeros((n, 3))
        t3[:, 0] = 1
        t2 = np.zeros((n, 3))
        t2[:, 1] = 1
        return cls(name, r, t3=t3, t2=t2, bead_length=step_sizes, **kwargs)

    @classmethod
    def gaussian_walk_polymer(cls, name: str, num_beads: int, step_lengths: np.ndarray, **kwargs):
        """Gaussian random walk drawn from numpy's global generator
        (chromo/util/poly_paths.py:269-295)."""
        r = gaussian_walk(num_beads - 1, np.asarray(step_lengths))
        t3, t2 = estimate_tangents_from_coordinates(r)
        return cls(name, r, t3=t3, t2=t2, bead_length=step_lengths, **kwargs)

    @classmethod
    def confined_gaussian_walk(cls, name: str, num_beads: int, step_lengths: np.ndarray,
                               confine_type: str, confine_length: float, **kwargs):
        step_lengths = np.ascontiguousarray(step_lengths)
        r = confined_gaussian_walk(num_beads, step_lengths, confine_type, confine_length)
        t3, t2 = estimate_tangents_from_coordinates(r)
        return cls(name, r, t3=t3, t2=t2, bead_length=step_lengths, **kwargs)


# natural twist of bare DNA per nm: 2 pi / 10.5 bp, 0.332 nm per bp
# (NATURAL_TWIST_BARE / LENGTH_BP, chromo/polymers.pyx:38-40)
NATURAL_TWIST_BARE = 2 * np.pi / 10.5
LENGTH_BP = 0.332


class SSTWLC(SSWLC):
    """Stretchable, shearable wormlike chain with twist (chromo/polymers.pyx:1889-2320).

    ``lt`` is the twist persistence length (nm).  Each bond's energy gains
    0.5 eps_twist dw^2 with eps_twist = lt / (delta lp) = lt / bead_length and
    dw the twist angle of the two beads' (t2, t3) frames minus the natural
    twist bead_length * (2 pi / 10.5) / 0.332, wrapped into [-pi, pi).  The MC
    kernels evaluate the twist terms in FP64."""

    def __init__(self, name, r, *, bead_length, lp, lt, bead_rad=5, t3=_empty_2d, t2=_empty_2d,
                 states=_mty_2d_int, binder_names=_empty_1d, chemical_mods=_mty_2d_int,
                 chemical_mod_names=_empty_1d, log_path="", max_binders=-1):
        self.lt = float(lt)
        super().__init__(name, r, bead_length=bead_length, lp=lp, bead_rad=bead_rad, t3=t3, t2=t2,
                         states=states, binder_names=binder_names, chemical_mods=chemical_mods,
                         chemical_mod_names=chemical_mod_names, log_path=log_path,
                         max_binders=max_binders)

    def _find_parameters(self, bead_length):
        super()._find_parameters(bead_length)
        # eps_twist = lt / (delta lp), delta = bead_length / lp (polymers.pyx:1957-2001)
        self.eps_twist = self.lt / (self.delta * self.lp)

    def natural_twist(self):
        """omega0 per bond: bead_length * (2 pi / 10.5) / 0.332 (polymers.pyx:2088-2090)."""
        return np.asarray(self.bead_length, dtype=np.float64) * NATURAL_TWIST_BARE / LENGTH_BP

    def twist_parameters(self):
        """(eps_twist, omega0) per bond, as the device takes them."""
        return np.asarray(self.eps_twist, dtype=np.float64), self.natural_twist()

    def __str__(self):
        return f"Polymer_Class<SSTWLC>, {PolymerBase.__str__(self)}"


class Chromatin(SSWLC):
    """SSWLC model of chromatin, lp = 53 nm (chromo/polymers.pyx:1821-1887)."""

    def __init__(self, name, r, *, bead_length, bead_rad=5, t3=_empty_2d, t2=_empty_2d,
                 states=_mty_2d_int, binder_names=_empty_1d, chemical_mods=_mty_2d_int,
                 chemical_mod_names=_empty_1d_str, log_path="", max_binders=-1, **kwargs):
        super().__init__(name, r, bead_length=bead_length, bead_rad=bead_rad, lp=53, t3=t3,
                         t2=t2, states=states, binder_names=binder_names, log_path=log_path,
                         chemical_mods=chemical_mods, chemical_mod_names=chemical_mod_names,
                         max_binders=max_binders)

    def construct_beads(self):
        self.beads = {i: Nucleosome(i, self.r[i], t3=self.t3[i], t2=self.t2[i],
                                    rad=self.bead_rad, states=self.states[i],
                                    binder_names=self.binder_names)
                      for i in range(self.r.shape[0])}


# ---- initial paths (chromo/util/poly_paths.py) ----

def gaussian_walk(num_steps: int, step_sizes: np.ndarray) -> np.ndarray:
    """Random walk of ``num_steps`` steps from the origin (num_steps + 1 points):
    step k points along a direction drawn isotropically (a normalised
    standard-normal 3-vector from numpy's global generator, all drawn as one
    block) and has length ``step_sizes[k]`` (chromo/util/poly_paths.py:269-295)."""
    dirs = np.random.standard_normal((num_steps, 3))
    dirs = dirs / np.linalg.norm(dirs, axis=1)[:, None]
    out = np.zeros((num_steps + 1, 3))
    out[1:] = np.cumsum(dirs * np.asarray(step_sizes)[:, None], axis=0)
    return out


def in_confinement(point, confine_type, confine_length):
    if confine_type == "":
        return True
    if confine_type == "Spherical":
        return np.linalg.norm(point) <= confine_length
    if confine_type == "Cubical":
        return bool(np.all(np.abs(point) <= confine_length / 2))
    raise ValueError(f"Confinement type {confine_type} not found.")


def confined_gaussian_walk(num_points, step_sizes, confine_type, confine_length):
    points = np.array([0.0, 0.0, 0.0])
    pts = [points]
    for i in range(num_points - 1):
        while True:
            step = np.random.standard_normal((1, 3))
            point = pts[-1] + np.divide(step, np.linalg.norm(step)) * step_sizes[i]
            if in_confinement(point, confine_type, confine_length):
                pts.append(point.reshape(3))
                break
    return np.vstack(pts)


def estimate_tangents_from_coordinates(coordinates: np.ndarray):
    """t3 from the neighbouring coordinates (one-sided at the two ends) and a
    unit t2 perpendicular to it (chromo/util/poly_paths.py:506-545)."""
    from .synthetic import tangents_from_coordinates
    return tangents_from_coordinates(np.asarray(coordinates, dtype=float))
