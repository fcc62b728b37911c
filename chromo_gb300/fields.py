"""Fields: the voxelised density field and the null field (chromo/fields.pyx).

``UniformDensityField`` keeps the reference's constructor and geometry
(``init_grid``, chromo/fields.pyx:536-575), binder prefactors
(``init_field_energy_prefactors``, :687-712) and accessible volumes
(``get_accessible_volumes``, :714-768).  The density grid itself lives on the
GPU as int64 fixed point (2^-40 of a unit trilinear weight per count); the
``density`` attribute returns it converted to the reference's layout and
units (n_bins x (num_binders + 1), bead weight / accessible volume).

``fast_field = 1`` selects the reference's pre-tabulated sub-bin weights, a
speed approximation for CPUs; the GPU always evaluates exact trilinear
weights, so the flag is accepted and recorded but does not change the
arithmetic.
"""

import numpy as np

FX_SCALE = 2.0 ** 40
_CONFINE_KIND = {"": 0, "Spherical": 1, "Cubical": 2}


class FieldBase:
    """A discretisation of space for computing energies (chromo/fields.pyx:46-120)."""

    def __init__(self, polymers, binders):
        self.polymers = list(polymers)
        self.n_polymers = len(self.polymers)
        self.binders = binders
        self.confine_type = ""
        self.confine_length = 0.0

    @property
    def name(self):
        return self.__class__.__name__

    def __contains__(self, poly):
        return any(p is poly for p in self.polymers)

    def __str__(self):
        return "Field<>"


class NullField(FieldBase):
    """No field energy beyond an optional confinement (chromo/fields.pyx:280-321)."""

    def __init__(self, polymers=None, confine_type="", confine_length=0.0):
        super().__init__([] if polymers is None else polymers, binders=None)
        if confine_type not in _CONFINE_KIND:
            raise ValueError(f"Confinement type {confine_type} not found.")
        self.confine_type = confine_type
        self.confine_length = confine_length


def spherical_accessible_volumes(nx, ny, nz, dx, dy, dz, radius, vol_bin, n_side=20):
    """Per-voxel volume inside a sphere of ``radius`` centred in an nx x ny x
    nz grid of dx x dy x dz voxels of volume ``vol_bin`` (chromo/fields.pyx:
    714-951): the full voxel away from the surface, else the voxel volume
    times the fraction of an n_side^3 point lattice in the voxel that lies
    inside."""
    n_bins = nx * ny * nz
    vols = np.full(n_bins, vol_bin)
    idx = np.arange(n_bins)
    ix, iy, iz = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    nxyz = np.array([nx, ny, nz])
    cen = np.stack([ix, iy, iz], axis=1) - (nxyz - 1) / 2
    coords = cen @ np.diag([dx, dy, dz])
    buffer_dist = np.sqrt(2) / 4 * max(dx, dy, dz)
    dist = np.sqrt((coords ** 2).sum(axis=1))
    split = ~((dist < radius - buffer_dist) | (dist > radius + buffer_dist))
    g = np.reshape(np.mgrid[0:n_side, 0:n_side, 0:n_side].T, (n_side ** 3, 3)).astype(float)
    g = g * np.array([dx / n_side, dy / n_side, dz / n_side])
    for i in np.nonzero(split)[0]:
        pts = g + (coords[i] - np.array([dx / 2, dy / 2, dz / 2]))
        d = np.linalg.norm(pts, axis=1)
        vols[i] = vol_bin * (np.count_nonzero(d < radius) / float(len(pts)))
    return vols


class UniformDensityField(FieldBase):
    """Rectilinear voxel grid with trilinear density deposition
    (chromo/fields.pyx:324-2316)."""

    def __init__(self, polymers, binders, x_width, nx, y_width, ny, z_width, nz,
                 confine_type="", confine_length=0.0, chi=1.0, assume_fully_accessible=1,
                 vf_limit=0.5, fast_field=0, n_points=1000):
        super().__init__(polymers=polymers, binders=binders)
        for poly in self.polymers:
            if poly.num_binders != len(binders):
                raise NotImplementedError("For now, all polymers must use all of the same binders.")
        if confine_type not in _CONFINE_KIND:
            raise ValueError(f"Confinement type {confine_type} not found.")
        self.x_width, self.y_width, self.z_width = float(x_width), float(y_width), float(z_width)
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.init_grid()
        self.num_binders = len(binders)
        self.confine_type = confine_type
        self.confine_length = float(confine_length)
        self.assume_fully_accessible = assume_fully_accessible
        self.chi = float(chi)
        self.vf_limit = float(vf_limit)
        self.fast_field = int(fast_field)
        # init_fast_field (chromo/fields.pyx:577-671) rounds n_points up to even;
        # the sub-bin weights are evaluated on the device from that count
        self.n_points = int(n_points) + int(n_points) % 2 if self.fast_field else int(n_points)
        self.init_field_energy_prefactors()
        self.binder_dict = self.binders.to_dict(orient="records")
        self.access_vols = self.get_accessible_volumes(20, assume_fully_accessible)
        self._density_fx = None  # int64 fixed-point grid mirrored from the GPU

    def init_grid(self):
        # chromo/fields.pyx:536-575
        self.dx = self.x_width / self.nx
        self.dy = self.y_width / self.ny
        self.dz = self.z_width / self.nz
        self.dxyz = np.array([self.dx, self.dy, self.dz])
        self.n_bins = self.nx * self.ny * self.nz
        self.vol_bin = self.x_width * self.y_width * self.z_width / self.n_bins
        self.width_xyz = np.array([self.x_width, self.y_width, self.z_width])
        self.half_width_xyz = 0.5 * self.width_xyz
        self.half_step_xyz = 0.5 * self.dxyz
        self.n_xyz_m1 = np.array([self.nx - 1, self.ny - 1, self.nz - 1])

    def init_field_energy_prefactors(self):
        # chromo/fields.pyx:687-712
        names = [self.binders.loc[i, "name"] for i in range(self.num_binders)]
        for i in range(self.num_binders):
            row = self.binders.iloc[i]
            self.binders.at[i, "field_energy_prefactor"] = (
                0.5 * row.interaction_energy * row.interaction_volume * self.vol_bin)
            self.binders.at[i, "interaction_energy_intranucleosome"] = (
                row.interaction_energy * (1 - row.interaction_volume / self.vol_bin))
            xp = self.binders.at[i, "cross_talk_field_energy_prefactor"]
            for other in names:
                if other in row.cross_talk_interaction_energy.keys():
                    xp[other] = (row.cross_talk_interaction_energy[other]
                                 * row.interaction_volume * self.vol_bin)
                else:
                    xp[other] = 0

    def prefactor_arrays(self):
        """(pref[nb], intra[nb], xpref[nb, nb]) in binder order."""
        nb = self.num_binders
        pref = np.array([r["field_energy_prefactor"] for r in self.binder_dict], dtype=np.float64)
        intra = np.array([r["interaction_energy_intranucleosome"] for r in self.binder_dict],
                         dtype=np.float64)
        xpref = np.zeros((nb, nb))
        for i, r in enumerate(self.binder_dict):
            for j, o in enumerate(self.binder_dict):
                xpref[i, j] = r["cross_talk_field_energy_prefactor"][o["name"]]
        return pref, intra, xpref

    def get_accessible_volumes(self, n_side, assume_fully_accessible):
        """Per-voxel accessible volume (chromo/fields.pyx:714-951): the full
        voxel, or for a spherical confinement the fraction of an n_side^3
        point lattice in each voxel near the boundary that lies inside."""
        if assume_fully_accessible == 1 or self.confine_type != "Spherical":
            return np.full(self.n_bins, self.vol_bin)
        return spherical_accessible_volumes(self.nx, self.ny, self.nz, self.dx, self.dy, self.dz,
                                            self.confine_length, self.vol_bin, n_side)

    @property
    def uniform_access(self):
        return bool(np.all(self.access_vols == self.vol_bin))

    @property
    def density(self):
        """Density per voxel in the reference's units (n_bins x (num_binders+1)).
        Computed on the GPU from the current polymer positions if no simulation
        has run yet."""
        if self._density_fx is None:
            from .mc.mc_sim import _deposit_field
            _deposit_field(self)
        return (self._density_fx.astype(np.float64) / FX_SCALE) / self.access_vols[:, None]

    @property
    def density_fixed_point(self):
        if self._density_fx is None:
            from .mc.mc_sim import _deposit_field
            _deposit_field(self)
        return self._density_fx

    def compute_E(self, poly):
        """Total field energy in the reference's form (chromo/fields.pyx:1939-2316):
        oligomerisation sum_b pref_b sum rho_b^2, intranucleosome term, and the
        nonspecific chi (V/Vb) vf (1 - vf) term (1e99 vf above vf_limit after
        rounding vf to two decimals).  Per-move dE follows a different form (see
        ``compute_E_consistent``)."""
        rho = self.density
        pref, intra, _ = self.prefactor_arrays()
        E = 0.0
        for b in range(self.num_binders):
            E += pref[b] * float(np.sum(rho[:, b + 1] ** 2))
            E += intra[b] * int(np.count_nonzero(np.asarray(poly.states)[:, b] == 2))
        bead_V = poly.beads[0].vol
        vf = rho[:, 0] * bead_V
        over = np.round(vf, 2) > self.vf_limit
        E += float(np.sum(np.where(over, 1e99 * vf, self.chi * (self.access_vols / bead_V) * vf * (1 - vf))))
        return E

    def compute_E_consistent(self, poly):
        """Field energy whose differences are the per-move field dE, in FP64 on
        the GPU (chi enters as +chi (V/Vb) vf^2 and cross talk is included)."""
        from .mc.mc_sim import _energies_of
        return _energies_of(poly, field=self)[2]

    def __str__(self):
        return f"UniformDensityField<nx={self.nx},ny={self.ny},nz={self.nz},npoly={len(self.polymers)}>"
