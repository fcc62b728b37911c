"""Reader proteins (binders), as in chromo/binders.pyx.

Same classes, presets and lookup as the reference:

* ``Binder`` / ``ReaderProtein`` with ``interaction_volume = 4/3 pi r^3``
  (chromo/binders.pyx:19-128);
* presets ``null_reader``, ``hp1`` (``'HP1'``) and ``prc1`` (``'PRC1'``)
  (:131-186); ``get_by_name`` returns the module-level object itself, so a
  script that sets ``get_by_name('HP1').chemical_potential`` changes the
  binder every bead of every polymer refers to, exactly as in the reference;
* ``make_binder_collection`` snapshots ``binder.dict()`` of each binder
  into a table (:210-238).  The reference returns a pandas DataFrame; this
  package does not depend on pandas, so the table is a small class with the
  DataFrame calls the field uses (``len``, ``.loc`` / ``.at`` [i, col],
  ``.iloc[i].attr``, ``to_dict('records')``, ``equals``).
"""
import inspect
import sys

import numpy as np


class Binder:
    """A component binding the polymer (chromo/binders.pyx:19-48)."""

    def __init__(self, name: str, sites_per_bead: int) -> None:
        self.name = name
        self.sites_per_bead = sites_per_bead
        self.binding_seq = np.zeros((sites_per_bead,), dtype=int)


class ReaderProtein(Binder):
    """Reader protein energetics (chromo/binders.pyx:51-128)."""

    def __init__(self, name: str, sites_per_bead: int, bind_energy_mod: float,
                 bind_energy_no_mod: float, interaction_energy: float, chemical_potential: float,
                 interaction_radius: float, cross_talk_interaction_energy: dict = None) -> None:
        super().__init__(name, sites_per_bead)
        self.bind_energy_mod = bind_energy_mod
        self.bind_energy_no_mod = bind_energy_no_mod
        self.interaction_energy = interaction_energy
        self.chemical_potential = chemical_potential
        self.interaction_radius = interaction_radius
        self.interaction_volume = (4.0 / 3.0) * np.pi * interaction_radius ** 3
        self.field_energy_prefactor = 0.0
        self.interaction_energy_intranucleosome = 0.0
        self.cross_talk_interaction_energy = ({} if cross_talk_interaction_energy is None
                                              else cross_talk_interaction_energy)
        self.cross_talk_field_energy_prefactor = {}

    def dict(self):
        return {
            "name": self.name,
            "sites_per_bead": self.sites_per_bead,
            "bind_energy_mod": self.bind_energy_mod,
            "bind_energy_no_mod": self.bind_energy_no_mod,
            "interaction_energy": self.interaction_energy,
            "chemical_potential": self.chemical_potential,
            "interaction_radius": self.interaction_radius,
            "interaction_volume": self.interaction_volume,
            "field_energy_prefactor": self.field_energy_prefactor,
            "interaction_energy_intranucleosome": self.interaction_energy_intranucleosome,
            "cross_talk_interaction_energy": self.cross_talk_interaction_energy,
            "cross_talk_field_energy_prefactor": self.cross_talk_field_energy_prefactor,
        }


null_reader = ReaderProtein(
    "null_reader", sites_per_bead=0, bind_energy_mod=0, bind_energy_no_mod=0,
    interaction_energy=0, chemical_potential=0, interaction_radius=0)

hp1 = ReaderProtein(
    "HP1", sites_per_bead=2, bind_energy_mod=-0.01, bind_energy_no_mod=1.52,
    interaction_energy=-4, chemical_potential=-1, interaction_radius=3,
    cross_talk_interaction_energy={"PRC1": 0})

prc1 = ReaderProtein(
    "PRC1", sites_per_bead=2, bind_energy_mod=-0.01, bind_energy_no_mod=1.52,
    interaction_energy=-4, chemical_potential=-1, interaction_radius=3,
    cross_talk_interaction_energy={"HP1": 0})


def get_by_name(name):
    """The module-level binder named ``name`` (chromo/binders.pyx:189-207)."""
    matches = [obj for _, obj in inspect.getmembers(sys.modules[__name__])
               if isinstance(obj, Binder) and obj.name == name]
    if not matches:
        raise ValueError(f"No binders found in {__name__} with name: {name}")
    if len(matches) > 1:
        raise ValueError(f"More than one binder has the name requested: {name}")
    return matches[0]


class _Row:
    def __init__(self, d):
        object.__setattr__(self, "_d", d)

    def __getattr__(self, k):
        try:
            return self._d[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __getitem__(self, k):
        return self._d[k]


class _Cell:
    def __init__(self, t):
        self._t = t

    def __getitem__(self, key):
        i, col = key
        return self._t._rows[i][col]

    def __setitem__(self, key, value):
        i, col = key
        self._t._rows[i][col] = value


class _ILoc:
    def __init__(self, t):
        self._t = t

    def __getitem__(self, i):
        return _Row(self._t._rows[i])


class BinderCollection:
    """Table of binder properties, one row per binder, in the order given."""

    columns = ["name", "sites_per_bead", "bind_energy_mod", "bind_energy_no_mod",
               "interaction_energy", "chemical_potential", "interaction_radius",
               "interaction_volume", "field_energy_prefactor",
               "interaction_energy_intranucleosome", "cross_talk_interaction_energy",
               "cross_talk_field_energy_prefactor"]

    def __init__(self, rows=()):
        self._rows = [dict(r) for r in rows]

    def __len__(self):
        return len(self._rows)

    @property
    def loc(self):
        return _Cell(self)

    @property
    def at(self):
        return _Cell(self)

    @property
    def iloc(self):
        return _ILoc(self)

    def to_dict(self, orient="records"):
        if orient != "records":
            raise ValueError("only orient='records' is supported")
        return [dict(r) for r in self._rows]

    def copy(self):
        """A copy of the table: new rows, with the nested cross-talk dicts
        shared, as a pandas deep copy leaves object cells."""
        return BinderCollection(self._rows)

    def equals(self, other):
        return isinstance(other, BinderCollection) and self._rows == other._rows

    def __iter__(self):
        return iter(self.columns)


def make_binder_collection(binders):
    """Summary table of binders (chromo/binders.pyx:210-238)."""
    if binders is None:
        return None
    if isinstance(binders, (str, Binder)):
        binders = [binders]
    rows = []
    for b in binders:
        if isinstance(b, str):
            b = get_by_name(b)
        d = b.dict()
        # the reference's DataFrame.append copies the row; nested dicts stay shared
        rows.append(d)
    return BinderCollection(rows)
