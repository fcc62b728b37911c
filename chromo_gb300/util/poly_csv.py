"""The reference's CSV snapshot format for polymers, without pandas.

``PolymerBase.to_csv`` in the reference (chromo/polymers.pyx:575-672) builds a
pandas DataFrame with two-level column labels and writes it with
``DataFrame.to_csv``; ``from_file`` (:729-758) reads it back with
``read_csv(header=[0, 1], index_col=0)``.  The same text is produced and
parsed here directly:

* header line 1: an empty index label, then the first-level labels;
  header line 2: an empty index label, then the second-level labels;
* columns, in order: ``r``, ``t3``, ``t2`` (second level ``x``, ``y``, ``z``);
  ``states`` (one per binder name) and ``chemical_mods`` (one per
  modification name); ``bead_length`` (N - 1 bond lengths, then 0);
  ``max_binders`` (repeated on every row); ``name`` and ``lp`` (first row
  only, the others empty).  Single-level columns have an empty second label;
* one row per bead, prefixed by its index; floats in shortest round-trip
  form (Python ``repr``), integers in decimal.
"""
import csv
import io
from typing import Dict, List, Optional, Tuple

import numpy as np

_XYZ = ("x", "y", "z")


def _fmt_float(x) -> str:
    return repr(float(x))


def polymer_columns(poly) -> Tuple[List[Tuple[str, str]], List[List[str]]]:
    """Column labels and the per-row cells of ``poly``'s snapshot."""
    n = int(poly.r.shape[0])
    cols: List[Tuple[str, str]] = []
    data: List[List[str]] = []
    for name in ("r", "t3", "t2"):
        arr = np.asarray(getattr(poly, name), dtype=np.float64)
        for j, ax in enumerate(_XYZ):
            cols.append((name, ax))
            data.append([_fmt_float(v) for v in arr[:, j]])
    if len(poly.chemical_mod_names) > 0:
        states = np.asarray(poly.states)
        for j, b in enumerate(poly.binder_names):
            cols.append(("states", str(b)))
            data.append([str(int(v)) for v in states[:, j]])
        mods = np.asarray(poly.chemical_mods)
        for j, m in enumerate(poly.chemical_mod_names):
            cols.append(("chemical_mods", str(m)))
            data.append([str(int(v)) for v in mods[:, j]])
    bl = np.append(np.asarray(poly.bead_length, dtype=np.float64), 0.0)
    cols.append(("bead_length", ""))
    data.append([_fmt_float(v) for v in bl[:n]])
    if hasattr(poly, "max_binders"):
        cols.append(("max_binders", ""))
        data.append([str(int(poly.max_binders))] * n)
    for name in ("name", "lp", "lt", "bp_wrap"):
        if hasattr(poly, name):
            val = getattr(poly, name)
            if name != "name":
                val = float(val)
            cols.append((name, ""))
            data.append([str(val)] + [""] * (n - 1))
    return cols, data


def to_csv_text(poly) -> str:
    cols, data = polymer_columns(poly)
    out = io.StringIO()
    w = csv.writer(out, lineterminator="\n")
    w.writerow([""] + [c[0] for c in cols])
    w.writerow([""] + [c[1] for c in cols])
    n = len(data[0]) if data else 0
    for i in range(n):
        w.writerow([str(i)] + [col[i] for col in data])
    return out.getvalue()


def read_csv_columns(src) -> Tuple[Dict[str, Dict[str, List[str]]], List[str]]:
    """Parse the two-header-line CSV into {level0: {level1: cells}} (column order kept)."""
    if hasattr(src, "read"):
        text = src.read()
    else:
        with open(src, newline="") as fh:
            text = fh.read()
    rows = list(csv.reader(io.StringIO(text)))
    if len(rows) < 2:
        raise ValueError("a polymer CSV needs two header lines")
    top, sub = rows[0][1:], rows[1][1:]
    body = [r[1:] for r in rows[2:] if r]
    cols: Dict[str, Dict[str, List[str]]] = {}
    order: List[str] = []
    for k, (a, b) in enumerate(zip(top, sub)):
        if a not in cols:
            cols[a] = {}
            order.append(a)
        cols[a][b] = [r[k] for r in body]
    return cols, order


def polymer_kwargs(src, name: Optional[str] = None) -> dict:
    """Constructor arguments of the polymer stored in ``src`` (path or text buffer)."""
    cols, _ = read_csv_columns(src)
    kw = {}
    for vec in ("r", "t3", "t2"):
        if vec in cols:
            kw[vec] = np.ascontiguousarray(
                np.stack([np.asarray(cols[vec][ax], dtype=np.float64) for ax in _XYZ], axis=1))
    if "states" in cols:
        kw["binder_names"] = np.array(list(cols["states"].keys()))
        kw["states"] = np.ascontiguousarray(
            np.stack([np.asarray(v, dtype=np.int64) for v in cols["states"].values()], axis=1))
    if "chemical_mods" in cols:
        kw["chemical_mod_names"] = np.array(list(cols["chemical_mods"].keys()))
        kw["chemical_mods"] = np.ascontiguousarray(
            np.stack([np.asarray(v, dtype=np.int64) for v in cols["chemical_mods"].values()], axis=1))
    if "bead_length" in cols:
        kw["bead_length"] = np.asarray(cols["bead_length"][""][:-1], dtype=np.float64)
    if "max_binders" in cols:
        kw["max_binders"] = int(cols["max_binders"][""][0])
    if name is not None:
        kw["name"] = name
    elif "name" in cols:
        kw["name"] = cols["name"][""][0]
    else:
        kw["name"] = "unnamed"
    for key in ("lp", "lt", "bp_wrap"):
        if key in cols:
            kw[key] = float(cols[key][""][0])
    return kw
