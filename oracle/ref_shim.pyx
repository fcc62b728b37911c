# cython: language_level=3
"""Shim that exposes the reference's ``cdef`` energy methods to Python.

Test infrastructure only (builds against the reference compiled by
``oracle/build_reference.py``).  ``PolymerBase.compute_dE``
(``chromo/polymers.pxd:33-38``), ``FieldBase.compute_dE`` and
``update_affected_densities`` (``chromo/fields.pxd:16-20``) are ``cdef``
methods, so the golden-vector generator reaches them through these wrappers.
"""
cimport chromo.polymers as poly
cimport chromo.fields as fld
import numpy as np


def poly_dE(poly.PolymerBase p, str move_name, inds):
    cdef long[:] v = np.ascontiguousarray(inds, dtype=np.int64)
    return p.compute_dE(move_name, v, v.shape[0])


def field_dE(fld.FieldBase f, poly.PolymerBase p, inds, bint state_change):
    cdef long[:] v = np.ascontiguousarray(inds, dtype=np.int64)
    return f.compute_dE(p, v, v.shape[0], 20, state_change)


def field_accept(fld.FieldBase f):
    f.update_affected_densities()
