"""Homogeneous transforms of the MC moves (chromo/util/linalg.pyx:23-199).

Host-side helpers for calling a move function directly
(``chromo_gb300.mc.move_funcs``); the MC loop itself builds its transforms
inside the GPU kernel.  A transform is a 4 x 4 matrix [[R, T], [0, 1]]
acting on (x, y, z, 1).
"""
import ctypes

import numpy as np

RAND_MAX = 2147483647.0
_libc = ctypes.CDLL(None)
_libc.rand.restype = ctypes.c_int


_sources = {"rand": None, "state": None}


def rand() -> int:
    """libc rand(), the reference's source of move randomness (seed it with
    ``srand``), unless ``set_random_source`` installed another."""
    f = _sources["rand"]
    return int(f()) if f is not None else int(_libc.rand())


def new_state(n_tails: int) -> int:
    """A new binding state in 0..n_tails: np.random.randint(0, n_tails + 1), as
    the reference draws it, unless ``set_random_source`` installed another."""
    f = _sources["state"]
    return int(f(n_tails)) if f is not None else int(np.random.randint(0, n_tails + 1))


def srand(seed: int) -> None:
    _libc.srand(ctypes.c_uint(int(seed) & 0xFFFFFFFF))


def set_random_source(rand_fn=None, state_fn=None) -> None:
    """Replace the draws of directly called moves: ``rand_fn()`` in place of
    rand() (values in 0..RAND_MAX) and ``state_fn(n_tails)`` in place of the
    binding-state draw (None restores the default)."""
    _sources["rand"], _sources["state"] = rand_fn, state_fn


def uniform_sample_unit_sphere() -> np.ndarray:
    """A direction uniform on the unit sphere: azimuth 2 pi u1, polar angle
    acos(2 u2 - 1), u = rand() / RAND_MAX (linalg.pyx:23-42)."""
    phi = rand() / RAND_MAX * (2.0 * np.pi)
    theta = np.arccos(rand() / RAND_MAX * 2 - 1)
    return np.array([np.cos(phi) * np.sin(theta), np.sin(phi) * np.sin(theta), np.cos(theta)])


def rotation_about_axis(axis, point, angle) -> np.ndarray:
    """4 x 4 transform rotating by `angle` (counterclockwise looking down the
    unit `axis`) about the line through `point` along `axis`: Rodrigues'
    rotation R = cos I + sin [a]x + (1 - cos) a a^T and T = p - R p."""
    a = np.asarray(axis, dtype=float)
    p = np.asarray(point, dtype=float)
    c, s = np.cos(angle), np.sin(angle)
    cross = np.array([[0.0, -a[2], a[1]], [a[2], 0.0, -a[0]], [-a[1], a[0], 0.0]])
    m = np.identity(4)
    m[:3, :3] = c * np.identity(3) + s * cross + (1 - c) * np.outer(a, a)
    m[:3, 3] = p - m[:3, :3] @ p
    return m


def arbitrary_axis_rotation(axis, point, rot_angle, poly) -> None:
    """Store the rotation of ``rotation_about_axis`` in
    ``poly.transformation_mat`` (linalg.pyx:62-139)."""
    poly.transformation_mat = rotation_about_axis(axis, point, rot_angle)


def return_arbitrary_axis_rotation(axis, point, rot_angle) -> np.ndarray:
    """The same transform, returned (linalg.pyx:142-169)."""
    return rotation_about_axis(axis, point, rot_angle)


def generate_translation_mat(delta, polymer) -> None:
    """Store the translation by `delta` in ``polymer.transformation_mat``
    (linalg.pyx:172-199)."""
    m = np.identity(4)
    m[:3, 3] = np.asarray(delta, dtype=float)
    polymer.transformation_mat = m
