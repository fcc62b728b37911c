"""A NumPy restatement of the replica energy for derivative checks.

E = SSWLC elastic energy (chromo/polymers.pyx:1348-1381) + binding free
energy (chromo/polymers.pyx:1383-1538, with the precomputed single-site
table) + field energy in the form whose differences are the per-move field
dE (chromo/fields.pyx:1675-1875), with exact FP64 densities (no fixed point).
Used by the tests only, as the function that central finite differences are
taken of."""
import numpy as np


def trilinear(r, widths, n):
    """(voxel index [N, 8], weight [N, 8]) as the reference's
    _generate_weight_vector_with_trial / _generate_index_vector_with_trial."""
    widths = np.asarray(widths, dtype=np.float64)
    n = np.asarray(n)
    d = widths / n
    x = np.mod(r + 0.5 * widths, widths) - 0.5 * d
    ind = np.floor(x / d).astype(np.int64)
    lo = np.where(ind == -1, n - 1, ind)
    hi = np.where(lo + 1 == n, 0, lo + 1)
    wl = 1.0 - (x / d - ind)
    idx = np.empty((r.shape[0], 8), dtype=np.int64)
    w = np.empty((r.shape[0], 8))
    for l in range(8):
        bx, by, bz = l & 1, (l >> 1) & 1, (l >> 2) & 1
        fx = np.where(bx, 1 - wl[:, 0], wl[:, 0])
        fy = np.where(by, 1 - wl[:, 1], wl[:, 1])
        fz = np.where(bz, 1 - wl[:, 2], wl[:, 2])
        w[:, l] = fx * fy * fz
        ix = np.where(bx, hi[:, 0], lo[:, 0])
        iy = np.where(by, hi[:, 1], lo[:, 1])
        iz = np.where(bz, hi[:, 2], lo[:, 2])
        idx[:, l] = ix + n[0] * (iy + n[1] * iz)
    return idx, w


def voxel_fraction(r, widths, n):
    """Fractional position of each coordinate inside its voxel (0 or 1 at a face)."""
    widths = np.asarray(widths, dtype=np.float64)
    d = widths / np.asarray(n)
    x = np.mod(r + 0.5 * widths, widths) - 0.5 * d
    t = x / d
    return t - np.floor(t)


def elastic(r, t3, bonds):
    dr = r[1:] - r[:-1]
    a0, a1 = t3[:-1], t3[1:]
    eb, g, ep, epp, eta = (bonds[:, k] for k in range(5))
    par = np.sum(a0 * dr, axis=1)
    dp = dr - a0 * par[:, None]
    bend = a1 + (-a0 - eta[:, None] * dp)
    return float(np.sum(0.5 * eb * np.sum(bend * bend, axis=1) + 0.5 * ep * (par - g) ** 2
                        + 0.5 * epp * np.sum(dp * dp, axis=1)))


def binding(states, marks, p):
    e = 0.0
    for b in range(states.shape[1]):
        s, nm = states[:, b], marks[:, b]
        mu = p["mu"][b]
        me = mu * (2 - p["adj"]) if mu > 0 else mu * p["adj"]
        e += float(np.sum(p["bind_f"][b, nm, s]) - np.sum(s) * me)
    return e


def field(r, states, p):
    idx, w = trilinear(r, p["widths"], p["n"])
    G = int(np.prod(p["n"]))
    nb = states.shape[1]
    W = np.zeros(G)
    np.add.at(W, idx.ravel(), w.ravel())
    Wb = np.zeros((nb, G))
    for b in range(nb):
        np.add.at(Wb[b], idx.ravel(), (w * states[:, b][:, None]).ravel())
    V = p["vol_bin"]
    rho = Wb / V
    vf = W / V * p["bead_vol"]
    e = 0.0
    for b in range(nb):
        e += p["pref"][b] * np.sum(rho[b] ** 2)
        for c in range(nb):
            e += p["xpref"][b][c] * np.sum(rho[b] * rho[c])
    sat = vf > p["vf_limit"]
    e += np.sum(np.where(sat, 1e99 * vf, p["chi"] * (V / p["bead_vol"]) * vf * vf))
    for b in range(nb):
        e += p["intra"][b] * np.sum(states[:, b] == 2)
    return float(e)


def energy(r, t3, states, marks, bonds, p):
    return elastic(r, t3, bonds) + binding(states, marks, p) + field(r, states, p)
