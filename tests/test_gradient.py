"""Energy derivatives (config "batched + differentiation"): dE/dr and
dE/d(chi, mu_0, mu_1, eps_00, eps_11, eps_01) from the GPU against FP64
central finite differences (h = 1e-4) of a NumPy restatement of the energy,
on 100 seeded configurations; the reweighting algebra on the CPU."""
import numpy as np
import pytest

from chromo_gb300.derivatives import (observable_coefficients, reweighting_sensitivity,
                                      terms_covariance, theta_coefficients)
from energy_model import energy, voxel_fraction

H = 1e-4


def test_reweighting_algebra_matches_direct_covariance():
    rng = np.random.default_rng(0)
    T = rng.normal(size=(500, 14)) @ rng.normal(size=(14, 14))
    sum_t, sum_tt = T.sum(0), T.T @ T
    cov = terms_covariance(sum_t, sum_tt, len(T))
    np.testing.assert_allclose(cov, np.cov(T.T, bias=True), rtol=1e-9, atol=1e-9)
    O = observable_coefficients(1000, 64000, 2)
    C = theta_coefficients([-0.5, 0.3], 1.0, [113.1, 113.1], 64000.0)
    got = reweighting_sensitivity(sum_t, sum_tt, len(T), O, C)
    o, g = T @ O.T, T @ C.T
    want = -(o.T @ g / len(T) - np.outer(o.mean(0), g.mean(0)))
    np.testing.assert_allclose(got, want, rtol=1e-8, atol=1e-8)
    assert C[2, 11] == -1.0  # mu_1 > 0 with mu_adjust_factor 1: f = 2 - 1


def _setup(R=100, n=300, nbins=10, seed=3):
    from chromo_gb300 import workloads as wl
    from chromo_gb300.energetics import binding_free_energy_table, dss_parameters, field_prefactors
    rng = np.random.default_rng(seed)
    w = wl.Workload("grad", np.full(R, n), nbins, 2, rng.uniform(-1, 0, size=(R, 2)),
                    rng.uniform(0.5, 2.0, size=R), [-4.0, -3.0], [{"PRC1": 1.0}, {}], 50, 0,
                    wl.BASE_SEED + 4)
    chains = wl.make_chains(w)
    for c in chains:
        c.states[:] = rng.integers(0, 3, size=c.states.shape)
    sim = wl.build_sim(w, chains, pos_fp64=True)
    vint = 4.0 / 3.0 * np.pi * wl.R_INT ** 3
    vol_bin = wl.VOXEL ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint] * 2, w.cross, wl.binder_names(2), vol_bin)
    table = binding_free_energy_table([wl.SITES] * 2, [wl.HP1_E_MOD] * 2, [wl.HP1_E_NOMOD] * 2)
    _, eb, g, ep, epp, eta = dss_parameters(np.full(n - 1, wl.BEAD_SPACING), wl.LP)
    bonds = np.stack([eb, g, ep, epp, eta], axis=1)
    params = []
    for r in range(R):
        params.append(dict(widths=(nbins * wl.VOXEL,) * 3, n=(nbins,) * 3, vol_bin=vol_bin,
                           bead_vol=4.0 / 3.0 * np.pi * wl.BEAD_RAD ** 3, chi=float(w.chi[r]),
                           vf_limit=0.5, pref=pref, intra=intra, xpref=xpref, mu=list(w.mu[r]),
                           adj=1.0, bind_f=np.asarray(table), eps=list(w.eps), vint=vint,
                           cross=w.cross))
    return w, chains, sim, bonds, params


@pytest.mark.gpu
def test_position_and_parameter_gradients_match_finite_differences():
    pytest.importorskip("torch")
    from chromo_gb300 import workloads as wl
    from chromo_gb300.energetics import field_prefactors
    w, chains, sim, bonds, params = _setup()
    try:
        g, T = sim.gradient()
        E_gpu = sim.energies()[:, :3].sum(1)
    finally:
        sim.close()
    rng = np.random.default_rng(11)
    n = int(w.lengths[0])
    worst_r, worst_t = 0.0, 0.0
    for r, c in enumerate(chains):
        p = params[r]
        E0 = energy(c.r, c.t3, c.states, c.marks, bonds, p)
        assert E0 == pytest.approx(E_gpu[r], rel=1e-9, abs=1e-9)
        frac = voxel_fraction(c.r, p["widths"], p["n"])
        for _ in range(8):
            i, j = int(rng.integers(n)), int(rng.integers(3))
            if min(frac[i, j], 1 - frac[i, j]) < 1e-3:
                continue  # the weights have a kink at a voxel face
            rp, rm = c.r.copy(), c.r.copy()
            rp[i, j] += H
            rm[i, j] -= H
            fd = (energy(rp, c.t3, c.states, c.marks, bonds, p)
                  - energy(rm, c.t3, c.states, c.marks, bonds, p)) / (2 * H)
            got = float(g[r * n + i, j])
            worst_r = max(worst_r, abs(got - fd) / max(1.0, abs(fd)))
        if r < 20:  # parameters: chi, mu_0, mu_1, eps_00, eps_11, eps_01
            C = theta_coefficients(p["mu"], p["adj"], [p["vint"]] * 2, p["vol_bin"])
            dth = C @ T[r]
            for k in range(6):
                q_plus, q_minus = dict(p), dict(p)
                for q, sgn in ((q_plus, 1.0), (q_minus, -1.0)):
                    if k == 0:
                        q["chi"] = p["chi"] + sgn * H
                    elif k in (1, 2):
                        q["mu"] = list(p["mu"])
                        q["mu"][k - 1] += sgn * H
                    else:
                        eps = list(p["eps"])
                        cross = [dict(x) for x in p["cross"]]
                        if k == 3:
                            eps[0] += sgn * H
                        elif k == 4:
                            eps[1] += sgn * H
                        else:
                            cross[0]["PRC1"] += sgn * H
                        q["pref"], q["intra"], q["xpref"] = field_prefactors(
                            eps, [p["vint"]] * 2, cross, wl.binder_names(2), p["vol_bin"])
                fd = (energy(c.r, c.t3, c.states, c.marks, bonds, q_plus)
                      - energy(c.r, c.t3, c.states, c.marks, bonds, q_minus)) / (2 * H)
                worst_t = max(worst_t, abs(dth[k] - fd) / max(1.0, abs(fd)))
    print(f"worst relative error: dE/dr {worst_r:.2e}, dE/dtheta {worst_t:.2e}")
    assert worst_r < 1e-4   # FP32 output of an FP64 evaluation
    assert worst_t < 1e-6


@pytest.mark.gpu
def test_sampled_sensitivities_are_finite_and_counted():
    pytest.importorskip("torch")
    from chromo_gb300.batched import ReplicaBatch
    from golden_cases import load
    from test_gpu_api import _setup as api_setup
    polys, fields, ctrls = [], [], []
    for _ in range(2):
        p, _, f, c = api_setup(load("two_binders"))
        polys.append(p)
        fields.append(f)
        ctrls.append(c)
    with ReplicaBatch(polys, fields, ctrls) as b:
        b.sample(50, 2, 123)
        s = b.sensitivities()
        assert s.shape == (2, polys[0].num_binders + 1, 6)
        assert np.all(np.isfinite(s))
        _, _, count = b.sim.samples()
        assert np.all(count == 50)
        per, theta = b.gradient()
        assert len(per) == 2 and per[0].shape == (polys[0].num_beads, 3)
        assert np.all(np.isfinite(theta))


@pytest.mark.gpu
def test_autograd_bridge_on_device_tensors():
    """replica_energy on CUDA tensors: energies equal cg_energies, dE/dr equals
    the gradient kernel's (FP32 output of cg_gradient, so within FP32
    rounding), dE/dt3 equals FP64 central differences of the NumPy energy
    (h = 1e-6; the energy is quadratic in t3), and every tensor stays on the
    device."""
    torch = pytest.importorskip("torch")
    from chromo_gb300.autograd import replica_energy
    from chromo_gb300.batched import ReplicaBatch
    from golden_cases import load
    from test_gpu_api import _setup as api_setup
    from energy_model import elastic
    polys, fields, ctrls = [], [], []
    for _ in range(3):
        p, _, f, c = api_setup(load("two_binders"))
        polys.append(p)
        fields.append(f)
        ctrls.append(c)
    with ReplicaBatch(polys, fields, ctrls, precision="fp64") as b:
        dev = torch.device("cuda")
        pos = torch.tensor(np.concatenate([p.r for p in polys]), dtype=torch.float64, device=dev,
                           requires_grad=True)
        t3 = torch.tensor(np.concatenate([p.t3 for p in polys]), dtype=torch.float64, device=dev,
                          requires_grad=True)
        E = replica_energy(pos, b, tangents=t3)
        assert E.is_cuda
        np.testing.assert_allclose(E.detach().cpu().numpy(), b.energies()[:, :3].sum(1), rtol=1e-12)
        weights = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64, device=dev)
        gr, gt = torch.autograd.grad((E * weights).sum(), (pos, t3))
        assert gr.is_cuda and gt.is_cuda
        per, _ = b.gradient()
        want = np.concatenate([w * g.astype(np.float64) for w, g in zip([1.0, -2.0, 0.5], per)])
        np.testing.assert_allclose(gr.cpu().numpy(), want, rtol=2e-6, atol=1e-6)
        # dE/dt3 of replica 0 against central differences of the elastic energy
        p0 = polys[0]
        n = p0.num_beads
        bonds = np.stack([p0.eps_bend, p0.gamma, p0.eps_par, p0.eps_perp, p0.eta], axis=1)
        r0, a0 = np.asarray(p0.r, dtype=np.float64), np.asarray(p0.t3, dtype=np.float64)
        h = 1e-6
        got = gt.cpu().numpy()[:n]
        for i in (0, 1, n // 2, n - 1):
            for j in range(3):
                up, dn = a0.copy(), a0.copy()
                up[i, j] += h
                dn[i, j] -= h
                fd = (elastic(r0, up, bonds) - elastic(r0, dn, bonds)) / (2 * h)
                assert got[i, j] == pytest.approx(fd, rel=1e-6, abs=1e-6), (i, j)


@pytest.mark.gpu
def test_device_sums_of_sampled_terms_equal_host_sums():
    """cg_sample_terms adds every replica's 14 terms T and T T^T to running sums
    on the device; after each of 12 sampled configurations the host reads the
    same terms (cg_gradient), and the device sums equal the host sums."""
    pytest.importorskip("torch")
    from chromo_gb300.batched import ReplicaBatch
    from golden_cases import load
    from test_gpu_api import _setup as api_setup
    polys, fields, ctrls = [], [], []
    for _ in range(2):
        p, _, f, c = api_setup(load("two_binders"))
        polys.append(p)
        fields.append(f)
        ctrls.append(c)
    with ReplicaBatch(polys, fields, ctrls) as b:
        b.sim.samples(reset=True)
        host_t, host_tt = 0.0, 0.0
        for k in range(12):
            b.sim.run(1, 500 + k)
            b.sim.sync()
            _, T = b.sim.gradient(positions=False, terms=True)
            host_t = host_t + T
            host_tt = host_tt + np.einsum("ri,rj->rij", T, T)
            b.sim.sample_terms()
        b.sim.sync()
        sum_t, sum_tt, count = b.sim.samples()
        assert np.all(count == 12)
        np.testing.assert_allclose(sum_t, host_t, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(sum_tt, host_tt, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_reweighting_sensitivity_equals_finite_difference_of_ensemble_means():
    """End to end: d<O>/dmu of the mean binder occupancy O from the on-device
    reweighting sums at mu_0 (-Cov(O, dE/dmu) = Cov(O, f N_bound), the
    fluctuation formula) against central finite differences of <O> measured
    in separate runs at mu_0 -+ 0.25 kT.  System of the reference-equilibrium
    fixture (100-bead chain, one binder, 6^3 periodic box); 64 independent
    replicas per run, 1,500 burn-in steps, 300 samples 20 steps apart; the
    two estimates must agree within 3 combined standard errors (replica to
    replica spread)."""
    pytest.importorskip("torch")
    from pathlib import Path
    from chromo_gb300.derivatives import observable_coefficients, reweighting_sensitivity, theta_coefficients
    from test_gpu_equilibrium import _replicas
    fixture = Path(__file__).resolve().parent / "golden" / "stats" / "eq_one_binder.npz"
    with np.load(fixture, allow_pickle=False) as z:
        g = {k: z[k] for k in z.files}
    R, seed, delta = 64, 7771, 0.25
    mu0 = float(g["mu"][0])
    n = len(g["r0"])
    vol_bin = float(np.prod(np.asarray(g["widths"], dtype=float) / np.asarray(g["nxyz"], dtype=float)))
    vint = 4.0 / 3.0 * np.pi * 3.0 ** 3
    O = observable_coefficients(n, int(np.prod(g["nxyz"])), 1)
    C = theta_coefficients([mu0], 1.0, [vint], vol_bin)

    def sampled(mu):
        gg = dict(g)
        gg["mu"] = np.array([mu])
        sim = _replicas(gg, R)
        try:
            sim.run(int(g["burn"]), seed)
            sim.samples(reset=True)
            for k in range(int(g["samples"])):
                sim.run(int(g["every"]), seed + 1 + k)
                sim.sample_terms()
            sim.sync()
            return sim.samples()
        finally:
            sim.close()

    sum_t, sum_tt, count = sampled(mu0)
    rw = np.array([reweighting_sensitivity(sum_t[r], sum_tt[r], count[r], O, C)[0, 1] for r in range(R)])
    means = {}
    for sign in (-1, 1):
        st, _, cnt = sampled(mu0 + sign * delta)
        means[sign] = (O[0] @ st.T) / cnt  # per replica <O>
    fd = (means[1] - means[-1]) / (2 * delta)
    m_rw, se_rw = rw.mean(), rw.std(ddof=1) / np.sqrt(R)
    m_fd, se_fd = fd.mean(), fd.std(ddof=1) / np.sqrt(R)
    zz = (m_rw - m_fd) / np.sqrt(se_rw ** 2 + se_fd ** 2)
    print(f"d<occupancy>/dmu: reweighting {m_rw:.4f} +- {se_rw:.4f}, finite difference {m_fd:.4f} +- {se_fd:.4f}, "
          f"z {zz:+.2f}")
    assert m_rw > 0 and abs(zz) <= 3.0
