"""cg_field_energy_static: the field energy of a chain computed in a static
device scratch grid, with no allocation inside the call.

Checked against the cg_sim path (cg_deposit + cg_energy, whose out[2] is the
same quantity) on the golden chains and on a 10,000-bead chain, on two calls
in a row (the second call reuses the scratch the first one left behind).
Kept in the last-collected file so that it also runs after every other test
in the same process."""
import ctypes as C

import numpy as np
import pytest

from golden_cases import CASES, gpu_sim, load

UNIFORM_CASES = [c for c in CASES if int(load(c)["field_kind"]) == 2]
REL = 1e-12  # FP64 sums over the same int64 grid, reduced in a different order


def _call(fp, n, r, states, out, stream):
    from chromo_gb300 import _native as nat
    rc = nat.lib().cg_field_energy_static(C.byref(fp), n, r, states, None, out, stream)
    nat.check(rc)


def _static_energies(fp, r_host, states_host, calls=2):
    import torch
    r = torch.tensor(np.ascontiguousarray(r_host, dtype=np.float64), device="cuda")
    st = torch.tensor(np.ascontiguousarray(states_host, dtype=np.int64), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    got = []
    for _ in range(calls):
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        _call(fp, int(r.shape[0]), r.data_ptr(), st.data_ptr(), out.data_ptr(), stream)
        torch.cuda.synchronize()
        got.append(out.cpu().numpy())
    return got


def _golden_field(g):
    from chromo_gb300.device import field_params
    return field_params(
        field_kind=2, confine_kind=int(g["confine_kind"]), confine_length=float(g["confine_length"]),
        nxyz=g["nxyz"], widths=g["widths"], n_binders=g["states0"].shape[1], chi=float(g["chi"]),
        vf_limit=float(g["vf_limit"]), bead_vol=4.0 / 3.0 * np.pi * float(g["bead_rad"]) ** 3,
        pref=g["pref"], intra=g["intra"], xpref=g["xpref"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", UNIFORM_CASES)
def test_static_field_energy_matches_sim_on_golden_chains(case):
    pytest.importorskip("torch")
    g = load(case)
    sim = gpu_sim(g, pos_fp64=True)
    try:
        want = sim.energy(0)[2]
    finally:
        sim.close()
    for got in _static_energies(_golden_field(g), g["r0"], g["states0"]):
        assert got[0] == pytest.approx(want, rel=REL, abs=1e-9)


@pytest.mark.gpu
def test_static_field_energy_matches_sim_on_10k_chain():
    pytest.importorskip("torch")
    from chromo_gb300 import workloads as wl
    from chromo_gb300.device import field_params
    from chromo_gb300.energetics import field_prefactors
    w = wl.make_workload("plain")
    chains = wl.make_chains(w)
    rng = np.random.default_rng(7)
    chains[0].states[:] = rng.integers(0, 3, size=chains[0].states.shape)
    sim = wl.build_sim(w, chains, pos_fp64=True)
    try:
        want = sim.energy(0)[2]
    finally:
        sim.close()
    nb = w.n_binders
    vint = 4.0 / 3.0 * np.pi * wl.R_INT ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint] * nb, w.cross, wl.binder_names(nb),
                                          wl.VOXEL ** 3)
    fp = field_params(field_kind=2, nxyz=(w.nbins,) * 3, widths=(w.nbins * wl.VOXEL,) * 3,
                      n_binders=nb, chi=float(w.chi[0]), vf_limit=0.5,
                      bead_vol=4.0 / 3.0 * np.pi * wl.BEAD_RAD ** 3, pref=pref, intra=intra,
                      xpref=xpref)
    first, second = _static_energies(fp, chains[0].r, chains[0].states)
    assert first[0] == pytest.approx(want, rel=REL)
    assert second[0] == first[0] and second[1] == first[1]


def _plain_field():
    from chromo_gb300 import workloads as wl
    from chromo_gb300.device import field_params
    from chromo_gb300.energetics import field_prefactors
    w = wl.make_workload("plain")
    vint = 4.0 / 3.0 * np.pi * wl.R_INT ** 3
    pref, intra, xpref = field_prefactors(w.eps, [vint], w.cross, wl.binder_names(1), wl.VOXEL ** 3)
    return w, field_params(field_kind=2, nxyz=(w.nbins,) * 3, widths=(w.nbins * wl.VOXEL,) * 3,
                           n_binders=1, chi=1.0, vf_limit=0.5,
                           bead_vol=4.0 / 3.0 * np.pi * wl.BEAD_RAD ** 3, pref=pref, intra=intra,
                           xpref=xpref)


@pytest.mark.gpu
def test_static_field_energy_reports_nonfinite_position():
    """A position that is not finite makes both outputs NaN (the call itself
    succeeds: the check runs on the device), and the next call with finite
    positions is correct again."""
    pytest.importorskip("torch")
    from chromo_gb300 import workloads as wl
    w, fp = _plain_field()
    c = wl.make_chains(w)[0]
    r = c.r.copy()
    r[17, 1] = np.nan
    bad = _static_energies(fp, r, c.states, calls=1)[0]
    assert np.isnan(bad).all()
    good = _static_energies(fp, c.r, c.states, calls=1)[0]
    assert np.isfinite(good).all()


@pytest.mark.gpu
def test_static_field_energy_second_call_allocates_nothing():
    """After the first call on the device (which may load the module), a call
    leaves the device's free memory exactly as it found it."""
    torch = pytest.importorskip("torch")
    from chromo_gb300 import workloads as wl
    w, fp = _plain_field()
    c = wl.make_chains(w)[0]
    r = torch.tensor(np.ascontiguousarray(c.r), device="cuda")
    st = torch.tensor(np.ascontiguousarray(c.states), device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _call(fp, int(r.shape[0]), r.data_ptr(), st.data_ptr(), out.data_ptr(), stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        _call(fp, int(r.shape[0]), r.data_ptr(), st.data_ptr(), out.data_ptr(), stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_field_energy_rejects_grid_beyond_scratch():
    """Checked before any CUDA call, so it runs without a GPU."""
    from chromo_gb300 import _native as nat
    from chromo_gb300.device import field_params
    try:
        nat.lib()
    except (OSError, RuntimeError) as e:
        pytest.skip(f"native library not loadable here: {e}")
    fp = field_params(field_kind=2, nxyz=(128, 128, 128), widths=(1.0, 1.0, 1.0), n_binders=1)
    buf = np.zeros(8)
    ptr = buf.ctypes.data
    with pytest.raises(nat.CgError) as ei:
        _call(fp, 1, ptr, ptr, ptr, None)
    assert ei.value.code == -1 and "static scratch" in str(ei.value)
