"""Host-side parts of the drop-in API, checked against the reference's values
(stored in the golden cases) and its documented behaviour."""
import numpy as np
import pytest

import chromo_gb300.binders as cb
from chromo_gb300.fields import NullField, UniformDensityField
from chromo_gb300.mc import get_amplitude_bounds
from chromo_gb300.mc.mc_controller import SimpleControl, all_moves
from chromo_gb300.polymers import SSTWLC, Chromatin
from golden_cases import CASES, load


def _poly_from_golden(g, state="0"):
    names = [str(x) for x in g["binder_names"]]
    for i, nm in enumerate(names):
        b = cb.get_by_name(nm)
        b.chemical_potential = float(g["mu"][i])
        b.interaction_energy = float(g["interaction_energy"][i])
        b.cross_talk_interaction_energy = {
            str(o): float(g["cross"][i, j]) for j, o in enumerate(names)
            if not np.isnan(g["cross"][i, j])}
    kw = dict(bead_length=g["bead_length"], t3=g["t3" + state], t2=g["t2" + state],
              states=g["states" + state], binder_names=np.array(names), chemical_mods=g["marks"],
              chemical_mod_names=np.array(names), max_binders=int(g["max_binders"]))
    if "lt" in g:  # an SSTWLC chain
        p = SSTWLC("p", g["r" + state], lp=float(g["lp"]), lt=float(g["lt"]), **kw)
    else:
        p = Chromatin("p", g["r" + state], **kw)
    binders = cb.make_binder_collection([cb.get_by_name(n) for n in names])
    return p, binders


@pytest.mark.parametrize("name", CASES)
def test_sswlc_parameters_match_reference(name):
    g = load(name)
    p, _ = _poly_from_golden(g)
    for k in ("eps_bend", "gamma", "eps_par", "eps_perp", "eta"):
        np.testing.assert_array_equal(getattr(p, k), g[k])
    if "lt" in g:  # SSTWLC: twist modulus (polymers.pyx:1957-2001) and natural twist
        eps, w0 = p.twist_parameters()
        np.testing.assert_array_equal(eps, g["eps_twist"])
        np.testing.assert_array_equal(w0, g["omega0"])


@pytest.mark.parametrize("name", [c for c in CASES if c != "null_spherical"])
def test_field_prefactors_match_reference(name):
    g = load(name)
    p, binders = _poly_from_golden(g)
    n = [int(x) for x in g["nxyz"]]
    w = [float(x) for x in g["widths"]]
    f = UniformDensityField([p], binders, w[0], n[0], w[1], n[1], w[2], n[2], chi=float(g["chi"]),
                            vf_limit=float(g["vf_limit"]))
    pref, intra, xpref = f.prefactor_arrays()
    np.testing.assert_array_equal(pref, g["pref"])
    np.testing.assert_array_equal(intra, g["intra"])
    np.testing.assert_array_equal(xpref, g["xpref"])
    assert f.vol_bin == pytest.approx(w[0] * w[1] * w[2] / (n[0] * n[1] * n[2]))


@pytest.mark.parametrize("name", [c for c in CASES if "access_vols" in load(c)])
def test_accessible_volumes_match_reference(name):
    """Voxels cut by a spherical confinement get the fraction of a 20^3 point
    lattice inside the sphere (chromo/fields.pyx:714-951), as the reference
    computed them for the golden case."""
    g = load(name)
    p, binders = _poly_from_golden(g)
    n = [int(x) for x in g["nxyz"]]
    w = [float(x) for x in g["widths"]]
    f = UniformDensityField([p], binders, w[0], n[0], w[1], n[1], w[2], n[2], confine_type="Spherical",
                            confine_length=float(g["confine_length"]), chi=float(g["chi"]),
                            assume_fully_accessible=0)
    assert not f.uniform_access
    np.testing.assert_array_equal(f.access_vols, g["access_vols"])


def test_binder_presets_and_lookup():
    assert cb.get_by_name("HP1") is cb.hp1
    assert cb.get_by_name("PRC1") is cb.prc1
    with pytest.raises(ValueError):
        cb.get_by_name("nope")
    t = cb.make_binder_collection(["HP1", cb.prc1])
    assert len(t) == 2 and t.loc[1, "name"] == "PRC1"
    assert t.iloc[0].interaction_volume == pytest.approx(4 / 3 * np.pi * 27)
    assert t.to_dict(orient="records")[0]["sites_per_bead"] == 2


def test_amplitude_bounds_and_controllers():
    p = Chromatin.straight_line_in_x("p", np.full(999, 16.5), binder_names=np.array(["HP1"]))
    bab, mab = get_amplitude_bounds([p])
    assert bab.bounds["crank_shaft"] == (30, 150)
    assert bab.bounds["end_pivot"] == (50, 150)
    assert bab.bounds["tangent_rotation"] == (1, 1000)
    assert mab.bounds["slide"] == pytest.approx((0.2 * 16.5, 0.3 * 16.5))
    cs = all_moves("/tmp", bab.bounds, mab.bounds, SimpleControl)
    assert [c.move.num_per_cycle for c in cs] == [30, 1, 60, 60, 10]
    assert [c.move.name for c in cs] == ["crank_shaft", "end_pivot", "slide", "tangent_rotation",
                                         "change_binding_state"]
    assert cs[0].move.amp_bead == 30 and cs[0].move.amp_move == pytest.approx(0.1 * np.pi)


def test_simple_control_rule_on_host():
    p = Chromatin.straight_line_in_x("p", np.full(99, 16.5), binder_names=np.array(["HP1"]))
    bab, mab = get_amplitude_bounds([p])
    c = all_moves("/tmp", bab.bounds, mab.bounds, SimpleControl)[2]
    c.move.acceptance_tracker.acceptance_rate = 0.9
    a0 = c.move.amp_move
    c.update_amplitudes()
    assert c.move.amp_move == pytest.approx(a0 / 0.95)
    c.move.acceptance_tracker.acceptance_rate = 0.1
    c.move.amp_move = mab.bounds["slide"][0] * 1.01
    c.update_amplitudes()
    assert c.move.amp_bead == max(bab.bounds["slide"][0], 10 - 1)
    assert c.move.amp_move == pytest.approx(mab.bounds["slide"][1])


def test_null_field_membership():
    p = Chromatin.straight_line_in_x("p", np.full(9, 16.5), binder_names=np.array(["HP1"]))
    f = NullField([p], confine_type="Spherical", confine_length=100.0)
    assert p in f
    assert Chromatin.straight_line_in_x("q", np.full(9, 16.5), binder_names=np.array(["HP1"])) not in f
    with pytest.raises(ValueError):
        NullField([p], confine_type="Tetrahedral")


def test_mc_step_runs_one_move_at_current_amplitudes(monkeypatch):
    """mc_step (chromo/mc/mc_sim.pyx:106-182) hands mc_sim one step of one
    uncontrolled move at the adapter's current amplitudes, drops the field
    when it is not active, restores num_per_cycle, and draws a fresh random
    stream on every call unless given a seed (the GPU run itself is mc_sim's)."""
    import importlib
    ms = importlib.import_module("chromo_gb300.mc.mc_sim")  # the package re-exports the function
    p = Chromatin.straight_line_in_x("p", np.full(99, 16.5), binder_names=np.array(["HP1"]))
    binders = cb.make_binder_collection([cb.get_by_name("HP1")])
    field = UniformDensityField([p], binders, 400, 10, 400, 10, 400, 10)
    bab, mab = get_amplitude_bounds([p])
    move = all_moves("/tmp", bab.bounds, mab.bounds, SimpleControl)[2].move  # slide
    move.amp_bead, move.amp_move = 7, 2.5
    calls = []

    def fake_mc_sim(polymers, readerproteins, n_steps, ctrls, fld, maf, seed):
        (c,) = ctrls
        calls.append(dict(polys=list(polymers), n=n_steps, kind=c.kind, bead=c.bead_amp_bounds,
                          amp=c.move_amp_bounds, npc=c.move.num_per_cycle, field=fld, seed=seed))

    monkeypatch.setattr(ms, "mc_sim", fake_mc_sim)
    ms.mc_step(move, p, binders, field, 1, 0)
    ms.mc_step(move, p, binders, field, 0, 0)
    ms.mc_step(move, p, binders, field, 1, 0, random_seed=42)
    assert [c["n"] for c in calls] == [1, 1, 1] and all(c["polys"] == [p] for c in calls)
    assert all(c["kind"] == 0 and c["npc"] == 1 for c in calls)
    assert calls[0]["bead"] == (7, 7) and calls[0]["amp"] == (2.5, 2.5)
    assert calls[0]["field"] is field and calls[1]["field"] is None
    assert calls[0]["seed"] != calls[1]["seed"] and calls[2]["seed"] == 42
    assert move.num_per_cycle == 60
    with pytest.raises(NotImplementedError):
        ms.mc_step(move, p, binders, field, 1, 1)


def test_continue_polymer_in_field_from_latest_snapshot(monkeypatch, tmp_path):
    """continue_polymer_in_field_simulation (chromo/mc/__init__.py:167-227)
    reads each polymer's latest <name>-<i>.csv, puts it in the field, and
    continues the snapshot numbering (the device runs are faked here)."""
    import chromo_gb300.mc as mc
    binders = cb.make_binder_collection([cb.get_by_name("HP1")])
    p = Chromatin.straight_line_in_x("chr", np.full(49, 16.5), binder_names=np.array(["HP1"]))
    p.to_csv(str(tmp_path / "chr-0.csv"))
    p.r[:, 1] += 3.0
    p.states[::2, 0] = 1
    p.to_csv(str(tmp_path / "chr-1.csv"))
    (tmp_path / "notes-x.csv").write_text("not a snapshot")
    field = UniformDensityField([p], binders, 400, 10, 400, 10, 400, 10)
    seen = []

    class FakeChain:  # the device steps, faked: each run shifts the chain by 1 in z
        def __init__(self, polymers, fld, ctrls):
            (self.q,) = polymers
            self.fld = fld

        def run(self, n_steps, maf, seed):
            q = self.q
            seen.append((q.r.copy(), q.states.copy(), self.fld is field and q in self.fld, n_steps))
            q.r[:, 2] += 1.0

        def close(self):
            pass

    monkeypatch.setattr(mc, "ResidentChain", FakeChain)
    assert {k: v[0] for k, v in mc.latest_snapshots(tmp_path).items()} == {"chr": 1}
    snaps = mc.continue_polymer_in_field_simulation(Chromatin, binders, field, str(tmp_path), 5, 2)
    assert len(snaps) == 2 and len(seen) == 2
    np.testing.assert_array_equal(seen[0][0], p.r)
    np.testing.assert_array_equal(seen[0][1], p.states)
    assert seen[0][2] and seen[0][3] == 5
    assert (tmp_path / "chr-2.csv").exists() and (tmp_path / "chr-3.csv").exists()
    q = Chromatin.from_file(str(tmp_path / "chr-3.csv"), "chr")
    np.testing.assert_allclose(q.r[:, 2], p.r[:, 2] + 2.0)
    with pytest.raises(FileNotFoundError):
        mc.continue_polymer_in_field_simulation(Chromatin, binders, field, str(tmp_path / "none"), 5, 1)


def test_confined_workload_chains_and_volumes():
    """The confined benchmark workload: every bead starts inside its sphere,
    and the accessible volumes it uploads are those UniformDensityField
    computes for the same grid and confinement (chromo/fields.pyx:714-951)."""
    from chromo_gb300 import workloads as wl
    w = wl.make_workload("sphere")
    chains = wl.make_chains(w)
    assert len(chains) == w.replicas == 256
    assert max(np.linalg.norm(c.r, axis=1).max() for c in chains[:16]) <= w.sphere_radius
    p = Chromatin("p", chains[0].r, bead_length=np.full(len(chains[0].r) - 1, wl.BEAD_SPACING),
                  binder_names=np.array(["HP1"]))
    width = w.nbins * wl.VOXEL
    f = UniformDensityField([p], cb.make_binder_collection([cb.get_by_name("HP1")]), width, w.nbins,
                            width, w.nbins, width, w.nbins, confine_type="Spherical",
                            confine_length=w.sphere_radius, assume_fully_accessible=0)
    np.testing.assert_array_equal(wl._sphere_volumes(w.nbins, w.sphere_radius), f.access_vols)
    assert f.access_vols.min() > 0


def _fake_chain_class(log, fail_at=None):
    class FakeChain:
        """Stands in for the resident device chain: run k moves every bead by k + 1 in x."""
        def __init__(self, polymers, fld, ctrls):
            (self.q,) = polymers
            self.k = 0
            log.append("init")

        def run(self, n_steps, maf, seed):
            self.k += 1
            self.q.r[:, 0] += self.k
            self.q.states[:, 0] = self.k % 2
            log.append(("run", n_steps, maf, seed))

        def close(self):
            log.append("close")
    return FakeChain


def test_polymer_in_field_writes_snapshots_in_the_background(monkeypatch, tmp_path):
    """polymer_in_field keeps one resident chain for all segments and writes each
    snapshot's CSV on a background thread from a frozen copy: the files hold
    the snapshots even though the polymer moves on before they are written;
    the segments get the mu_schedule factor and seeds drawn from random_seed."""
    import chromo_gb300.mc as mc
    from chromo_gb300.mc.moves import Bounds
    log = []
    monkeypatch.setattr(mc, "ResidentChain", _fake_chain_class(log))
    p = Chromatin.straight_line_in_x("chr", np.full(30, 16.5), binder_names=np.array(["HP1"]))
    binders = cb.make_binder_collection([cb.get_by_name("HP1")])
    field = UniformDensityField([p], binders, 400, 10, 400, 10, 400, 10)
    x0 = p.r[:, 0].copy()

    class Sched:
        @staticmethod
        def function(i, n):
            return 1.0 - 0.25 * i

    b = Bounds("b", {})
    snaps = mc.polymer_in_field([p], binders, field, 7, 3, b, b, mc_move_controllers=[object()],
                                random_seed=11, mu_schedule=Sched, output_dir=tmp_path, start_index=4)
    assert log[0] == "init" and log[-1] == "close" and len(log) == 5
    np.random.seed(11)
    seeds = [np.random.randint(0, 1E9) for _ in range(3)]
    assert [e[1:] for e in log[1:4]] == [(7, 1.0, seeds[0]), (7, 0.75, seeds[1]), (7, 0.5, seeds[2])]
    for i in range(3):
        q = Chromatin.from_file(str(tmp_path / f"chr-{4 + i}.csv"), "chr")
        np.testing.assert_array_equal(q.r, snaps[i][0]["r"])
        np.testing.assert_array_equal(q.states, snaps[i][0]["states"])
        np.testing.assert_allclose(q.r[:, 0], x0 + sum(range(1, i + 2)))
    np.testing.assert_array_equal(p.r, snaps[-1][0]["r"])


def test_polymer_in_field_reports_a_failed_snapshot_write(monkeypatch, tmp_path):
    """A snapshot that cannot be written raises from polymer_in_field (after the
    resident chain is closed)."""
    import chromo_gb300.mc as mc
    from chromo_gb300.mc.moves import Bounds
    log = []
    monkeypatch.setattr(mc, "ResidentChain", _fake_chain_class(log))
    p = Chromatin.straight_line_in_x("chr", np.full(10, 16.5), binder_names=np.array(["HP1"]))
    binders = cb.make_binder_collection([cb.get_by_name("HP1")])
    field = UniformDensityField([p], binders, 400, 10, 400, 10, 400, 10)
    b = Bounds("b", {})
    with pytest.raises(OSError):
        mc.polymer_in_field([p], binders, field, 2, 2, b, b, mc_move_controllers=[object()],
                            output_dir=tmp_path / "missing" / "dir")
    assert log[-1] == "close"
