"""Save / do schedules (interface/nsim/when.py) and the hysteresis loop
(interface/nmag/hysteresis.py:244-557) on the host, with a stand-in engine
that relaxes exponentially, so the control logic runs without a GPU."""
import math

import numpy as np
import pytest

import nmag
from nmag import SI
from nmag.when import at, every, never


def test_every_and_at_next_times():
    c = {"step": 3, "stage_step": 3, "time": 0.0, "stage_time": 0.0, "real_time": 0.0, "stage": 1,
         "convergence": False, "stage_end": False}
    w = every("step", 5)
    assert w.next_time("step", c) == 5 and not w.match_time(c)
    assert w.next_time("time", c) is False          # other counter: does it match now?
    c["step"] = 10
    assert w.match_time(c) and w.next_time("step", c) == 15
    w = every("step", 5, first=12, last=30)
    assert w.next_time("step", c) == 12
    c["step"] = 30
    assert w.next_time("step", c) is False
    # SI times become simulation units (1e-12 s)
    t = every("time", SI(2e-12, "s"))
    c["time"] = 3.0
    assert t.next_time("time", c) == pytest.approx(4.0)
    assert at("time", SI(5e-12, "s")).next_time("time", c) == pytest.approx(5.0)
    assert at("convergence").next_time("step", c) is True
    c["convergence"] = True
    assert at("convergence").match_time(c)
    # combinations (when.py:71-128)
    c["step"] = 0
    assert (every("step", 4) | every("step", 6)).next_time("step", c) == 4
    assert (every("step", 4) & every("step", 6)).next_time("step", c) == 12
    assert (every("step", 4) | at("convergence")).next_time("step", c) == 4
    assert never.next_time("step", c) is False and not never.match_time(c)
    with pytest.raises(ValueError):
        every("step", 0)
    with pytest.raises(ValueError):
        every("step", 5, first=10, last=5)


class RelaxingEngine(object):
    """Stand-in for nmag._lib.Engine: fixed steps of h, m relaxing towards
    +z with rate 1 (simulation units)."""

    def __init__(self, N=4, h=0.25):
        self.N, self.B, self.h = N, 1, h
        self.t, self.nst = 0.0, 0
        self.m = np.tile([1.0, 0.0, 0.0], (N, 1))
        self.mark = self.m.copy()
        self.H = None
        self.inits = 0

    def _shape3(self):
        return (self.N, 3)

    def set_m(self, m):
        self.m = np.array(m, dtype=float).reshape(self.N, 3)
        self.mark = self.m.copy()

    def get_m(self):
        return self.m.copy()

    def set_h_ext(self, h):
        self.H = np.array(h, dtype=float)

    def ts_init(self, t0, rtol, atol, q, k):
        self.t, self.nst, self.inits = t0, 0, self.inits + 1

    def ts_advance(self, target, exact_tstop, max_it):
        n = math.ceil((target - self.t) / self.h - 1e-12)
        if max_it is not None and max_it > 0:
            n = min(n, max_it)
        n = max(n, 0)
        self.t = min(self.t + n * self.h, target)
        self.nst += n
        a = math.exp(-self.t)
        self.m = np.tile([a, 0.0, math.sqrt(1 - a * a)], (self.N, 1))
        return self.t, {"nst": self.nst, "hcur": self.h}

    def timings(self):
        return np.zeros(8)

    def max_dm_step(self):
        d = float(np.abs(self.m - self.mark).max())
        self.mark = self.m.copy()
        return d

    def averages(self):
        return self.m.mean(0)

    def eval_fields(self):
        z = np.zeros((self.N, 3))
        return {"H_exch": z, "H_demag": z + 0.1, "H_anis": z, "H_total": z + 0.1, "dmdt": z,
                "phi": np.zeros(self.N), "rho": np.zeros(self.N)}

    def energy_density(self):
        return {k: np.full(self.N, 0.5) for k in ("E_exch", "E_demag", "E_ext", "E_anis", "E_total")}

    def csr(self):
        return (None,) * 5 + (np.array([1.0, 2.0, 3.0, 4.0]),)


def make_sim(tmp_path, monkeypatch, stop=1e-3):
    monkeypatch.chdir(tmp_path)
    sim = nmag.Simulation("hyst")
    eng = RelaxingEngine()
    sim.engine = eng
    sim.material = nmag.MagMaterial("Py")
    sim.mesh = nmag.mesh.Mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], [[0, 1, 2, 3]])
    sim._m = eng.get_m()
    sim._h_ext = np.zeros((eng.N, 3))
    sim.stopping_dm_dt = stop
    return sim, eng


def test_relax_runs_to_convergence_and_saves_at_stage_end(tmp_path, monkeypatch):
    sim, eng = make_sim(tmp_path, monkeypatch)
    sim.relax()
    assert sim.clock.stage_end and sim.clock.convergence
    assert sim.max_dm_dt < sim.stopping_dm_dt
    rows = [l for l in open("hyst_dat.ndt") if not l.startswith("#")]
    assert len(rows) == 1                        # averages at stage end only (the default save)
    from nmag import h5data
    tab = h5data.read(str(tmp_path / "hyst_dat.h5"))["tables"]
    assert len(tab["m"]) == 1                    # every field once, at the stage end
    assert sim.clock.id == 0                     # ids start at -1; one new id per averages row


def test_hysteresis_schedules(tmp_path, monkeypatch):
    sim, eng = make_sim(tmp_path, monkeypatch)
    seen = []

    def record(s):
        seen.append((s.clock.stage, s.clock.stage_step))
    H = [[0, 0, 0.1], [0, 0, 0.2], [0, 0, 0.3]]      # plain numbers: simulation units
    sim.hysteresis(H, save=[(record, every("stage_step", 6))],
                   do=[("next stage", at("stage_step", 12)), ("exit", at("step", 30))])
    # stage 1: steps 0, 6, 12 (ended by next_stage at 12); stage 2 likewise;
    # stage 3 exits at step 30 = stage step 6
    assert seen == [(1, 0), (1, 6), (1, 12), (2, 0), (2, 6), (2, 12), (3, 0), (3, 6)]
    assert sim.clock.exit_hysteresis and sim.clock.step == 30
    assert eng.inits == 3 and np.allclose(eng.H[0], [0, 0, 0.3])
    sim.set_H_ext([0, 0, 2e5], SI("A/m"))
    assert np.allclose(eng.H[0], [0, 0, 0.2])                 # 1 A/m = 1e-6 simulation units
    sim.set_H_ext([SI(0, "A/m"), SI(0, "A/m"), SI(1e5, "A/m")])
    assert np.allclose(eng.H[0], [0, 0, 0.1])


def test_hysteresis_time_schedule_and_errors(tmp_path, monkeypatch):
    sim, eng = make_sim(tmp_path, monkeypatch)
    times = []
    sim.relax(save=[(lambda s: times.append(round(s.clock.stage_time_su, 9)), every("time", SI(0.5e-12, "s")))],
              do=[("exit", at("stage_time", SI(2e-12, "s")))])
    assert times == [0.0, 0.5, 1.0, 1.5, 2.0]
    with pytest.raises(ValueError):
        sim.relax(save=[("teleport", at("stage_end"))])
    with pytest.raises(ValueError):
        sim.relax(save=[("averages", at("stage_end")), ("save averages", every("step", 3))])


def test_ndt_row_layout(tmp_path, monkeypatch):
    """main.py:2313-2480,2571-2634: a names line, a units line, then one
    row per save with the clock, the SI averages and the extra columns."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    sim.relax(save=[("averages", every("step", 10) | at("stage_end"))])
    lines = open("hyst_dat.ndt").read().splitlines()
    names, units = lines[0][1:].split(), lines[1][1:].split()
    rows = [l.split() for l in lines[2:]]
    assert names[:7] == ["time", "id", "step", "last_step_dt", "stage_time", "stage_step", "stage"]
    for col in ("m_Py_0", "m_Py_2", "M_Py_1", "H_total_Py_2", "dmdt_Py_0", "E_total_Py", "E_demag_Py",
                "H_demag_0", "H_ext_2", "phi", "rho", "pin", "maxangle_m_Py", "localtime", "unixtime"):
        assert col in names, col
    assert len(units) == len(names) and all(len(r) == len(names) for r in rows)
    u = dict(zip(names, units))
    assert u["time"] == "<s>" and u["H_demag_0"] == "<A/m>" and u["E_total_Py"] == "<kg/ms^2>" and u["m_Py_0"] == "<1>"
    assert u["dmdt_Py_0"] == "<A/ms>" and u["maxangle_m_Py"] == "<deg>"
    steps = [int(r[names.index("step")]) for r in rows]
    assert steps[:3] == [0, 10, 20] and steps == sorted(set(steps))     # every 10 steps, no step twice
    ids = [int(r[names.index("id")]) for r in rows]
    assert ids == list(range(len(rows)))
    last = dict(zip(names, rows[-1]))
    m = eng.get_m()
    V = np.array([1.0, 2.0, 3.0, 4.0])
    assert float(last["m_Py_2"]) == pytest.approx((m[:, 2] * V).sum() / V.sum(), rel=1e-12)
    assert float(last["H_demag_1"]) == pytest.approx(0.1 * 1e6, rel=1e-12)    # A/m from 0.1 su
    assert float(last["E_exch_Py"]) == pytest.approx(0.5 * 1e6, rel=1e-12)    # J/m^3 from 0.5 su
    assert float(last["pin"]) == 1.0 and float(last["maxangle_m_Py"]) == pytest.approx(0.0, abs=1e-6)


def test_subfield_averages(tmp_path, monkeypatch):
    """main.py:2234-2312: averages in SI numbers or objects; the subfield is
    the material name; M = Ms m."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    assert sim.get_subfield_average_siv("H_demag") == pytest.approx([0.1e6] * 3, rel=1e-12)
    E = sim.get_subfield_average("E_total", "Py")
    assert E.value == pytest.approx(0.5e6, rel=1e-12) and E.dims == SI("J/m^3").dims
    with pytest.raises(ValueError):
        sim.get_subfield_average_siv("m", "Co")
    M = sim.get_subfield("M_Py")
    assert np.allclose(M, eng.get_m() * 0.86e6, rtol=1e-11)


def test_subfield_names_probe_and_units(tmp_path, monkeypatch):
    """Subfield names as the reference resolves them (main.py:612-628): a
    per-material field with this material's suffix or bare, mesh fields bare;
    the probe interpolates in the simplex (None outside) and carries the
    reference's units."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    assert np.allclose(sim.get_subfield("m_Py"), eng.get_m())
    for bad in ("m_Co", "H_demag_Py", "E_total_Co", "Hdemag", "H_ext_x"):
        with pytest.raises(KeyError):
            sim.get_subfield(bad)
    with pytest.raises(KeyError):
        sim.set_m([1.0, 0.0, 0.0], "m_Co")
    assert np.allclose(sim.get_subfield("H_demag"), 0.1e6)
    inside = [0.2e-9, 0.2e-9, 0.2e-9]
    assert sim.probe_subfield_siv("H_demag", inside) == pytest.approx([0.1e6] * 3)
    assert sim.probe_subfield_siv("E_exch_Py", inside) == pytest.approx(0.5e6)
    assert sim.probe_subfield_siv("m", [5e-9, 0.0, 0.0]) is None
    d = sim.probe_subfield("dmdt_Py", [SI(v, "m") for v in inside])
    assert d[0].dims == SI("A/m s").dims
    H = sim.probe_subfield("H_total", [SI(v, "m") for v in inside])
    assert H[2].dims == SI("A/m").dims and H[2].value == pytest.approx(0.1e6)


def test_save_fields_and_restart_name(tmp_path, monkeypatch):
    """save_data(fields=...) appends rows to <name>_dat.h5 in the layout of
    nfem/hdf5_v01.py:685-1022 (tags, mesh, metadata, sites, one table per
    field with id / stage / step / time and the subfields in SI)."""
    from nmag import h5data
    sim, eng = make_sim(tmp_path, monkeypatch)
    sim.save_data(fields="all")
    d = h5data.read(str(tmp_path / "hyst_dat.h5"))
    assert {"m", "M", "H_demag", "E_total", "phi", "pin"} <= set(d["tables"])
    assert np.allclose(d["tables"]["H_demag"]["H_demag"], 0.1e6)
    assert ("m", "m_Py", repr(nmag.SI(1.0)), "[3]") in d["metadata"]
    assert np.array_equal(d["dofsites"]["m_Py"], np.arange(4))
    assert np.array_equal(d["mesh"].simplices, sim.mesh.simplices)
    sim.clock.step = 7
    sim.save_data(fields=["m"])
    t = h5data.read(str(tmp_path / "hyst_dat.h5"))["tables"]
    assert list(t["m"]["step"]) == [0, 7] and len(t["H_demag"]) == 1
    assert np.allclose(t["m"]["m_Py"][1], sim.get_subfield("m_Py"))
    with pytest.raises(KeyError):
        sim.save_data(fields=["B_field"])
    assert sim.get_restart_file_name() == "hyst_restart.h5"
    # the module-level read-out of saved fields (main.py:2915-3015)
    fn = str(tmp_path / "hyst_dat.h5")
    assert np.allclose(nmag.get_subfield_from_h5file(fn, "m_Py", row=1), sim.get_subfield("m_Py"), atol=1e-7)
    assert np.allclose(nmag.get_subfield_from_h5file(fn, "H_demag"), 0.1e6)
    id1 = int(t["m"]["id"][1])
    assert np.allclose(nmag.get_subfield_from_h5file(fn, "m_Py", id=id1),
                       nmag.get_subfield_from_h5file(fn, "m_Py", row=1))
    assert np.array_equal(nmag.get_subfield_sites_from_h5file(fn, "m_Py"), np.arange(4).reshape(-1, 1))
    assert np.allclose(nmag.get_subfield_positions_from_h5file(fn, "m_Py"), sim.mesh.points * 1e-9)
    with pytest.raises(KeyError):
        nmag.get_subfield_from_h5file(fn, "B_Py")


def test_restart_file_round_trip(tmp_path, monkeypatch):
    """save_restart_file / load_restart_file (main.py:2764-2883): m and the
    clock come back; a stage saved at convergence continues with the next
    stage; load_m_from_h5file reads the first row of /data/fields/m."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    m0 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [0.6, 0.8, 0.0]])
    sim.set_m(m0)
    sim.clock.step, sim.clock.stage, sim.clock.convergence = 42, 3, True
    sim.save_restart_file()
    assert (tmp_path / "hyst_restart.h5").exists() and not (tmp_path / "hyst_restart.h5.internal").exists()
    sim.set_m([0.0, 0.0, 1.0])
    sim.clock.step, sim.clock.stage, sim.clock.convergence = 0, 1, False
    sim.load_restart_file()
    assert np.allclose(sim.get_subfield("m_Py"), m0, atol=1e-7)   # stored as FP32
    assert sim.clock.step == 42 and sim.clock.stage == 4
    sim.set_m([0.0, 0.0, 1.0])
    sim.load_m_from_h5file(str(tmp_path / "hyst_restart.h5"))
    assert np.allclose(sim.get_subfield("m"), m0, atol=1e-7)
    sim.set_m([0.0, 0.0, 1.0])
    sim.load_restart_file(file_name=str(tmp_path / "hyst_restart.h5"))   # the reference's argument name
    assert np.allclose(sim.get_subfield("m"), m0, atol=1e-7)


def test_load_m_from_h5file_selects_a_row(tmp_path, monkeypatch):
    """load_m_from_h5file(filename, id=..., row=...): the row with that id,
    else the row-th row, else the first (hdf5_v01.py:1625-1679)."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    states = [np.tile(v, (4, 1)) for v in ([1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0])]
    for m in states:
        sim.set_m(m)
        sim.save_data(fields=["m"])
    fn = str(tmp_path / "hyst_dat.h5")
    ids = list(nmag.h5data.read(fn)["tables"]["m"]["id"])
    assert len(ids) == 3
    for k, m in enumerate(states):
        sim.set_m([0.6, 0.8, 0.0])
        sim.load_m_from_h5file(fn, row=k)
        assert np.allclose(sim.get_subfield("m"), m, atol=1e-7)
        sim.set_m([0.6, 0.8, 0.0])
        sim.load_m_from_h5file(fn, id=int(ids[k]))
        assert np.allclose(sim.get_subfield("m"), m, atol=1e-7)
    sim.load_m_from_h5file(fn)
    assert np.allclose(sim.get_subfield("m"), states[0], atol=1e-7)
    with pytest.raises(KeyError):
        sim.load_m_from_h5file(fn, id=12345)


def test_current_density_needs_a_polarisation(tmp_path, monkeypatch):
    sim, eng = make_sim(tmp_path, monkeypatch)
    with pytest.raises(KeyError):
        sim.set_current_density([1e12, 0, 0], unit=SI("A/m^2"))


def test_progress_file(tmp_path, monkeypatch):
    """hysteresis.py:25-40: <name>_progress.txt with the clock and the
    convergence state, at most every progress_message_minimum_delay seconds."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    sim.hysteresis([[0, 0, 0.1]], save=[], progress_message_minimum_delay=0)
    text = (tmp_path / "hyst_progress.txt").read_text()
    assert "stage_step" in text and "max_dm_dt" in text
    step_line = [l for l in text.splitlines() if l.startswith("step ")][0]
    assert int(step_line.split()[1]) == sim.clock.step


def test_load_m_from_a_whole_mesh_file(tmp_path, monkeypatch):
    """A data file of the whole mesh (vacuum nodes included, as the reference
    writes it) places m by the node numbers of the mesh as loaded: node k of
    the magnetic part is node node_map[k] of the file's mesh."""
    from nmag import h5data
    sim, eng = make_sim(tmp_path, monkeypatch)
    sim.node_map = np.array([1, 2, 4, 5])
    whole = nmag.mesh.Mesh(np.random.default_rng(0).standard_normal((6, 3)), [[0, 1, 2, 3], [2, 3, 4, 5]])
    file_nodes = np.array([5, 4, 2, 1])
    vals = np.array([[0.0, 0.0, 1.0], [0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.6, 0.0, 0.8]])
    row = {"id": 0, "stage": 1, "step": 3, "time": 0.0, "data": {"m_Py": vals}}
    h5data.write(str(tmp_path / "whole.h5"), whole, [("m", "m_Py", "SI(1.0, '')", "[3]")],
                 {"m_Py": file_nodes}, {"m": h5data.field_rows([("m_Py", None)], [row])})
    sim.load_m_from_h5file(str(tmp_path / "whole.h5"))
    want = {int(n): v for n, v in zip(file_nodes, vals)}
    got = sim.get_subfield("m_Py")
    for k, n in enumerate(sim.node_map):
        assert np.allclose(got[k], want[int(n)], atol=1e-7)


def test_reinitialise_tolerances_and_retired_methods(tmp_path, monkeypatch):
    """reinitialise(rel_tolerance, abs_tolerance, initial_time) as
    main.py:2707-2731; region_volume and save_fields refuse as the
    reference's retired methods do (main.py:2105-2107,2637-2639)."""
    sim, eng = make_sim(tmp_path, monkeypatch)
    seen = []
    eng.ts_init = lambda t0, rtol, atol, q, k: seen.append((t0, rtol, atol))
    sim.reinitialise(rel_tolerance=1e-8, abs_tolerance=1e-7, initial_time=0)
    assert seen[-1] == (0.0, 1e-8, 1e-7)
    sim.reinitialise()
    assert seen[-1][1:] == (1e-8, 1e-7)
    sim.reinitialise(initial_time=SI(2e-12, "s"))
    assert abs(seen[-1][0] - 2.0) < 1e-12 and abs(sim.clock.stage_time_su - 2.0) < 1e-12
    with pytest.raises(NotImplementedError):
        sim.region_volume("Py")
    with pytest.raises(RuntimeError):
        sim.save_fields()
    assert sim.get_subfield_average_siv(field_name="m") == sim.get_subfield_average_siv("m")
