"""nmag.Simulation on libnmaggpu: the drop-in for the LLG path of
interface/nmag/main.py (Simulation, main.py:776-2883), simulation_core.py
(relax/hysteresis entry points, :276-278), hysteresis.py (:207-557) and
convergence.py (:54-100).

State lives on the GPU in one ``nmg_handle``; the host keeps the "master
buffer" copy of m that the reference keeps (main.py:550-705): every
``advance_time`` copies m back once, exactly like the reference's
``_to_mbuf_copier("m")`` (main.py:1383), and computes max|dm| from it.
"""
from __future__ import annotations

import logging
import math
import os
import re
import time as _time

import numpy as np

from . import h5data as _h5data
from . import mesh as _mesh
from . import sites as _sites
from . import si as _si
from ._lib import Engine, Material, Options, NmagGpuError
from .material import MagMaterial
from .when import at, every, never
from .si import SI, simulation_units

log = logging.getLogger("nmag")

# SI units of the fields as the reference converts them (main.py:208-231),
# including its unit for dm/dt, SI("A/m s")
_FIELD_SI = {"H": SI(1.0, "A/m"), "E": SI(1.0, "J/m^3"), "phi": SI(1.0, "A"), "rho": SI(1.0, "A/m^2"),
             "dmdt": SI(1.0, "A/m s"), "J": SI(1.0, "A/m^2"), "M": SI(1.0, "A/m"), "m": SI(1.0, ""),
             "pin": SI(1.0, "")}
# averages written to the .ndt file (main.py:2313-2480): per material (the
# fields_on_space of main.py:202-204) and over the mesh (fields_on_materials)
_NDT_PER_MATERIAL = [("m", "m"), ("M", "M"), ("H_total", "H"), ("H_exch", "H"), ("H_anis", "H"), ("dmdt", "dmdt"),
                     ("E_total", "E"), ("E_exch", "E"), ("E_anis", "E"), ("E_demag", "E"), ("E_ext", "E")]
_NDT_MESH = [("H_demag", "H"), ("H_ext", "H"), ("phi", "phi"), ("rho", "rho"), ("pin", "pin")]
_NDT_HEADERS_DONE = set()


def _su_factor(kind):
    return 1.0 / simulation_units.of(_FIELD_SI[kind])


class Clock(dict):
    """Simulation clock (interface/nmag/clock.py): ids, steps, stage data."""

    def __init__(self):
        super().__init__(id=-1, stage=1, step=0, time_su=0.0, stage_step=0, stage_time_su=0.0,
                         real_time=0.0, stage_end=False, convergence=False, exit_hysteresis=False,
                         last_step_dt_su=0.0, time_reached_su=0.0, zero_stage_step=0, zero_stage_time_su=0.0)

    def view(self):
        """The counters the save / do schedules read (times in simulation
        units, real time in seconds)."""
        return {"step": self.step, "stage_step": self.stage_step, "time": self.time_su,
                "stage_time": self.stage_time_su, "real_time": self.real_time, "stage": self.stage,
                "convergence": bool(self.convergence), "stage_end": bool(self.stage_end),
                "zero_stage_step": self.zero_stage_step, "zero_stage_time": self.zero_stage_time_su}

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError:
            raise AttributeError(k)

    def __setattr__(self, k, v):
        self[k] = v


_SPACES = re.compile(r"[ \t]+")


def _normalise_action(name):
    """hysteresis.py:42-54: 'Save  Fields' -> 'save_fields'."""
    return _SPACES.sub("_", name.lower())


def _next_deltas(event, view, suggest=None, tols=None):
    """hysteresis.py:132-159: (steps, simulation time, real time) to the next
    firing of event, each None when it does not constrain that counter; the
    minimum with ``suggest``."""
    def delta(name):
        n = event.next_time(name, view, tols=tols)
        return None if isinstance(n, bool) else n - view[name]

    def least(vals):
        vals = [v for v in vals if v is not None]
        return min(vals) if vals else None
    ds, dt, dr = suggest if suggest is not None else (None, None, None)
    return (least([delta("step"), delta("stage_step"), ds]), least([delta("time"), delta("stage_time"), dt]),
            least([delta("real_time"), dr]))


def _next_time(event, view, tols=None):
    """hysteresis.py:161-198: (step, time, real time) of the next firing,
    counted from the start of the stage."""
    def at_(name, zero=None):
        n = event.next_time(name, view, tols=tols)
        if isinstance(n, bool):
            return None
        return n - view[zero] if zero else n

    def least(vals):
        vals = [v for v in vals if v is not None]
        return min(vals) if vals else None
    return (least([at_("step", "zero_stage_step"), at_("stage_step")]),
            least([at_("time", "zero_stage_time"), at_("stage_time")]), at_("real_time"))


# Newton-matrix Jacobians of the BDF timestepper, by level
JACOBIAN_LEVELS = ("approximate", "local", "exact")


class Simulation(object):
    """Micromagnetic simulation (main.py:776-845 constructor arguments)."""

    def __init__(self, name=None, phi_BEM=None, periodic_bc=None, do_demag=True, do_anisotropy_jacobian=False,
                 temperature=None, thermal_delta_t=None, user_seed_T=0, timestepper_max_order=2,
                 timestepper_krylov_max=300, ksp_tolerances=None, adjust_tolerances=False, use_pvode=True,
                 lam_debugfile=None, quirks="nmag", bem_precision="fp64", n_members=1, cg_precision="fp64",
                 bem_anchor=0.0, adjoint_cg_precision="fp64", anchor_product="fp32", cg_local_sweeps=0,
                 jacobian="approximate", jacobian_demag_rtol=1e-3, jv_precision="fp64", cg_coarse=True):
        if periodic_bc is not None:
            raise NotImplementedError("periodic boundary conditions are outside this path")
        if temperature is not None:
            raise NotImplementedError("thermal (Heun) integration is disabled in the reference (main.py:797-806)")
        # kept for the API: in the reference this flag only extends the
        # jacobian plan (nmag_lam.py:665-679), and jacobian plans are never
        # built ("old relic", nsim.ml:3266) -- the timestepper's Jacobian takes
        # its derivatives from phys_field_derivs, which ignore H_anis
        # (nmag_lam.py:689-693) -- so it changes no result
        self._do_anisotropy_jacobian = bool(do_anisotropy_jacobian)
        self.name = name or "nmag"
        self._do_demag = bool(do_demag)
        self.max_order = int(timestepper_max_order)
        self.krylov_max = int(timestepper_krylov_max)
        self.ksp_tolerances = dict(ksp_tolerances or {})
        self.quirks = quirks
        self.bem_precision = bem_precision
        # "fp32": the Poisson CG iterates in FP32 with FP64 residual refinement
        self.cg_precision = cg_precision
        # fp32x2 only: > 0 forms B x as B x0 + B32 (x - x0) while x stays within
        # this relative max-norm distance of the last compensated product's x0
        self.bem_anchor = float(bem_anchor)
        # ensemble anchored product's difference B (x - x0): "fp32" or "fp16"
        # (FP16 copy of B in tensor-core fragment order, FP32 accumulation)
        self.anchor_product = anchor_product
        # Poisson solves of the RK4 adjoint's backward pass ("fp32": FP32 CG
        # iterations with FP64 residual refinement to the same tolerance)
        self.adjoint_cg_precision = adjoint_cg_precision
        # FP32 inner CG: damped Jacobi sweeps on each thread block's own rows
        # in its preconditioner (0 or 1: Jacobi alone)
        self.cg_local_sweeps = int(cg_local_sweeps)
        # the BDF's Newton matrix: "approximate" (the reference's: exchange
        # only), "local" (+ anisotropy, C3 length term, local couplings) or
        # "exact" (+ the demag response, Poisson solves at jacobian_demag_rtol)
        if jacobian not in JACOBIAN_LEVELS:
            raise ValueError("jacobian must be one of %s" % ", ".join(JACOBIAN_LEVELS))
        self.jacobian = jacobian
        self.jacobian_demag_rtol = float(jacobian_demag_rtol)
        if not 0.0 < self.jacobian_demag_rtol < 1.0:
            raise ValueError("jacobian_demag_rtol must be in (0, 1)")
        # the approximate Jacobian's products and block preconditioner in FP32
        # arithmetic ("fp32") or FP64; the Newton residual stays FP64
        if jv_precision not in ("fp64", "fp32"):
            raise ValueError("jv_precision must be 'fp64' or 'fp32'")
        self.jv_precision = jv_precision
        # the Neumann CG's aggregation coarse level (False: Jacobi alone)
        self.cg_coarse = bool(cg_coarse)
        # several magnetic materials: the site layout (None: one material)
        self.layer = None
        self.materials = []
        # ensemble: n_members simulations on one mesh, integrated together;
        # per-node arrays then carry a leading member axis (GB300 extension)
        self.n_members = max(1, int(n_members))
        self.ts_rel_tol = 1e-6
        self.ts_abs_tol = 1e-6
        self.stopping_dm_dt = simulation_units.of(_si.degrees_per_ns)   # 1 deg/ns
        self._default_exact_tstop = True
        self.max_time_reached = simulation_units.of(SI(1.0, "s"))
        self.clock = Clock()
        self.max_dm_dt = None
        self._countdown_initial = 2
        self._countdown = 2
        self.engine = None
        self._timers = {}
        self.mesh = None
        self.node_map = None    # magnetic nodes -> nodes of the loaded mesh (vacuum present)
        self.material = None
        self._m = None          # host master buffer of m (N,3)
        self._h_ext = None
        self._ts_ready = False
        self._last_nst = 0
        self.last_stats = {}

    # ---- setup -----------------------------------------------------------
    def load_mesh(self, filename, region_names_and_mag_mats, unit_length, do_reorder=False, manual_distribution=None):
        """main.py:1075.  ``filename`` is an nmesh ASCII file or a ``nmag.mesh.Mesh``."""
        m = _mesh.load(filename)
        # region ids 1, 2, ... name the listed regions in order; 0 is vacuum
        mats = []
        for entry in region_names_and_mag_mats:
            region_name, mat = entry
            mats.extend(mat if isinstance(mat, (list, tuple)) else [mat])
        if not mats:
            raise ValueError("load_mesh: no magnetic material given")
        # distinct materials in order of appearance; several (or a region with
        # several) give every material its own m on its sites
        self.materials = []
        for mt in mats:
            if all(mt is not x for x in self.materials):
                self.materials.append(mt)
        c0 = mats[0].coefficients(self.quirks)
        several_in_a_region = any(isinstance(e[1], (list, tuple)) and len(e[1]) > 1 for e in region_names_and_mag_mats)
        self._multi = several_in_a_region or any(mt.coefficients(self.quirks) != c0 for mt in mats[1:])
        if not self._multi:
            self.materials = [mats[0]]
        nreg = int(m.regions.max()) if len(m.regions) else 0
        if nreg != len(region_names_and_mag_mats):   # main.py:1174-1180
            raise ValueError("Found inconsistency between the mesh you loaded and the provided list of "
                             "(region_name, materials). The mesh has %d regions but the provided list has "
                             "%d pairs." % (nreg, len(region_names_and_mag_mats)))
        # vacuum simplices carry no magnetisation; the magnetic part alone is
        # simulated (its open-boundary potential comes from the BEM), and
        # per-site arrays refer to its nodes, as nmag's m subfields do
        self.node_map = None
        if np.any(m.regions <= 0):
            m, self.node_map = _mesh.magnetic_part(m)
        self.material = mats[0]
        # regions of each material name (main.py:1182-1191: region ids 1, 2, ...)
        self._regions_by_material = {}
        for rid, (region_name, mat) in enumerate(region_names_and_mag_mats, start=1):
            for mt in (mat if isinstance(mat, (list, tuple)) else [mat]):
                self._regions_by_material.setdefault(mt.name, []).append(rid)
        scale = simulation_units.of(unit_length, compatible_with=SI("m"))
        self.mesh = _mesh.Mesh(m.points * scale, m.simplices, m.regions)
        opts = Options()
        opts.do_demag = int(self._do_demag)

        def tol(key, default):
            v = self.ksp_tolerances.get(key)
            return default if v is None else v
        opts.nbc_rtol, opts.nbc_atol, opts.nbc_maxits = tol("NBC.rtol", 1e-5), tol("NBC.atol", 1e-50), int(tol("NBC.maxits", 10000))
        opts.dbc_rtol, opts.dbc_atol, opts.dbc_maxits = tol("DBC.rtol", 1e-5), tol("DBC.atol", 1e-50), int(tol("DBC.maxits", 10000))
        # fp32: FP32 matrix; fp32x2: FP32 + BF16 residual matrix with compensated FP32 products;
        # bf16x3: three BF16 planes of matrix and vectors, six tensor-core products per term
        opts.bem_precision = {"fp64": 0, "fp32": 1, "fp32x2": 2, "bf16x3": 3}[self.bem_precision]
        opts.cg_precision = {"fp64": 0, "fp32": 1}[self.cg_precision]
        opts.n_members = self.n_members if self.n_members > 1 else 0
        opts.bem_anchor_tol = self.bem_anchor
        opts.adjoint_cg_precision = {"fp64": 0, "fp32": 1}[self.adjoint_cg_precision]
        opts.anchor_product = {"fp32": 0, "fp16": 1}[self.anchor_product]
        opts.cg_local_sweeps = self.cg_local_sweeps
        opts.jv_precision = {"fp64": 0, "fp32": 1}[self.jv_precision]
        opts.cg_no_coarse = 0 if self.cg_coarse else 1
        self.layer = None
        if self._multi:
            names = [mt.name for mt in self.materials]
            per_region = [[mt.name for mt in (mat if isinstance(mat, (list, tuple)) else [mat])]
                          for _, mat in region_names_and_mag_mats]
            for mt in self.materials:
                if mt.anisotropy_polynomial(self.quirks) is not None or mt.su_llg_stt_prefactor != 0.0:
                    raise NotImplementedError("several materials: polynomial anisotropies and spin-transfer "
                                              "torque are not available (material '%s')" % mt.name)
            self.layer = _sites.SiteLayer(self.mesh, per_region)
            self.engine = Engine.materials(self.mesh.points, self.mesh.simplices, self.mesh.regions,
                                           [[names.index(n) for n in r] for r in per_region],
                                           [self._material_struct(mt) for mt in self.materials], opts)
            self.engine.set_jacobian(JACOBIAN_LEVELS.index(self.jacobian), self.jacobian_demag_rtol)
            self._j = None
            shape = self.engine._shape3()
            self._m = np.zeros(shape)
            self.engine.max_dm_step()
            self._h_ext = np.zeros(shape)
            self._ts_ready = False
            return self.mesh
        self.engine = Engine(self.mesh.points, self.mesh.simplices, self._material_struct(), opts)
        self.engine.set_jacobian(JACOBIAN_LEVELS.index(self.jacobian), self.jacobian_demag_rtol)
        poly = self.material.anisotropy_polynomial(self.quirks)
        if poly is not None:
            self.engine.set_anisotropy_poly(*poly)
        self._j = None
        if self.material.su_llg_stt_prefactor != 0.0:   # llg_polarisation given: J starts at zero
            c = self.material.coefficients(self.quirks)
            self.engine.set_stt(c["C4"], c["C5"])
            self._j = np.zeros(self.engine._shape3())
        shape = self.engine._shape3()
        self._m = np.zeros(shape)
        self.engine.max_dm_step()   # the device's reference m for the first convergence check
        self._h_ext = np.zeros(shape)
        self._ts_ready = False
        return self.mesh

    def _material_struct(self, material=None):
        c = (material or self.material).coefficients(self.quirks)
        mt = Material()
        mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = c["Ms"], c["exch_coeff"], c["C1"], c["C2"], c["C3"]
        mt.K1 = c["K1"]
        for d in range(3):
            mt.axis[d] = c["axis"][d]
        mt.anis_coeff, mt.E_coeff_half, mt.E_coeff_ext = c["anis_coeff"], c["E_coeff_half"], c["E_coeff_ext"]
        return mt

    def set_local_magnetic_coupling(self, mat1, mat2, coupling):
        """main.py:1234-1263: couple the magnetisations of two materials
        whose sites share nodes (two species in one crystal).  coupling: an
        SI value in units of mu0 (or a pair, one per direction); H_lc of mat1
        gains (coupling/mu0) Ms_2 m_2, its energy density
        (coupling/mu0) (mu0 Ms_1 Ms_2 / 2) m_1 . m_2, and the other way round."""
        if self.layer is None:
            raise KeyError("set_local_magnetic_coupling: the simulation has one material")
        names = [mt.name for mt in self.materials]
        if mat1.name not in names or mat2.name not in names or mat1.name == mat2.name:
            raise ValueError("set_local_magnetic_coupling: two different materials of the simulation")
        done = getattr(self, "_couplings", set())
        if (mat1.name, mat2.name) in done or (mat2.name, mat1.name) in done:
            raise ValueError("A coupling %s-%s has been already specified!" % (mat1.name, mat2.name))
        pair = coupling if isinstance(coupling, (list, tuple)) else (coupling, coupling)
        c1, c2 = (float((x / _si.mu0).value) if isinstance(x, SI) else float(x) for x in pair)
        en_dens = simulation_units.of(0.5 * _si.mu0 * mat1.Ms * mat2.Ms, compatible_with=SI("J/m^3"))
        Ms1 = simulation_units.of(mat1.Ms, compatible_with=SI("A/m"))
        Ms2 = simulation_units.of(mat2.Ms, compatible_with=SI("A/m"))
        k1, k2 = names.index(mat1.name), names.index(mat2.name)
        self.engine.set_local_coupling(k1, k2, c1 * Ms2, en_dens * c1)
        self.engine.set_local_coupling(k2, k1, c2 * Ms1, en_dens * c2)
        done.add((mat1.name, mat2.name))
        self._couplings = done
        self._ts_ready = False

    def set_damping(self, llg_damping):
        """Change the material's damping (e.g. between relax and dynamics);
        with several materials, every material's."""
        if self.layer is not None:
            for k, mt in enumerate(self.materials):
                mt.set_damping(llg_damping)
                self.engine.set_site_material(k, self._material_struct(mt))
            self._ts_ready = False
            return
        self.material.set_damping(llg_damping)
        self.engine.set_material(self._material_struct())
        self._ts_ready = False

    def _positions_si(self):
        """Positions (m) of the sites: the mesh nodes, or with several
        materials every material's nodes in site order."""
        pts = self.mesh.points if self.layer is None else self.mesh.points[self.layer.site_node]
        return pts * simulation_units.conversion_factor_of(SI("m"))

    def _material_of(self, subfieldname, field):
        """With several materials: the material named by '<field>_<name>'
        (None for the bare field name, i.e. every material)."""
        if self.layer is None or subfieldname in (None, field):
            return None
        name = subfieldname[len(field) + 1:]
        for mt in self.materials:
            if mt.name == name:
                return mt
        raise KeyError("Couldn't find field for subfieldname '%s'" % subfieldname)

    def _sites_of(self, material):
        return self.layer.sites_of(material.name)

    def _vector_values(self, values):
        B = self.n_members
        if B > 1:
            if isinstance(values, (list, tuple)) and len(values) == B and not (
                    B == 3 and all(np.isscalar(v) or isinstance(v, SI) for v in values)):
                return np.stack([self._one_vector_values(v) for v in values])
            arr = None if callable(values) else np.asarray(values, dtype=np.float64)
            if arr is not None and arr.shape == (B, self.engine.N, 3):
                return arr.copy()
            one = self._one_vector_values(values)
            return np.broadcast_to(one, (B,) + one.shape).copy()
        return self._one_vector_values(values)

    def _one_vector_values(self, values):
        N = self.engine.N
        if callable(values):
            pos = self._positions_si()
            return np.array([values(p) for p in pos], dtype=np.float64).reshape(N, 3)
        arr = np.asarray(values, dtype=np.float64)
        if arr.shape == (3,):
            return np.broadcast_to(arr, (N, 3)).copy()
        return arr.reshape(N, 3).copy()

    def set_m(self, values, subfieldname=None):
        """main.py:1787: set m (auto-normalised); subfieldname 'm_<material>'
        or None (every material)."""
        if subfieldname is not None and self._field_of(subfieldname) != "m":
            raise KeyError("set_m: '%s' is not a magnetisation subfield" % subfieldname)
        m = self._vector_values(values)
        n = np.linalg.norm(m, axis=-1)
        if np.any(n == 0.0):
            raise ValueError("set_m: zero-length magnetisation vector")
        m = m / n[..., None]
        mat = self._material_of(subfieldname, "m") if subfieldname is not None else None
        if mat is not None:   # only that material's sites change
            s_ = self._sites_of(mat)
            full = np.array(self._m, copy=True)
            full[..., s_, :] = m[..., s_, :]
            m = full
        self._m = m
        self.engine.set_m(m)
        self._ts_ready = False

    def set_H_ext(self, values, unit=None):
        """main.py:1726-1785: values times unit (SI, compatible with A/m), or
        SI values; plain numbers without a unit are dimensionless, i.e.
        simulation units (map_terminals.SI_vector takes SI(""))."""
        if unit is None:
            if isinstance(values, (list, tuple)) and values and isinstance(values[0], SI):
                h = self._vector_values([simulation_units.of(v, compatible_with=SI("A/m")) for v in values])
            else:
                h = self._vector_values(values)
        else:
            h = self._vector_values(values) * simulation_units.of(unit, compatible_with=SI("A/m"))
        self._h_ext = h
        self.engine.set_h_ext(h)
        self._ts_ready = False

    def set_pinning(self, values):
        """main.py:1918-1935: the pinning factor of dm/dt per site (1 free,
        0 fixed): a number, a function of the position (SI) or N values.
        Shared by the members of an ensemble."""
        N = self.engine.N
        if callable(values):
            p = np.array([float(values(x)) for x in self._positions_si()], dtype=np.float64)
        else:
            p = np.broadcast_to(np.asarray(values, dtype=np.float64), (N,)).copy()
        self._pin = p
        self.engine.set_pinning(None if np.all(p == 1.0) else p)
        self._ts_ready = False

    def set_current_density(self, values, unit=None):
        """main.py:1934-1960: the current density of the spin-transfer
        torque, values times unit (SI, compatible with A/m^2), SI values, or
        plain numbers in simulation units.  The field exists only when the
        material has a spin polarisation (nmag_lam.py:195-202; main.py:570)."""
        if self.material is None or self.material.su_llg_stt_prefactor == 0.0:
            raise KeyError("set_current_density: no 'current_density' field (the material has no "
                           "llg_polarisation)")
        if unit is None:   # SI values, or plain numbers in simulation units (as set_H_ext)
            if isinstance(values, (list, tuple)) and values and isinstance(values[0], SI):
                j = self._vector_values([simulation_units.of(v, compatible_with=SI("A/m^2")) for v in values])
            else:
                j = self._vector_values(values)
        else:
            j = self._vector_values(values) * simulation_units.of(unit, compatible_with=SI("A/m^2"))
        self._j = j
        self.engine.set_current_density(j)
        self._ts_ready = False

    def set_params(self, stopping_dm_dt=None, ts_rel_tol=None, ts_abs_tol=None, exact_tstop=None):
        """main.py:1048-1073."""
        if stopping_dm_dt is not None:
            self.stopping_dm_dt = simulation_units.of(stopping_dm_dt, compatible_with=SI("1/s"))
        if ts_rel_tol is not None:
            self.ts_rel_tol = float(ts_rel_tol)
            self._ts_ready = False
        if ts_abs_tol is not None:
            self.ts_abs_tol = float(ts_abs_tol)
            self._ts_ready = False
        if exact_tstop is not None:
            self._default_exact_tstop = bool(exact_tstop)

    def reinitialise(self, rel_tolerance=None, abs_tolerance=None, initial_time=None):
        """main.py:2707-2731: (re)create the integrator at the current state,
        from initial_time (SI, or simulation units) when given, with new
        relative / absolute tolerances when given."""
        if rel_tolerance is not None:
            self.ts_rel_tol = float(rel_tolerance)
        if abs_tolerance is not None:
            self.ts_abs_tol = float(abs_tolerance)
        if initial_time is not None:
            t0 = (simulation_units.of(initial_time, compatible_with=SI("s")) if isinstance(initial_time, SI)
                  else float(initial_time))
            self.clock.stage_time_su = t0
            self.clock.stage_step = 0
        else:
            t0 = self.clock.stage_time_su
        self.engine.ts_init(t0, self.ts_rel_tol, self.ts_abs_tol, self.max_order, self.krylov_max)
        self._ts_t0 = t0
        self._last_nst = 0
        self._ts_ready = True

    # ---- dynamics ----------------------------------------------------------
    def advance_time(self, target_time, max_it=-1, exact_tstop=None):
        """main.py:1325-1460: integrate to target_time (SI), or max_it steps."""
        if max_it is None or max_it < 0:
            max_it = -1
        if exact_tstop is None:
            exact_tstop = self._default_exact_tstop
        target_su = simulation_units.of(target_time, compatible_with=SI("s")) if isinstance(target_time, SI) else float(target_time)
        if not self._ts_ready:
            self.reinitialise()
        if target_su == 0:
            return target_time
        prev_m = self._m
        wall0 = _time.time()
        t_stage, stats = self.engine.ts_advance(target_su, exact_tstop, max_it)
        self.clock.real_time += _time.time() - wall0   # clock.py: real time spent advancing
        self._timers["advance_time"] = self._timers.get("advance_time", 0.0) + self.engine.timings()[0] * 1e-3
        self._m = self.engine.get_m()
        delta_steps = stats["nst"] - self._last_nst
        self._last_nst = stats["nst"]
        delta_t = t_stage - self.clock.stage_time_su
        self.clock.stage_time_su = t_stage
        self.clock.time_su += delta_t
        self.clock.time_reached_su = self.clock.time_su
        self.clock.step += max(delta_steps, 0)
        self.clock.stage_step += max(delta_steps, 0)
        self.clock.last_step_dt_su = stats["hcur"]
        self.last_stats = stats
        # max |m - m before this advance| (the device remembers m at each
        # set_m and each advance), as the reference's mwe_norm_dist_fun
        dm = self.engine.max_dm_step()
        if prev_m is not None and delta_t > 0.0:
            self.max_dm_dt = dm / delta_t
        return SI(t_stage * simulation_units.conversion_factor_of(SI("s")), "s")

    def is_converged(self):
        """convergence.py:54-100 / main.py:2737-2760: max dm/dt below
        stopping_dm_dt twice in a row; sets clock.convergence.  The count of
        checks below the threshold restarts at convergence and at a check
        above it, not at a new stage, and a check with no max dm/dt yet
        (None, after a new stage) leaves it unchanged.  (The reference's
        tolerance-factor suggestions only act with adjust_tolerances=True, a
        debugging path that waits for console input; they are not made.)"""
        self.clock.convergence = False
        if self.max_dm_dt is None:
            return False
        if self.max_dm_dt < self.stopping_dm_dt:
            self._countdown -= 1
            if self._countdown < 1:
                self._countdown = self._countdown_initial
                self.clock.convergence = True
                return True
            return False
        self._countdown = self._countdown_initial
        return False

    # predefined things to save / do (simulation_core.py:180-200,256-271)
    @staticmethod
    def hysteresis_next_stage(sim):
        """End the current stage (the 'next_stage' action)."""
        sim.clock.stage_end = True

    @staticmethod
    def hysteresis_exit(sim):
        """Leave the hysteresis loop (the 'exit' action)."""
        sim.clock.exit_hysteresis = True
        sim.clock.stage_end = True

    _ACTIONS = {"save_averages": lambda sim: sim.save_data(avoid_same_step=True),
                "save_fields": lambda sim: sim.save_data(fields="all", avoid_same_step=True),
                "save_field_m": lambda sim: sim.save_data(fields=["m"], avoid_same_step=True),
                "save_restart": lambda sim: sim.save_restart_file(),
                "do_next_stage": lambda sim: Simulation.hysteresis_next_stage(sim),
                "do_exit": lambda sim: Simulation.hysteresis_exit(sim)}

    def _join_save_and_do(self, save, do):
        """hysteresis.py:56-130: (function, when, key) for every thing of the
        (thing, ..., when) tuples, the do list first; strings name the
        predefined actions ('averages', 'save fields', 'next_stage', ...)."""
        joint, keys = [], set()
        for prefix, items in (("do", do), ("save", save)):
            try:
                items = [list(t) for t in items]
            except TypeError:
                raise ValueError("hysteresis: '%s' must be a list of (thing, ..., when) tuples" % prefix)
            for item in items:
                if len(item) < 2:
                    raise ValueError("hysteresis: '%s' must be a list of (thing, ..., when) tuples" % prefix)
                when = item[-1]
                for thing in item[:-1]:
                    if callable(thing):
                        fn, key = thing, ("fn", id(thing))
                    elif isinstance(thing, str):
                        name = _normalise_action(prefix + " " + thing)
                        if name not in self._ACTIONS:
                            name = _normalise_action(thing)
                        if name not in self._ACTIONS:
                            raise ValueError("hysteresis: you want to %s '%s' but I don't know how to do it; "
                                             "available: %s" % (prefix, thing, ", ".join(sorted(self._ACTIONS))))
                        fn, key = self._ACTIONS[name], name
                    else:
                        raise ValueError("hysteresis: things to %s are strings or functions, not %r" % (prefix, thing))
                    if key in keys:
                        raise ValueError("hysteresis: %s is given twice in 'save' / 'do'; combine the schedules "
                                         "with | instead" % (thing,))
                    keys.add(key)
                    joint.append((fn, when, key))
        return joint

    def _update_progress_file(self, H, filename, min_delay):
        """hysteresis.py:25-40: at most every min_delay seconds, the time, the
        clock and the convergence state into <name>_progress.txt, and a log
        line."""
        now = _time.time()
        if now - getattr(self, "_progress_t", -1e300) < min_delay:
            return
        self._progress_t = now
        with open(filename, "w") as f:
            f.write(_time.asctime() + "\n")
            for k in ("id", "stage", "step", "stage_step", "time_su", "stage_time_su", "real_time",
                      "last_step_dt_su", "convergence", "stage_end"):
                f.write("%-16s %s\n" % (k, self.clock[k]))
            f.write("max_dm_dt %s (stop below %s, simulation units)\n" % (self.max_dm_dt, self.stopping_dm_dt))
        Hs = "None" if H is None else _si.str_of_SI_vector(
            H if isinstance(H, (list, tuple)) and H and isinstance(H[0], SI) else list(np.ravel(H))[:3])
        log.info("it %d, time %g s; stage %d; H_ext=%s" % (self.clock.step, self.clock.time_su * 1e-12,
                                                          self.clock.stage, Hs))

    def hysteresis(self, H_ext_list, save=(("averages", "fields", at("stage_end")),), do=(),
                   convergence_check=every("step", 5), progress_message_minimum_delay=60):
        """hysteresis.py:244-557: for each applied field (None keeps the
        current one) start a stage and integrate until converged, running
        the save / do actions whenever their schedules fire."""
        actions = self._join_save_and_do(save, do)
        tol_time = simulation_units.of(SI(1e-20, "s"))   # hysteresis.py:420-423
        tols = {"time": tol_time, "stage_time": tol_time}
        next_save = {}
        stage = self.clock.stage
        self.clock.exit_hysteresis = False
        for H in list(H_ext_list)[stage - 1:]:
            self.do_next_stage(stage=stage)
            stage = None
            self.clock.stage_end = False
            if H is not None:
                if isinstance(H, tuple) and len(H) == 2 and isinstance(H[1], SI):
                    self.set_H_ext(H[0], H[1])
                else:
                    self.set_H_ext(H)
            self.reinitialise(initial_time=0)   # the convergence countdown carries over, as in the reference
            for _, when, key in actions:
                next_save[key] = _next_time(when, self.clock.view(), tols)
            while True:
                self.clock.stage_end = self.is_converged()
                deltas = _next_deltas(convergence_check, self.clock.view(), tols=tols)
                for fn, when, key in actions:
                    v = self.clock.view()
                    nst = _next_time(when, v, tols)
                    if when.match_time(v) or nst != next_save[key]:
                        fn(self)
                    next_save[key] = nst
                    deltas = _next_deltas(when, self.clock.view(), suggest=deltas, tols=tols)
                d_step, d_time, _ = deltas
                if d_time is None:
                    target, max_it = self.max_time_reached, d_step
                else:
                    target, max_it = self.clock.stage_time_su + d_time, (-1 if d_step is None else d_step)
                if self.clock.exit_hysteresis:
                    return
                if self.clock.stage_end:
                    break
                t = self.advance_time(target, max_it=max_it)
                if simulation_units.of(t, compatible_with=SI("s")) > 0.99 * self.max_time_reached:
                    raise RuntimeError("Simulation time reached %s: are you starting from a zero torque "
                                       "configuration?" % self.max_time_reached)
                try:   # progress reports never stop the loop (hysteresis.py:541-551)
                    self._update_progress_file(H, self.name + "_progress.txt", progress_message_minimum_delay)
                except Exception as exc:
                    log.info("Problem when generating progress file: %s" % exc)

    def relax(self, H_applied=None, save=(("averages", "fields", at("stage_end")),), do=(),
              convergence_check=every("step", 5), progress_message_minimum_delay=60):
        """hysteresis.py:207-242: hysteresis([H_applied])."""
        return self.hysteresis([H_applied], save=save, do=do, convergence_check=convergence_check,
                               progress_message_minimum_delay=progress_message_minimum_delay)

    # ---- read-out ------------------------------------------------------------
    # fields per material (subfields <field>_<material>) and over the mesh
    # (main.py:199-206); the bare field name is accepted for the one material
    _PER_MATERIAL = ("E_total", "E_demag", "E_exch", "E_anis", "E_ext", "H_total", "H_exch", "H_anis", "dmdt",
                     "m", "M")
    _ON_MESH = ("H_demag", "H_ext", "phi", "rho", "pin", "current_density")
    _KIND = {"m": "m", "M": "M", "H_total": "H", "H_exch": "H", "H_anis": "H", "H_demag": "H", "H_ext": "H",
             "dmdt": "dmdt", "E_total": "E", "E_demag": "E", "E_exch": "E", "E_anis": "E", "E_ext": "E",
             "phi": "phi", "rho": "rho", "pin": "pin", "current_density": "J"}

    def _field_of(self, subfieldname):
        """The field of a subfield name; KeyError for names that name no
        subfield of this simulation (main.py:612-628)."""
        if subfieldname in self._ON_MESH:
            return subfieldname
        names = [mt.name for mt in getattr(self, "materials", None) or ([self.material] if self.material else [])]
        for f in self._PER_MATERIAL:
            if subfieldname == f:
                return f
            if subfieldname.startswith(f + "_"):
                if subfieldname[len(f) + 1:] not in names:
                    break
                return f
        raise KeyError("Couldn't find field for subfieldname '%s'" % subfieldname)

    def get_subfield(self, subfieldname, units=None, _snap=None):
        """main.py:1480-1568: field values per site in SI (the reference's unit
        table); m is dimensionless.  (_snap: fields and energy densities of
        one evaluation, for callers reading several subfields.)"""
        field = self._field_of(subfieldname)
        if self.layer is not None:
            return self._get_subfield_sites(subfieldname, field, _snap)
        if field == "m":
            return self._m.copy()
        if field == "M":   # M = Ms m (nmag_lam.py:463)
            return self._m * self.material.coefficients(self.quirks)["Ms"] * _su_factor("M")
        if field == "H_ext":
            return self._h_ext * _su_factor("H")
        if field == "pin":
            p = getattr(self, "_pin", None)
            return p.copy() if p is not None else np.ones(self.engine.N)
        if field == "current_density":
            j = self._j if getattr(self, "_j", None) is not None else np.zeros_like(self._h_ext)
            return j * _su_factor("J")
        if field.startswith("E_"):
            E = _snap["E"] if _snap else self.engine.energy_density()
            return E[field] * _su_factor("E")
        f = _snap["f"] if _snap else self.engine.eval_fields()
        return f[field] * _su_factor(self._KIND[field])

    _VECTOR = ("m", "M", "H_total", "H_exch", "H_anis", "H_demag", "H_ext", "dmdt", "current_density")

    def _get_subfield_sites(self, subfieldname, field, _snap):
        """Several materials: a per-material subfield on its material's sites
        (all sites for the bare name); a mesh field on the mesh nodes (the
        value of each node's first site)."""
        mat = self._material_of(subfieldname, field) if field in self._PER_MATERIAL else None
        if field in ("m", "M"):
            vals = np.array(self._m, copy=True)
            if field == "M":
                ms = np.array([mt.coefficients(self.quirks)["Ms"] for mt in self.materials])[self.layer.site_material]
                vals = vals * ms[:, None] * _su_factor("M")
        elif field == "H_ext":
            vals = self._h_ext * _su_factor("H")
        elif field == "pin":
            p = getattr(self, "_pin", None)
            vals = p.copy() if p is not None else np.ones(self.engine.N)
        elif field == "current_density":   # no spin-transfer torque with several materials: zero
            vals = np.zeros_like(np.asarray(self._h_ext))
        elif field.startswith("E_"):
            E = _snap["E"] if _snap else self.engine.energy_density()
            vals = E[field] * _su_factor("E")
        else:
            f = _snap["f"] if _snap else self.engine.eval_fields()
            vals = f[field] * _su_factor(self._KIND[field])
        axis = -2 if field in self._VECTOR else -1
        if field in self._ON_MESH:   # node values: each node's first site
            return np.take(vals, self.layer.node_site_idx[self.layer.node_site_ptr[:-1]], axis=axis)
        if mat is not None:
            return np.take(vals, self._sites_of(mat), axis=axis)
        return vals

    def _unit_of(self, subfieldname):
        return _FIELD_SI[self._KIND[self._field_of(subfieldname)]]

    def probe_subfield_siv(self, subfieldname, pos, unit=None):
        """main.py:1651-1700: the subfield at a position given in metres
        (floats), linearly interpolated in the simplex containing it; a float
        for scalar subfields, a list for vectors; None outside the magnetic
        mesh."""
        vals = self.get_subfield(subfieldname)
        if vals.ndim == 3:   # an ensemble: member 0, as get_subfield_average_siv
            vals = vals[0]
        pos_su = np.asarray(pos, dtype=np.float64) * simulation_units.of(SI(1.0, "m"))
        v = self.mesh.interpolate(vals, pos_su)
        if v is None:
            return None
        return float(v) if np.ndim(v) == 0 else [float(x) for x in v]

    def probe_subfield(self, subfieldname, pos, unit=None):
        """main.py:1570-1650: as probe_subfield_siv with the position a list of
        SI objects (or an SI vector) and the result SI objects."""
        pos_m = [simulation_units.of(p, compatible_with=SI("m")) * simulation_units.conversion_factor_of(SI("m"))
                 for p in pos]
        data = self.probe_subfield_siv(subfieldname, pos_m)
        if data is None:
            return None
        u = unit if unit is not None else self._unit_of(subfieldname)
        return [x * u for x in data] if isinstance(data, list) else data * u

    def probe_H_demag_siv(self, pos, pos_unit=SI("m"), epsilon=1e-7):
        """main.py:2124-2187: H_demag (A/m) at a position given in units of
        pos_unit.  Inside the magnetic mesh this is the probed H_demag field
        (nsimexec.ml:4248-4285 probes the field first); outside, the
        reference's parallel linalg machine has no potential evaluation
        (nsim.ml:3703, get_potential fails), and neither is there one here."""
        pos_m = np.asarray(pos, dtype=np.float64) * (simulation_units.of(pos_unit, compatible_with=SI("m"))
                                                     * simulation_units.conversion_factor_of(SI("m")))
        v = self.probe_subfield_siv("H_demag", list(pos_m))
        if v is None:
            raise NotImplementedError("probe_H_demag_siv: the exterior demag field (get_potential) is not "
                                      "available, as in the reference's parallel linalg machine")
        return v

    def get_subfield_sites(self, subfieldname):
        """main.py:2055-2077: node indices (of the loaded mesh) of the sites,
        one list per site."""
        self._unit_of(subfieldname)   # KeyError for unknown subfields
        nodes = self.node_map if self.node_map is not None else np.arange(self.mesh.n_nodes)
        return np.asarray(nodes, dtype=np.int64).reshape(-1, 1)

    def get_subfield_positions(self, subfieldname, pos_units=SI("m")):
        """main.py:2079-2103: site positions (site order, as get_subfield)
        in units of pos_units."""
        self._unit_of(subfieldname)
        return self.mesh.points / simulation_units.of(pos_units, compatible_with=SI("m"))

    def material_volume(self, material_name):
        """main.py:2189-2226: volume (simulation units) of the regions of a
        material; None: the whole magnetic mesh."""
        vol = self.mesh.tet_volumes()
        if material_name is None:
            return float(vol.sum())
        regions = self._regions_by_material[material_name]
        return float(vol[np.isin(self.mesh.regions, regions)].sum())

    def get_timers(self, timers=()):
        """main.py:1904-1916: (name, None, seconds) per timer; the device time
        of advance_time accumulated over the calls."""
        names = list(timers) or sorted(self._timers)
        return [(k, None, self._timers.get(k, 0.0)) for k in names]

    def region_volume(self, material_name):
        """main.py:2105-2107: retired in the reference, which points to
        material_volume."""
        raise NotImplementedError("Use material_volume instead")

    def save_fields(self, filename=None, fieldnames="all"):
        """main.py:2637-2639: retired in the reference in favour of
        save_data(fields=...)."""
        raise RuntimeError("Use save_data(fields=fields) to save fields")

    def save_mesh(self, filename, scontext=None):
        """main.py:1228-1232 / nmeshlib/lib1.py:498-515: the magnetic mesh in
        simulation units of length (as the reference's mesh object stores it),
        as nmesh HDF5 when the name ends in .h5, else as nmesh ASCII.
        (scontext, the reference's MPI context, has no use on one GPU.)"""
        if os.path.splitext(filename)[1].lower() == ".h5":
            _mesh.save_hdf5(self.mesh, filename)
        else:
            _mesh.save_ascii(self.mesh, filename)

    def do_next_stage(self, stage=None):
        """main.py:2733-2735 / clock.py:84-94: start the next stage (or the
        given one)."""
        self.max_dm_dt = None
        self.clock.stage = self.clock.stage + 1 if stage is None else stage
        self.clock.stage_step = 0
        self.clock.stage_time_su = 0.0
        self.clock.convergence = False
        self.clock.zero_stage_step = self.clock.step
        self.clock.zero_stage_time_su = self.clock.time_su
        self._ts_ready = False

    def get_subfield_average_siv(self, field_name, subfield_name=None):
        """main.py:2234-2290: volume average of a field in SI numbers (a
        list for vectors); ``subfield_name`` names the material of
        per-material fields ('m', 'Py' -> m_Py).  Member 0 of an ensemble."""
        field, subfield = field_name, subfield_name
        if self.layer is not None:   # several materials: averages over one material's sites
            names = [mt.name for mt in self.materials]
            name, base = subfield, field
            if name is None:
                for f in self._PER_MATERIAL:
                    if field.startswith(f + "_") and field[len(f) + 1:] in names:
                        name, base = field[len(f) + 1:], f
            if name is not None and name not in names:
                raise ValueError("You want to compute the average of '%s', but the subfield you specified (%s) is "
                                 "not one of its subfields" % (field, subfield))
            if base == "m" and name is not None:
                return list(self.engine.material_averages(names.index(name)))
            vals = self.get_subfield(base if name is None else "%s_%s" % (base, name))
            if self.n_members > 1:
                vals = vals[0]
            if name is not None:
                V = self._volumes()[self.layer.sites_of(name)]
            elif base in self._ON_MESH:
                V = self.layer.scatter(self._volumes())   # node volumes: the sum over each node's sites
            else:
                V = self._volumes()
            if vals.ndim == 2:
                return list((vals * V[:, None]).sum(0) / V.sum())
            return float((vals * V).sum() / V.sum())
        if subfield is not None and subfield != self.material.name:
            raise ValueError("You want to compute the average of '%s', but the subfield you specified (%s) is "
                             "not one of its subfields" % (field, subfield))
        if field == "m" or field.startswith("m_"):
            return list(self.engine.averages())
        vals = self.get_subfield(field)
        if vals.ndim == 3 or (vals.ndim == 2 and self.n_members > 1 and vals.shape[0] == self.n_members):
            vals = vals[0]
        V = self._volumes()
        if vals.ndim == 2:
            return list((vals * V[:, None]).sum(0) / V.sum())
        return float((vals * V).sum() / V.sum())

    def get_subfield_average(self, field_name, subfield_name=None):
        """main.py:2290-2312: as get_subfield_average_siv, as SI objects."""
        v = self.get_subfield_average_siv(field_name, subfield_name)
        u = self._unit_of(field_name)
        return [x * u for x in v] if isinstance(v, list) else v * u

    def get_member_average_m(self, member):
        """<m> of one ensemble member."""
        return list(self.engine.member_averages(member))

    def _volumes(self):
        if not hasattr(self, "_vol_cache"):
            self._vol_cache = self.engine.csr()[5]
        return self._vol_cache

    def energies(self):
        """Total energies (J) [E_exch, E_demag, E_ext, E_anis, E_total] at the current m."""
        self.engine.eval_fields()
        _, e = self.engine.averages(energies=True)
        return e * _su_factor("E") * (simulation_units.conversion_factor_of(SI("m")) ** 3)

    def _compute_averages(self):
        """main.py:2313-2480: (names, values, units) of one .ndt row: the
        clock, the volume average in SI of every field (member 0 of an
        ensemble), the largest angle between m at neighbouring nodes,
        the local and the unix time."""
        ck = self.clock
        to_si = simulation_units.conversion_factor_of(SI(1.0, "s"))
        names = ["time", "id", "step", "last_step_dt", "stage_time", "stage_step", "stage"]
        units = [SI(1.0, "s"), SI(1.0), SI(1.0), SI(1.0, "s"), SI(1.0, "s"), SI(1.0), SI(1.0)]
        values = [ck.time_su * to_si, int(ck.id), int(ck.step), ck.last_step_dt_su * to_si,
                  ck.stage_time_su * to_si, float(ck.stage_step), int(ck.stage)]
        f = self.engine.eval_fields()
        E = self.engine.energy_density()
        first = (lambda a: a[0]) if self.n_members > 1 else (lambda a: a)
        if self.layer is not None:
            return self._averages_sites(names, units, values, f, E, first)
        m = first(np.asarray(self._m))
        c = self.material.coefficients(self.quirks)
        su = {"m": m, "M": c["Ms"] * m, "H_ext": first(np.asarray(self._h_ext)),
              "phi": first(f["phi"]), "rho": first(f["rho"]),
              "pin": getattr(self, "_pin", None) if getattr(self, "_pin", None) is not None else np.ones(len(m))}
        for k in ("H_total", "H_exch", "H_anis", "H_demag", "dmdt"):
            su[k] = first(f[k])
        for k in ("E_total", "E_exch", "E_anis", "E_demag", "E_ext"):
            su[k] = first(E[k])
        mesh_fields = list(_NDT_MESH)
        if getattr(self, "_j", None) is not None:
            su["current_density"] = first(np.asarray(self._j))
            mesh_fields.append(("current_density", "J"))
        V = self._volumes()

        def average(a, kind):
            a = np.asarray(a, dtype=np.float64)
            s_ = (a * V[:, None]).sum(0) if a.ndim == 2 else (a * V).sum()
            return s_ / V.sum() * (1.0 / simulation_units.of(_FIELD_SI[kind]))
        mat = self.material.name
        for fname, kind in _NDT_PER_MATERIAL:
            names.append("%s_%s" % (fname, mat)); units.append(_FIELD_SI[kind]); values.append(average(su[fname], kind))
        for fname, kind in mesh_fields:
            names.append(fname); units.append(_FIELD_SI[kind]); values.append(average(su[fname], kind))
        # largest angle between m at the two ends of a mesh edge (degrees)
        t = self.mesh.simplices
        e = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)])
        mn = m / np.linalg.norm(m, axis=1)[:, None]
        cosang = np.clip(np.einsum("ij,ij->i", mn[e[:, 0]], mn[e[:, 1]]), -1.0, 1.0)
        names.append("maxangle_m_%s" % mat); units.append("<deg>")
        values.append(float(np.degrees(np.arccos(cosang.min()))) if len(cosang) else 0.0)
        lt = _time.localtime()
        names += ["localtime", "unixtime"]
        units += ["<>", SI(1.0, "s")]
        values += ["%04d/%02d/%02d-%02d:%02d:%02d" % lt[:6], _time.time()]
        return names, values, units

    def _averages_sites(self, names, units, values, f, E, first):
        """The .ndt row with several materials: every material's columns
        (averages over its sites with its box volumes, its largest
        neighbour angle), then the mesh fields over the nodes."""
        L = self.layer
        Vs = self._volumes()
        m = first(np.asarray(self._m))
        su = {"m": m, "H_ext": first(np.asarray(self._h_ext)), "phi": first(f["phi"]), "rho": first(f["rho"]),
              "pin": getattr(self, "_pin", None) if getattr(self, "_pin", None) is not None else np.ones(len(m))}
        ms = np.array([mt.coefficients(self.quirks)["Ms"] for mt in self.materials])[L.site_material]
        su["M"] = ms[:, None] * m
        for k in ("H_total", "H_exch", "H_anis", "H_demag", "dmdt"):
            su[k] = first(f[k])
        for k in ("E_total", "E_exch", "E_anis", "E_demag", "E_ext"):
            su[k] = first(E[k])

        def average(a, V, kind):
            a = np.asarray(a, dtype=np.float64)
            s_ = (a * V[:, None]).sum(0) if a.ndim == 2 else (a * V).sum()
            return s_ / V.sum() * (1.0 / simulation_units.of(_FIELD_SI[kind]))
        for k, mt in enumerate(self.materials):
            sx = L.sites_of(mt.name)
            for fname, kind in _NDT_PER_MATERIAL:
                names.append("%s_%s" % (fname, mt.name)); units.append(_FIELD_SI[kind])
                values.append(average(su[fname][sx], Vs[sx], kind))
        first_site = L.node_site_idx[L.node_site_ptr[:-1]]
        Vn = L.scatter(Vs)
        for fname, kind in _NDT_MESH:
            names.append(fname); units.append(_FIELD_SI[kind]); values.append(average(su[fname][first_site], Vn, kind))
        for k, mt in enumerate(self.materials):   # largest angle between m at the ends of an edge of the material
            t = L.site_tets[k] + L.offset[k]
            e = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)])
            mn = m / np.linalg.norm(m, axis=1)[:, None]
            cosang = np.clip(np.einsum("ij,ij->i", mn[e[:, 0]], mn[e[:, 1]]), -1.0, 1.0)
            names.append("maxangle_m_%s" % mt.name); units.append("<deg>")
            values.append(float(np.degrees(np.arccos(cosang.min()))) if len(cosang) else 0.0)
        lt = _time.localtime()
        names += ["localtime", "unixtime"]
        units += ["<>", SI(1.0, "s")]
        values += ["%04d/%02d/%02d-%02d:%02d:%02d" % lt[:6], _time.time()]
        return names, values, units

    @staticmethod
    def _save_data_table_to_ndt(names, values, units, filename):
        """main.py:2571-2634: one row of 25-character columns; a name line and
        a unit line first (once per file and process)."""
        cols = []
        for name, value, unit in zip(names, values, units):
            ustr = unit if isinstance(unit, str) else unit.dens_str()
            if np.ndim(value) == 0:
                cols.append((name, value, ustr))
            else:
                cols += [("%s_%d" % (name, k), float(v), ustr) for k, v in enumerate(value)]
        key = os.path.abspath(filename)
        new = not os.path.exists(filename)
        with open(filename, "a") as fh:
            if new or key not in _NDT_HEADERS_DONE:
                fh.write("#" + "".join("%-25s " % n for n, _, _ in cols) + "\n")
                fh.write("#" + "".join("%-25s " % u for _, _, u in cols) + "\n")
                _NDT_HEADERS_DONE.add(key)
            row = []
            for _, v, _ in cols:
                if isinstance(v, str):
                    row.append("% 25s " % v)
                elif isinstance(v, (int, np.integer)):
                    row.append("% 25d " % v)
                else:
                    row.append("% 25.13g " % float(v))
            fh.write("".join(row) + "\n")

    def save_data(self, fields=None, avoid_same_step=False):
        """main.py:2481-2536: append the averages to <name>_dat.ndt (a new
        clock id per row; with avoid_same_step a step already written is not
        written again) and, when fields are given ('all' or field names),
        append a row per field to <name>_dat.h5 (nfem/hdf5_v01.py:685-1022:
        the fields' subfields at their sites, in SI)."""
        saved = getattr(self, "_saved_steps", None)
        if saved is None:
            saved = self._saved_steps = set()
        if not (avoid_same_step and self.clock.step in saved):
            self.clock.id += 1
            saved.add(self.clock.step)
            names, values, units = self._compute_averages()
            self._save_data_table_to_ndt(names, values, units, "%s_dat.ndt" % self.name)
        if fields:
            all_fields = list(self._PER_MATERIAL) + list(self._ON_MESH)
            req = all_fields if fields == "all" else ([fields] if isinstance(fields, str) else list(fields))
            chosen = []
            for name in req:
                f = self._field_of(name)   # KeyError for unknown fields
                if f not in chosen:
                    chosen.append(f)
            self._append_h5_fields("%s_dat.h5" % self.name, chosen, all_fields)

    # ---- HDF5 data and restart files (nfem/hdf5_v01.py layout) ----
    def _subfields_of(self, field):
        """(subfield name, node index of each of its sites) of a field."""
        if field in self._ON_MESH:
            return [(field, np.arange(self.mesh.n_nodes))]
        mats = self.materials if self.layer is not None else [self.material]
        out = []
        for mt in mats:
            nodes = self.layer.site_node[self._sites_of(mt)] if self.layer is not None else np.arange(self.mesh.n_nodes)
            out.append(("%s_%s" % (field, mt.name), nodes))
        return out

    def _h5_metadata(self, fields):
        meta, sites = [], {}
        for f in fields:
            shape = "[3]" if f in self._VECTOR else "[]"
            unit = repr(_FIELD_SI[self._KIND[f]])
            for sub, nodes in self._subfields_of(f):
                meta.append((f, sub, unit, shape))
                sites[sub] = nodes
        return meta, sites

    def _h5_row(self, fields):
        snap = {"f": self.engine.eval_fields(), "E": self.engine.energy_density()}
        rows = {}
        for f in fields:
            data = {sub: self.get_subfield(sub, _snap=snap) for sub, _ in self._subfields_of(f)}
            rows[f] = {"id": self.clock.id, "stage": self.clock.stage, "step": self.clock.step,
                       "time": self.clock.time_su * 1e-12, "data": data}
        return rows

    def _append_h5_fields(self, path, fields, all_fields):
        meta, sites = self._h5_metadata(all_fields)
        old = _h5data.read(path) if os.path.exists(path) else None
        tables = dict(old["tables"]) if old else {}
        if old:
            meta, sites = old["metadata"], old["dofsites"]
        for f, row in self._h5_row(fields).items():
            new = _h5data.field_rows([(sub, None) for sub, _ in self._subfields_of(f)], [row])
            tables[f] = np.concatenate([tables[f], new]) if f in tables else new
        _h5data.write(path, self.mesh, meta, sites, tables, sim_units=repr(simulation_units))

    def get_restart_file_name(self):
        """The default restart file (simulation_core.py:343-345)."""
        return "%s_restart.h5" % self.name

    def save_restart_file(self, filename=None, fieldnames=("m",), all=False):
        """main.py:2764-2857: the fields (m by default, every field with
        all=True) and the clock, written to a temporary file and renamed;
        the clock is the attribute 'clock' of /data/fields/m."""
        fn = filename or self.get_restart_file_name()
        fields = list(self._PER_MATERIAL) + list(self._ON_MESH) if all else \
            [self._field_of(n) for n in fieldnames]
        if "m" not in fields:
            fields = ["m"] + fields
        meta, sites = self._h5_metadata(fields)
        tables = {f: _h5data.field_rows([(sub, None) for sub, _ in self._subfields_of(f)], [row])
                  for f, row in self._h5_row(fields).items()}
        _h5data.write(fn, self.mesh, meta, sites, tables, sim_units=repr(simulation_units),
                      clock=repr(dict(self.clock)))

    def load_m_from_h5file(self, filename, id=None, row=None, unit=None):
        """main.py:1876-1902: set m from a row of /data/fields/m of an nmag
        data or restart file -- the row with the given id, else row ``row``
        (the first by default; hdf5_v01.py:1625-1679) -- subfield by
        subfield, placed by the file's sites (the mesh must be the one the
        file was written with)."""
        if unit:
            raise NotImplementedError("This feature is not implemented yet (unit=*).")
        d = _h5data.read(filename)
        if "m" not in d["tables"]:
            raise IOError("File '%s' holds no field m" % filename)
        tab = d["tables"]["m"]
        if id is not None:
            hits = np.nonzero(tab["id"] == id)[0]
            if not len(hits):
                raise KeyError("no row with id %d for field 'm' in '%s'" % (id, filename))
            row = int(hits[0])
        row = tab[0 if row is None else row]
        m = np.array(self._m, copy=True)
        # a file of the whole mesh (vacuum included, as the reference writes
        # it) numbers the nodes of the mesh as loaded, not of its magnetic part
        whole = getattr(self, "node_map", None) is not None and len(d["mesh"].points) != self.mesh.n_nodes
        for sub, nodes in self._subfields_of("m"):
            if whole:
                nodes = np.asarray(self.node_map)[nodes]
            if sub not in row.dtype.names:
                continue
            vals = np.asarray(row[sub], dtype=np.float64)
            file_nodes = d["dofsites"].get(sub)
            if file_nodes is None or len(file_nodes) != len(nodes):
                raise ValueError("load_m_from_h5file: the sites of '%s' differ from this simulation's" % sub)
            pos = {int(n): k for k, n in enumerate(nodes)}
            if any(int(n) not in pos for n in file_nodes):
                raise ValueError("load_m_from_h5file: the sites of '%s' differ from this simulation's" % sub)
            idx = np.array([pos[int(n)] for n in file_nodes])
            target = self._sites_of(self._material_of(sub, "m"))[idx] if self.layer is not None else idx
            m[..., target, :] = vals
        self.set_m(m)

    def load_restart_file(self, file_name=None, filename=None):
        """main.py:2859-2883: m and the clock of a restart file (file_name,
        the reference's argument; filename is accepted too); a stage saved
        at convergence continues with the next stage."""
        fn = file_name or filename or self.get_restart_file_name()
        self.load_m_from_h5file(fn)
        clock = _h5data.read(fn)["clock"]
        if clock:
            import ast
            try:   # this package's clock (a dict); another writer's clock is not read
                values = ast.literal_eval(clock)
            except (ValueError, SyntaxError):
                log.warning("load_restart_file: the clock of '%s' is not readable; m only", fn)
                return
            self.clock.update(values)
            if self.clock.convergence:
                self.clock.stage += 1
