"""ctypes binding of libnmaggpu.so (include/nmag_gpu.h).

The library is the only compute path: if it is missing or cannot be loaded,
``lib()`` raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class Material(C.Structure):
    _fields_ = [("Ms", C.c_double), ("exch_coeff", C.c_double), ("C1", C.c_double), ("C2", C.c_double),
                ("C3", C.c_double), ("K1", C.c_double), ("axis", C.c_double * 3), ("anis_coeff", C.c_double),
                ("E_coeff_half", C.c_double), ("E_coeff_ext", C.c_double)]


class Options(C.Structure):
    _fields_ = [("do_demag", C.c_int), ("nbc_rtol", C.c_double), ("nbc_atol", C.c_double), ("nbc_maxits", C.c_int),
                ("dbc_rtol", C.c_double), ("dbc_atol", C.c_double), ("dbc_maxits", C.c_int),
                ("bem_precision", C.c_int), ("cg_precision", C.c_int), ("cg_no_coarse", C.c_int),
                ("n_members", C.c_int), ("bem_anchor_tol", C.c_double),
                ("adjoint_cg_precision", C.c_int), ("anchor_product", C.c_int), ("cg_local_sweeps", C.c_int),
                ("jv_precision", C.c_int)]


class Particle(C.Structure):
    _fields_ = [("coords", C.c_void_p), ("n_nodes", C.c_int), ("tets", C.c_void_p), ("n_tets", C.c_int),
                ("mat", Material), ("h_dir", C.c_double * 3)]


class BatchOptions(C.Structure):
    _fields_ = [("cg_rtol", C.c_double), ("cg_maxits", C.c_int), ("n_stages", C.c_int), ("rtol", C.c_double),
                ("atol", C.c_double), ("stop_dmdt", C.c_double), ("h_max", C.c_double), ("dt0", C.c_double),
                ("dt_max", C.c_double), ("fixed_dt", C.c_double), ("threads", C.c_int), ("budget", C.c_double),
                ("integrator", C.c_int), ("krylov_maxits", C.c_int), ("reserved", C.c_int * 2)]


class TsStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("nst", "nfe", "nni", "nli", "ncfn", "netf", "npe", "nps", "njv", "nje")] + \
               [("hcur", C.c_double), ("tcur", C.c_double), ("qcur", C.c_int32), ("last_cg_iters_nbc", C.c_int32),
                ("last_cg_iters_dbc", C.c_int32), ("pad", C.c_int32), ("time_rhs_ms", C.c_double),
                ("time_jv_ms", C.c_double), ("time_psolve_ms", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "pad"}


# every symbol declared in include/nmag_gpu.h
EXPORTS = ["nmg_version", "nmg_set_device", "nmg_last_error", "nmg_create", "nmg_destroy", "nmg_mesh_info", "nmg_get_csr",
           "nmg_export_operator", "nmg_get_boundary", "nmg_get_bem", "nmg_set_m", "nmg_get_m", "nmg_set_h_ext",
           "nmg_set_material", "nmg_set_anisotropy_poly", "nmg_set_stt", "nmg_set_current_density", "nmg_set_pinning", "nmg_eval_fields", "nmg_energy_density", "nmg_averages", "nmg_ts_init",
           "nmg_ts_advance", "nmg_max_dm", "nmg_max_dm_step", "nmg_rhs_device", "nmg_bem_apply", "nmg_set_jacobian",
           "nmg_jacobian_apply", "nmg_rk4_device", "nmg_get_timings", "nmg_profile",
           "nmg_profile_read", "nmg_launch_count", "nmg_cg_iterations", "nmg_bem_anchor_stats", "nmg_max_dm_static",
           "nmg_set_element_params", "nmg_clear_element_params", "nmg_rk4_forward", "nmg_rk4_adjoint",
           "nmg_member_averages", "nmg_create_materials", "nmg_site_info", "nmg_set_site_material", "nmg_set_local_coupling",
           "nmg_material_averages", "nmg_batch_last_error", "nmg_batch_create", "nmg_batch_destroy", "nmg_batch_info",
           "nmg_batch_set_m", "nmg_batch_get_m", "nmg_batch_eval", "nmg_batch_run", "nmg_batch_state",
           "nmg_batch_set_schedule", "nmg_batch_autotune"]

PROFILED_KERNELS = ["bem_gemv", "cg_neumann", "cg_dirichlet", "heff_llg", "jv_psolve", "bem_anchor_delta"]

_lib = None


class NmagGpuError(RuntimeError):
    pass


def lib_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load libnmaggpu.so (building it in-tree with nvcc if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB) or not _build.up_to_date():
        if not build_if_missing:
            raise NmagGpuError("libnmaggpu.so is not built (run nmag._build.build())")
        _build.build()
    L = C.CDLL(_build.LIB)
    vp = C.c_void_p
    L.nmg_version.restype = C.c_int
    L.nmg_set_device.argtypes = [C.c_int]
    L.nmg_last_error.argtypes = [vp]
    L.nmg_last_error.restype = C.c_char_p
    L.nmg_create.argtypes = [_f64p, C.c_int, _i32p, C.c_int, C.POINTER(Material), C.POINTER(Options), C.POINTER(vp)]
    L.nmg_destroy.argtypes = [vp]
    L.nmg_mesh_info.argtypes = [vp, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")]
    L.nmg_get_csr.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.nmg_export_operator.argtypes = [vp, C.c_int, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int), vp, vp, vp]
    L.nmg_get_boundary.argtypes = [vp, vp, vp, vp, vp]
    L.nmg_get_bem.argtypes = [vp, _f64p]
    L.nmg_set_m.argtypes = [vp, _f64p]
    L.nmg_get_m.argtypes = [vp, _f64p]
    L.nmg_set_h_ext.argtypes = [vp, _f64p]
    L.nmg_set_material.argtypes = [vp, C.POINTER(Material)]
    L.nmg_set_anisotropy_poly.argtypes = [vp, C.c_int, vp, vp, C.c_int, vp, vp]
    L.nmg_set_stt.argtypes = [vp, C.c_double, C.c_double]
    L.nmg_set_current_density.argtypes = [vp, vp]
    L.nmg_set_pinning.argtypes = [vp, vp]
    L.nmg_eval_fields.argtypes = [vp, vp, vp]
    L.nmg_energy_density.argtypes = [vp, _f64p]
    L.nmg_averages.argtypes = [vp, _f64p, vp]
    L.nmg_ts_init.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
    L.nmg_ts_advance.argtypes = [vp, C.c_double, C.c_int, C.c_int64, C.POINTER(C.c_double), C.POINTER(TsStats)]
    L.nmg_max_dm.argtypes = [vp, _f64p, C.POINTER(C.c_double)]
    L.nmg_max_dm_step.argtypes = [vp, C.POINTER(C.c_double)]
    L.nmg_rhs_device.argtypes = [vp, vp, vp]
    L.nmg_bem_apply.argtypes = [vp, vp, vp, C.c_int]
    L.nmg_set_jacobian.argtypes = [vp, C.c_int, C.c_double]
    L.nmg_jacobian_apply.argtypes = [vp, vp, vp, vp]
    L.nmg_create_materials.argtypes = [_f64p, C.c_int, _i32p, C.c_int, _i32p, C.c_int, _i32p, _i32p, vp, C.c_int,
                                       C.POINTER(Options), C.POINTER(vp)]
    L.nmg_site_info.argtypes = [vp, vp, vp]
    L.nmg_set_site_material.argtypes = [vp, C.c_int, C.POINTER(Material)]
    L.nmg_set_local_coupling.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double]
    L.nmg_material_averages.argtypes = [vp, C.c_int, C.c_int, _f64p, vp]
    L.nmg_rk4_device.argtypes = [vp, vp, C.c_double, C.c_int]
    L.nmg_get_timings.argtypes = [vp, _f64p]
    L.nmg_profile.argtypes = [vp, C.c_int]
    L.nmg_profile_read.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.nmg_launch_count.argtypes = [vp]
    L.nmg_launch_count.restype = C.c_int64
    L.nmg_cg_iterations.argtypes = [vp, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")]
    L.nmg_bem_anchor_stats.argtypes = [vp, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")]
    L.nmg_max_dm_static.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_double)]
    L.nmg_member_averages.argtypes = [vp, C.c_int, _f64p, vp]
    L.nmg_batch_last_error.argtypes = [vp]
    L.nmg_batch_last_error.restype = C.c_char_p
    L.nmg_batch_create.argtypes = [vp, C.c_int, C.POINTER(BatchOptions), C.POINTER(vp)]
    L.nmg_batch_destroy.argtypes = [vp]
    L.nmg_batch_info.argtypes = [vp, vp, vp, vp]
    L.nmg_batch_set_m.argtypes = [vp, _f64p]
    L.nmg_batch_get_m.argtypes = [vp, _f64p]
    L.nmg_batch_eval.argtypes = [vp, vp, vp]
    L.nmg_batch_run.argtypes = [vp, C.c_int]
    L.nmg_batch_state.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.nmg_batch_set_schedule.argtypes = [vp, C.c_int, C.c_double]
    L.nmg_batch_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.nmg_set_element_params.argtypes = [vp, vp, vp, vp, _f64p]
    L.nmg_clear_element_params.argtypes = [vp]
    L.nmg_rk4_forward.argtypes = [vp, vp, C.c_double, C.c_int, C.c_int, vp, C.c_int, C.c_int, vp, vp]
    L.nmg_rk4_adjoint.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    _lib = L
    return L


def set_device(device):
    """GPU for the engines created next on this thread (the library's own CUDA
    runtime does not follow torch.cuda.set_device)."""
    check(lib().nmg_set_device(int(device)), None, "set_device")


def check(rc, handle=None, what="call"):
    if rc != 0:
        msg = lib().nmg_last_error(handle)
        raise NmagGpuError("%s failed (status %d): %s" % (what, rc, msg.decode() if msg else ""))


class Engine(object):
    """Owns one nmg_handle: the device state of one simulation."""

    def __init__(self, points, simplices, material: Material, options: Options):
        L = lib()
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
        sim = np.ascontiguousarray(simplices, dtype=np.int32).reshape(-1)
        h = C.c_void_p()
        rc = L.nmg_create(pts, len(pts) // 3, sim, len(sim) // 4, C.byref(material), C.byref(options), C.byref(h))
        if rc != 0:
            raise NmagGpuError("nmg_create failed (status %d): %s" % (rc, L.nmg_last_error(None).decode()))
        self.h = h
        info = np.zeros(6, np.int64)
        L.nmg_mesh_info(h, info)
        self.N, self.T, self.nnz, self.nb, self.ntri, self.nouter = (int(v) for v in info)
        self.B = max(1, int(options.n_members))   # ensemble members (arrays gain a leading member axis)

    @classmethod
    def materials(cls, points, simplices, regions, region_materials, materials, options: Options):
        """Several magnetic materials (nmg_create_materials): regions (T,) of
        ids 1..R; region_materials[r - 1] lists the material indices region
        r carries; materials: Material structs.  Per-site arrays then hold
        one entry per site (self.N sites, material by material)."""
        L = lib()
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
        sim = np.ascontiguousarray(simplices, dtype=np.int32).reshape(-1)
        reg = np.ascontiguousarray(regions, dtype=np.int32).reshape(-1)
        ptr = np.zeros(len(region_materials) + 1, np.int32)
        for r, ms in enumerate(region_materials):
            ptr[r + 1] = ptr[r] + len(ms)
        idx = np.ascontiguousarray([k for ms in region_materials for k in ms], dtype=np.int32)
        arr = (Material * len(materials))(*materials)
        h = C.c_void_p()
        rc = L.nmg_create_materials(pts, len(pts) // 3, sim, len(sim) // 4, reg, len(region_materials), ptr, idx,
                                    C.cast(arr, C.c_void_p), len(materials), C.byref(options), C.byref(h))
        if rc != 0:
            raise NmagGpuError("nmg_create_materials failed (status %d): %s" % (rc, L.nmg_last_error(None).decode()))
        self = cls.__new__(cls)
        self.h = h
        info = np.zeros(6, np.int64)
        L.nmg_mesh_info(h, info)
        self.N, self.T, self.nnz, self.nb, self.ntri, self.nouter = (int(v) for v in info)
        self.B = max(1, int(options.n_members))
        self.n_materials = len(materials)
        return self

    def site_info(self):
        """(site_node, site_material) of a several-materials handle."""
        node = np.zeros(self.N, np.int32)
        mat = np.zeros(self.N, np.int32)
        check(lib().nmg_site_info(self.h, node.ctypes.data, mat.ctypes.data), self.h, "site_info")
        return node, mat

    def set_site_material(self, k, mat: Material):
        check(lib().nmg_set_site_material(self.h, int(k), C.byref(mat)), self.h, "set_site_material")

    def set_local_coupling(self, k1, k2, h_coeff, e_coeff):
        """H_lc of material k1 gains h_coeff m_k2, E_lc gains e_coeff m_k1 . m_k2 (shared nodes)."""
        check(lib().nmg_set_local_coupling(self.h, int(k1), int(k2), float(h_coeff), float(e_coeff)), self.h,
              "set_local_coupling")

    def material_averages(self, k, member=0, energies=False):
        a = np.zeros(3)
        e = np.zeros(5)
        check(lib().nmg_material_averages(self.h, int(k), int(member), a, e.ctypes.data if energies else None),
              self.h, "material_averages")
        return (a, e) if energies else a

    def _shape3(self):
        return (self.B, self.N, 3) if self.B > 1 else (self.N, 3)

    def close(self):
        if getattr(self, "h", None):
            lib().nmg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state ----
    def set_m(self, m):
        check(lib().nmg_set_m(self.h, np.ascontiguousarray(m, dtype=np.float64).reshape(-1)), self.h, "set_m")

    def get_m(self):
        out = np.zeros(3 * self.N * self.B)
        check(lib().nmg_get_m(self.h, out), self.h, "get_m")
        return out.reshape(self._shape3())

    def set_h_ext(self, h):
        h = np.broadcast_to(np.asarray(h, dtype=np.float64), self._shape3())
        check(lib().nmg_set_h_ext(self.h, np.ascontiguousarray(h).reshape(-1)), self.h, "set_h_ext")

    def set_material(self, mat: Material):
        check(lib().nmg_set_material(self.h, C.byref(mat)), self.h, "set_material")

    def set_stt(self, c4, c5):
        """Spin-transfer coefficients LLG_C4 (adiabatic), LLG_C5 (non-adiabatic)."""
        check(lib().nmg_set_stt(self.h, float(c4), float(c5)), self.h, "set_stt")

    def set_current_density(self, j=None):
        """Current density (simulation units), broadcast like set_h_ext; None = zero."""
        if j is None:
            check(lib().nmg_set_current_density(self.h, None), self.h, "set_current_density")
            return
        j = np.ascontiguousarray(np.broadcast_to(np.asarray(j, dtype=np.float64), self._shape3())).reshape(-1)
        check(lib().nmg_set_current_density(self.h, j.ctypes.data), self.h, "set_current_density")

    def set_pinning(self, pin=None):
        """Pinning factor per node (N values, shared by ensemble members); None = 1."""
        if pin is None:
            check(lib().nmg_set_pinning(self.h, None), self.h, "set_pinning")
            return
        p = np.ascontiguousarray(np.broadcast_to(np.asarray(pin, dtype=np.float64), (self.N,)))
        check(lib().nmg_set_pinning(self.h, p.ctypes.data), self.h, "set_pinning")

    def set_anisotropy_poly(self, e_pow=(), e_coef=(), h_pow=(), h_coef=()):
        """Polynomial anisotropy (nmg_set_anisotropy_poly): exponents packed
        a | b << 4 | c << 8; h_coef holds three coefficients per field term.
        Empty tables remove it."""
        ep = np.ascontiguousarray(e_pow, dtype=np.int32)
        ec = np.ascontiguousarray(e_coef, dtype=np.float64)
        hp = np.ascontiguousarray(h_pow, dtype=np.int32)
        hc = np.ascontiguousarray(h_coef, dtype=np.float64).reshape(-1)
        if ec.size != ep.size or hc.size != 3 * hp.size:
            raise ValueError("set_anisotropy_poly: coefficient and exponent tables differ in length")
        check(lib().nmg_set_anisotropy_poly(self.h, ep.size, ep.ctypes.data, ec.ctypes.data, hp.size, hp.ctypes.data,
                                            hc.ctypes.data), self.h, "set_anisotropy_poly")

    # ---- evaluation ----
    def eval_fields(self):
        n = self.N * self.B
        f = np.zeros(15 * n)
        s = np.zeros(2 * n)
        check(lib().nmg_eval_fields(self.h, f.ctypes.data, s.ctypes.data), self.h, "eval_fields")
        f = f.reshape((5,) + self._shape3())
        sh = (self.B, self.N) if self.B > 1 else (self.N,)
        return {"H_exch": f[0], "H_demag": f[1], "H_anis": f[2], "H_total": f[3], "dmdt": f[4],
                "phi": s[:n].reshape(sh), "rho": s[n:].reshape(sh)}

    def energy_density(self):
        E = np.zeros(5 * self.N * self.B)
        check(lib().nmg_energy_density(self.h, E), self.h, "energy_density")
        E = E.reshape((5, self.B, self.N) if self.B > 1 else (5, self.N))
        return {"E_exch": E[0], "E_demag": E[1], "E_ext": E[2], "E_anis": E[3], "E_total": E[4]}

    def averages(self, energies=False):
        a = np.zeros(3)
        e = np.zeros(5)
        check(lib().nmg_averages(self.h, a, e.ctypes.data if energies else None), self.h, "averages")
        return (a, e) if energies else a

    def member_averages(self, member, energies=False):
        a = np.zeros(3)
        e = np.zeros(5)
        check(lib().nmg_member_averages(self.h, int(member), a, e.ctypes.data if energies else None), self.h,
              "member_averages")
        return (a, e) if energies else a

    # ---- time integration ----
    def ts_init(self, t0=0.0, rtol=1e-6, atol=1e-6, max_order=2, krylov_max=300):
        check(lib().nmg_ts_init(self.h, t0, rtol, atol, max_order, krylov_max), self.h, "ts_init")

    def ts_advance(self, t, exact_tstop=True, max_steps=-1):
        tr = C.c_double()
        st = TsStats()
        check(lib().nmg_ts_advance(self.h, t, int(bool(exact_tstop)), int(max_steps), C.byref(tr), C.byref(st)),
              self.h, "ts_advance")
        return tr.value, st.as_dict()

    def max_dm(self, m_prev):
        out = C.c_double()
        check(lib().nmg_max_dm(self.h, np.ascontiguousarray(m_prev, dtype=np.float64).reshape(-1), C.byref(out)),
              self.h, "max_dm")
        return out.value

    def max_dm_step(self):
        """max |m - m at the previous call or set_m| on the device (0 the first time)."""
        out = C.c_double()
        check(lib().nmg_max_dm_step(self.h, C.byref(out)), self.h, "max_dm_step")
        return out.value

    def timings(self):
        t = np.zeros(8)
        lib().nmg_get_timings(self.h, t)
        return t

    def profile(self, enable):
        check(lib().nmg_profile(self.h, int(bool(enable))), self.h, "profile")

    def profile_read(self):
        """{kernel: (launches, total device ms)} since the last profile(True)."""
        out = {}
        for k, name in enumerate(PROFILED_KERNELS):
            n, ms = C.c_int64(), C.c_double()
            check(lib().nmg_profile_read(self.h, k, C.byref(n), C.byref(ms)), self.h, "profile_read")
            out[name] = (n.value, ms.value)
        return out

    def launch_count(self):
        return int(lib().nmg_launch_count(self.h))

    def cg_iterations(self):
        out = np.zeros(2, np.int64)
        check(lib().nmg_cg_iterations(self.h, out), self.h, "cg_iterations")
        return int(out[0]), int(out[1])

    def bem_anchor_stats(self):
        """(BEM products, anchor refreshes) of the anchored compensated product."""
        out = np.zeros(2, np.int64)
        check(lib().nmg_bem_anchor_stats(self.h, out), self.h, "bem_anchor_stats")
        return int(out[0]), int(out[1])

    # ---- inspection (parity tests) ----
    def csr(self):
        N, nnz = self.N, self.nnz
        rp = np.zeros(N + 1, np.int32); ci = np.zeros(nnz, np.int32); K = np.zeros(nnz)
        G = np.zeros(3 * nnz); D = np.zeros(3 * nnz); V = np.zeros(N)
        check(lib().nmg_get_csr(self.h, rp.ctypes.data, ci.ctypes.data, K.ctypes.data, G.ctypes.data, D.ctypes.data,
                                V.ctypes.data), self.h, "get_csr")
        return rp, ci, K, G.reshape(3, nnz), D.reshape(3, nnz), V

    def export_operator(self, which, coeff=1.0):
        L = lib()
        r, c, n = C.c_int(), C.c_int(), C.c_int()
        check(L.nmg_export_operator(self.h, which, coeff, C.byref(r), C.byref(c), C.byref(n), None, None, None),
              self.h, "export_operator")
        rp = np.zeros(r.value + 1, np.int32); ci = np.zeros(n.value, np.int32); va = np.zeros(n.value)
        check(L.nmg_export_operator(self.h, which, coeff, C.byref(r), C.byref(c), C.byref(n), rp.ctypes.data,
                                    ci.ctypes.data, va.ctypes.data), self.h, "export_operator")
        return rp, ci, va, (r.value, c.value)

    def boundary(self):
        nob = np.zeros(self.nb, np.int32); tri = np.zeros(3 * self.ntri, np.int32)
        nrm = np.zeros(3 * self.ntri); sa = np.zeros(self.nb)
        check(lib().nmg_get_boundary(self.h, nob.ctypes.data, tri.ctypes.data, nrm.ctypes.data, sa.ctypes.data),
              self.h, "get_boundary")
        return nob, tri.reshape(-1, 3), nrm.reshape(-1, 3), sa

    def bem(self):
        out = np.zeros(self.nb * self.nb)
        check(lib().nmg_get_bem(self.h, out), self.h, "get_bem")
        return out.reshape(self.nb, self.nb)

    # ---- device pointers (torch tensors) ----
    def rhs_device(self, d_m, d_dmdt):
        check(lib().nmg_rhs_device(self.h, C.c_void_p(d_m), C.c_void_p(d_dmdt)), self.h, "rhs_device")

    def bem_apply_device(self, d_x, d_y, n_rhs):
        """y_n = B x_n for n_rhs member-major boundary vectors (device addresses)."""
        check(lib().nmg_bem_apply(self.h, C.c_void_p(d_x), C.c_void_p(d_y), int(n_rhs)), self.h, "bem_apply")

    def set_jacobian(self, level, demag_rtol=1e-3):
        """The Newton matrix's Jacobian: 0 the reference's (exchange only), 1 + the local
        terms, 2 + the demag response (Poisson solves at demag_rtol)."""
        check(lib().nmg_set_jacobian(self.h, int(level), float(demag_rtol)), self.h, "set_jacobian")

    def jacobian_apply_device(self, d_m, d_v, d_out):
        """out = J(m) v at the handle's Jacobian level (device addresses)."""
        check(lib().nmg_jacobian_apply(self.h, C.c_void_p(d_m), C.c_void_p(d_v), C.c_void_p(d_out)), self.h,
              "jacobian_apply")

    def rk4_device(self, d_m, dt, nsteps):
        check(lib().nmg_rk4_device(self.h, C.c_void_p(d_m), dt, nsteps), self.h, "rk4_device")

    # ---- differentiation form (device pointers; 0 = NULL) ----
    def set_element_params(self, d_wK, d_wD, d_kappa, axis):
        ax = np.ascontiguousarray(axis, dtype=np.float64)
        check(lib().nmg_set_element_params(self.h, C.c_void_p(d_wK or None), C.c_void_p(d_wD or None),
                                           C.c_void_p(d_kappa or None), ax), self.h, "set_element_params")

    def clear_element_params(self):
        check(lib().nmg_clear_element_params(self.h), self.h, "clear_element_params")

    def rk4_forward(self, d_m0, dt, nsteps, ckpt_every, d_pulses, n_pulses, steps_per_pulse, d_m_final, d_hist):
        check(lib().nmg_rk4_forward(self.h, C.c_void_p(d_m0), dt, nsteps, ckpt_every, C.c_void_p(d_pulses or None),
                                    n_pulses, steps_per_pulse, C.c_void_p(d_m_final), C.c_void_p(d_hist or None)),
              self.h, "rk4_forward")

    def rk4_adjoint(self, d_mT_bar, d_hist_bar, d_m0_bar, d_wK_bar, d_wD_bar, d_kappa_bar, d_pulses_bar):
        ptrs = [C.c_void_p(p or None) for p in (d_mT_bar, d_hist_bar, d_m0_bar, d_wK_bar, d_wD_bar, d_kappa_bar,
                                                  d_pulses_bar)]
        check(lib().nmg_rk4_adjoint(self.h, *ptrs), self.h, "rk4_adjoint")
