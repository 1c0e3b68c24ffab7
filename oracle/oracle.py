"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, to produce expected results.  The product never
imports it.

The oracle restates nsim's LLG right-hand side and CVODE-style integrator on
the CPU (see nmag_oracle.h for the reference citations).  Its BEM fill is
pinned to the reference's own code: the reference's plain-C Lindholm stub
(src/bem3d_stubs.c), compiled unmodified against a minimal caml shim into
_ref/ (ref_bem), fills the same matrix bit for bit; the reference's
structured mesher (utils/cubicmesh/cubicmesh.c) is built there too
(ref_cubicmesh) and its files pin the nmesh text reader.  The rest of the path has
no compilable reference (OCaml, PETSc, SUNDIALS are absent), so known-answer
tests pin the restatement there.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class OmMesh(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_tets", C.c_int),
                ("coords", C.POINTER(C.c_double)), ("tets", C.POINTER(C.c_int32)),
                ("nt_ptr", C.POINTER(C.c_int32)), ("nt_idx", C.POINTER(C.c_int32)),
                ("dL", C.POINTER(C.c_double)), ("adet", C.POINTER(C.c_double)),
                ("nbr", C.POINTER(C.c_int32)),
                ("nnz", C.c_int), ("row_ptr", C.POINTER(C.c_int32)), ("col_idx", C.POINTER(C.c_int32)),
                ("K", C.POINTER(C.c_double)), ("G", C.POINTER(C.c_double) * 3), ("D", C.POINTER(C.c_double) * 3),
                ("vol", C.POINTER(C.c_double)),
                ("nb", C.c_int), ("b_of_node", C.POINTER(C.c_int32)), ("node_of_b", C.POINTER(C.c_int32)),
                ("ntri", C.c_int), ("tri", C.POINTER(C.c_int32)), ("tri_normal", C.POINTER(C.c_double)),
                ("solid_angle", C.POINTER(C.c_double)), ("bem", C.POINTER(C.c_double))]


class OmMaterial(C.Structure):
    _fields_ = [("Ms", C.c_double), ("exch_coeff", C.c_double), ("C1", C.c_double), ("C2", C.c_double),
                ("C3", C.c_double), ("K1", C.c_double), ("axis", C.c_double * 3), ("anis_coeff", C.c_double),
                ("E_coeff_half", C.c_double), ("E_coeff_ext", C.c_double)]


class OmSolver(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("maxits", C.c_int)]


class OmState(C.Structure):
    _fields_ = [("M", C.POINTER(OmMesh)), ("mat", OmMaterial), ("nbc", OmSolver), ("dbc", OmSolver),
                ("do_demag", C.c_int),
                ("phi1", C.POINTER(C.c_double)), ("phi2", C.POINTER(C.c_double)), ("h_ext", C.POINTER(C.c_double)),
                ("h_exch", C.POINTER(C.c_double)), ("h_demag", C.POINTER(C.c_double)),
                ("h_anis", C.POINTER(C.c_double)), ("h_total", C.POINTER(C.c_double)),
                ("rho", C.POINTER(C.c_double)), ("phi", C.POINTER(C.c_double)), ("dmdt", C.POINTER(C.c_double)),
                ("tmp_b1", C.POINTER(C.c_double)), ("tmp_b2", C.POINTER(C.c_double)),
                ("last_iters_nbc", C.c_int), ("last_iters_dbc", C.c_int), ("n_rhs", C.c_longlong),
                ("nthreads", C.c_int),
                ("basis_b", C.POINTER(C.c_double) * 2), ("basis_x", C.POINTER(C.c_double) * 2),
                ("gram", (C.c_double * 100) * 2), ("bcount", C.c_int * 2), ("bhead", C.c_int * 2),
                ("an_ne", C.c_int), ("an_nh", C.c_int), ("an_epow", C.POINTER(C.c_int32)),
                ("an_hpow", C.POINTER(C.c_int32)), ("an_ecoef", C.POINTER(C.c_double)),
                ("an_hcoef", C.POINTER(C.c_double)), ("stt_c4", C.c_double), ("stt_c5", C.c_double),
                ("stt_j", C.POINTER(C.c_double)), ("stt_dmdc", C.POINTER(C.c_double)),
                ("pin", C.POINTER(C.c_double))]


class OmStats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("nst", "nfe", "nni", "nli", "ncfn", "netf", "npe", "nps", "njv", "nje")] + \
               [("hcur", C.c_double), ("tcur", C.c_double), ("qcur", C.c_int)]


_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB) or any(
            os.path.getmtime(os.path.join(HERE, f)) > os.path.getmtime(LIB)
            for f in ("nmag_oracle.c", "nmag_bdf.c", "nmag_oracle.h")):
        subprocess.check_call(["make", "-s", "-C", HERE])


REF_SRC = os.environ.get("NMAG_REFERENCE_SRC", "/root/reference/src")
REF_LIB = os.path.join(HERE, "_ref", "libref_bem.so")
_ref = None


def build_ref():
    """Compile the reference's own Lindholm stub (REF_SRC/bem3d_stubs.c,
    unmodified) with the harness into _ref/ when the reference tree is
    present; return whether the library exists afterwards."""
    if os.path.exists(os.path.join(REF_SRC, "bem3d_stubs.c")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF_SRC=" + REF_SRC])
    return os.path.exists(REF_LIB)


REF_UTILS = os.environ.get("NMAG_REFERENCE_UTILS", os.path.join(os.path.dirname(REF_SRC), "utils"))
REF_CUBICMESH = os.path.join(HERE, "_ref", "cubicmesh")


def build_ref_cubicmesh():
    """Compile the reference's structured mesher (REF_UTILS/cubicmesh/
    cubicmesh.c, unmodified) into _ref/ when the reference tree is present;
    return whether the program exists afterwards."""
    if os.path.exists(os.path.join(REF_UTILS, "cubicmesh", "cubicmesh.c")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref-cubicmesh", "REF_SRC=" + REF_SRC,
                               "REF_UTILS=" + REF_UTILS])
    return os.path.exists(REF_CUBICMESH)


def ref_cubicmesh(path, sizes, divisions, region_filter=None):
    """Run the reference's mesher: ``cubicmesh path,lx:nx,ly:ny,lz:nz
    [filter]`` writes an nmesh text file to path (cubicmesh.c:402-441)."""
    if not os.path.exists(REF_CUBICMESH):
        raise RuntimeError("reference mesher not built (oracle/_ref)")
    spec = ",".join([path] + ["%r:%d" % (float(a), int(n)) for a, n in zip(sizes, divisions)])
    cmd = [REF_CUBICMESH, spec] + ([region_filter] if region_filter else [])
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return path


def ref_lib():
    """The reference-built BEM library, or None when it was not built (the
    reference tree is absent, e.g. where only the committed fixtures exist)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            return None
        L = C.CDLL(REF_LIB)
        L.ref_fill_bem.argtypes = [C.c_int, _f64p, C.c_int, _i32p, _f64p, _f64p, _f64p]
        L.ref_fill_bem.restype = C.c_int
        _ref = L
    return _ref


def ref_bem(omesh):
    """The BEM matrix of an OracleMesh as the reference's own stub fills it
    (bem3d.ml:938-1047 around bem3d_stubs.c:413-610), from the oracle's
    boundary numbering, surface triangles, normals and solid angles."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference BEM library not built (oracle/_ref)")
    nb = omesh.nb
    obs = np.ascontiguousarray(omesh.points[omesh.node_of_b], dtype=np.float64)
    out = np.zeros((nb, nb))
    rc = L.ref_fill_bem(nb, obs.reshape(-1), omesh.ntri, np.ascontiguousarray(omesh.tri, np.int32).reshape(-1),
                        np.ascontiguousarray(omesh.tri_normal).reshape(-1), np.ascontiguousarray(omesh.solid_angle),
                        out.reshape(-1))
    if rc != 0:
        raise MemoryError("ref_fill_bem failed")
    return out


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.om_build.argtypes = [C.POINTER(OmMesh), C.c_int, _f64p, C.c_int, _i32p]
        L.om_fill_bem.argtypes = [C.POINTER(OmMesh), C.c_int]
        L.om_free.argtypes = [C.POINTER(OmMesh)]
        L.om_export_operator.argtypes = [C.POINTER(OmMesh), C.c_int, C.c_double, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_void_p,
                                         C.c_void_p]
        L.om_state_init.argtypes = [C.POINTER(OmState), C.POINTER(OmMesh), C.POINTER(OmMaterial),
                                    C.POINTER(OmSolver), C.POINTER(OmSolver), C.c_int, C.c_int]
        L.om_state_free.argtypes = [C.POINTER(OmState)]
        L.om_rhs.argtypes = [C.POINTER(OmState), _f64p, C.c_void_p]
        L.om_set_anisotropy_poly.argtypes = [C.POINTER(OmState), C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                             C.c_void_p, C.c_void_p]
        L.om_set_stt.argtypes = [C.POINTER(OmState), C.c_double, C.c_double, C.c_void_p]
        L.om_set_pinning.argtypes = [C.POINTER(OmState), C.c_void_p]
        L.om_energy_density.argtypes = [C.POINTER(OmState), _f64p, _f64p]
        L.om_jv.argtypes = [C.POINTER(OmState), _f64p, _f64p, _f64p, _f64p]
        L.om_bdf_create.argtypes = [C.POINTER(OmState), C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double]
        L.om_bdf_create.restype = C.c_void_p
        L.om_bdf_free.argtypes = [C.c_void_p]
        L.om_bdf_init.argtypes = [C.c_void_p, C.c_double, _f64p]
        L.om_bdf_advance.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_longlong, C.POINTER(C.c_double), _f64p]
        L.om_bdf_stats.argtypes = [C.c_void_p, C.POINTER(OmStats)]
        L.om_bdf_set_precond.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.om_bdf_pc_iterations.argtypes = [C.c_void_p]
        L.om_bdf_pc_iterations.restype = C.c_longlong
        L.om_pc_matrix_apply.argtypes = [C.POINTER(OmState), _f64p, _f64p, C.c_double, _f64p, _f64p]
        L.om_rk4.argtypes = [C.POINTER(OmState), _f64p, C.c_double, C.c_int]
        L.om_triangle_space_angle.argtypes = [_f64p, _f64p, _f64p, _f64p]
        L.om_triangle_space_angle.restype = C.c_double
        L.om_lindholm_single.argtypes = [_f64p, _f64p, _f64p, _f64p, _f64p, _f64p]
        _lib = L
    return _lib


def lindholm_single(p0, p1, p2, normal, obs):
    """Double-layer weights of one triangle for one observer."""
    f = lambda v: np.ascontiguousarray(v, dtype=np.float64)
    lh = np.zeros(3)
    lib().om_lindholm_single(f(p0), f(p1), f(p2), f(normal), f(obs), lh)
    return lh


def solid_angle(obs, p0, p1, p2):
    f = lambda v: np.ascontiguousarray(v, dtype=np.float64)
    return lib().om_triangle_space_angle(f(obs), f(p0), f(p1), f(p2))


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class OracleMesh(object):
    """Topology, CSR and BEM of a tetrahedral mesh, computed by the oracle."""

    def __init__(self, points, simplices, fill_bem=True, nthreads=0):
        L = lib()
        self._m = OmMesh()
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
        sim = np.ascontiguousarray(simplices, dtype=np.int32).reshape(-1)
        st = L.om_build(C.byref(self._m), len(pts) // 3, pts, len(sim) // 4, sim)
        if st != 0:
            raise ValueError("oracle mesh build failed (%d)" % st)
        if fill_bem:
            L.om_fill_bem(C.byref(self._m), nthreads)
        m = self._m
        N, T, nnz, nb = m.n_nodes, m.n_tets, m.nnz, m.nb
        self.n_nodes, self.n_tets, self.nnz, self.nb, self.ntri = N, T, nnz, nb, m.ntri
        self.points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        self.row_ptr = _arr(m.row_ptr, N + 1, np.int32)
        self.col_idx = _arr(m.col_idx, nnz, np.int32)
        self.K = _arr(m.K, nnz, np.float64)
        self.G = np.stack([_arr(m.G[d], nnz, np.float64) for d in range(3)])
        self.D = np.stack([_arr(m.D[d], nnz, np.float64) for d in range(3)])
        self.vol = _arr(m.vol, N, np.float64)
        self.b_of_node = _arr(m.b_of_node, N, np.int32)
        self.node_of_b = _arr(m.node_of_b, nb, np.int32)
        self.tri = _arr(m.tri, 3 * m.ntri, np.int32).reshape(-1, 3)
        self.tri_normal = _arr(m.tri_normal, 3 * m.ntri, np.float64).reshape(-1, 3)
        self.solid_angle = _arr(m.solid_angle, nb, np.float64)
        self.nbr = _arr(m.nbr, 4 * T, np.int32).reshape(-1, 4)
        self.dL = _arr(m.dL, 12 * T, np.float64).reshape(-1, 4, 3)
        self.adet = _arr(m.adet, T, np.float64)
        self._filled = fill_bem

    @property
    def bem(self):
        """The dense BEM (row-major nb x nb), copied out on first access."""
        if not self._filled:
            return None
        if not hasattr(self, "_bem"):
            self._bem = _arr(self._m.bem, self.nb * self.nb, np.float64).reshape(self.nb, self.nb)
        return self._bem

    def export_operator(self, which, coeff=1.0):
        L = lib()
        r, c, n = C.c_int(), C.c_int(), C.c_int()
        L.om_export_operator(C.byref(self._m), which, coeff, C.byref(r), C.byref(c), C.byref(n), None, None, None)
        rp = np.zeros(r.value + 1, np.int32)
        ci = np.zeros(n.value, np.int32)
        va = np.zeros(n.value, np.float64)
        L.om_export_operator(C.byref(self._m), which, coeff, C.byref(r), C.byref(c), C.byref(n),
                             rp.ctypes.data, ci.ctypes.data, va.ctypes.data)
        return rp, ci, va, (r.value, c.value)

    def __del__(self):
        try:
            lib().om_free(C.byref(self._m))
        except Exception:
            pass


class OracleSim(object):
    """RHS + BDF integration on the oracle for one material."""

    def __init__(self, omesh, coeffs, do_demag=True, nbc=(1e-5, 1e-50, 10000), dbc=(1e-5, 1e-50, 10000),
                 nthreads=0):
        L = lib()
        self.omesh = omesh
        mat = OmMaterial()
        mat.Ms = coeffs["Ms"]; mat.exch_coeff = coeffs["exch_coeff"]
        mat.C1 = coeffs["C1"]; mat.C2 = coeffs["C2"]; mat.C3 = coeffs["C3"]
        mat.K1 = coeffs.get("K1", 0.0)
        ax = coeffs.get("axis", (0.0, 0.0, 1.0))
        for d in range(3):
            mat.axis[d] = ax[d]
        mat.anis_coeff = coeffs.get("anis_coeff", 0.0)
        mat.E_coeff_half = coeffs.get("E_coeff_half", 0.0)
        mat.E_coeff_ext = coeffs.get("E_coeff_ext", 0.0)
        self._s = OmState()
        n1 = OmSolver(nbc[0], nbc[1], int(nbc[2]))
        n2 = OmSolver(dbc[0], dbc[1], int(dbc[2]))
        L.om_state_init(C.byref(self._s), C.byref(omesh._m), C.byref(mat), C.byref(n1), C.byref(n2),
                        int(bool(do_demag)), nthreads)
        poly = coeffs.get("anis_poly")
        if poly is not None:
            ep, ec, hp, hc = (np.ascontiguousarray(poly[0], dtype=np.int32), np.ascontiguousarray(poly[1], dtype=np.float64),
                              np.ascontiguousarray(poly[2], dtype=np.int32), np.ascontiguousarray(poly[3], dtype=np.float64))
            L.om_set_anisotropy_poly(C.byref(self._s), ep.size, ep.ctypes.data, ec.ctypes.data, hp.size,
                                     hp.ctypes.data, hc.ctypes.data)
        self.N = omesh.n_nodes
        self._bdf = None

    def set_stt(self, c4, c5, j=None):
        """Spin-transfer coefficients and current density (3N or broadcast)."""
        jj = None if j is None else np.ascontiguousarray(np.broadcast_to(np.asarray(j, dtype=np.float64),
                                                                         (self.N, 3))).reshape(-1)
        lib().om_set_stt(C.byref(self._s), float(c4), float(c5), None if jj is None else jj.ctypes.data)

    def set_pinning(self, pin=None):
        """Pinning factor per node (N values; None = 1 everywhere)."""
        pp = None if pin is None else np.ascontiguousarray(np.broadcast_to(np.asarray(pin, dtype=np.float64),
                                                                           (self.N,)))
        self._pin = pp   # the C side copies; kept for reference
        lib().om_set_pinning(C.byref(self._s), None if pp is None else pp.ctypes.data)

    def set_h_ext(self, h):
        h = np.broadcast_to(np.asarray(h, dtype=np.float64), (self.N, 3)).reshape(-1)
        np.ctypeslib.as_array(self._s.h_ext, shape=(3 * self.N,))[:] = h

    def rhs(self, m):
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        out = np.zeros(3 * self.N)
        st = lib().om_rhs(C.byref(self._s), m, out.ctypes.data)
        if st:
            raise RuntimeError("oracle rhs failed: %d" % st)
        return out

    def field(self, name):
        n = self.N
        ptr = getattr(self._s, {"H_exch": "h_exch", "H_demag": "h_demag", "H_anis": "h_anis",
                                "H_total": "h_total", "H_ext": "h_ext", "dmdt": "dmdt",
                                "dm_dcurrent": "stt_dmdc"}[name])
        return np.ctypeslib.as_array(ptr, shape=(3 * n,)).copy().reshape(n, 3)

    def scalar_field(self, name):
        ptr = getattr(self._s, {"phi": "phi", "rho": "rho", "phi1": "phi1", "phi2": "phi2"}[name])
        return np.ctypeslib.as_array(ptr, shape=(self.N,)).copy()

    @property
    def iters(self):
        return self._s.last_iters_nbc, self._s.last_iters_dbc

    def energy_density(self, m):
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        E = np.zeros(5 * self.N)
        lib().om_energy_density(C.byref(self._s), m, E)
        return E.reshape(5, self.N)

    def jv(self, mJ, HJ, v):
        out = np.zeros(3 * self.N)
        lib().om_jv(C.byref(self._s), np.ascontiguousarray(mJ, dtype=np.float64).reshape(-1),
                    np.ascontiguousarray(HJ, dtype=np.float64).reshape(-1),
                    np.ascontiguousarray(v, dtype=np.float64).reshape(-1), out)
        return out

    def pc_matrix_apply(self, mJ, HJ, gamma, v):
        """(I - gamma J(mJ, HJ)) v from the matrix the reference's
        preconditioner assembles."""
        out = np.zeros(3 * self.N)
        lib().om_pc_matrix_apply(C.byref(self._s), np.ascontiguousarray(mJ, dtype=np.float64).reshape(-1),
                                 np.ascontiguousarray(HJ, dtype=np.float64).reshape(-1), float(gamma),
                                 np.ascontiguousarray(v, dtype=np.float64).reshape(-1), out)
        return out

    def ts_init(self, m0, t0=0.0, rtol=1e-6, atol=1e-6, max_order=2, krylov_max=300, pc_rtol=1e-2, pc_atol=1e-7,
                precond="block", pc_restart=30, pc_maxit=10000):
        """precond: "block" (one exact 3x3 block-Jacobi sweep, as on the
        device) or "reference" (P = I - gamma J assembled, GMRES(pc_restart)
        with ILU(0) to pc_rtol / pc_atol, nsim.ml:2210-2262,2419-2483)."""
        L = lib()
        if self._bdf:
            L.om_bdf_free(self._bdf)
        self._bdf = L.om_bdf_create(C.byref(self._s), max_order, krylov_max, rtol, atol, pc_rtol, pc_atol)
        L.om_bdf_set_precond(self._bdf, {"block": 0, "reference": 1}[precond], pc_restart, pc_maxit)
        st = L.om_bdf_init(self._bdf, t0, np.ascontiguousarray(m0, dtype=np.float64).reshape(-1))
        if st:
            raise RuntimeError("oracle ts init failed: %d" % st)

    def ts_advance(self, t, exact_tstop=True, max_steps=-1):
        out = np.zeros(3 * self.N)
        tr = C.c_double()
        st = lib().om_bdf_advance(self._bdf, t, int(bool(exact_tstop)), max_steps, C.byref(tr), out)
        if st:
            raise RuntimeError("oracle ts advance failed: %d" % st)
        return tr.value, out.reshape(self.N, 3)

    def ts_stats(self):
        s = OmStats()
        lib().om_bdf_stats(self._bdf, C.byref(s))
        out = {n: getattr(s, n) for n, _ in OmStats._fields_}
        out["pc_iterations"] = lib().om_bdf_pc_iterations(self._bdf)
        return out

    def rk4(self, m, dt, nsteps):
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1).copy()
        st = lib().om_rk4(C.byref(self._s), m, dt, nsteps)
        if st:
            raise RuntimeError("oracle rk4 failed")
        return m.reshape(self.N, 3)

    def __del__(self):
        try:
            if self._bdf:
                lib().om_bdf_free(self._bdf)
            lib().om_state_free(C.byref(self._s))
        except Exception:
            pass
