"""Batching form: many independent magnetic particles, each with its own
mesh, material and field-sweep direction, advanced together on the GPU in
one persistent launch per step batch (nmg_batch_* of libnmaggpu.so).

Each particle runs the reference's hysteresis protocol
(interface/nmag/hysteresis.py:244-557): at each field of the sweep it relaxes
until max |dm/dt| < stop_dmdt twice in a row, then moves to the next field,
H_k = h_max (1 - 2k/(n-1)) along its direction.  The right-hand side is the
single path's (nmag_lam.py:734-832); time integration is either the embedded
Bogacki-Shampine 3(2) pair (integrator="bs3", explicit) or the linearly
implicit ROS2 W-method (integrator="ros2": L-stable, steps limited by accuracy
rather than by the exchange stiffness; each stage solves I - gamma tau J by
BiCGSTAB with the exchange + site Jacobian of nsim.ml:967-1050), both with
per-particle step control.
"""
import ctypes as C

import numpy as np

from ._lib import BatchOptions, Material, NmagGpuError, Particle, lib

__all__ = ["ParticleBatch"]


def _material_struct(coeffs):
    if coeffs.get("anis_poly") is not None:
        raise NotImplementedError("particle batches take the second-order uniaxial anisotropy only")
    if coeffs.get("C4", 0.0) != 0.0 or coeffs.get("C5", 0.0) != 0.0:
        raise NotImplementedError("particle batches have no spin-transfer torque")
    mt = Material()
    mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = (coeffs["Ms"], coeffs["exch_coeff"], coeffs["C1"], coeffs["C2"],
                                                 coeffs["C3"])
    mt.K1 = coeffs["K1"]
    for d in range(3):
        mt.axis[d] = coeffs["axis"][d]
    mt.anis_coeff, mt.E_coeff_half, mt.E_coeff_ext = coeffs["anis_coeff"], coeffs["E_coeff_half"], coeffs["E_coeff_ext"]
    return mt


class ParticleBatch(object):
    """particles: list of (points_su (n,3), simplices (t,4), coefficients dict
    as MagMaterial.coefficients() gives, h_dir (3,)).  Options in simulation
    units (stop_dmdt default 1 deg/ns, h_max the sweep amplitude)."""

    def __init__(self, particles, n_stages=81, h_max=0.0, stop_dmdt=1.7453292519943295e-05, rtol=1e-5, atol=1e-5,
                 cg_rtol=1e-6, cg_maxits=5000, dt0=0.01, dt_max=5.0, fixed_dt=0.0, threads=256, budget=0.0,
                 integrator="bs3", krylov_maxits=200):
        L = lib()
        self._keep = []
        arr = (Particle * len(particles))()
        self.sizes = []
        for k, (pts, sim, coeffs, hdir) in enumerate(particles):
            p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1)
            t = np.ascontiguousarray(sim, dtype=np.int32).reshape(-1)
            self._keep += [p, t]
            arr[k].coords = p.ctypes.data
            arr[k].n_nodes = len(p) // 3
            arr[k].tets = t.ctypes.data
            arr[k].n_tets = len(t) // 4
            arr[k].mat = _material_struct(coeffs)
            for d in range(3):
                arr[k].h_dir[d] = float(hdir[d])
            self.sizes.append(len(p) // 3)
        o = BatchOptions()
        o.cg_rtol, o.cg_maxits, o.n_stages = cg_rtol, cg_maxits, n_stages
        o.rtol, o.atol, o.stop_dmdt, o.h_max = rtol, atol, stop_dmdt, h_max
        o.dt0, o.dt_max, o.fixed_dt, o.threads, o.budget = dt0, dt_max, fixed_dt, threads, budget
        o.integrator = {"bs3": 0, "ros2": 1}[integrator]
        o.krylov_maxits = krylov_maxits
        h = C.c_void_p()
        rc = L.nmg_batch_create(arr, len(particles), C.byref(o), C.byref(h))
        if rc != 0:
            raise NmagGpuError("nmg_batch_create failed (status %d): %s" % (rc, L.nmg_batch_last_error(None).decode()))
        self.h = h
        self.P = len(particles)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        self.N = int(self.offsets[-1])

    def _check(self, rc, what):
        if rc != 0:
            raise NmagGpuError("%s failed (status %d): %s" % (what, rc, lib().nmg_batch_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            lib().nmg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def split(self, flat):
        return [flat[self.offsets[k]:self.offsets[k + 1]] for k in range(self.P)]

    def set_m(self, ms):
        flat = np.concatenate([np.asarray(m, np.float64).reshape(-1, 3) for m in ms])
        self._check(lib().nmg_batch_set_m(self.h, np.ascontiguousarray(flat).reshape(-1)), "batch_set_m")

    def get_m(self):
        out = np.zeros(3 * self.N)
        self._check(lib().nmg_batch_get_m(self.h, out), "batch_get_m")
        return self.split(out.reshape(-1, 3))

    def eval(self):
        f = np.zeros(3 * self.N)
        H = np.zeros(3 * self.N)
        self._check(lib().nmg_batch_eval(self.h, f.ctypes.data, H.ctypes.data), "batch_eval")
        return self.split(f.reshape(-1, 3)), self.split(H.reshape(-1, 3))

    def run(self, launches=1):
        self._check(lib().nmg_batch_run(self.h, int(launches)), "batch_run")

    def state(self):
        t = np.zeros(self.P)
        stage = np.zeros(self.P, np.int32)
        steps = np.zeros(self.P, np.int64)
        rhs = np.zeros(self.P, np.int64)
        done = np.zeros(self.P, np.int32)
        dmdt = np.zeros(self.P)
        self._check(lib().nmg_batch_state(self.h, t.ctypes.data, stage.ctypes.data, steps.ctypes.data,
                                          rhs.ctypes.data, done.ctypes.data, dmdt.ctypes.data), "batch_state")
        return {"t": t, "stage": stage, "steps": steps, "rhs": rhs, "done": done, "max_dmdt": dmdt}

    def set_schedule(self, threads, budget):
        self._check(lib().nmg_batch_set_schedule(self.h, int(threads), float(budget)), "batch_set_schedule")

    def autotune(self, trial_launches=2):
        t, b = C.c_int(), C.c_double()
        self._check(lib().nmg_batch_autotune(self.h, int(trial_launches), C.byref(t), C.byref(b)), "batch_autotune")
        return t.value, b.value
