"""Differentiation form: a fixed-step RK4 LLG trajectory whose per-element
Ms, per-element K1 and applied-field pulse amplitudes are parameters, with
gradients from the library's hand-written discrete adjoint
(nmg_rk4_forward / nmg_rk4_adjoint) behind a torch.autograd.Function.

The reference has one scalar Ms and K1 per material
(interface/nmag/main.py:347-465); per-element values extend its RHS
(interface/nmag/nmag_lam.py:734-832) through the element weights

    wK_T = Ms / Ms_T          exchange prefactor 2A/(mu0 Ms_T) per element
    wD_T = Ms_T / Ms          magnetic charge Ms_T m per element
    kappa_T = 2 K1_T / (mu0 Ms_T)   uniaxial anisotropy field per element

(Ms = the material's Ms).  The chain rule from (Ms_T, K1_T) to the weights
runs in torch; the trajectory and its adjoint run in CUDA.  torch is used
here only for device memory and for the autograd boundary.
"""
import numpy as np
import torch

__all__ = ["RK4Trajectory", "element_weights", "rk4_trajectory", "film_loss"]


def _ptr(t):
    return int(t.data_ptr()) if t is not None and t.numel() > 0 else 0


def _check(t, name, n=None):
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise TypeError("%s must be a contiguous float64 CUDA tensor" % name)
    if n is not None and t.numel() != n:
        raise ValueError("%s has %d values, expected %d" % (name, t.numel(), n))


class RK4Trajectory(torch.autograd.Function):
    """(m0, wK, wD, kappa, pulses) -> (m_final, <m> after every step).

    Non-tensor arguments: the engine (nmag._lib.Engine), the anisotropy axis,
    dt (simulation units), the number of steps, the checkpoint interval and the
    steps per pulse.  backward() runs the adjoint of the most recent forward on
    the same engine; another forward in between is an error."""

    @staticmethod
    def forward(ctx, m0, wK, wD, kappa, pulses, eng, axis, dt, nsteps, ckpt_every, steps_per_pulse):
        N, T = eng.N, eng.T
        _check(m0, "m0", 3 * N)
        for t, name in ((wK, "wK"), (wD, "wD"), (kappa, "kappa")):
            _check(t, name, T)
        _check(pulses, "pulses")
        n_pulses = pulses.numel() // 3
        torch.cuda.synchronize()
        eng.set_element_params(_ptr(wK), _ptr(wD), _ptr(kappa), axis)
        mT = torch.empty_like(m0)
        hist = torch.empty(nsteps, 3, dtype=torch.float64, device=m0.device)
        eng.rk4_forward(_ptr(m0), float(dt), int(nsteps), int(ckpt_every), _ptr(pulses), n_pulses,
                        int(steps_per_pulse), _ptr(mT), _ptr(hist))
        eng._rk4_token = getattr(eng, "_rk4_token", 0) + 1
        ctx.eng, ctx.token, ctx.axis = eng, eng._rk4_token, axis
        ctx.n_pulses = n_pulses
        ctx.save_for_backward(wK, wD, kappa)
        return mT, hist

    @staticmethod
    def backward(ctx, g_mT, g_hist):
        eng = ctx.eng
        if getattr(eng, "_rk4_token", None) != ctx.token:
            raise RuntimeError("RK4Trajectory.backward: another forward ran on this engine since")
        wK, wD, kappa = ctx.saved_tensors
        dev = wK.device
        g_mT = torch.zeros(3 * eng.N, dtype=torch.float64, device=dev) if g_mT is None else g_mT.contiguous()
        g_hist = None if g_hist is None else g_hist.contiguous()
        g_m0 = torch.empty(3 * eng.N, dtype=torch.float64, device=dev)
        g_wK = torch.empty(eng.T, dtype=torch.float64, device=dev)
        g_wD = torch.empty_like(g_wK)
        g_kap = torch.empty_like(g_wK)
        g_pul = torch.zeros(3 * max(ctx.n_pulses, 1), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        eng.set_element_params(_ptr(wK), _ptr(wD), _ptr(kappa), ctx.axis)
        eng.rk4_adjoint(_ptr(g_mT), _ptr(g_hist), _ptr(g_m0), _ptr(g_wK), _ptr(g_wD), _ptr(g_kap),
                        _ptr(g_pul) if ctx.n_pulses else 0)
        g_pul = g_pul[:3 * ctx.n_pulses]
        return g_m0, g_wK, g_wD, g_kap, g_pul, None, None, None, None, None, None


def element_weights(Ms_T, K1_T, Ms, mu0):
    """(wK, wD, kappa) from per-element Ms_T and K1_T (simulation units)."""
    wK = Ms / Ms_T
    wD = Ms_T / Ms
    kappa = 2.0 * K1_T / (mu0 * Ms_T)
    return wK, wD, kappa


def rk4_trajectory(eng, m0, Ms_T, K1_T, pulses, axis, Ms, mu0, dt, nsteps, ckpt_every=50, steps_per_pulse=1):
    """Differentiable RK4 trajectory: returns (m_final, <m> history)."""
    wK, wD, kappa = element_weights(Ms_T, K1_T, Ms, mu0)
    return RK4Trajectory.apply(m0, wK.contiguous(), wD.contiguous(), kappa.contiguous(), pulses.reshape(-1),
                               eng, np.asarray(axis, np.float64), dt, nsteps, ckpt_every, steps_per_pulse)


def film_loss(hist, target=(0.0, 1.0, 0.0), weight=1e-3):
    """||<m>(T) - target||^2 + weight * mean over steps of <m>_x^2."""
    tgt = torch.as_tensor(target, dtype=hist.dtype, device=hist.device)
    return ((hist[-1] - tgt) ** 2).sum() + weight * (hist[:, 0] ** 2).mean()
