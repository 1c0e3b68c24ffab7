"""Dense FP64 torch restatement of the LLG right-hand side with per-element
parameters and of its fixed-step RK4 trajectory.  Test infrastructure: its
autograd gradient is the reference the CUDA discrete adjoint is checked
against, and its RHS is itself checked against the C oracle.

Model (interface/nmag/nmag_lam.py:734-832 with per-element weights):
  H_exch = -c_exch / V * (sum_T wK_T K_T) m
  rho_i  = Ms sum_T wD_T (|det_T|/24) grad(lambda_a) . sum_{b in T} m_b
  phi1   = K^+ rho (mean-free), phi2 = BEM harmonic extension of B phi1_b
  H_demag = -G (phi1 + phi2) / V
  H_anis = c (a.m)(a - (a.m) m), c = sum_T (|det_T|/24) kappa_T / V
  dm/dt  = C1 m x H + C2 m x (m x H) + C3 (1 - m.m) m
Element matrices come from the tetrahedra's coordinates here (inverse of
the 4x4 point matrix), independently of the device and oracle assembly.
"""
import numpy as np
import torch

f64 = torch.float64


class DenseLLG(object):
    def __init__(self, points, tets, bem, node_of_b, coeffs, axis=(0.0, 0.0, 1.0)):
        P = torch.as_tensor(np.asarray(points, np.float64))
        Tt = torch.as_tensor(np.asarray(tets, np.int64))
        N, T = P.shape[0], Tt.shape[0]
        self.N, self.T, self.tets = N, T, Tt
        X = P[Tt]                                                   # T,4,3
        Mpt = torch.cat([torch.ones(T, 4, 1, dtype=f64), X], dim=2)  # rows [1, x_b]
        Cinv = torch.linalg.inv(Mpt)                                # lambda_a = Cinv[:, :, a] . [1, x]
        g = Cinv[:, 1:4, :].transpose(1, 2).contiguous()            # T,4,3 gradients
        adet = torch.linalg.det(Mpt).abs()
        self.g, self.adet = g, adet
        self.V = torch.zeros(N, dtype=f64).index_add_(0, Tt.reshape(-1), (adet / 24.0).repeat_interleave(4))
        I = Tt[:, :, None].expand(T, 4, 4).reshape(-1)
        J = Tt[:, None, :].expand(T, 4, 4).reshape(-1)
        self.I, self.J = I, J
        self.Kloc = (adet / 6.0)[:, None, None] * (g @ g.transpose(1, 2))   # T,4,4
        K = torch.zeros(N, N, dtype=f64).index_put_((I, J), self.Kloc.reshape(-1), accumulate=True)
        self.K = K
        # G_c[i][j] = sum_T (|det|/24) d_c lambda_j
        self.G = []
        for c in range(3):
            Gl = (adet / 24.0)[:, None, None] * g[:, None, :, c].expand(T, 4, 4)
            self.G.append(torch.zeros(N, N, dtype=f64).index_put_((I, J), Gl.reshape(-1), accumulate=True))
        self.Ainv = torch.linalg.inv(K + 1.0 / N)
        nob = torch.as_tensor(np.asarray(node_of_b, np.int64))
        self.nob = nob
        isb = torch.zeros(N, dtype=torch.bool)
        isb[nob] = True
        inner = torch.nonzero(~isb).reshape(-1)
        nb = nob.numel()
        Dmap = torch.zeros(N, nb, dtype=f64)
        Dmap[nob, torch.arange(nb)] = 1.0
        if inner.numel():
            Dmap[inner] = -torch.linalg.solve(K[inner][:, inner], K[inner][:, nob])
        self.Dmap = Dmap
        self.B = torch.as_tensor(np.asarray(bem, np.float64))
        self.c = coeffs
        a = torch.as_tensor(np.asarray(axis, np.float64))
        self.axis = a / a.norm()

    def operators(self, wK, wD, kappa):
        """Parameter-dependent pieces: the weighted exchange matrix, the
        per-element charge factors and the per-node anisotropy coefficient."""
        Kx = torch.zeros(self.N, self.N, dtype=f64).index_put(
            (self.I, self.J), (wK[:, None, None] * self.Kloc).reshape(-1), accumulate=True)
        qfac = (self.c["Ms"] * wD * self.adet / 24.0)[:, None, None] * self.g          # T,4,3
        can = torch.zeros(self.N, dtype=f64).index_add(
            0, self.tets.reshape(-1), ((self.adet / 24.0) * kappa).repeat_interleave(4)) / self.V
        return Kx, qfac, can

    def rhs(self, m, ops, hext, demag=True):
        Kx, qfac, can = ops
        c = self.c
        V = self.V[:, None]
        H = hext - c["exch_coeff"] * (Kx @ m) / V
        if demag:
            msum = m[self.tets].sum(1)                                                   # T,3
            q = (qfac * msum[:, None, :]).sum(-1)                                        # T,4
            rho = torch.zeros(self.N, dtype=f64).index_add(0, self.tets.reshape(-1), q.reshape(-1))
            phi1 = self.Ainv @ (rho - rho.mean())
            phi = phi1 + self.Dmap @ (self.B @ phi1[self.nob])
            H = H - torch.stack([Gc @ phi for Gc in self.G], dim=1) / V
        a = self.axis
        am = m @ a
        H = H + can[:, None] * am[:, None] * (a[None, :] - am[:, None] * m)
        mxH = torch.cross(m, H, dim=1)
        mm = (m * m).sum(1, keepdim=True)
        return c["C1"] * mxH + c["C2"] * torch.cross(m, mxH, dim=1) + c["C3"] * (1.0 - mm) * m, H

    def average(self, m):
        return (self.V[:, None] * m).sum(0) / self.V.sum()

    def trajectory(self, m0, wK, wD, kappa, pulses, hbase, dt, nsteps, steps_per_pulse, demag=True):
        ops = self.operators(wK, wD, kappa)
        m = m0.reshape(self.N, 3)
        pul = pulses.reshape(-1, 3)
        hist = []
        for n in range(nsteps):
            k = n // steps_per_pulse
            he = hbase + pul[k][None, :] if k < pul.shape[0] else hbase
            k1, _ = self.rhs(m, ops, he, demag)
            k2, _ = self.rhs(m + 0.5 * dt * k1, ops, he, demag)
            k3, _ = self.rhs(m + 0.5 * dt * k2, ops, he, demag)
            k4, _ = self.rhs(m + dt * k3, ops, he, demag)
            m = m + (dt / 6.0) * (((k1 + 2.0 * k2) + 2.0 * k3) + k4)
            hist.append(self.average(m))
        return m.reshape(-1), torch.stack(hist)
