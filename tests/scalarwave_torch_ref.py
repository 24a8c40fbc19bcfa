"""PyTorch-autograd reference of the differentiated ScalarWave problem.

The same discrete forward problem as nrpytutorial_gb300.adjoint's
ScalarWaveExtraction on a spherical-type grid (Gaussian pulse
uu = A exp(-(r - r0)^2 / w^2), vv = 0; the curvilinear scalar-wave RHS of
ScalarWave/ScalarWaveCurvilinear_RHSs.py:43-98 at interior points; the
library's RK4 step with the extrapolation + inner-parity boundary
conditions after every substep; J = sqrt(sum_n dt sum_q w_q uu(shell_q)^2)
on the i0 = const shell), written with differentiable torch ops (float64,
CPU) so that torch.autograd gives a reference gradient.  The reference
metric and the boundary map come from the oracle (oracle/grid.py,
oracle/bcs.py); this module is test infrastructure.
"""
import numpy as np
import torch

import oracle.bcs as obc
import oracle.grid as og
from oracle.fd import coeff_table


class TorchScalarWave:
    def __init__(self, gp, shell_i0, shell_weights, n_steps, CFL=0.5, wavespeed=1.0):
        self.gp = gp
        self.ng = g = gp.NGHOSTS
        self.dt = og.find_timestep(gp, CFL)
        self.n_steps = n_steps
        self.c2 = wavespeed * wavespeed
        c = coeff_table(gp.FD_order)
        self.R = R = gp.FD_order // 2
        self.w1 = [float(c[0][R + k]) for k in range(R + 1)]
        self.w2 = [float(c[1][R + k]) for k in range(R + 1)]
        q = og.hatted_grid(gp, interior=True)
        gUU, G = q["ghatUU"], q["GammahatUDD"]
        contracted = np.einsum("ij...,kij...->k...", gUU, G)
        shape = tuple(n - 2 * g for n in reversed(gp.np))  # interior (n2, n1, n0)
        self.gd = [torch.tensor(np.broadcast_to(gUU[d, d], shape).copy()) for d in range(3)]
        self.Gd = [torch.tensor(np.broadcast_to(contracted[d], shape).copy()) for d in range(3)]
        self.layers = []
        for outer_dirs, (idst, isrc, ipar) in obc.build_bcstruct(gp):
            outer = [(torch.tensor(a[:, 0]), torch.tensor(a[:, 1])) for a in outer_dirs if len(a)]
            inner = None
            if len(idst):
                inner = (torch.tensor(idst), torch.tensor(isrc), torch.tensor(ipar[:, 0], dtype=torch.float64))
            self.layers.append((outer, inner))
        self.i0 = shell_i0
        self.sw = torch.tensor(np.asarray(shell_weights), dtype=torch.float64)
        z, y, x = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
        if gp.CoordSystem == og.CART:
            r = np.sqrt(x * x + y * y + z * z)
        else:
            # the Cartesian radius |r(xx0)| (r(xx0) < 0 at the inner ghost points)
            r = np.broadcast_to(np.abs(og.radial(gp.CoordSystem, gp.xx[0], gp.AMPL, gp.SINHW)[0]), x.shape)
        self.r = torch.tensor(np.ascontiguousarray(r))

    def initial_data(self, A, r0, w):
        u = A * torch.exp(-((self.r - r0) / w) ** 2)
        return torch.stack([u, torch.zeros_like(u)])

    def _S(self, f, o):
        g = self.ng
        n2, n1, n0 = f.shape
        return f[g + o[2]:n2 - g + o[2], g + o[1]:n1 - g + o[1], g + o[0]:n0 - g + o[0]]

    @staticmethod
    def _off(d, k):
        o = [0, 0, 0]
        o[d] = k
        return o

    def d1(self, f, d):
        acc = 0
        for k in range(1, self.R + 1):
            acc = acc + self.w1[k] * (self._S(f, self._off(d, k)) - self._S(f, self._off(d, -k)))
        return acc * self.gp.invdx[d]

    def d2(self, f, d):
        acc = self.w2[0] * self._S(f, [0, 0, 0])
        for k in range(1, self.R + 1):
            acc = acc + self.w2[k] * (self._S(f, self._off(d, k)) + self._S(f, self._off(d, -k)))
        return acc * self.gp.invdx[d] ** 2

    def rhs(self, y):
        uu, vv = y[0], y[1]
        acc = 0
        for d in range(3):
            acc = acc + self.gd[d] * self.d2(uu, d) - self.Gd[d] * self.d1(uu, d)
        g = self.ng
        full = torch.zeros_like(y)
        full[:, g:-g, g:-g, g:-g] = torch.stack([self._S(vv, [0, 0, 0]), self.c2 * acc])
        return full

    def bcs(self, y):
        flat = y.reshape(2, -1)
        for outer, inner in self.layers:
            for idx, st in outer:
                v = 3.0 * flat[:, idx + st] - 3.0 * flat[:, idx + 2 * st] + flat[:, idx + 3 * st]
                flat = flat.index_copy(1, idx, v)
            if inner is not None:
                idst, isrc, par = inner
                flat = flat.index_copy(1, idst, par * flat[:, isrc])
        return flat.reshape(y.shape)

    def step(self, y):
        dt = self.dt
        k1 = self.rhs(y)
        y1 = self.bcs(y + k1 * (dt / 2))
        k2 = self.rhs(y1)
        y2 = self.bcs(y + k2 * (dt / 2))
        k3 = self.rhs(y2)
        y3 = self.bcs(y + k3 * dt)
        k4 = self.rhs(y3)
        return self.bcs(y + (k1 * (dt / 6) + k2 * (dt / 3) + k3 * (dt / 3)) + k4 * (dt / 6))

    def observable(self, A, r0, w):
        y = self.initial_data(A, r0, w)
        g = self.ng
        J2 = 0
        for _ in range(self.n_steps):
            y = self.step(y)
            s = y[0, g:-g, g:-g, self.i0].reshape(-1)  # q = j1 + Nxx1 * j2
            J2 = J2 + self.dt * (self.sw * s * s).sum()
        return torch.sqrt(J2)

    def gradient(self, A, r0, w):
        p = [torch.tensor(float(v), dtype=torch.float64, requires_grad=True) for v in (A, r0, w)]
        J = self.observable(*p)
        gr = torch.autograd.grad(J, p)
        return float(J.detach()), np.array([float(v) for v in gr])
