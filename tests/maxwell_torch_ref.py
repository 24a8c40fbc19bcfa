"""PyTorch-autograd reference of the differentiated Maxwell problem.

The same discrete forward problem as nrpytutorial_gb300.adjoint (toroidal
dipole data, Maxwell System I RHS with FD4 on a Cartesian grid, the library's
RK4 step with the outer boundary conditions after every substep, tricubic
sampling on an extraction sphere, J = sqrt(sum_n dt sum_p w_p |E|^2)),
written with differentiable torch ops (float64, CPU) so that torch.autograd
gives a reference gradient.  The boundary map comes from the oracle
(oracle/bcs.py); this module is test infrastructure.
"""
import numpy as np
import torch

import oracle.bcs as obc
import oracle.grid as og
from oracle.fd import coeff_table


class TorchMaxwell:
    def __init__(self, N, domain, sphere_points, sphere_weights, n_steps, CFL=0.5, fd_order=4):
        self.gp = og.GridParams("Cartesian", (N, N, N), fd_order // 2 + 1, fd_order, domain=domain)
        gp = self.gp
        self.ng = gp.NGHOSTS
        self.dt = og.find_timestep(gp, CFL)
        self.n_steps = n_steps
        c = coeff_table(fd_order)  # full stencils, offsets -R..R
        self.R = R = fd_order // 2
        self.c1 = [float(c[0][R + k]) for k in range(R + 1)]  # c1[k], k = 0..R (c1[0] = 0)
        self.c2 = [float(c[1][R + k]) for k in range(R + 1)]
        self.layers = []
        for outer_dirs, _ in obc.build_bcstruct(gp):
            ph = []
            for arr in outer_dirs:
                if len(arr):
                    ph.append((torch.tensor(arr[:, 0]), torch.tensor(arr[:, 1])))
            self.layers.append(ph)
        # tricubic weights (numpy, constant)
        idx, w = [], []
        n = gp.np
        for x in sphere_points:
            base, ws = [], []
            for d in range(3):
                j = (x[d] - gp.xxmin[d]) / gp.dxx[d] + gp.NGHOSTS - 0.5
                f = np.floor(j)
                s = j - f
                base.append(int(f) - 1)
                ws.append([-s * (s - 1) * (s - 2) / 6, (s + 1) * (s - 1) * (s - 2) / 2,
                           -(s + 1) * s * (s - 2) / 2, (s + 1) * s * (s - 1) / 6])
            ii, ww = [], []
            for cc in range(4):
                for b in range(4):
                    for a in range(4):
                        ii.append((base[0] + a) + n[0] * ((base[1] + b) + n[1] * (base[2] + cc)))
                        ww.append(ws[0][a] * ws[1][b] * ws[2][cc])
            idx.append(ii)
            w.append(ww)
        self.sidx = torch.tensor(np.array(idx), dtype=torch.int64)
        self.sw = torch.tensor(np.array(w), dtype=torch.float64)
        self.pw = torch.tensor(np.asarray(sphere_weights), dtype=torch.float64)

    def initial_data(self, amp, lam):
        gp = self.gp
        z, y, x = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
        x, y, z = (torch.tensor(a) for a in (x, y, z))
        r = torch.sqrt(x * x + y * y + z * z)
        u, v = r, -r  # t = 0
        eu, ev = torch.exp(-lam * u ** 2), torch.exp(-lam * v ** 2)
        deu, dev = -2 * lam * u * eu, -2 * lam * v * ev
        F = amp / r * ((ev - eu) / r ** 2 - 2 * lam * (v * ev + u * eu) / r)
        dF = amp / r * ((dev - deu) / r ** 2 - 2 * lam * (ev + v * dev + eu + u * deu) / r)
        zero = torch.zeros_like(x)
        return torch.stack([-y * F, x * F, zero, y * dF, -x * dF, zero, zero])

    def _S(self, f, o):
        g = self.ng
        n2, n1, n0 = f.shape
        return f[g + o[2]:n2 - g + o[2], g + o[1]:n1 - g + o[1], g + o[0]:n0 - g + o[0]]

    def _off(self, d, k):
        o = [0, 0, 0]
        o[d] = k
        return o

    def d1(self, f, d):
        acc = 0
        for k in range(1, self.R + 1):
            acc = acc + self.c1[k] * (self._S(f, self._off(d, k)) - self._S(f, self._off(d, -k)))
        return acc * self.gp.invdx[d]

    def d2(self, f, d):
        acc = self.c2[0] * self._S(f, [0, 0, 0])
        for k in range(1, self.R + 1):
            acc = acc + self.c2[k] * (self._S(f, self._off(d, k)) + self._S(f, self._off(d, -k)))
        return acc * self.gp.invdx[d] ** 2

    def d11(self, f, d, e):
        acc = 0
        for a in range(1, self.R + 1):
            inner = 0
            for b in range(1, self.R + 1):
                def o(sa, sb):
                    v = [0, 0, 0]
                    v[d] += sa * a
                    v[e] += sb * b
                    return v
                inner = inner + self.c1[b] * ((self._S(f, o(1, 1)) - self._S(f, o(1, -1)))
                                              - (self._S(f, o(-1, 1)) - self._S(f, o(-1, -1))))
            acc = acc + self.c1[a] * inner
        return acc * self.gp.invdx[d] * self.gp.invdx[e]

    def rhs(self, y):
        A, E, psi = y[0:3], y[3:6], y[6]
        out = []
        for i in range(3):
            out.append(-self._S(E[i], [0, 0, 0]) - self.d1(psi, i))
        for i in range(3):
            acc = 0
            for j in range(3):
                if j != i:
                    acc = acc - self.d2(A[i], j) + self.d11(A[j], j, i)
            out.append(acc)
        out.append(-(self.d1(A[0], 0) + self.d1(A[1], 1) + self.d1(A[2], 2)))
        full = torch.zeros_like(y)
        g = self.ng
        full[:, g:-g, g:-g, g:-g] = torch.stack(out)
        return full

    def bcs(self, y):
        flat = y.reshape(7, -1)
        for phases in self.layers:
            for idx, st in phases:
                v = 3.0 * flat[:, idx + st] - 3.0 * flat[:, idx + 2 * st] + flat[:, idx + 3 * st]
                flat = flat.index_copy(1, idx, v)
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

    def observable(self, amp, lam):
        y = self.initial_data(amp, lam)
        J2 = 0
        for _ in range(self.n_steps):
            y = self.step(y)
            E = y[3:6].reshape(3, -1)
            s = (E[:, self.sidx] * self.sw).sum(-1)  # (3, npts)
            J2 = J2 + self.dt * (self.pw * (s * s).sum(0)).sum()
        return torch.sqrt(J2)

    def gradient(self, amp, lam):
        a = torch.tensor(float(amp), dtype=torch.float64, requires_grad=True)
        l = torch.tensor(float(lam), dtype=torch.float64, requires_grad=True)
        J = self.observable(a, l)
        ga, gl = torch.autograd.grad(J, (a, l))
        return float(J.detach()), np.array([float(ga), float(gl)])
