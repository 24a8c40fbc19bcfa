"""Gradients of an observable of a BSSN evolution with respect to the
Brill-Lindquist masses and positions, by forward mode (tangent-linear
evolution).

The forward problem is a BSSN evolution (BSSN/BSSN_RHSs.py:28-328 with the
gauge RHSs of BSSN/BSSN_gauge_RHSs.py) from Brill-Lindquist data
(BSSN/BrillLindquist.py:36-82: masses m1, m2 at x1, x2), the reference's RK4
step with its curvilinear boundary conditions and det(gammabar) rescale
after every substep, FP64.  The observable is the L2 norm of the lapse's
departure from 1 over a radial shell and the evolution,

    J = sqrt( sum_{n=1..N} dt sum_q w_q (alpha(q, t_n) - 1)^2 ),

on the i0 = const shell (spherical-type grids: weights r^2 sin(theta)
dtheta dphi; Cartesian grids: the x = const plane with weights dy dz).

BSSN is nonlinear, so the derivative needs the Jacobian of every step along
the trajectory.  With up to four parameters at a time, the state and one
tangent state per parameter evolve together (BSSN_tangent_step: the RHS
algebra instantiated with dual numbers, the boundary conditions applied to
each tangent, the linearised rescale), and the gradient accumulates along
the way: one pass, no stored trajectory, no recomputation.  The derivative
is exact for the discretised problem.  The same code with no tangents is
the plain evolution (value_only), so the finite-difference checks compare
the very discrete map that is differentiated.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .grid import Grid

PARAMS = ("m1", "m2", "x1", "y1", "z1", "x2", "y2", "z2")
NUM_EVOL_GFS = 24
ALPHA = 6


def shell_weights_any(grid: Grid, i0):
    """Weights of the shell i0: r^2 sin(theta) dtheta dphi on spherical-type
    grids, dxx1 dxx2 on Cartesian grids (q = j1 + Nxx1 * j2 order)."""
    from .adjoint import shell_weights
    pr = grid.params
    if pr.CoordSystem == 0:
        return np.full(pr.Nxx1 * pr.Nxx2, pr.dxx1 * pr.dxx2)
    return shell_weights(grid, i0)


class BrillLindquistGradient:
    """J and dJ/d(params) for a BSSN evolution of n_steps from
    Brill-Lindquist data; params: up to four names of PARAMS."""

    def __init__(self, grid: Grid, shell_i0, n_steps, CFL=0.5, params=("m1", "m2", "z1", "z2"), device="cuda"):
        from .mol import Evolution
        params = tuple(params)
        if not params or len(params) > 4 or any(p not in PARAMS for p in params):
            raise ValueError("params: one to four of %s" % (PARAMS,))
        pr = grid.params
        if not (pr.NGHOSTS <= shell_i0 < pr.Nxx_plus_2NGHOSTS0 - pr.NGHOSTS):
            raise ValueError("shell_i0 must be an interior index")
        self.lib = _lib.load()
        # the grid's reference-metric tables and boundary map (its state buffers stay unused)
        self.ev = Evolution("BSSN", grid, precision="fp64", device=device)
        self.grid, self.device = grid, self.ev.device
        self.params = params
        self.pidx = (C.c_int * 4)(*([PARAMS.index(p) for p in params] + [0] * (4 - len(params))))
        self.ntan = len(params) if len(params) != 3 else 4  # built for 0, 1, 2, 4 tangents
        self.i0 = int(shell_i0)
        self.n_steps = int(n_steps)
        self.dt = grid.find_timestep(CFL)
        self.wts = torch.tensor(shell_weights_any(grid, shell_i0), dtype=torch.float64, device=self.device)
        self.p = C.byref(pr)
        self.ntot = grid.ntot

    def _run(self, m1, x1, m2, x2, ntan):
        ev = self.ev
        ev._sync_stream()
        z = dict(dtype=torch.float64, device=self.device)
        Y = torch.zeros(((ntan + 1) * NUM_EVOL_GFS,) + tuple(self.grid.shape), **z)
        scratch = torch.zeros((ntan + 1) * 78 * self.ntot, **z)
        accum = torch.zeros(5, **z)
        X1 = (C.c_double * 3)(*[float(v) for v in x1])
        X2 = (C.c_double * 3)(*[float(v) for v in x2])
        _lib.check(self.lib.BSSN_tangent_initial_data_BrillLindquist(self.p, float(m1), X1, float(m2), X2, ntan,
                                                                     self.pidx, _lib.ptr(Y)),
                   "BSSN_tangent_initial_data_BrillLindquist")
        for _ in range(self.n_steps):
            _lib.check(self.lib.BSSN_tangent_step(ev._rfm(), self.p, C.byref(ev.bc), ntan, _lib.ptr(Y),
                                                  _lib.ptr(scratch), float(self.dt)), "BSSN_tangent_step")
            _lib.check(self.lib.BSSN_tangent_shell_accumulate(self.p, ntan, _lib.ptr(Y), ALPHA, self.i0,
                                                              _lib.ptr(self.wts), float(self.dt), 1.0,
                                                              _lib.ptr(accum)), "BSSN_tangent_shell_accumulate")
        a = accum.cpu().numpy()
        J = float(np.sqrt(a[0]))
        return J, a[1:1 + ntan] / (2.0 * J) if ntan else np.zeros(0)

    def value_only(self, m1, x1, m2, x2):
        """J alone (the same discrete evolution, no tangents)."""
        return self._run(m1, x1, m2, x2, 0)[0]

    def value_and_gradient(self, m1, x1, m2, x2):
        """(J, dJ/d(params)) in the order of `params`."""
        J, g = self._run(m1, x1, m2, x2, self.ntan)
        return J, g[:len(self.params)]

    @staticmethod
    def unpack(theta):
        """(m1, x1, m2, x2) from the 8 parameters in PARAMS order."""
        t = [float(v) for v in theta]
        return t[0], t[2:5], t[1], t[5:8]


class _BLFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, model):
        m1, x1, m2, x2 = BrillLindquistGradient.unpack(theta.detach().cpu().numpy())
        J, g = model.value_and_gradient(m1, x1, m2, x2)
        full = np.zeros(8)
        for k, name in enumerate(model.params):
            full[PARAMS.index(name)] = g[k]
        ctx.grad = torch.tensor(full, dtype=theta.dtype, device=theta.device)
        return torch.tensor(J, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, gJ):
        return gJ * ctx.grad, None


def brill_lindquist_observable(theta, model: BrillLindquistGradient):
    """J as a differentiable torch function of theta = (m1, m2, x1, y1, z1,
    x2, y2, z2); the gradient is exact in the model's params and zero in
    the others."""
    return _BLFn.apply(theta, model)
