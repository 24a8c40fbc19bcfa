"""Gradients of wave-extraction observables of linear evolutions with
respect to their initial-data parameters, by the discrete adjoint.

Two forward problems, both this library's RK4 evolution
(MoL_step_forward_in_time, the outer boundary conditions after every
substep):

* MaxwellExtraction: vacuum Maxwell System I
  (Maxwell/VacuumMaxwell_Flat_Evol_Cartesian.py:54-74) on a Cartesian grid
  from toroidal-dipole data (Maxwell/InitialData.py:41-104) with amplitude
  `amp` and width parameter `lam`; the observable is the L2 norm of E over
  an extraction sphere and the evolution,
      J(amp, lam) = sqrt( sum_{n=1..N} dt sum_p w_p |E(x_p, t_n)|^2 ),
  with tricubic interpolation to the sphere points x_p and surface weights
  w_p = r^2 sin(theta) dtheta dphi.
* ScalarWaveExtraction: the scalar wave equation
  (ScalarWave/ScalarWaveCurvilinear_RHSs.py:43-98) on a Cartesian or
  curvilinear grid from a Gaussian pulse uu = A exp(-(r - r0)^2 / w^2),
  vv = 0; the observable is the L2 norm of uu over a radial shell (the
  i0 = const surface of a spherical-type grid, its grid points themselves,
  no interpolation) and the evolution,
      J(A, r0, w) = sqrt( sum_{n=1..N} dt sum_q w_q uu(shell_q, t_n)^2 ),
  w_q = r^2 sin(theta) dtheta dphi at the shell points.

Gradients come from the hand-written transposes in libnrgpu
(MoL_adjoint_step_backward, nrgpu_sphere_sample_adjoint,
nrgpu_shell_sample_adjoint), exact for the discretised problem, and are
exposed as torch.autograd.Functions.

Checkpoints: the forward pass keeps the state every `checkpoint_every`
steps.  By default it also keeps the observable's samples of every step (a
few MB), which is all the backward pass needs because the systems are
linear; with keep_samples=False it keeps only the checkpoints and the
backward pass recomputes each segment's samples from its checkpoint (the
general scheme for observables along the trajectory), with identical
results.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .grid import Grid


class ExtractionSphere:
    """Midpoint-rule sphere of radius r: ntheta x nphi points, weights
    r^2 sin(theta) dtheta dphi (they sum to ~4 pi r^2)."""

    def __init__(self, radius, ntheta=32, nphi=64, center=(0.0, 0.0, 0.0)):
        th = (np.arange(ntheta) + 0.5) * np.pi / ntheta
        ph = (np.arange(nphi) + 0.5) * 2 * np.pi / nphi
        T, P = np.meshgrid(th, ph, indexing="ij")
        self.radius = float(radius)
        self.points = np.stack([center[0] + radius * np.sin(T) * np.cos(P),
                                center[1] + radius * np.sin(T) * np.sin(P),
                                center[2] + radius * np.cos(T)], axis=-1).reshape(-1, 3)
        self.weights = (radius ** 2 * np.sin(T) * (np.pi / ntheta) * (2 * np.pi / nphi)).reshape(-1)

    @property
    def n(self):
        return self.points.shape[0]


class _AdjointExtraction:
    """Checkpointed forward evolution of a linear system, an observable
    J = sqrt(sum_n dt * samples_n), and its adjoint gradient.  Subclasses
    give the initial data with parameter derivatives and the sampling."""

    system = None
    NPARAM = 0

    def __init__(self, grid: Grid, n_steps, CFL, checkpoint_every, keep_samples, device, sample_shape):
        from .mol import Evolution
        self.lib = _lib.load()
        self.ev = Evolution(self.system, grid, precision="fp64", device=device)
        self.grid = grid
        self.device = self.ev.device
        self.n_steps = int(n_steps)
        self.dt = grid.find_timestep(CFL)
        self.K = int(checkpoint_every)
        self.keep_samples = keep_samples
        z = dict(dtype=torch.float64, device=self.device)
        nsamp = self.n_steps if keep_samples else self.K
        self.samples = torch.zeros((nsamp,) + tuple(sample_shape), **z)
        self.J2 = torch.zeros(1, **z)
        self.scratch_J2 = torch.zeros(1, **z)
        self.checkpoints = {}
        self.params = None
        self.p = C.byref(grid.params)

    # -- subclass hooks
    def _sample(self, y, out, accum):
        raise NotImplementedError

    def _sample_adjoint(self, samples, target):
        raise NotImplementedError

    def _check_samples(self):
        pass

    def initial_data(self, *params, out=None, derivs=None):
        raise NotImplementedError

    # -- pieces
    def _sync(self):
        self.ev._sync_stream()

    # -- forward
    def forward(self, *params):
        """Evolves n_steps from the data of `params`; returns J (float)."""
        if len(params) != self.NPARAM:
            raise ValueError("expected %d parameters" % self.NPARAM)
        self._sync()
        self.params = tuple(float(v) for v in params)
        ev = self.ev
        self.initial_data(*self.params, out=ev.y_n)
        self.J2.zero_()
        self.checkpoints = {0: ev.y_n.clone()}
        for n in range(1, self.n_steps + 1):
            ev.step(self.dt)
            slot = (n - 1) if self.keep_samples else (n - 1) % self.K
            self._sample(ev.y_n, self.samples[slot], self.J2)
            if n % self.K == 0 or n == self.n_steps:
                self.checkpoints[n] = ev.y_n.clone()
        self._check_samples()
        return float(torch.sqrt(self.J2).item())

    def _segment_samples(self, start, stop):
        """Recomputes the samples of steps start+1..stop from checkpoint `start`."""
        ev = self.ev
        ev.y_n.copy_(self.checkpoints[start])
        for n in range(start + 1, stop + 1):
            ev.step(self.dt)
            self._sample(ev.y_n, self.samples[n - start - 1], self.scratch_J2)

    def adjoint_initial_state(self):
        """dJ/dy_0 (the adjoint at the initial state) as a device tensor."""
        if self.params is None:
            raise RuntimeError("run forward() first")
        self._sync()
        ev = self.ev
        shape = ev.y_n.shape
        z = dict(dtype=torch.float64, device=self.device)
        lam_a = torch.zeros(shape, **z)
        lam_b = torch.zeros(shape, **z)
        scratch = torch.zeros((4,) + tuple(shape), **z)
        N, K = self.n_steps, self.K
        seg_start = ((N - 1) // K) * K
        if not self.keep_samples:
            self._segment_samples(seg_start, N)

        def seed(n, target):
            # gradient of J with respect to y_n (n >= 1)
            slot = (n - 1) if self.keep_samples else (n - 1 - seg_start)
            self._sample_adjoint(self.samples[slot], target)

        seed(N, lam_a)
        for n in range(N, 0, -1):
            _lib.check(self.lib.MoL_adjoint_step_backward(ev.sys_id, ev._rfm(), self.p, C.byref(ev.bc),
                                                          _lib.ptr(lam_a), _lib.ptr(lam_b), _lib.ptr(scratch),
                                                          float(self.dt)), "MoL_adjoint_step_backward")
            lam_a, lam_b = lam_b, lam_a
            m = n - 1  # lam_a is now dJ/dy_m (without y_m's own samples)
            if m >= 1:
                if not self.keep_samples and m <= seg_start:
                    seg_start -= K
                    self._segment_samples(seg_start, seg_start + K)
                seed(m, lam_a)
        if not self.keep_samples:  # leave the evolution at the final state, as after forward()
            ev.y_n.copy_(self.checkpoints[N])
        return lam_a

    # -- backward
    def gradient(self):
        """dJ/d(params) by the discrete adjoint (float64 numpy array)."""
        lam = self.adjoint_initial_state()
        z = dict(dtype=torch.float64, device=self.device)
        derivs = [torch.zeros_like(lam) for _ in range(self.NPARAM)]
        self.initial_data(*self.params, derivs=derivs)
        res = torch.zeros(self.NPARAM, **z)
        part = torch.zeros(1024, **z)
        n = lam.numel()
        for k, d in enumerate(derivs):
            _lib.check(self.lib.nrgpu_dot(_lib.ptr(lam), _lib.ptr(d), n, _lib.ptr(part), 1024,
                                          _lib.ptr(res[k:k + 1])), "nrgpu_dot")
        return res.cpu().numpy()


class MaxwellExtraction(_AdjointExtraction):
    """Maxwell System I from toroidal-dipole data (amp, lam); J over an
    extraction sphere."""

    system = "Maxwell"
    NPARAM = 2
    E0, NE = 3, 3  # EU0..EU2 in the alphabetical gf order AU0-2, EU0-2, psi

    def __init__(self, grid: Grid, sphere: ExtractionSphere, n_steps, CFL=0.5, checkpoint_every=20,
                 keep_samples=True, device="cuda"):
        if grid.params.CoordSystem != 0:
            raise ValueError("Maxwell System I is Cartesian only")
        super().__init__(grid, n_steps, CFL, checkpoint_every, keep_samples, device, (sphere.n, self.NE))
        z = dict(dtype=torch.float64, device=self.device)
        self.pts = torch.tensor(sphere.points, **z).contiguous()
        self.wts = torch.tensor(sphere.weights, **z).contiguous()
        self.npts = sphere.n

    def _sample(self, y, out, accum):
        _lib.check(self.lib.nrgpu_sphere_sample(self.p, _lib.ptr(y), self.E0, self.NE, _lib.ptr(self.pts),
                                                _lib.ptr(self.wts), self.npts, float(self.dt), _lib.ptr(out),
                                                _lib.ptr(accum)), "nrgpu_sphere_sample")

    def _sample_adjoint(self, samples, target):
        _lib.check(self.lib.nrgpu_sphere_sample_adjoint(
            self.p, _lib.ptr(samples), self.E0, self.NE, _lib.ptr(self.pts), _lib.ptr(self.wts),
            self.npts, float(self.dt), _lib.ptr(self.J2), _lib.ptr(target)), "nrgpu_sphere_sample_adjoint")

    def _check_samples(self):
        flag = C.c_int()
        _lib.check(self.lib.nrgpu_sphere_check(self.p, C.byref(flag)), "nrgpu_sphere_check")
        if flag.value:
            raise ValueError("extraction sphere leaves the grid (tricubic stencil out of range)")

    def initial_data(self, amp, lam, out=None, derivs=None, d_amp=None, d_lam=None):
        if derivs is not None:
            d_amp, d_lam = derivs
        self._sync()
        _lib.check(self.lib.Maxwell_initial_data_toroidal_dipole(self.p, float(amp), float(lam), 0.0,
                                                                 _lib.ptr(out), _lib.ptr(d_amp), _lib.ptr(d_lam)),
                   "Maxwell_initial_data_toroidal_dipole")


# Coordinate systems whose xx0 is a radius and (xx1, xx2) = (theta, phi).
_SPHERICAL_TYPE = {1, 2, 3}  # Spherical, SinhSpherical, SinhSphericalv2


def shell_weights(grid: Grid, i0):
    """Surface weights r^2 sin(theta) dtheta dphi at the Nxx1*Nxx2 interior
    points of shell i0 of a spherical-type grid (q = j1 + Nxx1 * j2 order),
    r the shell's radius from the library's xx_to_Cart."""
    pr = grid.params
    if pr.CoordSystem not in _SPHERICAL_TYPE:
        raise ValueError("radial shells need a spherical-type CoordSystem (Spherical, SinhSpherical(v2))")
    lib = _lib.load()
    g = pr.NGHOSTS
    x = (C.c_double * 3)()
    _lib.check(lib.xx_to_Cart(C.byref(pr), None, int(i0), g, g, x), "xx_to_Cart")
    r = float(np.sqrt(x[0] ** 2 + x[1] ** 2 + x[2] ** 2))
    th = pr.xxmin1 + (np.arange(pr.Nxx1) + 0.5) * pr.dxx1
    w = r * r * np.sin(th)[None, :] * pr.dxx1 * pr.dxx2 * np.ones((pr.Nxx2, 1))
    return np.ascontiguousarray(w.reshape(-1))  # q = j1 + Nxx1 * j2


class ScalarWaveExtraction(_AdjointExtraction):
    """ScalarWave from a Gaussian pulse (A, r0, w); J over the radial shell
    i0 = shell_i0 of a spherical-type grid."""

    system = "ScalarWave"
    NPARAM = 3

    def __init__(self, grid: Grid, shell_i0, n_steps, CFL=0.5, checkpoint_every=20, keep_samples=True,
                 device="cuda"):
        pr = grid.params
        if not (pr.NGHOSTS <= shell_i0 < pr.Nxx_plus_2NGHOSTS0 - pr.NGHOSTS):
            raise ValueError("shell_i0 must be an interior index")
        w = shell_weights(grid, shell_i0)
        super().__init__(grid, n_steps, CFL, checkpoint_every, keep_samples, device, (w.size,))
        self.i0 = int(shell_i0)
        self.wts = torch.tensor(w, dtype=torch.float64, device=self.device)

    def _sample(self, y, out, accum):
        _lib.check(self.lib.nrgpu_shell_sample(self.p, _lib.ptr(y), 0, self.i0, _lib.ptr(self.wts),
                                               float(self.dt), _lib.ptr(out), _lib.ptr(accum)),
                   "nrgpu_shell_sample")

    def _sample_adjoint(self, samples, target):
        _lib.check(self.lib.nrgpu_shell_sample_adjoint(self.p, _lib.ptr(samples), 0, self.i0, _lib.ptr(self.wts),
                                                       float(self.dt), _lib.ptr(self.J2), _lib.ptr(target)),
                   "nrgpu_shell_sample_adjoint")

    def initial_data(self, A, r0, w, out=None, derivs=None):
        d = derivs if derivs is not None else (None, None, None)
        self._sync()
        _lib.check(self.lib.ScalarWave_initial_data_gaussian(self.p, float(A), float(r0), float(w), _lib.ptr(out),
                                                             _lib.ptr(d[0]), _lib.ptr(d[1]), _lib.ptr(d[2])),
                   "ScalarWave_initial_data_gaussian")


class _ExtractionFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, model):
        J = model.forward(*[float(v) for v in params])
        ctx.model = model
        return torch.tensor(J, dtype=torch.float64, device=params.device)

    @staticmethod
    def backward(ctx, gJ):
        g = torch.tensor(ctx.model.gradient(), dtype=torch.float64, device=gJ.device)
        return gJ * g, None


def extraction_observable(params, model: _AdjointExtraction):
    """J as a differentiable torch function of params ([amp, lam] for
    MaxwellExtraction, [A, r0, w] for ScalarWaveExtraction)."""
    return _ExtractionFn.apply(params, model)
