"""Gradients of a wave-extraction observable of a Maxwell evolution with
respect to its initial-data parameters, by the discrete adjoint.

The forward problem is this library's evolution of vacuum Maxwell System I
(Maxwell/VacuumMaxwell_Flat_Evol_Cartesian.py:54-74) from toroidal-dipole
data (Maxwell/InitialData.py:41-104) with amplitude `amp` and width
parameter `lam`, RK4 (MoL_step_forward_in_time) with the outer boundary
conditions after every substep.  The observable is the L2 norm of E over an
extraction sphere and the evolution,

    J(amp, lam) = sqrt( sum_{n=1..N} dt sum_p w_p |E(x_p, t_n)|^2 ),

with tricubic interpolation to the sphere points x_p and surface weights
w_p = r^2 sin(theta) dtheta dphi.  Its gradient is computed by the
hand-written transposes in libnrgpu (MoL_adjoint_step_backward,
nrgpu_sphere_sample_adjoint), exact for the discretised problem, and exposed
as a torch.autograd.Function.

Checkpoints: the forward pass keeps the state every `checkpoint_every`
steps.  By default it also keeps the sphere samples of every step (a few
MB), which is all the backward pass needs because the system is linear;
with keep_samples=False it keeps only the checkpoints and the backward pass
recomputes each segment's samples from its checkpoint (the general scheme
for observables along the trajectory), with identical results.
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


class MaxwellExtraction:
    """Forward evolution + observable, and its adjoint gradient."""

    E0, NE = 3, 3  # EU0..EU2 in the alphabetical gf order AU0-2, EU0-2, psi

    def __init__(self, grid: Grid, sphere: ExtractionSphere, n_steps, CFL=0.5, checkpoint_every=20,
                 keep_samples=True, device="cuda"):
        from .mol import Evolution
        if grid.params.CoordSystem != 0:
            raise ValueError("Maxwell System I is Cartesian only")
        self.lib = _lib.load()
        self.ev = Evolution("Maxwell", grid, precision="fp64", device=device)
        self.grid = grid
        self.device = self.ev.device
        self.n_steps = int(n_steps)
        self.dt = grid.find_timestep(CFL)
        self.K = int(checkpoint_every)
        self.keep_samples = keep_samples
        z = dict(dtype=torch.float64, device=self.device)
        self.pts = torch.tensor(sphere.points, **z).contiguous()
        self.wts = torch.tensor(sphere.weights, **z).contiguous()
        self.npts = sphere.n
        nsamp = self.n_steps if keep_samples else self.K
        self.samples = torch.zeros((nsamp, self.npts, self.NE), **z)
        self.J2 = torch.zeros(1, **z)
        self.scratch_J2 = torch.zeros(1, **z)
        self.checkpoints = {}
        self.params = None
        self.p = C.byref(grid.params)

    # -- pieces
    def _sync(self):
        self.ev._sync_stream()

    def _sample(self, y, out, accum):
        _lib.check(self.lib.nrgpu_sphere_sample(self.p, _lib.ptr(y), self.E0, self.NE, _lib.ptr(self.pts),
                                                _lib.ptr(self.wts), self.npts, float(self.dt), _lib.ptr(out),
                                                _lib.ptr(accum)), "nrgpu_sphere_sample")

    def _check_sphere(self):
        flag = C.c_int()
        _lib.check(self.lib.nrgpu_sphere_check(self.p, C.byref(flag)), "nrgpu_sphere_check")
        if flag.value:
            raise ValueError("extraction sphere leaves the grid (tricubic stencil out of range)")

    def initial_data(self, amp, lam, out=None, d_amp=None, d_lam=None):
        self._sync()
        _lib.check(self.lib.Maxwell_initial_data_toroidal_dipole(self.p, float(amp), float(lam), 0.0,
                                                                 _lib.ptr(out), _lib.ptr(d_amp), _lib.ptr(d_lam)),
                   "Maxwell_initial_data_toroidal_dipole")

    # -- forward
    def forward(self, amp, lam):
        """Evolves n_steps from the (amp, lam) data; returns J (float)."""
        self._sync()
        self.params = (float(amp), float(lam))
        ev = self.ev
        self.initial_data(amp, lam, out=ev.y_n)
        self.J2.zero_()
        self.checkpoints = {0: ev.y_n.clone()}
        for n in range(1, self.n_steps + 1):
            ev.step(self.dt)
            slot = (n - 1) if self.keep_samples else (n - 1) % self.K
            self._sample(ev.y_n, self.samples[slot], self.J2)
            if n % self.K == 0 or n == self.n_steps:
                self.checkpoints[n] = ev.y_n.clone()
        self._check_sphere()
        return float(torch.sqrt(self.J2).item())

    def _segment_samples(self, start, stop):
        """Recomputes the samples of steps start+1..stop from checkpoint `start`."""
        ev = self.ev
        ev.y_n.copy_(self.checkpoints[start])
        for n in range(start + 1, stop + 1):
            ev.step(self.dt)
            self._sample(ev.y_n, self.samples[n - start - 1], self.scratch_J2)

    # -- backward
    def gradient(self):
        """dJ/d(amp, lam) by the discrete adjoint (float64 numpy array)."""
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
            _lib.check(self.lib.nrgpu_sphere_sample_adjoint(
                self.p, _lib.ptr(self.samples[slot]), self.E0, self.NE, _lib.ptr(self.pts), _lib.ptr(self.wts),
                self.npts, float(self.dt), _lib.ptr(self.J2), _lib.ptr(target)), "nrgpu_sphere_sample_adjoint")

        seed(N, lam_a)
        for n in range(N, 0, -1):
            _lib.check(self.lib.MoL_adjoint_step_backward(1, self.p, C.byref(ev.bc), _lib.ptr(lam_a),
                                                          _lib.ptr(lam_b), _lib.ptr(scratch),
                                                          float(self.dt)), "MoL_adjoint_step_backward")
            lam_a, lam_b = lam_b, lam_a
            m = n - 1  # lam_a is now dJ/dy_m (without y_m's own samples)
            if m >= 1:
                if not self.keep_samples and m <= seg_start:
                    seg_start -= K
                    self._segment_samples(seg_start, seg_start + K)
                seed(m, lam_a)
        d_amp = torch.zeros(shape, **z)
        d_lam = torch.zeros(shape, **z)
        self.initial_data(*self.params, d_amp=d_amp, d_lam=d_lam)
        res = torch.zeros(2, **z)
        part = torch.zeros(1024, **z)
        n = lam_a.numel()
        for k, d in enumerate((d_amp, d_lam)):
            _lib.check(self.lib.nrgpu_dot(_lib.ptr(lam_a), _lib.ptr(d), n, _lib.ptr(part), 1024,
                                          _lib.ptr(res[k:k + 1])), "nrgpu_dot")
        if not self.keep_samples:  # leave the evolution at the final state, as after forward()
            ev.y_n.copy_(self.checkpoints[N])
        return res.cpu().numpy()


class _ExtractionFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, model):
        J = model.forward(float(params[0]), float(params[1]))
        ctx.model = model
        return torch.tensor(J, dtype=torch.float64, device=params.device)

    @staticmethod
    def backward(ctx, gJ):
        g = torch.tensor(ctx.model.gradient(), dtype=torch.float64, device=gJ.device)
        return gJ * g, None


def extraction_observable(params, model: MaxwellExtraction):
    """J(amp, lam) as a differentiable torch function of params = [amp, lam]."""
    return _ExtractionFn.apply(params, model)
