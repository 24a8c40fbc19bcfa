"""Batched curvilinear ScalarWave evolutions through the libnrgpu C ABI.

`ScalarWaveBatch` holds many independent ScalarWave evolutions on Spherical
or SinhSpherical grids that share Ntheta and Nphi but not Nr, each identical
to the single-grid evolution of Tutorial-Start_to_Finish-ScalarWaveCurvilinear
(ScalarWave/ScalarWaveCurvilinear_RHSs.py:43-98 RHS, RK4 MoL step,
apply_bcs_curvilinear), with its own CFL time step.  The state of all
instances is packed into one device array per RK4 buffer; `instance(i)`
returns a (2, n2, n1, n0) view of instance i's gridfunctions uu, vv.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib


class ScalarWaveBatch:
    def __init__(self, Nr, Ntheta=32, Nphi=8, CoordSystem="Spherical", RMAX=10.0, AMPL=10.0, SINHW=0.2,
                 wavespeed=1.0, CFL_FACTOR=0.5, precision="mixed", device="cuda"):
        self.lib = _lib.load()
        if precision not in _lib.PREC:
            raise ValueError("precision must be one of %s" % sorted(_lib.PREC))
        self.Nr = [int(n) for n in Nr]
        self.ninst = len(self.Nr)
        self.precision = precision
        self.device = torch.device(device)
        self._sync_stream()
        handle = C.c_void_p()
        nr = (C.c_int * self.ninst)(*self.Nr)
        _lib.check(self.lib.nrgpu_batch_create(self.ninst, nr, int(Ntheta), int(Nphi), _lib.COORD[CoordSystem],
                                               float(RMAX), float(AMPL), float(SINHW), float(wavespeed),
                                               float(CFL_FACTOR), _lib.PREC[precision], C.byref(handle)),
                   "nrgpu_batch_create")
        self.handle = handle
        self.total = int(self.lib.nrgpu_batch_total_points(handle))
        base = (C.c_longlong * self.ninst)()
        ntot = (C.c_longlong * self.ninst)()
        dims = (C.c_int * (3 * self.ninst))()
        _lib.check(self.lib.nrgpu_batch_offsets(handle, base, ntot, dims), "nrgpu_batch_offsets")
        self.base = np.array(base[:], dtype=np.int64)
        self.ntot = np.array(ntot[:], dtype=np.int64)
        self.dims = np.array(dims[:], dtype=np.int64).reshape(-1, 3)
        dt = (C.c_double * self.ninst)()
        _lib.check(self.lib.nrgpu_batch_timesteps(handle, dt), "nrgpu_batch_timesteps")
        self.dt = np.array(dt[:])
        stage = torch.float64 if precision == "fp64" else torch.float32
        z = dict(device=self.device)
        self.y_n = torch.zeros(self.total, dtype=torch.float64, **z)
        self.rt = torch.zeros(self.total, dtype=torch.float64, **z)
        # compensated: stage buffers of FP32 (hi, lo) pairs
        kshape = (self.total, 2) if precision == "compensated" else (self.total,)
        self.k_odd = torch.zeros(kshape, dtype=stage, **z)
        self.k_even = torch.zeros(kshape, dtype=stage, **z)
        self.gfs = _lib.MoL_gridfunctions(_lib.PREC[precision], self.y_n.data_ptr(), self.rt.data_ptr(),
                                          self.k_odd.data_ptr(), self.k_even.data_ptr(), None)
        self.steps_taken = 0

    # -- plumbing
    def _sync_stream(self):
        _lib.set_stream(torch.cuda.current_stream(self.device))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nrgpu_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def instance(self, i, buf=None):
        """(2, n2, n1, n0) view of instance i in a packed buffer (default y_n)."""
        buf = self.y_n if buf is None else buf
        n0, n1, n2 = (int(v) for v in self.dims[i])
        b, n = int(self.base[i]), int(self.ntot[i])
        return buf[b:b + 2 * n].view((2, n2, n1, n0) + tuple(buf.shape[1:]))

    def interior_points(self):
        """Interior grid points summed over instances (one RK4 step updates each once)."""
        return int(sum((n0 - 4) * (n1 - 4) * (n2 - 4) for n0, n1, n2 in self.dims))

    # -- set-up
    def initial_data_gaussian(self, A, r0, w):
        """u = A exp(-(r-r0)^2/w^2), v = 0 on every instance (all points)."""
        arr = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (self.ninst,)))
               for v in (A, r0, w)]
        self._sync_stream()
        dp = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in arr]
        _lib.check(self.lib.nrgpu_batch_initial_data_gaussian(self.handle, *dp, _lib.ptr(self.y_n)),
                   "nrgpu_batch_initial_data_gaussian")

    def set_timesteps(self, dt):
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (self.ninst,)))
        _lib.check(self.lib.nrgpu_batch_set_timesteps(self.handle, dt.ctypes.data_as(C.POINTER(C.c_double))),
                   "nrgpu_batch_set_timesteps")
        self.dt = dt.copy()

    def autotune(self, reps=5):
        """Chooses the RHS tile shape and persistent grid size by timing;
        returns (tx, ty, grid, ms)."""
        self._sync_stream()
        if self.precision == "fp64":
            src = self.y_n
        elif self.precision == "compensated":
            hi = self.y_n.to(torch.float32)
            src = torch.stack([hi, (self.y_n - hi.double()).to(torch.float32)], dim=-1).contiguous()
        else:
            src = self.y_n.to(torch.float32)
        ms = C.c_float()
        _lib.check(self.lib.nrgpu_batch_autotune(self.handle, _lib.ptr(src), _lib.ptr(self.k_odd), int(reps),
                                                 C.byref(ms)), "nrgpu_batch_autotune")
        return self.get_tile() + (ms.value,)

    def set_tile(self, tx, ty, grid):
        _lib.check(self.lib.nrgpu_batch_set_tile(self.handle, int(tx), int(ty), int(grid)), "nrgpu_batch_set_tile")

    def get_tile(self):
        tx, ty, g = C.c_int(), C.c_int(), C.c_int()
        _lib.check(self.lib.nrgpu_batch_get_tile(self.handle, C.byref(tx), C.byref(ty), C.byref(g)),
                   "nrgpu_batch_get_tile")
        return tx.value, ty.value, g.value

    # -- the hot path
    def rhs_eval(self, in_gfs, rhs_gfs):
        self._sync_stream()
        _lib.check(self.lib.nrgpu_batch_rhs_eval(self.handle, _lib.ptr(in_gfs), _lib.ptr(rhs_gfs)),
                   "nrgpu_batch_rhs_eval")

    def apply_bcs(self, gfs):
        self._sync_stream()
        kind = 1 if gfs.dtype == torch.float64 else (2 if gfs.dim() == 2 and gfs.shape[-1] == 2 else 0)
        _lib.check(self.lib.nrgpu_batch_apply_bcs(self.handle, _lib.ptr(gfs), kind), "nrgpu_batch_apply_bcs")

    def step(self):
        """One RK4 step of every instance, each with its own time step."""
        self._sync_stream()
        _lib.check(self.lib.nrgpu_batch_step(self.handle, C.byref(self.gfs)), "nrgpu_batch_step")
        self.steps_taken += 1

    def capture(self, n_steps=1):
        """Captures n_steps batched RK4 steps into a CUDA graph; returns a
        callable that replays them on the current stream."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        snapshot = self.y_n.clone()  # before the side stream waits: the warm-up step rewrites y_n
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.step()  # warm-up outside the graph
        torch.cuda.current_stream(self.device).wait_stream(side)
        with torch.cuda.graph(g):
            for _ in range(n_steps):
                self.step()
        self.y_n.copy_(snapshot)
        self.steps_taken -= n_steps + 1
        self._sync_stream()

        def replay():
            g.replay()
            self.steps_taken += n_steps
        replay.graph = g
        return replay
