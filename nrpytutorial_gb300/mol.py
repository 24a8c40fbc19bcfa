"""Method-of-lines evolutions on the GPU through the libnrgpu C ABI.

`Evolution` owns the RK4 buffers of RK_Allocate_Memory.h (y_n, running total,
k_odd, k_even; MoLtimestepping/C_Code_Generation.py:97-103) as torch CUDA
tensors, the reference-metric tables and the boundary-condition map, and
calls the library's entry points on the current torch stream.  PyTorch only
provides device memory and streams here; every numerical operation is a
libnrgpu kernel.
"""
import ctypes as C

import torch

from . import _lib
from .grid import AUXEVOL_GFS, SYSTEM_GFS, T4UU_GFS, Grid


class Evolution:
    def __init__(self, system, grid: Grid, precision="fp64", device="cuda", boundary="extrapolation"):
        self.lib = _lib.load()
        if boundary not in ("extrapolation", "sommerfeld", "none"):
            raise ValueError("boundary must be 'extrapolation', 'sommerfeld' or 'none'")
        if boundary == "sommerfeld" and precision != "fp64":
            raise ValueError("the Sommerfeld step is FP64")
        self.boundary = boundary
        if system not in SYSTEM_GFS:
            raise ValueError("unknown system %r" % system)
        if precision not in _lib.PREC:
            raise ValueError("precision must be one of %s" % sorted(_lib.PREC))
        self.system = system
        self.sys_id = _lib.SYSTEM[system]
        self.grid = grid
        self.precision = precision
        self.device = torch.device(device)
        names, parity = SYSTEM_GFS[system]
        self.gf_names = names
        self.parity = (C.c_int8 * len(parity))(*parity)
        self.ngf = len(names)
        shape = (self.ngf,) + grid.shape
        stage = torch.float64 if precision == "fp64" else torch.float32
        z = dict(device=self.device)
        self.y_n = torch.zeros(shape, dtype=torch.float64, **z)
        self.rt = torch.zeros(shape, dtype=torch.float64, **z)
        # compensated: stage buffers hold FP32 (hi, lo) pairs of the FP64 stage values
        # (both compensated modes; compensated_fp64rk keeps the RK accumulation in FP64)
        kshape = shape + (2,) if precision.startswith("compensated") else shape
        self.k_odd = torch.zeros(kshape, dtype=stage, **z)
        self.k_even = torch.zeros(kshape, dtype=stage, **z)
        naux = len(AUXEVOL_GFS.get(system, []))
        self.sources = system == "BSSN" and bool(grid.params.enable_stress_energy_source_terms)
        if self.sources:
            naux += len(T4UU_GFS)
            self.T4UU = torch.zeros((len(T4UU_GFS),) + grid.shape, dtype=torch.float64, **z)
        self.auxevol = torch.zeros((max(naux, 1),) + grid.shape, dtype=stage, **z)
        self.gfs = _lib.MoL_gridfunctions(_lib.PREC[precision], self.y_n.data_ptr(), self.rt.data_ptr(),
                                          self.k_odd.data_ptr(), self.k_even.data_ptr(),
                                          self.auxevol.data_ptr())
        self._sync_stream()
        self.rfm = _lib.rfm_struct()
        self._rfm_ok = False
        if grid.params.CoordSystem != 0:
            _lib.check(self.lib.rfm_struct__malloc(C.byref(grid.params), C.byref(self.rfm)), "rfm_struct__malloc")
            _lib.check(self.lib.rfm_struct__define(C.byref(grid.params), C.byref(self.rfm)), "rfm_struct__define")
            self._rfm_ok = True
        # boundary="none": no boundary map (a slab of a grid split over ranks,
        # whose boundary conditions the slab driver applies); step() is refused
        self.bc = _lib.bc_struct()
        if boundary != "none":
            _lib.check(self.lib.driver_bcstruct(C.byref(grid.params), C.byref(self.bc)), "driver_bcstruct")
            self._bc_ok = True
        self.time = 0.0

    # -- plumbing
    def _sync_stream(self):
        _lib.set_stream(torch.cuda.current_stream(self.device))

    def _need_bc(self):
        if self.boundary == "none":
            raise RuntimeError("this Evolution has no boundary map (boundary='none')")

    def _rfm(self):
        return C.byref(self.rfm) if self._rfm_ok else None

    def close(self):
        if getattr(self, "_rfm_ok", False):
            self.lib.rfm_struct__freemem(C.byref(self.rfm))
            self._rfm_ok = False
        if getattr(self, "_bc_ok", False):
            self.lib.bcstruct_freemem(C.byref(self.bc))
            self._bc_ok = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the hot path
    def step(self, dt, fused=True):
        """One RK4 step (MoLtimestepping/RK_MoL.h).  With boundary="sommerfeld"
        the radiation condition acts on each stage's RHS instead
        (MoL_step_forward_in_time_sommerfeld; FP64)."""
        self._need_bc()
        self._sync_stream()
        if self.boundary == "sommerfeld":
            f = self.lib.MoL_step_forward_in_time_sommerfeld
        else:
            f = self.lib.MoL_step_forward_in_time if fused else self.lib.MoL_step_forward_in_time_unfused
        _lib.check(f(self.sys_id, self._rfm(), C.byref(self.grid.params), C.byref(self.bc),
                     C.byref(self.gfs), float(dt)), "MoL_step_forward_in_time")
        self.time += dt

    def capture(self, dt, n_steps=1, fused=True):
        """Captures n_steps RK4 steps into a CUDA graph; returns a callable
        that replays them on the current stream.  The step path launches
        kernels only (no allocation, no host synchronisation), so the graph
        holds the same launches the eager step would issue; dt and every
        buffer address are fixed at capture time."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        snapshot = self.y_n.clone()
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.step(dt, fused)  # warm-up launch outside the graph (module load, first-use costs)
        torch.cuda.current_stream(self.device).wait_stream(side)
        with torch.cuda.graph(g):
            for _ in range(n_steps):
                self.step(dt, fused)
        self.y_n.copy_(snapshot)  # undo the warm-up step
        self.time -= dt * (n_steps + 1)
        self._sync_stream()

        def replay():
            g.replay()
            self.time += dt * n_steps
        replay.graph = g
        return replay

    def substep_rhs(self, dt, stage=1, which=0):
        """One substep's kernels before its BCs (timing and profiling; run a
        full step first).  which: 0 all of them, 1 BSSN Ricci, 2 BSSN RHS,
        3 the RHS kernel(s) without a split step's update kernel, 4 that
        update kernel alone."""
        self._sync_stream()
        _lib.check(self.lib.MoL_substep_rhs(self.sys_id, self._rfm(), C.byref(self.grid.params),
                                            C.byref(self.gfs), int(stage), float(dt), int(which)),
                   "MoL_substep_rhs")

    def evolve_host(self, y_host, dt, n_steps):
        """Host-buffer evolution: y_host (numpy float64, IDX4S) in, state out."""
        self._sync_stream()
        _lib.check(self.lib.MoL_evolve_host(self.sys_id, self._rfm(), C.byref(self.grid.params),
                                            C.byref(self.bc), C.byref(self.gfs), float(dt), int(n_steps),
                                            y_host.ctypes.data_as(C.POINTER(C.c_double))),
                   "MoL_evolve_host")

    def rhs_eval(self, in_gfs, rhs_gfs, auxevol=None):
        """The system's rhs_eval (plain store at interior points)."""
        self._sync_stream()
        p = C.byref(self.grid.params)
        f32 = in_gfs.dtype == torch.float32
        sfx = "_f32" if f32 else ""
        if self.system == "ScalarWave":
            if self.grid.params.CoordSystem == 0:
                st = getattr(self.lib, "ScalarWave_rhs_eval" + sfx)(p, _lib.ptr(in_gfs), _lib.ptr(rhs_gfs))
            else:
                st = getattr(self.lib, "ScalarWaveCurvilinear_rhs_eval" + sfx)(
                    self._rfm(), p, _lib.ptr(in_gfs), _lib.ptr(rhs_gfs))
        elif self.system == "Maxwell":
            st = getattr(self.lib, "Maxwell_rhs_eval" + sfx)(p, _lib.ptr(in_gfs), _lib.ptr(rhs_gfs))
        elif self.system == "MaxwellCurvilinear":
            st = getattr(self.lib, "MaxwellCurvilinear_rhs_eval" + sfx)(self._rfm(), p, _lib.ptr(in_gfs),
                                                                        _lib.ptr(rhs_gfs))
        else:
            aux = self.auxevol if auxevol is None else auxevol
            _lib.check(getattr(self.lib, "BSSN_Ricci_eval" + sfx)(self._rfm(), p, _lib.ptr(in_gfs), _lib.ptr(aux)),
                       "BSSN_Ricci_eval")
            st = getattr(self.lib, "BSSN_rhs_eval" + sfx)(self._rfm(), p, _lib.ptr(aux), _lib.ptr(in_gfs),
                                                          _lib.ptr(rhs_gfs))
        _lib.check(st, "rhs_eval")

    def rhs_eval_given_ricci(self, in_gfs, auxevol, rhs_gfs):
        """BSSN rhs_eval alone, with RbarDD supplied in auxevol (the reference's
        LeaveRicciSymbolic form: rhs_eval(rfmstruct, params, auxevol_gfs,
        in_gfs, rhs_gfs) after a separate Ricci_eval)."""
        self._sync_stream()
        sfx = "_f32" if in_gfs.dtype == torch.float32 else ""
        _lib.check(getattr(self.lib, "BSSN_rhs_eval" + sfx)(self._rfm(), C.byref(self.grid.params),
                                                            _lib.ptr(auxevol), _lib.ptr(in_gfs),
                                                            _lib.ptr(rhs_gfs)), "BSSN_rhs_eval")

    def ricci_eval(self, in_gfs, auxevol):
        self._sync_stream()
        sfx = "_f32" if in_gfs.dtype == torch.float32 else ""
        _lib.check(getattr(self.lib, "BSSN_Ricci_eval" + sfx)(self._rfm(), C.byref(self.grid.params),
                                                              _lib.ptr(in_gfs), _lib.ptr(auxevol)),
                   "BSSN_Ricci_eval")

    def apply_bcs(self, gfs):
        self._need_bc()
        self._sync_stream()
        f = self.lib.apply_bcs_curvilinear_f32 if gfs.dtype == torch.float32 else self.lib.apply_bcs_curvilinear
        _lib.check(f(C.byref(self.grid.params), C.byref(self.bc), gfs.shape[0],
                     C.cast(self.parity, C.POINTER(C.c_int8)), _lib.ptr(gfs)), "apply_bcs_curvilinear")

    def initial_data_scalarwave(self, kind="PlaneWave", time=0.0, k=(1.0, 1.0, 1.0), sigma=3.0, out=None):
        """ScalarWave/InitialData.py data ("PlaneWave" or "SphericalGaussian") at all points."""
        self._sync_stream()
        out = self.y_n if out is None else out
        kk = (C.c_double * 3)(*[float(v) for v in k])
        _lib.check(self.lib.ScalarWave_initial_data(C.byref(self.grid.params), {"PlaneWave": 0,
                                                    "SphericalGaussian": 1}[kind], float(time), kk, float(sigma),
                                                    _lib.ptr(out)), "ScalarWave_initial_data")

    def apply_sommerfeld(self, gfs, rhs, xx=None):
        """Sommerfeld radiation condition on rhs (FP64) from the state gfs."""
        self._sync_stream()
        xxp = None
        if xx is not None:
            xxp = (C.c_void_p * 3)(*[x.data_ptr() for x in xx])
        _lib.check(self.lib.apply_bcs_sommerfeld(C.byref(self.grid.params), xxp, C.byref(self.bc), gfs.shape[0],
                                                 C.cast(self.parity, C.POINTER(C.c_int8)), _lib.ptr(gfs),
                                                 _lib.ptr(rhs)), "apply_bcs_sommerfeld")

    def enforce_detgammabar(self, gfs):
        self._sync_stream()
        f = (self.lib.BSSN_enforce_detgammabar_constraint_f32 if gfs.dtype == torch.float32
             else self.lib.BSSN_enforce_detgammabar_constraint)
        _lib.check(f(self._rfm(), C.byref(self.grid.params), _lib.ptr(gfs)), "enforce_detgammabar_constraint")

    def set_stress_energy(self, T4UU):
        """Stress-energy tensor T^{mu nu} for the BSSN source terms: (10, n2,
        n1, n0) in the order T4UU00, 01, 02, 03, 11, 12, 13, 22, 23, 33.
        Kept in FP64 for the constraints and copied into auxevol[6:16] in
        the stage precision for the RHS kernels."""
        if not self.sources:
            raise ValueError("build the Grid with stress_energy_source_terms=True")
        self.T4UU.copy_(T4UU)
        self.auxevol[6:16].copy_(self.T4UU)

    def hamiltonian(self, gfs=None):
        """Hamiltonian constraint at interior points (FP64); with source
        terms on, including -16 pi rho."""
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        H = torch.zeros((1,) + self.grid.shape, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.BSSN_Hamiltonian_constraint(self._rfm(), C.byref(self.grid.params), _lib.ptr(gfs),
                                                        _lib.ptr(H)), "BSSN_Hamiltonian_constraint")
        if self.sources:
            _lib.check(self.lib.BSSN_constraints_add_source_terms(self._rfm(), C.byref(self.grid.params),
                                                                  _lib.ptr(gfs), _lib.ptr(self.T4UU), _lib.ptr(H),
                                                                  None), "BSSN_constraints_add_source_terms")
        return H

    def momentum(self, gfs=None):
        """Momentum constraint M^i (3 gfs) at interior points (FP64)."""
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        M = torch.zeros((3,) + self.grid.shape, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.BSSN_momentum_constraint(self._rfm(), C.byref(self.grid.params), _lib.ptr(gfs),
                                                     _lib.ptr(M)), "BSSN_momentum_constraint")
        if self.sources:
            _lib.check(self.lib.BSSN_constraints_add_source_terms(self._rfm(), C.byref(self.grid.params),
                                                                  _lib.ptr(gfs), _lib.ptr(self.T4UU), None,
                                                                  _lib.ptr(M)), "BSSN_constraints_add_source_terms")
        return M

    def psi4(self, gfs=None, i0_range=None, out=None):
        """psi_4 (quasi-Kinnersley tetrad) as 2 gridfunctions (Re, Im) at
        interior points, optionally only for i0 in [i0_range[0], i0_range[1])
        (an extraction shell).  FP64 state in, FP64 out."""
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        if out is None:
            out = torch.zeros((2,) + self.grid.shape, dtype=torch.float64, device=self.device)
        lo, hi = (-1, -1) if i0_range is None else (int(i0_range[0]), int(i0_range[1]))
        _lib.check(self.lib.BSSN_psi4(self._rfm(), C.byref(self.grid.params), _lib.ptr(gfs), _lib.ptr(out), lo, hi),
                   "BSSN_psi4")
        return out

    def psi4_modes(self, i0, l_max=8, gfs=None):
        """Spin-weight -2 modes of psi_4 on the shell of radial index i0:
        returns ({(l, m): complex}, extraction radius).  psi_4 is evaluated
        on that shell only."""
        import numpy as np
        p4 = self.psi4(gfs, (i0, i0 + 1))
        n_modes = (l_max + 1) ** 2 - 4
        modes = torch.zeros(2 * n_modes, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.BSSN_psi4_spinweightm2_decomposition(C.byref(self.grid.params), _lib.ptr(p4), int(i0),
                                                                 int(l_max), _lib.ptr(modes)),
                   "BSSN_psi4_spinweightm2_decomposition")
        v = modes.cpu().numpy()
        out, q = {}, 0
        for l in range(2, l_max + 1):
            for m in range(-l, l + 1):
                out[(l, m)] = complex(v[2 * q], v[2 * q + 1])
                q += 1
        x0 = float(self.grid.xx[0][i0])
        p = self.grid.params
        r = x0 if p.CoordSystem == 1 else p.AMPL * np.sinh(x0 / p.SINHW) / np.sinh(1.0 / p.SINHW)
        if p.CoordSystem == 3:  # SinhSphericalv2 (reference_metric.py:142-143)
            r += p.AMPL * p.const_dr * x0
        return out, r

    def maxwell_curvilinear_constraints(self, gfs=None):
        """(C, G) of curvilinear Maxwell System II at interior points (FP64)."""
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        out = torch.zeros((2,) + self.grid.shape, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.MaxwellCurvilinear_constraints(self._rfm(), C.byref(self.grid.params), _lib.ptr(gfs),
                                                           _lib.ptr(out)), "MaxwellCurvilinear_constraints")
        return out

    def initial_data_toroidal_dipole(self, amp=1.0, lam=1.0, time=0.0, gfs=None):
        """Toroidal-dipole data (Maxwell/InitialData.py) for Maxwell (System I,
        Cartesian) or MaxwellCurvilinear (System II in the grid's basis)."""
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        p = C.byref(self.grid.params)
        if self.system == "MaxwellCurvilinear":
            st = self.lib.MaxwellCurvilinear_initial_data_toroidal_dipole(p, float(amp), float(lam), float(time),
                                                                          _lib.ptr(gfs))
        elif self.system == "Maxwell":
            st = self.lib.Maxwell_initial_data_toroidal_dipole(p, float(amp), float(lam), float(time), _lib.ptr(gfs),
                                                               None, None)
        else:
            raise ValueError("toroidal-dipole data belong to the Maxwell systems")
        _lib.check(st, "initial_data_toroidal_dipole")

    def maxwell_constraint(self, gfs=None):
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        Cc = torch.zeros((1,) + self.grid.shape, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.Maxwell_Constraints(C.byref(self.grid.params), _lib.ptr(gfs), _lib.ptr(Cc)),
                   "Maxwell_Constraints")
        return Cc

    def l2_norm(self, gfs, gf=0):
        """RMS over interior points of gridfunction `gf` of an FP64 array."""
        self._sync_stream()
        nblk = 1024
        scratch = torch.empty(nblk, dtype=torch.float64, device=self.device)
        res = torch.empty(2, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.nrgpu_l2_norm_sq(C.byref(self.grid.params), _lib.ptr(gfs), gf, _lib.ptr(scratch),
                                             nblk, _lib.ptr(res)), "nrgpu_l2_norm_sq")
        s, n = res.tolist()
        return (s / n) ** 0.5

    def initial_data_brill_lindquist(self, m1, pos1, m2, pos2, gfs=None):
        self._sync_stream()
        gfs = self.y_n if gfs is None else gfs
        _lib.check(self.lib.BSSN_initial_data_BrillLindquist(
            C.byref(self.grid.params), float(m1), (C.c_double * 3)(*pos1), float(m2), (C.c_double * 3)(*pos2),
            _lib.ptr(gfs)), "BSSN_initial_data_BrillLindquist")

    def rfm_table(self):
        import numpy as np
        host = np.zeros((self.rfm.nquant, self.rfm.N1, self.rfm.N0))
        _lib.check(self.lib.rfm_struct__download(C.byref(self.rfm), host.ctypes.data_as(C.POINTER(C.c_double))),
                   "rfm_struct__download")
        return host

    def bc_map(self):
        import numpy as np
        b = self.bc
        arrs = [np.zeros(max(b.total_outer, 1), dtype=np.int32) for _ in range(2)] + \
               [np.zeros(max(b.total_inner, 1), dtype=np.int32) for _ in range(3)]
        _lib.check(self.lib.bcstruct_download(C.byref(b), *[a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs]),
                   "bcstruct_download")
        return dict(outer_dest=arrs[0][:b.total_outer], outer_step=arrs[1][:b.total_outer],
                    inner_dest=arrs[2][:b.total_inner], inner_src=arrs[3][:b.total_inner],
                    inner_parity=arrs[4][:b.total_inner],
                    num_ob=list(b.num_ob_gz_pts)[:b.NGHOSTS], num_ib=list(b.num_ib_gz_pts)[:b.NGHOSTS],
                    ob_dir_start=[list(b.ob_dir_start[g]) for g in range(b.NGHOSTS)],
                    ib_start=list(b.ib_start)[:b.NGHOSTS])
