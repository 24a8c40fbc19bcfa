"""Grids and gridfunction registries for the GB300 MoL evolution library.

Mirrors the reference's driver set-up: paramstruct filled by
set_Nxx_dxx_invdx_params__and__xx (reference_metric.py:1330-1395), cell-
centred coordinate arrays xx[3], IDX4S layout (gf outermost, i0 fastest)
and alphabetically sorted evolved gridfunctions (grid.py:226-243).
"""
import ctypes as C

import numpy as np

from . import _lib

# Evolved gridfunctions in memory order, with curvilinear parity types
# (CurviBoundaryConditions.py:122-213).
SYSTEM_GFS = {
    "ScalarWave": (["uu", "vv"], [0, 0]),
    "Maxwell": (["AU0", "AU1", "AU2", "EU0", "EU1", "EU2", "psi"], [1, 2, 3, 1, 2, 3, 0]),
    "MaxwellCurvilinear": (["Gamma", "aU0", "aU1", "aU2", "eU0", "eU1", "eU2", "psi"], [0, 1, 2, 3, 1, 2, 3, 0]),
    "BSSN": (["aDD00", "aDD01", "aDD02", "aDD11", "aDD12", "aDD22", "alpha",
              "betU0", "betU1", "betU2", "cf",
              "hDD00", "hDD01", "hDD02", "hDD11", "hDD12", "hDD22",
              "lambdaU0", "lambdaU1", "lambdaU2", "trK", "vetU0", "vetU1", "vetU2"],
             [4, 5, 6, 7, 8, 9, 0, 1, 2, 3, 0, 4, 5, 6, 7, 8, 9, 1, 2, 3, 0, 1, 2, 3]),
}
AUXEVOL_GFS = {"BSSN": ["RbarDD00", "RbarDD01", "RbarDD02", "RbarDD11", "RbarDD12", "RbarDD22"]}
# With stress-energy source terms the T4UU gridfunctions follow RbarDD in auxevol
# (alphabetical registration order, as the reference's generated code has them).
T4UU_GFS = ["T4UU00", "T4UU01", "T4UU02", "T4UU03", "T4UU11", "T4UU12", "T4UU13", "T4UU22", "T4UU23", "T4UU33"]


def default_nghosts(system, fd_order):
    """ScalarWave drivers use FD_order/2 ghosts; the upwinded BSSN and the
    Maxwell drivers use FD_order/2 + 1 (Tutorial-Start_to_Finish-ScalarWave.ipynb,
    ...BSSNCurvilinear-Two_BHs_Collide.ipynb:835)."""
    return fd_order // 2 if system == "ScalarWave" else fd_order // 2 + 1


class Grid:
    """Numerical grid: paramstruct + cell-centred xx arrays (host, FP64)."""

    def __init__(self, CoordSystem, Nxx, FD_order=4, NGHOSTS=2, *, AMPL=10.0, SINHW=0.2,
                 RMAX=10.0, domain=(-10.0, 10.0), eta=2.0, wavespeed=1.0, EigenCoord=0, diss_strength=0.0,
                 stress_energy_source_terms=False, const_dr=0.0625, RHOMAX=10.0, ZMIN=-10.0, ZMAX=10.0,
                 AMPLRHO=10.0, SINHWRHO=0.2, AMPLZ=10.0, SINHWZ=0.2, const_drho=0.0625, const_dz=0.0625,
                 bScale=0.5, SINHWAA=0.2, AMAX=10.0):
        lib = _lib.load()
        p = _lib.paramstruct()
        p.CoordSystem = _lib.COORD[CoordSystem] if isinstance(CoordSystem, str) else int(CoordSystem)
        p.FD_order = FD_order
        p.NGHOSTS = NGHOSTS
        p.AMPL, p.SINHW, p.RMAX = AMPL, SINHW, RMAX
        p.const_dr = const_dr  # SinhSphericalv2's constant-spacing term (reference default 0.0625)
        p.RHOMAX, p.ZMIN, p.ZMAX = RHOMAX, ZMIN, ZMAX  # Cylindrical domain (reference defaults)
        p.AMPLRHO, p.SINHWRHO, p.AMPLZ, p.SINHWZ = AMPLRHO, SINHWRHO, AMPLZ, SINHWZ  # SinhCylindrical
        p.const_drho, p.const_dz = const_drho, const_dz  # SinhCylindricalv2
        p.bScale, p.SINHWAA, p.AMAX = bScale, SINHWAA, AMAX  # SymTP family (reference defaults)
        # Cartesian extent: (lo, hi) on every axis, or one (lo, hi) per axis
        ext = [tuple(d) for d in domain] if np.ndim(domain) == 2 else [tuple(domain)] * 3
        (p.xmin, p.xmax), (p.ymin, p.ymax), (p.zmin, p.zmax) = ext
        p.eta, p.wavespeed, p.time = eta, wavespeed, 0.0
        p.diss_strength = diss_strength  # Kreiss-Oliger dissipation of the BSSN RHSs (0 = off)
        p.enable_stress_energy_source_terms = int(bool(stress_energy_source_terms))  # T4UU in auxevol 6..15
        n = [int(v) for v in Nxx]
        np_ = [v + 2 * NGHOSTS for v in n]
        self.xx = [np.zeros(np_[d]) for d in range(3)]
        arr = (C.POINTER(C.c_double) * 3)(*[x.ctypes.data_as(C.POINTER(C.c_double)) for x in self.xx])
        _lib.check(lib.set_Nxx_dxx_invdx_params__and__xx(EigenCoord, (C.c_int * 3)(*n), C.byref(p), arr),
                   "set_Nxx_dxx_invdx_params__and__xx")
        self.params = p
        self.CoordSystem = CoordSystem
        self.Nxx = tuple(n)
        self.NGHOSTS = NGHOSTS
        self.FD_order = FD_order
        self.shape = (np_[2], np_[1], np_[0])  # (i2, i1, i0) numpy order
        self.ntot = np_[0] * np_[1] * np_[2]

    def slab(self, w0, w1):
        """The planes w0 <= i2 < w1 of this grid as a grid of their own (its
        interior the planes w0 + NGHOSTS .. w1 - NGHOSTS - 1): the same
        paramstruct with Nxx2 = w1 - w0 - 2 NGHOSTS and xxmin2 moved to the
        slab, for the library's interior kernels on one rank's slab."""
        g = self.NGHOSTS
        if not (0 <= w0 and w1 <= self.shape[0] and w1 - w0 > 2 * g):
            raise ValueError("slab planes [%d, %d) invalid" % (w0, w1))
        s = Grid.__new__(Grid)
        p = _lib.paramstruct()
        C.memmove(C.byref(p), C.byref(self.params), C.sizeof(p))
        p.Nxx2 = w1 - w0 - 2 * g
        p.Nxx_plus_2NGHOSTS2 = w1 - w0
        p.xxmin2 = self.params.xxmin2 + w0 * self.params.dxx2
        p.xxmax2 = p.xxmin2 + p.Nxx2 * self.params.dxx2
        s.params = p
        s.xx = [self.xx[0], self.xx[1], np.ascontiguousarray(self.xx[2][w0:w1])]
        s.CoordSystem, s.NGHOSTS, s.FD_order = self.CoordSystem, g, self.FD_order
        s.Nxx = (self.Nxx[0], self.Nxx[1], p.Nxx2)
        s.shape = (w1 - w0, self.shape[1], self.shape[2])
        s.ntot = s.shape[0] * s.shape[1] * s.shape[2]
        return s

    @property
    def interior(self):
        g = self.NGHOSTS
        return (slice(g, -g), slice(g, -g), slice(g, -g))

    def n_interior(self):
        return self.Nxx[0] * self.Nxx[1] * self.Nxx[2]

    def find_timestep(self, CFL_FACTOR):
        return float(_lib.load().find_timestep(C.byref(self.params), CFL_FACTOR))
