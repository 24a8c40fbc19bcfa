"""ctypes access to the reference-generated kernels (oracle/_ref/lib).

TEST INFRASTRUCTURE (see oracle/__init__.py).  Each configuration's library
exports ref_defaults / ref_set(name, value) (its generated paramstruct) and
ref_rhs_eval, ref_Ricci_eval, ref_Hamiltonian_constraint,
ref_enforce_detgammabar_constraint, ref_initial_data operating on numpy
FP64 arrays in IDX4S layout.
"""
import ctypes as C
import os

import numpy as np

from .ref_build import LIB, configs

DP = C.POINTER(C.c_double)


def available(cfg, flavour="strict"):
    return os.path.exists(os.path.join(LIB, "%s.%s.so" % (cfg, flavour)))


class RefKernels:
    def __init__(self, cfg, gp, flavour="strict", extra=None):
        path = os.path.join(LIB, "%s.%s.so" % (cfg, flavour))
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.lib.ref_set.argtypes = [C.c_char_p, C.c_double]
        self.lib.ref_set.restype = C.c_int
        self.lib.ref_defaults()
        self.gp = gp
        vals = {"Nxx0": gp.Nxx[0], "Nxx1": gp.Nxx[1], "Nxx2": gp.Nxx[2],
                "Nxx_plus_2NGHOSTS0": gp.np[0], "Nxx_plus_2NGHOSTS1": gp.np[1], "Nxx_plus_2NGHOSTS2": gp.np[2],
                "dxx0": gp.dxx[0], "dxx1": gp.dxx[1], "dxx2": gp.dxx[2],
                "invdx0": gp.invdx[0], "invdx1": gp.invdx[1], "invdx2": gp.invdx[2],
                "AMPL": gp.AMPL, "SINHW": gp.SINHW, "RMAX": gp.RMAX, "eta": gp.eta, "wavespeed": gp.wavespeed,
                "const_dr": getattr(gp, "const_dr", 0.0625)}
        for k in ("RHOMAX", "ZMIN", "ZMAX", "AMPLRHO", "SINHWRHO", "AMPLZ", "SINHWZ", "const_drho", "const_dz",
                  "bScale", "SINHWAA", "AMAX"):
            if hasattr(gp, k):
                vals[k] = getattr(gp, k)
        vals.update(extra or {})
        for k, v in vals.items():
            self.lib.ref_set(k.encode(), float(v))
        if self.lib.ref_nghosts() != gp.NGHOSTS:
            raise ValueError("library built for NGHOSTS=%d, grid has %d" % (self.lib.ref_nghosts(), gp.NGHOSTS))
        self.xx = [np.ascontiguousarray(x, dtype=np.float64) for x in gp.xx]

    def _x(self):
        return [x.ctypes.data_as(DP) for x in self.xx]

    @staticmethod
    def _p(a):
        assert a.dtype == np.float64 and a.flags.c_contiguous
        return a.ctypes.data_as(DP)

    def rhs_eval(self, in_gfs, aux=None, out=None):
        out = np.zeros_like(in_gfs) if out is None else out
        aux = np.zeros(1) if aux is None else aux
        self.lib.ref_rhs_eval(*self._x(), self._p(aux), self._p(in_gfs), self._p(out))
        return out

    def ricci(self, in_gfs, aux=None):
        aux = np.zeros((6,) + in_gfs.shape[1:]) if aux is None else aux
        self.lib.ref_Ricci_eval(*self._x(), self._p(in_gfs), self._p(aux))
        return aux

    def hamiltonian(self, in_gfs):
        # the generated H writes aux gridfunction HGF (the only AUX gf: index 0)
        aux = np.zeros((1,) + in_gfs.shape[1:])
        self.lib.ref_Hamiltonian_constraint(*self._x(), self._p(in_gfs), self._p(aux))
        return aux[0]

    def enforce(self, in_gfs):
        g = in_gfs.copy()
        self.lib.ref_enforce_detgammabar_constraint(*self._x(), self._p(g))
        return g

    def psi4(self, in_gfs):
        """psi4_eval: (re, im) sums of the six generated pieces (aux order
        psi4i_0pt..2pt, psi4r_0pt..2pt) and the pieces themselves."""
        aux = np.zeros((6,) + in_gfs.shape[1:])
        self.lib.ref_psi4_eval(*self._x(), self._p(in_gfs), self._p(aux))
        return np.array([aux[3] + aux[4] + aux[5], aux[0] + aux[1] + aux[2]]), aux

    def initial_data(self, shape24):
        g = np.zeros(shape24)
        self.lib.ref_initial_data(*self._x(), self._p(g))
        return g


__all__ = ["RefKernels", "available", "configs"]
