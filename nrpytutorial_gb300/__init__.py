"""GB300 (sm_103a) method-of-lines finite-difference evolution for NRPy+-style
PDE systems: ScalarWave, vacuum Maxwell (System I) and BSSN, with RK4 time
stepping, curvilinear boundary conditions and the det(gammabar) rescale.

The compute path is libnrgpu.so (hand-written CUDA behind a C ABI,
include/nrgpu.h); this package is its Python host side.
"""
from ._lib import COORD, PREC, SYSTEM, NrgpuError, load  # noqa: F401
from .grid import AUXEVOL_GFS, SYSTEM_GFS, Grid, default_nghosts  # noqa: F401


def Evolution(*args, **kwargs):  # noqa: N802  (factory keeps torch import lazy)
    from .mol import Evolution as _E
    return _E(*args, **kwargs)
