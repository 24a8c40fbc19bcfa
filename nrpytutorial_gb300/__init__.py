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


def sommerfeld_params(fd_order=2, speed=None, f_inf=None, radial_falloff_power=None):
    """Sommerfeld parameters (sommerfeld_boundary_condition_class): FD order
    of d_r, and per-gridfunction wave speed, value at infinity and radial
    falloff power (sequences; None leaves the current values)."""
    import ctypes as C
    lib = load()
    arrs = [None if v is None else (C.c_double * len(v))(*[float(x) for x in v])
            for v in (speed, f_inf, radial_falloff_power)]
    n = max([len(v) for v in (speed, f_inf, radial_falloff_power) if v is not None] or [0])
    from ._lib import check
    check(lib.nrgpu_sommerfeld_params(int(fd_order), n, *arrs), "nrgpu_sommerfeld_params")
