"""GB300 (sm_103a) method-of-lines finite-difference evolution for NRPy+-style
PDE systems: ScalarWave, vacuum Maxwell (System I) and BSSN, with RK4 time
stepping, curvilinear boundary conditions and the det(gammabar) rescale.

The compute path is libnrgpu.so (hand-written CUDA behind a C ABI,
include/nrgpu.h); this package is its Python host side.
"""
from ._lib import BSSN_KERNELS, COORD, PREC, SYSTEM, NrgpuError, load  # noqa: F401
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


def set_bssn_kernels(mode):
    """Selects the BSSN Ricci/RHS kernels: "auto" (shared-memory staged where
    the grid allows), "point", "staged" or "fused" (nrgpu_set_bssn_kernels);
    returns the previous mode's name."""
    from ._lib import check
    lib = load()
    names = {v: k for k, v in BSSN_KERNELS.items()}
    prev = names[lib.nrgpu_get_bssn_kernels()]
    check(lib.nrgpu_set_bssn_kernels(BSSN_KERNELS[mode]), "nrgpu_set_bssn_kernels")
    return prev


def device_status(clear=True):
    """The library's device status word (nonzero after a kernel's bounded wait
    for its own copies gave up); clears it by default."""
    v = load().nrgpu_device_status(1 if clear else 0)
    if v < 0:
        from ._lib import check
        check(-v, "nrgpu_device_status")
    return v
