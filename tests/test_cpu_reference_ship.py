"""The reference's BSSN step in its shipping form (oracle/gen_ref_ship.py:
rfm_precompute, SIMD-macro loops, FD functions, the generated RK_MoL.h and
the reference's curvilinear boundary conditions), which bench.py times as
the reference arm, against the reference's no-precompute generated kernels
driven by the oracle's RK4 step and boundary conditions: the same initial
state and, after two RK4 steps on the headline configuration's coordinates
(SinhSpherical AMPL 64, SINHW 0.2, FD4) at a small grid, the same state to
roundoff.  Both are strict FP64 builds.  Skipped where the generated
sources are absent (they come from the reference checkout)."""
import ctypes as C

import numpy as np
import pytest

import oracle.bcs as ob
import oracle.grid as og
from oracle import ref_build
from oracle.ref import RefKernels, available


def _ship(flavour="strict"):
    import os
    path = os.path.join(ref_build.LIB, "bssn_ship_sinhsph_fd4.%s.so" % flavour)
    if not os.path.exists(path):
        ref_build.build_if_present()
    if not os.path.exists(path):
        pytest.skip("shipping-form reference step not generated (oracle/gen_ref_ship.py)")
    lib = C.CDLL(path)
    lib.ship_setup.argtypes = [C.c_int] * 3 + [C.c_double] * 7
    lib.ship_step.argtypes = [C.c_double]
    lib.ship_ntot.restype = C.c_longlong
    return lib


def test_shipping_form_step_matches_generated_kernels_with_oracle_step():
    if not available("bssn_sinhsph_fd4"):
        pytest.skip("reference-generated kernels not built")
    lib = _ship()
    N = (16, 8, 8)
    gp = og.GridParams("SinhSpherical", N, 3, 4, AMPL=64.0, SINHW=0.2, eta=2.0)
    lib.ship_setup(*N, 64.0, 0.2, 2.0, 0.5, 0.5, 0.5, -0.5)
    shape = (24,) + gp.shape
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    xx = [np.zeros(n) for n in gp.np]
    lib.ship_get_xx(*[dp(a) for a in xx])
    for a, b in zip(xx, gp.xx):
        assert np.abs(a - b).max() < 1e-15
    y = np.zeros(shape)
    lib.ship_get_state(dp(y))
    R = RefKernels("bssn_sinhsph_fd4", gp,
                   extra={"BH1_mass": 0.5, "BH1_posn_z": 0.5, "BH2_mass": 0.5, "BH2_posn_z": -0.5})
    from nrpytutorial_gb300.grid import SYSTEM_GFS
    parity = SYSTEM_GFS["BSSN"][1]
    layers = ob.build_bcstruct(gp)

    def post(u):
        ob.apply_bcs(layers, u, parity)
        u[...] = R.enforce(u)

    y0 = R.initial_data(shape)
    post(y0)
    assert np.abs(y - y0).max() <= 1e-14 * np.abs(y0).max()
    dt = og.find_timestep(gp, 0.5)
    yo = y0.copy()
    for _ in range(2):
        lib.ship_step(dt)
        yo, _, _ = ob.rk4_step(yo, dt, lambda u: R.rhs_eval(u, aux=R.ricci(u)), post, 3)
    lib.ship_get_state(dp(y))
    # the step changed the state by O(1e-3); the two paths agree to roundoff
    assert np.abs(yo - y0).max() > 1e-6
    assert np.abs(y - yo).max() <= 1e-13 * np.abs(y0).max()
