"""The reference's own BSSN validation run, end to end on the GPU, against
the same run through the reference's generated kernels
(tests/golden/ref_bssn_bl_spherical_axisym.npz, made by make_golden.py
`evolve`): head-on Brill-Lindquist data (m = 0.5 at z = +-0.5) on the
axisymmetric Spherical grids 72x12x2 and 96x16x2 (RMAX 7.5, FD4, RK4,
CFL 1.0), evolved to t_final = 7.5 as Tutorial-Start_to_Finish-
BSSNCurvilinear-Two_BHs_Collide.ipynb runs it: the same time step and step
count, the final state and the Hamiltonian constraint at t_final."""
import os

import numpy as np
import pytest

from tests.helpers import per_gf_rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RMAX, CFL, T_FINAL = 7.5, 1.0, 7.5


def _state_rel(y, ref):
    """Max over gridfunctions of the normwise relative error.  The phi
    components (h_{r phi}, a_{theta phi}, beta^phi, ...) vanish in this
    axisymmetric run; the reference carries ~1e-47 of roundoff there, so
    they are checked to stay at roundoff instead."""
    big = max(np.linalg.norm(r) for r in ref)
    worst = 0.0
    for g in range(ref.shape[0]):
        if np.linalg.norm(ref[g]) < 1e-30 * big:
            assert np.abs(y[g]).max() < 1e-14, g
            continue
        worst = max(worst, per_gf_rel(y[g][None], ref[g][None]))
    return worst


def _run(cuda, N, prec):
    import torch
    from nrpytutorial_gb300 import Evolution, Grid
    G = Grid("Spherical", N, FD_order=4, NGHOSTS=3, RMAX=RMAX, eta=2.0)
    ev = Evolution("BSSN", G, precision=prec, device=cuda)
    ev.initial_data_brill_lindquist(0.5, (0.0, 0.0, 0.5), 0.5, (0.0, 0.0, -0.5))
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    dt = G.find_timestep(CFL)
    n = int(T_FINAL / dt + 0.5)
    ev.capture(dt, n_steps=n)()
    torch.cuda.synchronize()
    g = 3
    H = ev.hamiltonian()[0].cpu().numpy()[g:-g, g:-g, g:-g]
    y = ev.y_n.cpu().numpy()[:, g:-g, g:-g, g:-g]
    return dt, n, y, H


@pytest.mark.parametrize("N", [(72, 12, 2), (96, 16, 2)])
def test_validation_run_matches_reference_generated_c(cuda, N):
    z = np.load(os.path.join(GOLD, "ref_bssn_bl_spherical_axisym.npz"))
    tag = "%dx%dx%d" % N
    dt, n, y, H = _run(cuda, N, "fp64")
    assert dt == pytest.approx(float(z["dt_" + tag]), rel=1e-15)
    assert n == int(z["n_final_" + tag])
    # hundreds of RK4 steps of a puncture evolution: roundoff differences of
    # the two FP64 implementations grow, but stay far below any truncation
    # error; H (a sum of cancelling terms) is compared relative to its norm
    errH = per_gf_rel(H[None], z["H_" + tag][None])
    print(tag, "H rel", errH)
    assert errH < 1e-10
    if "state_" + tag in z.files:
        errY = _state_rel(y, z["state_" + tag])
        print(tag, "state rel", errY)
        assert errY < 1e-9


def test_validation_run_compensated_precision(cuda):
    """The same 72x12x2 run in compensated precision (FP32 RHS on FP32 pairs,
    float-float RK accumulation), 550 steps: the whole state within 1e-6 of
    the reference's FP64 run and every field within 1e-5 (the error of the
    FP32 RHS arithmetic grows with the step count; the 200-step headline run
    stays below 1e-6 in every field)."""
    from tests.helpers import rel_l2
    z = np.load(os.path.join(GOLD, "ref_bssn_bl_spherical_axisym.npz"))
    _, _, y, H = _run(cuda, (72, 12, 2), "compensated")
    ref = z["state_72x12x2"]
    worst = _state_rel(y, ref)
    whole = rel_l2(y, ref)
    print("compensated: state rel", whole, "worst field", worst,
          "H rel", per_gf_rel(H[None], z["H_72x12x2"][None]))
    assert whole < 1e-6
    assert worst < 1e-5


SW_AMPL, SW_SINHW, SW_T = 10.0, 0.4, 7.0


@pytest.mark.parametrize("prec", ["fp64", "compensated"])
def test_scalarwave_validation_run_matches_reference_generated_c(cuda, prec):
    """The reference's curvilinear ScalarWave validation run
    (Tutorial-Start_to_Finish-ScalarWaveCurvilinear.ipynb: SinhSpherical,
    domain 10, sinh width 0.4, FD4, RK4, CFL 1, extrapolation BCs, plane wave,
    16x8x16 and 24x12x24 to t = 7): the same dt and step counts, the state of
    the 16x8x16 run and both runs' error norms against the exact solution as
    the reference's generated rhs_eval gives them, and the 4th-order
    convergence the notebook validates."""
    import torch
    from nrpytutorial_gb300 import Evolution, Grid
    import oracle.grid as og
    import oracle.wave_maxwell as ow
    z = np.load(os.path.join(GOLD, "ref_sw_planewave_sinhsph.npz"))
    errs = []
    for N in ((16, 8, 16), (24, 12, 24)):
        tag = "%dx%dx%d" % N
        G = Grid("SinhSpherical", N, FD_order=4, NGHOSTS=2, AMPL=SW_AMPL, SINHW=SW_SINHW, wavespeed=1.0)
        gp = og.GridParams("SinhSpherical", N, 2, 4, AMPL=SW_AMPL, SINHW=SW_SINHW)
        ev = Evolution("ScalarWave", G, precision=prec, device=cuda)
        ev.initial_data_scalarwave("PlaneWave", 0.0)
        dt = G.find_timestep(1.0)
        n = int(SW_T / dt + 0.5)
        assert dt == pytest.approx(float(z["dt_" + tag]), rel=1e-15) and n == int(z["n_final_" + tag])
        ev.capture(dt, n_steps=n)()
        torch.cuda.synchronize()
        y = ev.y_n.cpu().numpy()
        g = 2
        exact = ow.scalarwave_id_grid(gp, "PlaneWave", n * dt)
        X2, X1, X0 = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
        m = np.zeros(gp.shape, dtype=bool)
        m[g:-g, g:-g, g:-g] = True
        m &= og.radial(gp.CoordSystem, X0, gp.AMPL, gp.SINHW)[0] < 0.3 * SW_AMPL
        err = float(np.sqrt(np.mean((y[0][m] - exact[0][m]) ** 2)))
        errs.append(err)
        want = float(z["l2_error_" + tag])
        print(prec, tag, "error norm", err, "reference", want)
        # FP64: the norm itself to 1e-10; compensated (2379 steps of FP32 RHS
        # arithmetic at 24x12x24): the difference within 1e-6 of the solution
        # (u = 2 + sin(...)), not of the error norm, which is ~1% of it
        scale = want if prec == "fp64" else float(np.abs(exact[0][m]).max())
        assert abs(err - want) <= (1e-10 if prec == "fp64" else 1e-6) * scale
        if "state_" + tag in z.files:
            rel = per_gf_rel(y[:, g:-g, g:-g, g:-g], z["state_" + tag])
            print(prec, tag, "state rel", rel)
            # compensated: FP32 RHS arithmetic over 707 steps, within the 1e-6 budget
            assert rel < (1e-11 if prec == "fp64" else 1e-6)
    order = np.log(errs[0] / errs[1]) / np.log(1.5)
    assert 3.7 < order < 4.3, (errs, order)


def test_maxwell_curvilinear_validation_run_converges(cuda):
    """The reference's curvilinear Maxwell validation run
    (Tutorial-Start_to_Finish-Solving_Maxwells_Equations_in_Vacuum-
    Curvilinear.ipynb:153-194, 752-753, 819-823, 1342-1353): System II on
    SinhCylindrical with AMPLRHO = AMPLZ = 10 (domain_size) and SINHWRHO =
    SINHWZ = 0.4, FD4, RK4, CFL 0.5, Sommerfeld boundaries (FD4 d_r, falloff
    power 3, speed 1), toroidal dipole amp = lam = 1, grids 50x4x100 and
    80x4x160 to t = 0.5 domain_size.  The notebook validates convergence of
    E^i and A^i to the exact solution; here the error in r < 4 (the pulse
    has not reached the boundary region) falls at 4th order."""
    import oracle.grid as og
    from nrpytutorial_gb300 import Evolution, Grid, sommerfeld_params
    sommerfeld_params(4, speed=[1.0] * 8, f_inf=[0.0] * 8, radial_falloff_power=[3.0] * 8)
    try:
        errs = _maxwell_runs(cuda, og, Evolution, Grid)
    finally:
        sommerfeld_params()  # the library's defaults again, for whatever runs next
    order = np.log(errs[0] / errs[1]) / np.log(1.6)
    print("Maxwell SinhCylindrical errors", errs, "order", order)
    assert 3.5 < order < 4.6, (errs, order)


def _maxwell_runs(cuda, og, Evolution, Grid):
    import torch
    kw = dict(AMPLRHO=10.0, SINHWRHO=0.4, AMPLZ=10.0, SINHWZ=0.4)
    errs = []
    for N in ((50, 4, 100), (80, 4, 160)):
        G = Grid("SinhCylindrical", N, FD_order=4, NGHOSTS=3, **kw)
        gp = og.GridParams("SinhCylindrical", N, 3, 4, **kw)
        ev = Evolution("MaxwellCurvilinear", G, device=cuda, boundary="sommerfeld")
        ev.initial_data_toroidal_dipole(1.0, 1.0, 0.0)
        dt = G.find_timestep(0.5)
        n = int(5.0 / dt + 0.5)
        ev.capture(dt, n_steps=n)()
        exact = torch.zeros_like(ev.y_n)
        ev.initial_data_toroidal_dipole(1.0, 1.0, n * dt, gfs=exact)
        torch.cuda.synchronize()
        got, want = ev.y_n.cpu().numpy(), exact.cpu().numpy()
        X2, X1, X0 = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
        (rho, _), (z, _) = og.cylinder_maps(gp, X0, X2)
        g = 3
        m = np.zeros(gp.shape, dtype=bool)
        m[g:-g, g:-g, g:-g] = True
        m &= np.sqrt(rho ** 2 + z ** 2) < 4.0
        # a^i and e^i (gridfunctions 1-6), rescaled components
        d = sum(np.mean((got[k][m] - want[k][m]) ** 2) for k in range(1, 7))
        errs.append(float(np.sqrt(d)))
    return errs
