"""ScalarWave on the GPU vs the CPU oracle: rhs_eval (Cartesian and
curvilinear, FP64 and FP32), the RK4 step (fused and unfused) with boundary
conditions, and 4th-order convergence to the exact plane wave."""
import numpy as np
import pytest

import oracle.bcs as ob
import oracle.wave_maxwell as ow
from tests.helpers import grids, per_gf_rel, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12   # normwise relative, FP64 vs FP64 oracle
FP32_TOL = 2e-5    # normwise relative, FP32 RHS vs FP64 oracle


def _evo(cuda, G, prec="fp64"):
    from nrpytutorial_gb300 import Evolution
    return Evolution("ScalarWave", G, precision=prec, device=cuda)


@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_cartesian_rhs_matches_oracle(cuda, order):
    import torch
    G, gp = grids("ScalarWave", "Cartesian", (12, 10, 14), order)
    ev = _evo(cuda, G)
    rng = np.random.default_rng(order)
    f = rng.standard_normal((2,) + gp.shape)
    inp = torch.tensor(f, device=cuda)
    out = torch.zeros_like(inp)
    ev.rhs_eval(inp, out)
    ref = ow.scalarwave_rhs_grid(gp, f)
    assert per_gf_rel(out.cpu().numpy(), ref, gp.NGHOSTS) < FP64_TOL
    # ghost zones are not written by rhs_eval
    assert float(out[:, :gp.NGHOSTS].abs().max()) == 0.0


@pytest.mark.parametrize("coord", ["Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical", "SinhCylindrical",
                                   "SinhCylindricalv2", "SymTP", "SinhSymTP"])
@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_curvilinear_rhs_matches_oracle(cuda, coord, order):
    import torch
    G, gp = grids("ScalarWave", coord, (10, 8, 6), order, AMPL=5.0, SINHW=0.3, RMAX=5.0)
    ev = _evo(cuda, G)
    f = np.random.default_rng(7).standard_normal((2,) + gp.shape)
    inp = torch.tensor(f, device=cuda)
    out = torch.zeros_like(inp)
    ev.rhs_eval(inp, out)
    ref = ow.scalarwave_rhs_grid(gp, f)
    assert per_gf_rel(out.cpu().numpy(), ref, gp.NGHOSTS) < FP64_TOL


def test_fp32_rhs_close_to_oracle(cuda):
    import torch
    G, gp = grids("ScalarWave", "SinhSpherical", (10, 8, 6), 4)
    ev = _evo(cuda, G, "mixed")
    f = np.random.default_rng(3).standard_normal((2,) + gp.shape)
    inp = torch.tensor(f, device=cuda, dtype=torch.float32)
    out = torch.zeros_like(inp)
    ev.rhs_eval(inp, out)
    ref = ow.scalarwave_rhs_grid(gp, inp.double().cpu().numpy())
    assert per_gf_rel(out.double().cpu().numpy(), ref, gp.NGHOSTS) < FP32_TOL


@pytest.mark.parametrize("coord", ["Cartesian", "SinhSpherical"])
@pytest.mark.parametrize("fused", [True, False])
def test_rk4_step_matches_oracle(cuda, coord, fused):
    import torch
    G, gp = grids("ScalarWave", coord, (8, 8, 6), 4, AMPL=5.0, SINHW=0.3)
    ev = _evo(cuda, G)
    rng = np.random.default_rng(11)
    y = rng.standard_normal((2,) + gp.shape)
    layers = ob.build_bcstruct(gp)

    def post(x):
        ob.apply_bcs(layers, x, [0, 0])

    post(y)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    dt = 0.1 * min(gp.dxx)
    yo = y.copy()
    for _ in range(3):
        ev.step(dt, fused=fused)
        yo, _, _ = ob.rk4_step(yo, dt, lambda u: ow.scalarwave_rhs_grid(gp, u), post, gp.NGHOSTS)
    got = ev.y_n.cpu().numpy()
    assert per_gf_rel(got, yo) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "compensated"])
def test_plane_wave_fourth_order_convergence(cuda, prec):
    """Plane wave u = sin(k.x - |k|t) on [-10,10]^3, FD4, RK4, CFL 0.5,
    quadratic-extrapolation outer BCs.  The error at fixed t must fall like
    N^-4 (Tutorial-Start_to_Finish-ScalarWave.ipynb's convergence check), in
    FP64 and with FP32 RHS arithmetic on compensated stage buffers."""
    import torch
    errs = []
    T = 2.0
    for N in (24, 48):
        G, gp = grids("ScalarWave", "Cartesian", (N, N, N), 4)
        ev = _evo(cuda, G, prec)
        ev.y_n.copy_(torch.tensor(ow.plane_wave(gp, 0.0), device=cuda))
        dt = 0.5 * min(gp.dxx)
        nsteps = int(round(T / dt))
        for _ in range(nsteps):
            ev.step(dt)
        exact = ow.plane_wave(gp, nsteps * dt)
        g = gp.NGHOSTS + N // 4
        num = ev.y_n.cpu().numpy()[0][g:-g, g:-g, g:-g]
        errs.append(np.abs(num - exact[0][g:-g, g:-g, g:-g]).max())
    order = np.log2(errs[0] / errs[1])
    assert 3.5 < order < 4.6, (errs, order)


@pytest.mark.parametrize("coord", ["Cartesian", "Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical",
                                   "SinhCylindrical", "SymTP", "SinhSymTP"])
@pytest.mark.parametrize("kind", ["PlaneWave", "SphericalGaussian"])
def test_initial_data_matches_oracle(cuda, coord, kind):
    G, gp = grids("ScalarWave", coord, (10, 8, 6), 4, AMPL=5.0, SINHW=0.3, RMAX=5.0, wavespeed=0.7)
    ev = _evo(cuda, G)
    ev.initial_data_scalarwave(kind, time=0.4, k=(0.3, -1.0, 0.5), sigma=1.5)
    ref = ow.scalarwave_id_grid(gp, kind, 0.4, (0.3, -1.0, 0.5), 1.5)
    assert np.allclose(ev.y_n.cpu().numpy(), ref, rtol=1e-13, atol=1e-13)
