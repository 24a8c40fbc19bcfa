"""Curvilinear rescaled vacuum Maxwell (System II) on the GPU: against the
reference's own generated rhs_eval, against the oracle (coordinate systems
x FD orders, FP64 and FP32), constraints, toroidal-dipole data, the RK4 step
with boundary conditions, compensated precision, and 4th-order convergence
of an evolved toroidal dipole to the exact solution."""
import os

import numpy as np
import pytest

import oracle.bcs as ob
import oracle.wave_maxwell as ow
from tests.helpers import grids, per_gf_rel, rel_l2

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0))
CASES = [("Cartesian", (8, 8, 8), 4), ("Spherical", (10, 8, 6), 2), ("Spherical", (10, 8, 6), 4),
         ("SinhSpherical", (10, 8, 8), 4), ("SinhSphericalv2", (10, 8, 8), 4), ("SinhCylindrical", (10, 8, 8), 4),
         ("Cylindrical", (8, 6, 8), 2), ("SinhCylindricalv2", (8, 8, 6), 4), ("SinhSymTP", (10, 8, 6), 4),
         ("SymTP", (8, 6, 6), 2)]
PARITY = [0, 1, 2, 3, 1, 2, 3, 0]


def _evo(cuda, coord, Nxx, order, prec="fp64", **kw):
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("MaxwellCurvilinear", coord, Nxx, order, **dict(KW, **kw))
    return Evolution("MaxwellCurvilinear", G, precision=prec, device=cuda), gp


def _state(gp, seed):
    return np.random.default_rng(seed).standard_normal((8,) + gp.shape)


def test_rhs_matches_reference_generated_c(cuda):
    import torch
    z = np.load(os.path.join(GOLD, "ref_maxwell_curvi_sinhsph_fd4.npz"))
    ev, gp = _evo(cuda, "SinhSpherical", tuple(z["Nxx"]), int(z["fd"]))
    f = np.random.default_rng(int(z["seed"])).standard_normal((8,) + gp.shape)
    t = torch.tensor(f, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out)
    g = gp.NGHOSTS
    got = out.cpu().numpy()[:, g:-g, g:-g, g:-g]
    # gridfunction order Gamma, aU0-2, eU0-2, psi, as the reference's gridfunction_defines.h has it
    assert per_gf_rel(got, z["rhs"]) < 1e-12


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_rhs_matches_oracle(cuda, coord, Nxx, order):
    import torch
    ev, gp = _evo(cuda, coord, Nxx, order)
    f = _state(gp, 3 + order)
    t = torch.tensor(f, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out)
    assert per_gf_rel(out.cpu().numpy(), ow.maxwell_curvi_rhs_grid(gp, f), gp.NGHOSTS) < 1e-12
    # FP32 arithmetic on FP32 storage
    t32 = t.float()
    o32 = torch.zeros_like(t32)
    ev.rhs_eval(t32, o32)
    ref32 = ow.maxwell_curvi_rhs_grid(gp, f.astype(np.float32).astype(np.float64))
    assert per_gf_rel(o32.double().cpu().numpy(), ref32, gp.NGHOSTS) < 5e-5


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_constraints_match_oracle(cuda, coord, Nxx, order):
    import torch
    ev, gp = _evo(cuda, coord, Nxx, order)
    f = _state(gp, 11)
    got = ev.maxwell_curvilinear_constraints(torch.tensor(f, device=cuda)).cpu().numpy()
    assert per_gf_rel(got, ow.maxwell_curvi_constraints_grid(gp, f), gp.NGHOSTS) < 1e-12


@pytest.mark.parametrize("coord", ["Cartesian", "Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical",
                                   "SinhCylindrical", "SymTP", "SinhSymTP"])
def test_toroidal_dipole_data_match_oracle(cuda, coord):
    ev, gp = _evo(cuda, coord, (10, 8, 6), 4)
    ev.initial_data_toroidal_dipole(1.2, 0.9, 0.3)
    want = ow.maxwell_curvi_toroidal_dipole(gp, 0.3, 1.2, 0.9)
    got = ev.y_n.cpu().numpy()
    # per vector (a, e), relative to the vector's largest component: the
    # toroidal field's radial and polar components are zero up to roundoff
    for comps in ((1, 2, 3), (4, 5, 6)):
        scale = max(np.linalg.norm(want[k]) for k in comps)
        for k in comps:
            assert np.linalg.norm(got[k] - want[k]) <= 1e-13 * scale, k
    assert float(np.abs(got[0]).max()) == 0.0 and float(np.abs(got[7]).max()) == 0.0


@pytest.mark.parametrize("fused", [True, False])
def test_rk4_step_matches_oracle(cuda, fused):
    import torch
    ev, gp = _evo(cuda, "SinhSpherical", (10, 8, 8), 4)
    layers = ob.build_bcstruct(gp)

    def post(x):
        ob.apply_bcs(layers, x, PARITY)

    y = _state(gp, 21)
    post(y)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    dt = 0.1 * min(gp.dxx)
    for _ in range(2):
        ev.step(dt, fused=fused)
    yo = y
    for _ in range(2):
        yo, _, _ = ob.rk4_step(yo, dt, lambda u: ow.maxwell_curvi_rhs_grid(gp, u), post, gp.NGHOSTS)
    assert per_gf_rel(ev.y_n.cpu().numpy(), yo) < 1e-12


def test_compensated_step_close_to_fp64(cuda):
    import torch
    runs = {}
    for prec in ("fp64", "mixed", "compensated"):
        ev, gp = _evo(cuda, "Spherical", (16, 12, 8), 4, prec=prec, RMAX=10.0)
        ev.initial_data_toroidal_dipole(1.0, 1.0, 0.0)
        dt = ev.grid.find_timestep(0.5)
        for _ in range(20):
            ev.step(dt)
        torch.cuda.synchronize()
        runs[prec] = ev.y_n.cpu().numpy()
    e_c = rel_l2(runs["compensated"], runs["fp64"])
    e_m = rel_l2(runs["mixed"], runs["fp64"])
    assert e_c < 1e-7 and e_c < e_m / 3, (e_c, e_m)


def test_evolved_toroidal_dipole_converges_at_fourth_order(cuda):
    """Toroidal dipole (amp = lam = 1) evolved to t = 1.5 on Spherical grids
    at two resolutions: the error against the exact solution at r < 5 (the
    pulse has not reached the outer boundary at r = 12) falls by ~2^4."""
    import torch
    errs = []
    for Nr, Nth in ((48, 24), (96, 48)):
        ev, gp = _evo(cuda, "Spherical", (Nr, Nth, 4), 4, RMAX=12.0)
        ev.initial_data_toroidal_dipole(1.0, 1.0, 0.0)
        T = 1.5
        dt0 = ev.grid.find_timestep(0.5)
        n = int(np.ceil(T / dt0))
        replay = ev.capture(T / n, n_steps=n)
        replay()
        torch.cuda.synchronize()
        got = ev.y_n.cpu().numpy()
        want = ow.maxwell_curvi_toroidal_dipole(gp, T, 1.0, 1.0)
        g = gp.NGHOSTS
        r = np.asarray(gp.xx[0])[None, None, :] * np.ones(gp.shape)
        m = np.zeros(gp.shape, dtype=bool)
        m[g:-g, g:-g, g:-g] = True
        m &= r < 5.0
        # E^theta-rescaled etc.: compare all three E components on the mask
        d = np.sqrt(sum(np.mean((got[4 + i][m] - want[4 + i][m]) ** 2) for i in range(3)))
        errs.append(float(d))
    order = np.log2(errs[0] / errs[1])
    assert 3.0 < order < 5.5, (errs, order)
