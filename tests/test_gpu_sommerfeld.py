"""Sommerfeld radiation boundary condition on the GPU vs the reference's own
generated apply_bcs_sommerfeld (CurviBoundaryConditions.py:259-658, fixture
tests/golden/ref_sommerfeld.npz: Spherical and SinhSpherical at d_r orders 2
and 4) and vs the oracle (the RHS at ghost points for every coordinate
family at FD orders 2 and 4, and RK4 steps of the reference's Sommerfeld
driver form)."""
import os
import numpy as np
import pytest

import oracle.bcs as ob
import oracle.wave_maxwell as ow
from tests.helpers import SOMMERFELD_CFGS, SOMMERFELD_GRID, grids, per_gf_rel, sommerfeld_inputs

pytestmark = pytest.mark.gpu

KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-3.0, 3.0))


def _set(fd, ngf, falloff=3.0):
    from nrpytutorial_gb300 import sommerfeld_params
    sommerfeld_params(fd, speed=[1.0] * ngf, f_inf=[0.0] * ngf, radial_falloff_power=[falloff] * ngf)


@pytest.mark.parametrize("cfg", sorted(SOMMERFELD_CFGS))
def test_sommerfeld_rhs_matches_reference_generated_c(cuda, cfg):
    import torch
    from nrpytutorial_gb300 import Evolution
    coord, dr = SOMMERFELD_CFGS[cfg]
    g = SOMMERFELD_GRID
    G, gp = grids("ScalarWave", coord, g["Nxx"], 4, AMPL=g["AMPL"], SINHW=g["SINHW"], RMAX=g["RMAX"])
    ev = Evolution("ScalarWave", G, device=cuda, boundary="sommerfeld")
    _set(dr, 2)
    f, rhs = sommerfeld_inputs(SOMMERFELD_CFGS[cfg], gp.shape)
    want = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_sommerfeld.npz"))[cfg]
    got = torch.tensor(rhs, device=cuda)
    ev.apply_sommerfeld(torch.tensor(f, device=cuda), got)
    assert per_gf_rel(got.cpu().numpy(), want) < 1e-12


@pytest.mark.parametrize("system,coord,Nxx,order,fd", [
    ("ScalarWave", "Cartesian", (10, 10, 10), 4, 2),
    ("ScalarWave", "Cartesian", (10, 10, 10), 4, 4),
    ("Maxwell", "Cartesian", (10, 8, 12), 4, 2),
    ("ScalarWave", "Spherical", (10, 8, 6), 4, 2),
    ("ScalarWave", "SinhSpherical", (10, 8, 6), 4, 4),
    ("ScalarWave", "SinhSphericalv2", (10, 8, 6), 4, 4),
    ("ScalarWave", "SinhCylindrical", (10, 8, 8), 4, 4),
    ("ScalarWave", "Cylindrical", (8, 6, 8), 4, 2),
    ("ScalarWave", "SinhCylindricalv2", (8, 6, 8), 4, 4),
    ("ScalarWave", "SinhSymTP", (10, 8, 6), 4, 4),
    ("ScalarWave", "SymTP", (8, 6, 6), 4, 2),
])
def test_sommerfeld_rhs_matches_oracle(cuda, system, coord, Nxx, order, fd):
    import torch
    from nrpytutorial_gb300 import SYSTEM_GFS, Evolution
    G, gp = grids(system, coord, Nxx, order, **KW)
    ev = Evolution(system, G, device=cuda, boundary="sommerfeld")
    parity = SYSTEM_GFS[system][1]
    ngf = len(parity)
    _set(fd, ngf)
    rng = np.random.default_rng(fd + ngf)
    f = rng.standard_normal((ngf,) + gp.shape)
    rhs = rng.standard_normal((ngf,) + gp.shape)
    layers = ob.build_bcstruct(gp)
    ref = ob.apply_sommerfeld(gp, layers, f, rhs.copy(), parity, fd)
    got = torch.tensor(rhs, device=cuda)
    ev.apply_sommerfeld(torch.tensor(f, device=cuda), got)
    assert per_gf_rel(got.cpu().numpy(), ref) < 1e-12
    # the caller's coordinate arrays give the same result
    got2 = torch.tensor(rhs, device=cuda)
    xx = [torch.tensor(np.asarray(G.xx[d]), dtype=torch.float64, device=cuda) for d in range(3)]
    ev.apply_sommerfeld(torch.tensor(f, device=cuda), got2, xx=xx)
    assert torch.equal(got, got2)


@pytest.mark.parametrize("system,coord,Nxx", [("ScalarWave", "SinhSpherical", (10, 8, 6)),
                                              ("Maxwell", "Cartesian", (10, 10, 10))])
def test_sommerfeld_rk4_steps_match_oracle(cuda, system, coord, Nxx):
    import torch
    from nrpytutorial_gb300 import SYSTEM_GFS, Evolution
    G, gp = grids(system, coord, Nxx, 4, **KW)
    ev = Evolution(system, G, device=cuda, boundary="sommerfeld")
    parity = SYSTEM_GFS[system][1]
    ngf = len(parity)
    _set(2, ngf)
    y = 0.1 * np.random.default_rng(4).standard_normal((ngf,) + gp.shape)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    layers = ob.build_bcstruct(gp)
    rhs_grid = ow.scalarwave_rhs_grid if system == "ScalarWave" else ow.maxwell_rhs_grid

    def rhs_fn(u):
        r = rhs_grid(gp, u)
        return ob.apply_sommerfeld(gp, layers, u, r, parity, 2)

    dt = 0.2 * min(gp.dxx)
    yo = y.copy()
    for _ in range(3):
        ev.step(dt)
        yo = ob.rk4_step_sommerfeld(yo, dt, rhs_fn, gp.NGHOSTS)
    assert per_gf_rel(ev.y_n.cpu().numpy(), yo) < 1e-12


def test_sommerfeld_absorbs_an_outgoing_pulse_better_than_extrapolation(cuda):
    """A spherical Gaussian pulse of the scalar wave leaves [-10,10]^3: after
    it has crossed the boundary, the energy left in the box is smaller with
    the radiation condition than with quadratic extrapolation."""
    import torch
    from nrpytutorial_gb300 import Evolution
    _set(2, 2)
    res = {}
    for bc in ("extrapolation", "sommerfeld"):
        G, gp = grids("ScalarWave", "Cartesian", (40, 40, 40), 4, domain=(-10.0, 10.0))
        ev = Evolution("ScalarWave", G, device=cuda, boundary=bc)
        z, y, x = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
        r = np.sqrt(x * x + y * y + z * z)
        u = np.exp(-((r - 3.0) / 1.0) ** 2)
        v = 2 * (r - 3.0) * u  # outgoing: u(r - t)
        ev.y_n.copy_(torch.tensor(np.stack([u, v]), device=cuda))
        dt = G.find_timestep(0.5)
        for _ in range(int(16.0 / dt)):
            ev.step(dt)
        g = gp.NGHOSTS
        res[bc] = float((ev.y_n[:, g:-g, g:-g, g:-g] ** 2).sum())
    assert res["sommerfeld"] < res["extrapolation"], res
