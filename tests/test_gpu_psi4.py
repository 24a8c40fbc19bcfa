"""psi_4 on the GPU: against the reference's own generated psi4 C, against
the oracle (every built coordinate system / FD order), the extraction-shell
restriction, the spin-weight -2 mode decomposition against the oracle, the
orthonormality of the modes, and a physics check (psi_4 of a single
Schwarzschild black hole converges to zero with resolution)."""
import os

import numpy as np
import pytest

import oracle.grid as og
import oracle.psi4 as op
from tests.helpers import bssn_random_state, grids, per_gf_rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0), eta=2.0)
CASES = [("Cartesian", (8, 6, 10), 4), ("Cartesian", (8, 8, 6), 6), ("Cartesian", (8, 6, 6), 2),
         ("Cartesian", (10, 8, 8), 8),
         ("SinhSpherical", (10, 8, 8), 4), ("Spherical", (8, 8, 6), 4), ("SinhSphericalv2", (10, 8, 8), 4),
         ("SinhCylindrical", (10, 8, 8), 4), ("SinhCylindricalv2", (8, 8, 6), 4), ("SinhSymTP", (10, 8, 6), 4),
         ("SymTP", (8, 6, 6), 4)]


def _evo(cuda, coord, Nxx, order, **kw):
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", coord, Nxx, order, **dict(KW, **kw))
    return Evolution("BSSN", G, device=cuda), gp


def test_psi4_matches_reference_generated_c(cuda):
    import torch
    z = np.load(os.path.join(GOLD, "ref_bssn_psi4_sph_fd4.npz"))
    ev, gp = _evo(cuda, "Spherical", tuple(z["Nxx"]), int(z["fd"]))
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    p4 = ev.psi4(torch.tensor(f, device=cuda)).cpu().numpy()
    g = gp.NGHOSTS
    parts = z["psi4_parts"]
    want = np.array([parts[3] + parts[4] + parts[5], parts[0] + parts[1] + parts[2]])
    assert per_gf_rel(p4[:, g:-g, g:-g, g:-g], want) < 1e-12


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_psi4_matches_oracle(cuda, coord, Nxx, order):
    import torch
    ev, gp = _evo(cuda, coord, Nxx, order)
    f = bssn_random_state(gp.shape, seed=61 + order)
    got = ev.psi4(torch.tensor(f, device=cuda)).cpu().numpy()
    ref = op.psi4_grid(gp, f)
    assert per_gf_rel(got, ref, gp.NGHOSTS) < 1e-12


def test_psi4_shell_range_writes_only_that_shell(cuda):
    import torch
    ev, gp = _evo(cuda, "SinhSpherical", (10, 8, 8), 4)
    t = torch.tensor(bssn_random_state(gp.shape, seed=5), device=cuda)
    full = ev.psi4(t).cpu().numpy()
    i0 = gp.NGHOSTS + 4
    shell = ev.psi4(t, (i0, i0 + 1)).cpu().numpy()
    assert np.array_equal(shell[..., i0], full[..., i0])
    mask = np.ones(gp.shape[2], dtype=bool)
    mask[i0] = False
    assert float(np.abs(shell[..., mask]).max()) == 0.0
    from nrpytutorial_gb300 import NrgpuError
    with pytest.raises(NrgpuError):
        ev.psi4(t, (0, 1))  # ghost shell


@pytest.mark.parametrize("coord", ["Spherical", "SinhSpherical", "SinhSphericalv2"])
def test_psi4_modes_match_oracle(cuda, coord):
    import torch
    ev, gp = _evo(cuda, coord, (8, 12, 16), 4)
    f = bssn_random_state(gp.shape, seed=71, amp=0.05)
    i0 = gp.NGHOSTS + 5
    modes, r = ev.psi4_modes(i0, l_max=8, gfs=torch.tensor(f, device=cuda))
    p4 = op.psi4_grid(gp, f)
    ref = op.swm2_modes(gp, p4, i0, l_max=8)
    scale = max(abs(complex(*v)) for v in ref.values())
    assert len(modes) == len(ref) == 77
    for k, (a, b) in ref.items():
        assert abs(modes[k] - complex(a, b)) <= 1e-12 * scale, (k, modes[k], (a, b))
    x0 = gp.xx[0][i0]
    want_r = float(og.radial(gp.CoordSystem, x0, gp.AMPL, gp.SINHW, gp.const_dr)[0])
    assert r == pytest.approx(want_r, rel=1e-14)


def test_mode_decomposition_is_orthonormal(cuda):
    """psi_4 set to c sY_{2,2} + d sY_{3,-1} on a shell: the decomposition
    returns c and d (midpoint rule on 64 x 64 cells) and ~0 elsewhere."""
    import ctypes as C
    import torch
    from nrpytutorial_gb300 import Grid, _lib
    G = Grid("Spherical", (4, 64, 64), FD_order=4, NGHOSTS=3, RMAX=10.0)
    gp = og.GridParams("Spherical", (4, 64, 64), 3, 4, RMAX=10.0)
    lib = _lib.load()
    c, d = 1.0 + 0.5j, -0.25 + 0.75j
    th = np.asarray(gp.xx[1])[None, :, None]
    ph = np.asarray(gp.xx[2])[:, None, None]
    y22 = complex(1, 0) * op.swsh_m2(2, 2, th, ph)[0] + 1j * op.swsh_m2(2, 2, th, ph)[1]
    y31 = op.swsh_m2(3, -1, th, ph)[0] + 1j * op.swsh_m2(3, -1, th, ph)[1]
    psi = np.broadcast_to(c * y22 + d * y31, gp.shape)
    t = torch.tensor(np.array([psi.real, psi.imag]), device=cuda)
    modes = torch.zeros(2 * 77, dtype=torch.float64, device=cuda)
    _lib.set_stream(torch.cuda.current_stream())
    _lib.check(lib.BSSN_psi4_spinweightm2_decomposition(C.byref(G.params), _lib.ptr(t), 5, 8, _lib.ptr(modes)),
               "decomposition")
    v = modes.cpu().numpy()
    q = 0
    for l in range(2, 9):
        for m in range(-l, l + 1):
            got = complex(v[2 * q], v[2 * q + 1])
            want = c if (l, m) == (2, 2) else d if (l, m) == (3, -1) else 0.0
            assert abs(got - want) < 2e-3, (l, m, got)
            q += 1


def test_psi4_modes_of_head_on_brill_lindquist_obey_its_symmetries(cuda):
    """Two equal masses on the z axis (time-symmetric Brill-Lindquist data):
    psi_4 is axisymmetric and reflection-symmetric, so on a shell its
    spin-weight -2 content is in m = 0, even-l modes; every m != 0 or odd-l
    mode vanishes to roundoff.  A single mass (Schwarzschild) has psi_4 = 0."""
    from nrpytutorial_gb300 import Evolution, Grid
    G = Grid("Spherical", (48, 32, 16), FD_order=4, NGHOSTS=3, RMAX=8.0)
    ev = Evolution("BSSN", G, device=cuda)
    ev.initial_data_brill_lindquist(0.5, (0.0, 0.0, 0.5), 0.5, (0.0, 0.0, -0.5))
    ev.apply_bcs(ev.y_n)
    i0 = 3 + int(np.argmin(np.abs(np.asarray(G.xx[0][3:-3]) - 4.0)))
    modes, r = ev.psi4_modes(i0, l_max=6)
    big = abs(modes[(2, 0)])
    assert big > 1e-5, modes[(2, 0)]
    assert abs(modes[(4, 0)]) < big
    for (l, m), v in modes.items():
        if m != 0 or l % 2:
            assert abs(v) < 1e-10 * big, ((l, m), v, big)
    ev.initial_data_brill_lindquist(1.0, (0.0, 0.0, 0.0), 0.0, (0.0, 0.0, 0.0))
    ev.apply_bcs(ev.y_n)
    p4 = ev.psi4(ev.y_n, (i0, i0 + 1)).cpu().numpy()[:, 3:-3, 3:-3, i0]
    assert float(np.abs(p4).max()) < 1e-6 * big, float(np.abs(p4).max())
