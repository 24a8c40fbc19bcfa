"""BSSN on the GPU vs the CPU oracle: reference-metric tables, Ricci,
rhs_eval, det(gammabar) rescale, Hamiltonian constraint, and the RK4 step,
in FP64 (1e-12 normwise relative) and FP32 (mixed-precision bound)."""
import numpy as np
import pytest

import oracle.bcs as ob
import oracle.bssn as obs
import oracle.grid as og
from tests.helpers import bssn_random_state, grids, per_gf_rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 5e-5

CASES = [("Cartesian", (8, 8, 8), 4), ("Cartesian", (8, 6, 10), 6),
         ("SinhSpherical", (10, 8, 8), 4), ("Spherical", (8, 8, 6), 4),
         ("Cartesian", (8, 6, 6), 2), ("Cartesian", (6, 8, 6), 8), ("SinhSphericalv2", (10, 8, 8), 4),
         ("SinhCylindrical", (10, 8, 8), 4), ("Cylindrical", (8, 6, 8), 4), ("SinhCylindricalv2", (8, 8, 6), 4),
         ("SymTP", (8, 6, 6), 4), ("SinhSymTP", (10, 8, 6), 4)]
KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0), eta=2.0)


def _setup(cuda, coord, Nxx, order, prec="fp64"):
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", coord, Nxx, order, **KW)
    return Evolution("BSSN", G, precision=prec, device=cuda), gp


@pytest.mark.parametrize("coord", ["SinhSpherical", "Spherical", "SinhSphericalv2", "Cylindrical", "SinhCylindrical",
                                   "SinhCylindricalv2", "SymTP", "SinhSymTP"])
def test_rfm_tables_match_oracle(cuda, coord):
    ev, gp = _setup(cuda, coord, (10, 8, 6), 4)
    tab = ev.rfm_table()
    q = og.hatted(gp)
    slots = [("ReU", 0), ("ReUdD", 3), ("ReUdDD", 12), ("ReDD", 39), ("ReDDdD", 48), ("ReDDdDD", 75),
             ("ghatDD", 156), ("ghatUU", 165), ("ghatDDdD", 174), ("ghatDDdDD", 201), ("GammahatUDD", 282),
             ("GammahatUDDdD", 309), ("detgammahat", 390), ("detgammahatdD", 391), ("detgammahatdDD", 394)]
    for name, off in slots:
        a = q[name]
        n = int(np.prod(a.shape[:-2]))
        got = tab[off:off + n].reshape(a.shape)
        scale = np.abs(a).max() + 1e-300
        assert np.abs(got - a).max() / scale < 1e-13, name


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_ricci_matches_oracle(cuda, bssn_kernels, coord, Nxx, order):
    import torch
    ev, gp = _setup(cuda, coord, Nxx, order)
    f = bssn_random_state(gp.shape, seed=order)
    t = torch.tensor(f, device=cuda)
    aux = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
    ev.ricci_eval(t, aux)
    ref = obs.ricci_grid(gp, f)
    assert per_gf_rel(aux.cpu().numpy(), ref, gp.NGHOSTS) < FP64_TOL


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_rhs_matches_oracle(cuda, bssn_kernels, coord, Nxx, order):
    import torch
    ev, gp = _setup(cuda, coord, Nxx, order)
    f = bssn_random_state(gp.shape, seed=100 + order)
    t = torch.tensor(f, device=cuda)
    aux = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out, auxevol=aux)  # Ricci then rhs (LeaveRicciSymbolic form)
    ref = obs.rhs_grid(gp, f, RbarDD6=aux.cpu().numpy())
    assert per_gf_rel(out.cpu().numpy(), ref, gp.NGHOSTS) < FP64_TOL
    # and with the oracle's own Ricci
    ref2 = obs.rhs_grid(gp, f)
    assert per_gf_rel(out.cpu().numpy(), ref2, gp.NGHOSTS) < FP64_TOL


@pytest.mark.parametrize("coord,Nxx,order", CASES[:3])
def test_fp32_rhs_close_to_fp64(cuda, coord, Nxx, order):
    import torch
    ev, gp = _setup(cuda, coord, Nxx, order, prec="mixed")
    f = bssn_random_state(gp.shape, seed=7, amp=0.05).astype(np.float32)
    t = torch.tensor(f, device=cuda)
    aux = torch.zeros((6,) + gp.shape, dtype=torch.float32, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out, auxevol=aux)
    ref = obs.rhs_grid(gp, f.astype(np.float64))
    assert per_gf_rel(out.double().cpu().numpy(), ref, gp.NGHOSTS) < FP32_TOL


@pytest.mark.parametrize("coord", ["Cartesian", "SinhSpherical"])
def test_enforce_detgammabar_matches_oracle(cuda, coord):
    import torch
    ev, gp = _setup(cuda, coord, (8, 8, 6), 4)
    f = bssn_random_state(gp.shape, seed=3)
    t = torch.tensor(f, device=cuda)
    ev.enforce_detgammabar(t)
    ref = obs.enforce_detgammabar(gp, f)
    assert per_gf_rel(t.cpu().numpy(), ref) < 1e-14
    # FP32 storage, FP64 arithmetic
    t32 = torch.tensor(f.astype(np.float32), device=cuda)
    ev.enforce_detgammabar(t32)
    ref32 = obs.enforce_detgammabar(gp, f.astype(np.float32).astype(np.float64))
    assert per_gf_rel(t32.double().cpu().numpy(), ref32) < 1e-7


@pytest.mark.parametrize("coord,Nxx,order", CASES[:3])
def test_hamiltonian_matches_oracle(cuda, bssn_kernels, coord, Nxx, order):
    ev, gp = _setup(cuda, coord, Nxx, order)
    import torch
    f = bssn_random_state(gp.shape, seed=9)
    H = ev.hamiltonian(torch.tensor(f, device=cuda)).cpu().numpy()[0]
    ref = obs.hamiltonian_grid(gp, f)
    g = gp.NGHOSTS
    assert per_gf_rel(H[None, g:-g, g:-g, g:-g], ref[None, g:-g, g:-g, g:-g]) < FP64_TOL


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_no_precompute_signature_matches_table_path(cuda, coord, Nxx, order):
    """BSSN_Ricci_eval_xx / BSSN_rhs_eval_xx (reference metric evaluated
    from the caller's xx arrays) agree with the precomputed-table path and
    with the oracle."""
    import ctypes as C
    import torch
    from nrpytutorial_gb300 import _lib
    ev, gp = _setup(cuda, coord, Nxx, order)
    f = bssn_random_state(gp.shape, seed=23)
    t = torch.tensor(f, device=cuda)
    xx = [torch.tensor(np.asarray(ev.grid.xx[d]), dtype=torch.float64, device=cuda) for d in range(3)]
    xxp = (C.c_void_p * 3)(*[x.data_ptr() for x in xx])
    p = C.byref(ev.grid.params)
    aux_a = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
    aux_b = torch.zeros_like(aux_a)
    out_a = torch.zeros_like(t)
    out_b = torch.zeros_like(t)
    ev.rhs_eval(t, out_a, auxevol=aux_a)
    _lib.check(ev.lib.BSSN_Ricci_eval_xx(p, xxp, _lib.ptr(t), _lib.ptr(aux_b)), "Ricci_eval_xx")
    _lib.check(ev.lib.BSSN_rhs_eval_xx(p, xxp, _lib.ptr(aux_b), _lib.ptr(t), _lib.ptr(out_b)), "rhs_eval_xx")
    assert per_gf_rel(aux_b.cpu().numpy(), aux_a.cpu().numpy(), gp.NGHOSTS) < 1e-14
    assert per_gf_rel(out_b.cpu().numpy(), out_a.cpu().numpy(), gp.NGHOSTS) < 1e-14
    assert per_gf_rel(out_b.cpu().numpy(), obs.rhs_grid(gp, f), gp.NGHOSTS) < FP64_TOL


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_momentum_constraint_matches_oracle(cuda, coord, Nxx, order):
    import torch
    ev, gp = _setup(cuda, coord, Nxx, order)
    f = bssn_random_state(gp.shape, seed=19)
    M = ev.momentum(torch.tensor(f, device=cuda)).cpu().numpy()
    ref = obs.momentum_grid(gp, f)
    assert per_gf_rel(M, ref, gp.NGHOSTS) < FP64_TOL


@pytest.mark.parametrize("coord,Nxx,order", [CASES[0], CASES[2]])
@pytest.mark.parametrize("fused", [True, False])
def test_rk4_step_matches_oracle(cuda, bssn_kernels, coord, Nxx, order, fused):
    import torch
    from nrpytutorial_gb300 import SYSTEM_GFS
    ev, gp = _setup(cuda, coord, Nxx, order)
    parity = SYSTEM_GFS["BSSN"][1]
    layers = ob.build_bcstruct(gp)

    def post(x):
        ob.apply_bcs(layers, x, parity)
        x[...] = obs.enforce_detgammabar(gp, x)

    y = bssn_random_state(gp.shape, seed=21, amp=0.02)
    post(y)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    dt = 0.05 * min(gp.dxx)
    ev.step(dt, fused=fused)
    yo, _, _ = ob.rk4_step(y, dt, lambda u: obs.rhs_grid(gp, u), post, gp.NGHOSTS)
    assert per_gf_rel(ev.y_n.cpu().numpy(), yo) < 1e-12


def test_cuda_graph_replay_matches_eager_steps(cuda, bssn_kernels):
    """Three RK4 steps replayed from a captured CUDA graph give the same bits
    as three eager steps."""
    import torch
    ev, gp = _setup(cuda, "SinhSpherical", (10, 8, 8), 4)
    y = bssn_random_state(gp.shape, seed=31, amp=0.02)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    y0 = ev.y_n.clone()
    dt = 0.02 * min(gp.dxx)
    for _ in range(3):
        ev.step(dt)
    eager = ev.y_n.clone()
    ev.y_n.copy_(y0)
    replay = ev.capture(dt, n_steps=3)
    assert torch.equal(ev.y_n, y0)  # capturing leaves the state as it was
    replay()
    torch.cuda.synchronize()
    assert torch.equal(ev.y_n, eager)


KO_DISS = 0.25


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_kreiss_oliger_rhs_matches_oracle(cuda, coord, Nxx, order):
    """diss_strength != 0 adds Kreiss-Oliger dissipation to all 24 RHSs."""
    import torch
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", coord, Nxx, order, diss_strength=KO_DISS, **KW)
    ev = Evolution("BSSN", G, device=cuda)
    f = bssn_random_state(gp.shape, seed=41 + order)
    t = torch.tensor(f, device=cuda)
    aux = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out, auxevol=aux)
    ref = obs.rhs_grid(gp, f, diss_strength=KO_DISS)
    assert per_gf_rel(out.cpu().numpy(), ref, gp.NGHOSTS) < FP64_TOL
    assert per_gf_rel(obs.rhs_grid(gp, f), ref, gp.NGHOSTS) > 1e-4  # the term is not negligible


def test_kreiss_oliger_fp32_rhs(cuda):
    """The FP32 instantiation (plain FP32 stage input); the (hi, lo) pair
    instantiation is checked through the compensated RK4 step below."""
    import torch
    from nrpytutorial_gb300 import Evolution
    coord, Nxx, order = CASES[2]
    G, gp = grids("BSSN", coord, Nxx, order, diss_strength=KO_DISS, **KW)
    ev = Evolution("BSSN", G, precision="mixed", device=cuda)
    f = bssn_random_state(gp.shape, seed=7, amp=0.05).astype(np.float32)
    t = torch.tensor(f, device=cuda)
    aux = torch.zeros((6,) + gp.shape, dtype=torch.float32, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out, auxevol=aux)
    ref = obs.rhs_grid(gp, f.astype(np.float64), diss_strength=KO_DISS)
    assert per_gf_rel(out.double().cpu().numpy(), ref, gp.NGHOSTS) < FP32_TOL


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("compensated", 1e-6)])
@pytest.mark.parametrize("fused", [True, False])
def test_kreiss_oliger_rk4_step_matches_oracle(cuda, prec, tol, fused):
    import torch
    from nrpytutorial_gb300 import SYSTEM_GFS, Evolution
    coord, Nxx, order = CASES[2]
    G, gp = grids("BSSN", coord, Nxx, order, diss_strength=KO_DISS, **KW)
    ev = Evolution("BSSN", G, precision=prec, device=cuda)
    parity = SYSTEM_GFS["BSSN"][1]
    layers = ob.build_bcstruct(gp)

    def post(x):
        ob.apply_bcs(layers, x, parity)
        x[...] = obs.enforce_detgammabar(gp, x)

    y = bssn_random_state(gp.shape, seed=43, amp=0.02)
    post(y)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    dt = 0.05 * min(gp.dxx)
    ev.step(dt, fused=fused)
    yo, _, _ = ob.rk4_step(y, dt, lambda u: obs.rhs_grid(gp, u, diss_strength=KO_DISS), post, gp.NGHOSTS)
    assert per_gf_rel(ev.y_n.cpu().numpy(), yo) < tol


def test_kreiss_oliger_damps_the_grid_scale_mode(cuda):
    """The dissipation is dissipative: on flat space plus a checkerboard in
    trK (the grid-scale mode, where every KO stencil gives -1 x f) the
    dissipated RHS differs from the plain one by exactly
    -diss_strength * (invdx0 + invdx1 + invdx2) * trK, and nowhere else."""
    import torch
    from nrpytutorial_gb300 import Evolution
    from oracle.bssn import GF
    coord, Nxx, order = "Cartesian", (12, 10, 8), 4
    outs = {}
    for diss in (0.0, 0.5):
        G, gp = grids("BSSN", coord, Nxx, order, diss_strength=diss, **KW)
        ev = Evolution("BSSN", G, device=cuda)
        y = bssn_random_state(gp.shape, seed=1, amp=0.0)
        i2, i1, i0 = np.indices(gp.shape)
        y[GF["trK"]] += 1e-3 * (-1.0) ** (i0 + i1 + i2)
        t = torch.tensor(y, device=cuda)
        aux = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
        out = torch.zeros_like(t)
        ev.rhs_eval(t, out, auxevol=aux)
        outs[diss] = out.cpu().numpy()
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    d = (outs[0.5] - outs[0.0])[I]
    want = -0.5 * sum(gp.invdx) * y[GF["trK"]][I[1:]]
    assert np.allclose(d[GF["trK"]], want, rtol=1e-12, atol=0.0)
    others = [k for k in range(24) if k != GF["trK"]]
    assert np.abs(d[others]).max() <= 1e-14


def _t4uu(shape, seed):
    """Seeded T^{mu nu} (10 gfs), T^00 > 0."""
    T = 0.05 * np.random.default_rng(seed).standard_normal((10,) + tuple(shape))
    T[0] = np.abs(T[0]) + 0.01
    return T


@pytest.mark.parametrize("coord,Nxx,order", CASES)
def test_source_terms_rhs_matches_oracle(cuda, coord, Nxx, order):
    """T^{mu nu} source terms on, with and without Kreiss-Oliger dissipation."""
    import torch
    from nrpytutorial_gb300 import Evolution
    for diss in (0.0, KO_DISS):
        G, gp = grids("BSSN", coord, Nxx, order, stress_energy_source_terms=True, diss_strength=diss, **KW)
        ev = Evolution("BSSN", G, device=cuda)
        f = bssn_random_state(gp.shape, seed=51 + order)
        T = _t4uu(gp.shape, 52 + order)
        ev.set_stress_energy(torch.tensor(T, device=cuda))
        t = torch.tensor(f, device=cuda)
        out = torch.zeros_like(t)
        ev.rhs_eval(t, out)
        ref = obs.rhs_grid(gp, f, diss_strength=diss, T4UU10=T)
        assert per_gf_rel(out.cpu().numpy(), ref, gp.NGHOSTS) < FP64_TOL, diss
        assert per_gf_rel(obs.rhs_grid(gp, f, diss_strength=diss), ref, gp.NGHOSTS) > 1e-4


def test_source_terms_constraints_match_oracle(cuda):
    import torch
    from nrpytutorial_gb300 import Evolution
    coord, Nxx, order = CASES[2]
    G, gp = grids("BSSN", coord, Nxx, order, stress_energy_source_terms=True, **KW)
    ev = Evolution("BSSN", G, device=cuda)
    f = bssn_random_state(gp.shape, seed=53)
    T = _t4uu(gp.shape, 54)
    ev.set_stress_energy(torch.tensor(T, device=cuda))
    t = torch.tensor(f, device=cuda)
    H = ev.hamiltonian(t).cpu().numpy()
    M = ev.momentum(t).cpu().numpy()
    g = gp.NGHOSTS
    assert per_gf_rel(H, obs.hamiltonian_grid(gp, f, T4UU10=T)[None], g) < FP64_TOL
    assert per_gf_rel(M, obs.momentum_grid(gp, f, T4UU10=T), g) < FP64_TOL


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("compensated", 1e-6), ("mixed", 1e-4)])
def test_source_terms_rk4_step_matches_oracle(cuda, prec, tol):
    import torch
    from nrpytutorial_gb300 import SYSTEM_GFS, Evolution
    coord, Nxx, order = CASES[2]
    G, gp = grids("BSSN", coord, Nxx, order, stress_energy_source_terms=True, **KW)
    ev = Evolution("BSSN", G, precision=prec, device=cuda)
    T = _t4uu(gp.shape, 56)
    ev.set_stress_energy(torch.tensor(T, device=cuda))
    parity = SYSTEM_GFS["BSSN"][1]
    layers = ob.build_bcstruct(gp)

    def post(x):
        ob.apply_bcs(layers, x, parity)
        x[...] = obs.enforce_detgammabar(gp, x)

    y = bssn_random_state(gp.shape, seed=55, amp=0.02)
    post(y)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    dt = 0.05 * min(gp.dxx)
    ev.step(dt)
    yo, _, _ = ob.rk4_step(y, dt, lambda u: obs.rhs_grid(gp, u, T4UU10=T), post, gp.NGHOSTS)
    assert per_gf_rel(ev.y_n.cpu().numpy(), yo) < tol
