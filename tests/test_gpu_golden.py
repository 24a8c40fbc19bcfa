"""The CUDA path against the reference directly: outputs of the reference's
own generated C (tests/golden/ref_*.npz, strict FP64 build) on the same
seeded inputs, the SENR curvilinear-BC golden file, and the reference's
Brill-Lindquist initial_data."""
import os

import numpy as np
import pytest

from tests.helpers import bssn_random_state, grids, per_gf_rel
from tests.test_cpu_oracle_pins import SENR_PARITY, senr_bc_case

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0), eta=2.0)
CFGS = {"bssn_cart_fd2": "Cartesian", "bssn_cart_fd4": "Cartesian", "bssn_cart_fd6": "Cartesian",
        "bssn_cart_fd8": "Cartesian", "bssn_sinhsph_fd4": "SinhSpherical", "bssn_sph_fd4": "Spherical",
        "bssn_sinhv2_fd4": "SinhSphericalv2", "bssn_sinhcyl_fd4": "SinhCylindrical",
        "bssn_sinhcylv2_fd4": "SinhCylindricalv2", "bssn_sinhsymtp_fd4": "SinhSymTP"}
TOL = 1e-12


def _load(cfg):
    return np.load(os.path.join(GOLD, "ref_%s.npz" % cfg))


@pytest.mark.parametrize("cfg", sorted(CFGS))
def test_bssn_matches_reference_generated_c(cuda, bssn_kernels, cfg):
    import torch
    from nrpytutorial_gb300 import Evolution
    z = _load(cfg)
    G, gp = grids("BSSN", CFGS[cfg], tuple(z["Nxx"]), int(z["fd"]), ng=int(z["ng"]), **KW)
    ev = Evolution("BSSN", G, device=cuda)
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    t = torch.tensor(f, device=cuda)
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    aux = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
    ev.ricci_eval(t, aux)
    assert per_gf_rel(aux.cpu().numpy()[I], z["ricci"]) < TOL
    # rhs_eval with the reference's RbarDD as auxevol input
    aux_ref = np.zeros((6,) + gp.shape)
    aux_ref[I] = z["ricci"]
    out = torch.zeros_like(t)
    ev.rhs_eval_given_ricci(t, torch.tensor(aux_ref, device=cuda), out)
    assert per_gf_rel(out.cpu().numpy()[I], z["rhs"]) < TOL
    H = ev.hamiltonian(t).cpu().numpy()[0]
    assert per_gf_rel(H[None, g:-g, g:-g, g:-g], z["hamiltonian"][None]) < TOL
    t2 = t.clone()
    ev.enforce_detgammabar(t2)
    assert per_gf_rel(t2.cpu().numpy()[11:17], z["enforce_hDD"]) < 1e-14


@pytest.mark.parametrize("cfg,cs", [("bssn_ko_sinhsph_fd4", "SinhSpherical"), ("bssn_ko_cart_fd2", "Cartesian"),
                                    ("bssn_ko_cart_fd6", "Cartesian"), ("bssn_ko_cart_fd8", "Cartesian")])
def test_kreiss_oliger_rhs_matches_reference_generated_c(cuda, cfg, cs):
    """rhs_eval with Kreiss-Oliger dissipation (diss_strength in the
    paramstruct) against the reference's generated C of the same RHSs, on
    both the table path (BSSN_rhs_eval) and the no-precompute signature
    (BSSN_rhs_eval_xx)."""
    import ctypes as C
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    z = _load(cfg)
    diss = float(z["diss_strength"])
    G, gp = grids("BSSN", cs, tuple(z["Nxx"]), int(z["fd"]), ng=int(z["ng"]), diss_strength=diss, **KW)
    ev = Evolution("BSSN", G, device=cuda)
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    t = torch.tensor(f, device=cuda)
    aux = torch.tensor(z["aux"], device=cuda)
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    out = torch.zeros_like(t)
    ev.rhs_eval_given_ricci(t, aux, out)
    assert per_gf_rel(out.cpu().numpy()[I], z["rhs"]) < TOL
    xx = [torch.tensor(np.asarray(G.xx[d]), dtype=torch.float64, device=cuda) for d in range(3)]
    xxp = (C.c_void_p * 3)(*[x.data_ptr() for x in xx])
    out_xx = torch.zeros_like(t)
    _lib.check(ev.lib.BSSN_rhs_eval_xx(C.byref(G.params), xxp, _lib.ptr(aux), _lib.ptr(t), _lib.ptr(out_xx)),
               "BSSN_rhs_eval_xx")
    torch.cuda.synchronize()
    assert per_gf_rel(out_xx.cpu().numpy()[I], z["rhs"]) < TOL


def test_source_terms_rhs_matches_reference_generated_c(cuda):
    """rhs_eval with T^{mu nu} source terms (auxevol = RbarDD + T4UU) against
    the reference's generated C, table path and no-precompute signature."""
    import ctypes as C
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    z = _load("bssn_src_sinhsph_fd4")
    G, gp = grids("BSSN", "SinhSpherical", tuple(z["Nxx"]), int(z["fd"]), ng=int(z["ng"]),
                  stress_energy_source_terms=True, **KW)
    ev = Evolution("BSSN", G, device=cuda)
    t = torch.tensor(bssn_random_state(gp.shape, seed=int(z["seed"])), device=cuda)
    aux = torch.tensor(z["aux"], device=cuda)
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    out = torch.zeros_like(t)
    ev.rhs_eval_given_ricci(t, aux, out)
    assert per_gf_rel(out.cpu().numpy()[I], z["rhs"]) < TOL
    xx = [torch.tensor(np.asarray(G.xx[d]), dtype=torch.float64, device=cuda) for d in range(3)]
    xxp = (C.c_void_p * 3)(*[x.data_ptr() for x in xx])
    out_xx = torch.zeros_like(t)
    _lib.check(ev.lib.BSSN_rhs_eval_xx(C.byref(G.params), xxp, _lib.ptr(aux), _lib.ptr(t), _lib.ptr(out_xx)),
               "BSSN_rhs_eval_xx")
    torch.cuda.synchronize()
    assert per_gf_rel(out_xx.cpu().numpy()[I], z["rhs"]) < TOL


@pytest.mark.parametrize("cfg", sorted(CFGS))
def test_brill_lindquist_matches_reference_initial_data(cuda, cfg):
    import torch
    from nrpytutorial_gb300 import Evolution
    z = _load(cfg)
    G, gp = grids("BSSN", CFGS[cfg], tuple(z["Nxx"]), int(z["fd"]), ng=int(z["ng"]), **KW)
    ev = Evolution("BSSN", G, device=cuda)
    ev.initial_data_brill_lindquist(0.5, (0.0, 0.0, 0.5), 0.5, (0.0, 0.0, -0.5))
    g = gp.NGHOSTS
    got = ev.y_n.cpu().numpy()[:, g:-g, g:-g, g:-g]
    want = z["bl_id"]
    # every gf: normwise relative, or absolute for identically-zero ones
    for k in range(24):
        nb = np.linalg.norm(want[k])
        err = np.linalg.norm(got[k] - want[k])
        assert err <= 1e-12 * max(nb, 1.0), (k, err, nb)


@pytest.mark.parametrize("cfg,cs,system,ngf", [("sw_cart_fd4", "Cartesian", "ScalarWave", 2),
                                              ("sw_sinhsph_fd4", "SinhSpherical", "ScalarWave", 2),
                                              ("maxwell_cart_fd4", "Cartesian", "Maxwell", 7),
                                              ("sw_sinhcyl_fd4", "SinhCylindrical", "ScalarWave", 2),
                                              ("maxwell_curvi_sinhcyl_fd4", "SinhCylindrical", "MaxwellCurvilinear",
                                               8)])
def test_wave_maxwell_match_reference_generated_c(cuda, cfg, cs, system, ngf):
    import torch
    from nrpytutorial_gb300 import Evolution
    z = _load(cfg)
    G, gp = grids(system, cs, tuple(z["Nxx"]), int(z["fd"]), ng=int(z["ng"]), **KW)
    ev = Evolution(system, G, device=cuda)
    f = np.random.default_rng(int(z["seed"])).standard_normal((ngf,) + gp.shape)
    t = torch.tensor(f, device=cuda)
    out = torch.zeros_like(t)
    ev.rhs_eval(t, out)
    g = gp.NGHOSTS
    assert per_gf_rel(out.cpu().numpy()[:, g:-g, g:-g, g:-g], z["rhs"]) < TOL


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_gpu_bcs_match_senr_golden_file(cuda, dtype):
    import torch
    from nrpytutorial_gb300 import Grid, _lib
    import ctypes as C
    want = np.load(os.path.join(GOLD, "senr_bc_spherical_4x4x4.npz"))["values"]
    lib = _lib.load()

    def apply(gp, f):
        G = Grid("Spherical", (4, 4, 4), FD_order=4, NGHOSTS=3)
        bc = _lib.bc_struct()
        _lib.check(lib.driver_bcstruct(C.byref(G.params), C.byref(bc)), "driver_bcstruct")
        t = torch.tensor(f.astype(dtype), device=cuda)
        _lib.set_stream(torch.cuda.current_stream())
        par = (C.c_int8 * 10)(*SENR_PARITY)
        fn = lib.apply_bcs_curvilinear if dtype == "float64" else lib.apply_bcs_curvilinear_f32
        _lib.check(fn(C.byref(G.params), C.byref(bc), 10, C.cast(par, C.POINTER(C.c_int8)), _lib.ptr(t)), "bcs")
        out = t.double().cpu().numpy()
        lib.bcstruct_freemem(C.byref(bc))
        return out

    got = senr_bc_case(apply)
    assert not np.isnan(got).any()
    assert np.array_equal(got.astype(np.int64), want.astype(np.int64))
