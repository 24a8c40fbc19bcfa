"""Pins the CPU oracle to the reference (no GPU):

1. the reference's trusted-value unit tests (md5-seeded symbol values in,
   30-digit expected values out) for BSSN_RHSs, BSSN_gauge_RHSs, the
   conformal Ricci tensor, the Hamiltonian constraint, ScalarWave (Cartesian
   and curvilinear), Maxwell System I, and the reference metric
   (Spherical, SinhSpherical, Cartesian);
2. outputs of the reference's own generated C (strict FP64 build) on seeded
   grids, stored in tests/golden/ref_*.npz by tests/golden/make_golden.py;
3. the SENR curvilinear-boundary-condition golden file (Spherical 4x4x4,
   NGHOSTS 3), from the reference's Tutorial-Start_to_Finish-Curvilinear_BCs test.
"""
import itertools
import json
import os

import numpy as np
import pytest

import oracle.bcs as ob
import oracle.bssn as obs
import oracle.grid as og
import oracle.wave_maxwell as ow
from tests.helpers import bssn_random_state, per_gf_rel

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TV = json.load(open(os.path.join(GOLD, "trusted_values.json")))

RANK = {"hDD": 2, "aDD": 2, "lambdaU": 1, "vetU": 1, "betU": 1, "alpha": 0, "cf": 0, "trK": 0,
        "uu": 0, "vv": 0, "EU": 1, "AU": 1, "psi": 0}
SYMM2 = {"hDD", "aDD"}


def symbols(inputs, bases):
    """Arrays of gridfunction and derivative symbol values, completed by the
    reference's index symmetries (sym01 gridfunctions, symmetric 2nd
    derivatives); symbols absent from the expressions are 0."""
    v = {}

    def name(base, op, idx):
        r = RANK[base]
        a = list(idx[:r])
        d = list(idx[r:])
        if base in SYMM2:
            a = sorted(a)
        if op == "dDD":
            d = sorted(d)
        return base + ("_" + op if op else "") + "".join(map(str, a + d))

    for base in bases:
        r = RANK[base]
        for op, nd in (("", 0), ("dD", 1), ("dupD", 1), ("dDD", 2)):
            arr = np.zeros((3,) * (r + nd) + (1,))
            for idx in itertools.product(range(3), repeat=r + nd):
                arr[idx] = inputs.get(name(base, op, idx), 0.0)
            v[base + ("_" + op if op else "")] = arr if r + nd else arr.reshape(1)
    return v


def expect(case):
    return {k: float(x) for k, x in TV[case]["expected"].items()}


def close(got, want, rtol):
    return abs(got - want) <= rtol * max(abs(want), 1e-300) or abs(got - want) < 1e-12


def _bssn_case(case):
    inp = TV[case]["inputs"]
    v = symbols(inp, ["hDD", "aDD", "lambdaU", "vetU", "betU", "alpha", "cf", "trK"])
    q = og.hatted_at("Spherical", inp.get("xx0", 0.0), inp.get("xx1", 0.0))
    q = {k: a[..., 0] for k, a in q.items()}  # point shape (1,)
    return inp, v, q


def test_trusted_bssn_rhss():
    inp, v, q = _bssn_case("BSSN_RHSs")
    out = obs.rhs(v, q, inp.get("eta", 0.0))
    ex = expect("BSSN_RHSs")
    for k, want in ex.items():
        if k == "cf_rhs":
            got = out["cf"][0]
        elif k == "trK_rhs":
            got = out["trK"][0]
        else:
            base, idx = k.split("[", 1)
            ij = sorted(int(c) for c in idx if c.isdigit())
            nm = {"lambda_rhsU": "lambdaU", "a_rhsDD": "aDD", "h_rhsDD": "hDD"}[base]
            got = out[nm + "".join(map(str, ij))][0]
        assert close(got, want, 1e-11), (k, got, want)


def test_trusted_bssn_gauge_rhss():
    inp, v, q = _bssn_case("gauge_RHSs")
    out = obs.rhs(v, q, inp["eta"])
    for k, want in expect("gauge_RHSs").items():
        if k == "alpha_rhs":
            got = out["alpha"][0]
        else:
            base, idx = k.split("[")
            nm = {"bet_rhsU": "betU", "vet_rhsU": "vetU"}[base]
            got = out[nm + idx[0]][0]
        assert close(got, want, 1e-11), (k, got, want)


def test_trusted_ricci_and_delta():
    inp, v, q = _bssn_case("Ricci")
    Q = obs._Q(v, q)
    R = obs.ricci(v, q, Q)
    for k, want in expect("Ricci").items():
        idx = [int(c) for c in k if c.isdigit()]
        got = R[idx[0], idx[1], 0] if k.startswith("RbarDD") else Q.DGammaU[idx[0], 0]
        assert close(got, want, 1e-11), (k, got, want)


def test_trusted_hamiltonian():
    inp, v, q = _bssn_case("constraints")
    H = obs.hamiltonian(v, q)[0]
    want = expect("constraints")["H"]
    assert close(H, want, 1e-11), (H, want)


@pytest.mark.parametrize("kind", ["PlaneWave", "SphericalGaussian"])
def test_trusted_scalarwave_initial_data(kind):
    inp = TV["SW_ID_" + kind]["inputs"]
    ex = expect("SW_ID_" + kind)
    uu, vv = ow.scalarwave_id_pointwise(kind, inp["xx0"], inp["xx1"], inp["xx2"], inp["time"], inp["wavespeed"],
                                        (inp.get("kk0"), inp.get("kk1"), inp.get("kk2")), inp.get("sigma"))
    assert close(uu, ex["uu_ID"], 1e-13), (uu, ex)
    assert close(vv, ex["vv_ID"], 1e-13), (vv, ex)


def test_trusted_momentum_constraint():
    inp, v, q = _bssn_case("constraints")
    M = obs.momentum(v, q)
    ex = expect("constraints")
    for i in range(3):
        want = ex["MU[%d]" % i]
        assert close(M[i, 0], want, 1e-11), (i, M[i, 0], want)


def _tmunu_case(case):
    inp = TV[case]["inputs"]
    v = symbols(inp, ["hDD", "vetU", "alpha", "cf"])
    v = {k: a for k, a in v.items()}
    q = og.hatted_at("Spherical", inp.get("xx0", 0.0), inp.get("xx1", 0.0))
    q = {k: a[..., 0] for k, a in q.items()}
    T10 = np.array([[inp.get("T4UU%d%d" % ab, 0.0)] for ab in obs.T4])
    return inp, v, q, obs.t4uu_full(T10)


def test_trusted_stress_energy_projections():
    inp, v, q, T = _tmunu_case("Tmunu_BSSN")
    SDD, SD, S, rho = obs.stress_energy(v, q, T)
    for k, want in expect("Tmunu_BSSN").items():
        idx = [int(c) for c in k if c.isdigit()]
        got = {"SDD": lambda: SDD[idx[0], idx[1], 0], "SD": lambda: SD[idx[0], 0], "S": lambda: S[0],
               "rho": lambda: rho[0]}[k.split("[")[0]]()
        assert close(float(got), want, 1e-12), (k, got, want)


def test_trusted_stress_energy_rhs_sources():
    inp, v, q, T = _tmunu_case("Tmunu_RHS_sources")
    src, LamU = obs.source_terms(v, q, T, PI=inp["PI"])
    for k, want in expect("Tmunu_RHS_sources").items():
        idx = [int(c) for c in k if c.isdigit()]
        base = k.split("[")[0]
        if base == "sourceterm_trK_rhs":
            got = src["trK"][0]
        elif base == "sourceterm_a_rhsDD":
            got = src["aDD%d%d" % tuple(sorted(idx))][0]
        elif base == "sourceterm_lambda_rhsU":
            got = src["lambdaU%d" % idx[0]][0]
        else:
            got = LamU[idx[0], 0]
        assert close(float(got), want, 1e-12), (k, got, want)


def _complex(sv):
    return complex(sv.replace(" ", ""))


def test_trusted_psi4_with_symbolic_tetrad():
    """Psi4(specify_tetrad=False): psi_4's six pieces from md5-seeded BSSN
    symbols, reference-metric coordinates and tetrad components."""
    import oracle.psi4 as op
    inp = TV["Psi4"]["inputs"]
    v = symbols(inp, ["hDD", "aDD", "cf", "trK"])
    q = og.hatted_at("Spherical", inp.get("xx0", 0.0), inp.get("xx1", 0.0))
    q = {k: a[..., 0] for k, a in q.items()}
    adm = op.adm_from_bssn(v, q)
    tet = {b: [np.array([inp.get("%s%d" % (b, m), 0.0)]) for m in range(4)] for b in ("n4U", "mre4U", "mim4U")}
    re, im = op.psi4_parts(adm, tet["n4U"], tet["mre4U"], tet["mim4U"])
    ex = TV["Psi4"]["expected"]
    for part in range(3):
        assert close(float(re[part][0]), float(ex["psi4_re_pt[%d]" % part]), 1e-11), part
        assert close(float(im[part][0]), float(ex["psi4_im_pt[%d]" % part]), 1e-11), part


def test_trusted_psi4_tetrads():
    """Psi4_tetrads(): the quasi-Kinnersley tetrad from md5-seeded hDD, cf
    and Spherical coordinates (for these random values the metric is not
    positive definite and some normalisations are imaginary, as in the
    reference's own trusted values)."""
    import oracle.psi4 as op
    inp = TV["Psi4_tetrads"]["inputs"]
    x0, x1, x2 = inp["xx0"], inp["xx1"], inp["xx2"]
    q = og.hatted_at("Spherical", x0, x1)
    q = {k: a[..., 0] for k, a in q.items()}
    h = np.zeros((3, 3, 1))
    for (i, j) in [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]:
        h[i, j] = h[j, i] = inp.get("hDD%d%d" % (i, j), 0.0)
    gamma = (h * q["ReDD"] + q["ghatDD"]) / inp["cf"] ** 2
    l4, n4, mre, mim = op.tetrad(gamma, og.SPH, np.array([x0]), np.array([x1]), np.array([x2]))
    got = {"l4U": l4, "n4U": n4, "mre4U": mre, "mim4U": mim}
    for k, sv in TV["Psi4_tetrads"]["expected"].items():
        base, idx = k.split("[")
        g = complex(np.ravel(got[base][int(idx[0])])[0])
        w = _complex(sv)
        assert abs(g - w) <= 1e-12 * max(abs(w), 1.0), (k, g, w)


@pytest.mark.parametrize("case,cart", [("ScalarWave_RHSs", True), ("ScalarWaveCurvilinear_RHSs", False)])
def test_trusted_scalarwave(case, cart):
    inp = TV[case]["inputs"]
    v = symbols(inp, ["uu", "vv"])
    q = og.hatted_at("Spherical", inp.get("xx0", 0.0), inp.get("xx1", 0.0))
    q = {k: a[..., 0] for k, a in q.items()}
    u, w = ow.scalarwave_pointwise(v, q, inp.get("wavespeed", 1.0), cart)
    ex = expect(case)
    assert close(float(np.ravel(u)[0]), ex["uu_rhs"], 1e-13)
    assert close(float(np.ravel(w)[0]), ex["vv_rhs"], 1e-12)


def test_trusted_maxwell_curvilinear_rescaled():
    """VacuumMaxwellRHSs_rescaled (System II, Spherical): a, e, psi, Gamma
    RHSs and the C, G constraints from md5-seeded symbols."""
    inp = TV["Maxwell_Curvi"]["inputs"]
    R3_ = range(3)
    v = {"aU": np.array([[inp.get("aU%d" % i, 0.0)] for i in R3_]),
         "eU": np.array([[inp.get("eU%d" % i, 0.0)] for i in R3_]),
         "Gamma": np.array([inp.get("Gamma", 0.0)]),
         "aU_dD": np.array([[[inp.get("aU_dD%d%d" % (i, j), 0.0)] for j in R3_] for i in R3_]),
         "eU_dD": np.array([[[inp.get("eU_dD%d%d" % (i, j), 0.0)] for j in R3_] for i in R3_]),
         "aU_dDD": np.array([[[[inp.get("aU_dDD%d%d%d" % ((i,) + tuple(sorted((j, k)))), 0.0)] for k in R3_]
                              for j in R3_] for i in R3_]),
         "psi_dD": np.array([[inp.get("psi_dD%d" % j, 0.0)] for j in R3_]),
         "psi_dDD": np.array([[[inp.get("psi_dDD%d%d" % tuple(sorted((j, k))), 0.0)] for k in R3_] for j in R3_]),
         "Gamma_dD": np.array([[inp.get("Gamma_dD%d" % j, 0.0)] for j in R3_])}
    q = og.hatted_at("Spherical", inp.get("xx0", 0.0), inp.get("xx1", 0.0))
    q = {k: a[..., 0] for k, a in q.items()}
    arhs, erhs, psi_rhs, Grhs, Cc, Gc = ow.maxwell_curvi_pointwise(v, q)
    ex = expect("Maxwell_Curvi")
    for i in R3_:
        assert close(float(arhs[i][0]), ex["arhsU[%d]" % i], 1e-12)
        assert close(float(erhs[i][0]), ex["erhsU[%d]" % i], 1e-12)
    assert close(float(psi_rhs[0]), ex["psi_rhs"], 1e-12)
    assert close(float(Grhs[0]), ex["Gamma_rhs"], 1e-12)
    assert close(float(Cc[0]), ex["C"], 1e-12)
    assert close(float(Gc[0]), ex["G"], 1e-12)
    # AU_Cart, EU_Cart: J^i_j A^j with J = d x_Cart / d xx
    import oracle.psi4 as op
    _, J = op.cart_and_jacobian(og.SPH, inp.get("xx0", 0.0), inp.get("xx1", 0.0), inp.get("xx2", 0.0))
    for nm, base in (("AU_Cart", "aU"), ("EU_Cart", "eU")):
        V = v[base][:, 0] * q["ReU"][:, 0]
        for i in R3_:
            got = float(sum(J[i, j] * V[j] for j in R3_))
            assert close(got, ex["%s[%d]" % (nm, i)], 1e-12), nm

def test_trusted_maxwell_system_I():
    inp = TV["Maxwell_I"]["inputs"]
    v = symbols(inp, ["EU", "AU", "psi"])
    A, E, psi, C = ow.maxwell_pointwise(v)
    ex = expect("Maxwell_I")
    for i in range(3):
        assert close(float(A[i][0]), ex["ArhsU[%d]" % i], 1e-13)
        assert close(float(E[i][0]), ex["ErhsU[%d]" % i], 1e-13)
    assert close(float(psi[0]), ex["psi_rhs"], 1e-13)
    assert close(float(C[0]), ex["C"], 1e-13)


@pytest.mark.parametrize("cs", ["Spherical", "SinhSpherical", "SinhSphericalv2", "Cylindrical", "SinhCylindrical",
                                "SinhCylindricalv2", "SymTP", "SinhSymTP", "Cartesian"])
def test_trusted_reference_metric(cs):
    inp = TV["rfm_" + cs]["inputs"]
    cyl = {k: inp[k] for k in ("AMPLRHO", "SINHWRHO", "AMPLZ", "SINHWZ", "const_drho", "const_dz", "bScale",
                                "SINHWAA", "AMAX") if k in inp}
    q = og.hatted_at(cs, inp.get("xx0", 0.0), inp.get("xx1", 0.0), inp.get("AMPL", 10.0), inp.get("SINHW", 0.2),
                     inp.get("const_dr", 0.0625), xx2=inp.get("xx2", 0.0), **cyl)
    n = 0
    for k, want in expect("rfm_" + cs).items():
        base, _, rest = k.partition("[")
        idx = tuple(int(c) for c in rest if c.isdigit())
        got = float(q[base][idx][0, 0]) if idx else float(q[base][0, 0])
        assert close(got, want, 1e-12), (k, got, want)
        n += 1
    assert n == 403


# ------------------------------------------------- reference-generated C
KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0), eta=2.0)
CFGS = {"bssn_cart_fd2": "Cartesian", "bssn_cart_fd4": "Cartesian", "bssn_cart_fd6": "Cartesian",
        "bssn_cart_fd8": "Cartesian", "bssn_sinhsph_fd4": "SinhSpherical", "bssn_sph_fd4": "Spherical",
        "bssn_sinhv2_fd4": "SinhSphericalv2", "bssn_sinhcyl_fd4": "SinhCylindrical",
        "bssn_sinhcylv2_fd4": "SinhCylindricalv2", "bssn_sinhsymtp_fd4": "SinhSymTP"}


@pytest.mark.parametrize("cfg", sorted(CFGS))
def test_oracle_matches_reference_generated_bssn(cfg):
    z = np.load(os.path.join(GOLD, "ref_%s.npz" % cfg))
    gp = og.GridParams(CFGS[cfg], tuple(z["Nxx"]), int(z["ng"]), int(z["fd"]), **KW)
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    ric = obs.ricci_grid(gp, f)
    assert per_gf_rel(ric[I], z["ricci"]) < 1e-13
    # rhs_eval fed the reference's own RbarDD (LeaveRicciSymbolic form)
    R6 = np.zeros((6,) + gp.shape)
    R6[I] = z["ricci"]
    assert per_gf_rel(obs.rhs_grid(gp, f, RbarDD6=R6)[I], z["rhs"]) < 1e-13
    assert per_gf_rel(obs.hamiltonian_grid(gp, f)[None, g:-g, g:-g, g:-g], z["hamiltonian"][None]) < 1e-13
    assert per_gf_rel(obs.enforce_detgammabar(gp, f)[11:17], z["enforce_hDD"]) < 1e-14


@pytest.mark.parametrize("cfg,cs", [("bssn_ko_sinhsph_fd4", "SinhSpherical"), ("bssn_ko_cart_fd2", "Cartesian"),
                                    ("bssn_ko_cart_fd6", "Cartesian"), ("bssn_ko_cart_fd8", "Cartesian")])
def test_oracle_kreiss_oliger_matches_reference_generated_bssn(cfg, cs):
    """rhs_eval with Kreiss-Oliger dissipation on every gridfunction
    (reference-generated C of the BaikalETK construction) against the
    oracle; the dissipation term itself is a sizeable part of the RHS."""
    z = np.load(os.path.join(GOLD, "ref_%s.npz" % cfg))
    gp = og.GridParams(cs, tuple(z["Nxx"]), int(z["ng"]), int(z["fd"]), **KW)
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    diss = float(z["diss_strength"])
    got = obs.rhs_grid(gp, f, RbarDD6=z["aux"], diss_strength=diss)[I]
    assert per_gf_rel(got, z["rhs"]) < 1e-13
    plain = obs.rhs_grid(gp, f, RbarDD6=z["aux"])[I]
    assert per_gf_rel(plain, z["rhs"]) > 1e-6


def test_oracle_source_terms_match_reference_generated_bssn():
    """rhs_eval with T^{mu nu} source terms (reference-generated C of the
    BaikalETK construction; auxevol = RbarDD + T4UU) against the oracle."""
    z = np.load(os.path.join(GOLD, "ref_bssn_src_sinhsph_fd4.npz"))
    gp = og.GridParams("SinhSpherical", tuple(z["Nxx"]), int(z["ng"]), int(z["fd"]), **KW)
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    g = gp.NGHOSTS
    I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    aux = z["aux"]
    got = obs.rhs_grid(gp, f, RbarDD6=aux[:6], T4UU10=aux[6:])[I]
    assert per_gf_rel(got, z["rhs"]) < 1e-13
    assert per_gf_rel(obs.rhs_grid(gp, f, RbarDD6=aux[:6])[I], z["rhs"]) > 1e-6


def test_oracle_fd_coefficients_match_reference_exactly():
    """Exact rational weights of finite_difference.compute_fdcoeffs_fdstencl
    (first, second, dupD, ddnD and Kreiss-Oliger derivatives, orders 2-8)."""
    from fractions import Fraction
    from oracle.fd import fd_weights, ko_weights
    want = json.load(open(os.path.join(GOLD, "fd_coefficients.json")))
    for order in (2, 4, 6, 8):
        cases = {"dD": fd_weights(order, 1), "dDD": fd_weights(order, 2), "dupD": fd_weights(order, 1, +1),
                 "ddnD": fd_weights(order, 1, -1), "dKOD": ko_weights(order)}
        for op, (offs, w) in cases.items():
            nz = [(o, c) for o, c in zip(offs, w) if c != 0]
            ref = want["%d_%s" % (order, op)]
            assert [o for o, _ in nz] == ref["offsets"], (order, op)
            assert [c for _, c in nz] == [Fraction(x) for x in ref["coeffs"]], (order, op)


def test_oracle_psi4_matches_reference_generated_c():
    """psi_4 on a seeded Spherical FD4 grid against the reference's own
    generated psi4 C (quasi-Kinnersley tetrad, six pieces summed)."""
    import oracle.psi4 as op
    z = np.load(os.path.join(GOLD, "ref_bssn_psi4_sph_fd4.npz"))
    gp = og.GridParams("Spherical", tuple(z["Nxx"]), int(z["ng"]), int(z["fd"]), **KW)
    f = bssn_random_state(gp.shape, seed=int(z["seed"]))
    g = gp.NGHOSTS
    got = op.psi4_grid(gp, f)[:, g:-g, g:-g, g:-g]
    parts = z["psi4_parts"]
    want = np.array([parts[3] + parts[4] + parts[5], parts[0] + parts[1] + parts[2]])
    assert per_gf_rel(got, want) < 1e-12


def test_oracle_swsh_matches_reference_generated_c():
    """Goldberg's formula (s = -2, l <= 8) against the reference's generated
    SpinWeight_minus2_SphHarmonics C at five (theta, phi) points."""
    import oracle.psi4 as op
    rows = json.load(open(os.path.join(GOLD, "swsh_m2.json")))
    assert len(rows) == 5 * 81
    for l, m, th, ph, re, im in rows:
        r, i = op.swsh_m2(l, m, th, ph)
        scale = max(abs(re), abs(im), 1e-2)  # harmonics are O(1): absolute 1e-14 near their zeros
        assert abs(float(r) - re) <= 1e-12 * scale and abs(float(i) - im) <= 1e-12 * scale, (l, m, th, ph)


@pytest.mark.parametrize("cfg,cs,fn,ngf", [("sw_cart_fd4", "Cartesian", ow.scalarwave_rhs_grid, 2),
                                          ("sw_sinhsph_fd4", "SinhSpherical", ow.scalarwave_rhs_grid, 2),
                                          ("maxwell_cart_fd4", "Cartesian", ow.maxwell_rhs_grid, 7),
                                          ("maxwell_curvi_sinhsph_fd4", "SinhSpherical", ow.maxwell_curvi_rhs_grid,
                                           8),
                                          ("sw_sinhcyl_fd4", "SinhCylindrical", ow.scalarwave_rhs_grid, 2),
                                          ("maxwell_curvi_sinhcyl_fd4", "SinhCylindrical", ow.maxwell_curvi_rhs_grid,
                                           8)])
def test_oracle_matches_reference_generated_wave_maxwell(cfg, cs, fn, ngf):
    z = np.load(os.path.join(GOLD, "ref_%s.npz" % cfg))
    gp = og.GridParams(cs, tuple(z["Nxx"]), int(z["ng"]), int(z["fd"]), **KW)
    f = np.random.default_rng(int(z["seed"])).standard_normal((ngf,) + gp.shape)
    g = gp.NGHOSTS
    assert per_gf_rel(fn(gp, f)[:, g:-g, g:-g, g:-g], z["rhs"]) < 1e-13


# ---------------------------------------------------------- SENR BC file
SENR_PARITY = [1, 2, 3, 4, 5, 6, 7, 8, 9, 0]  # rankoneU0-2, ranktwosymmDD00..22, rankzero


def senr_bc_case(apply):
    """The Discrete test of Tutorial-Start_to_Finish-Curvilinear_BCs.ipynb:
    value = linear index over all 10 gfs, ghosts set to NaN, BCs applied."""
    gp = og.GridParams("Spherical", (4, 4, 4), 3, 4)
    f = np.arange(10 * 1000, dtype=np.float64).reshape((10,) + gp.shape)
    ng = 3
    for i2, i1, i0 in itertools.product(range(10), repeat=3):
        if min(i0, i1, i2) < ng or max(i0, i1, i2) >= 10 - ng:
            f[:, i2, i1, i0] = np.nan
    f = apply(gp, f)
    return f.reshape(10, -1).T  # (points i0-fastest, gfs)


def test_oracle_bcs_match_senr_golden_file():
    want = np.load(os.path.join(GOLD, "senr_bc_spherical_4x4x4.npz"))["values"]
    got = senr_bc_case(lambda gp, f: ob.apply_bcs(ob.build_bcstruct(gp), f, SENR_PARITY))
    assert not np.isnan(got).any()
    assert np.array_equal(got.astype(np.int64), want.astype(np.int64))


def test_parity_types_follow_the_reference_naming_rule():
    """Every system's gridfunction parity types (the product's table) are
    what CurviBoundaryConditions.py:122-160 derives from the names."""
    import oracle.bcs as ob
    from nrpytutorial_gb300.grid import SYSTEM_GFS
    for system, (names, par) in SYSTEM_GFS.items():
        assert [ob.parity_type(n) for n in names] == list(par), system
