"""BSSN in reference-metric form: pointwise algebra and grid drivers (numpy).

TEST INFRASTRUCTURE (see oracle/__init__.py).

Every tensor array has its tensor indices first and point axes last.  The
pointwise functions take the values of the reference's free symbols:
gridfunctions (hDD, aDD, lambdaU, vetU, betU, trK, cf, alpha), their finite-
difference derivative symbols (hDD_dD, hDD_dupD, hDD_dDD, aDD_dupD,
lambdaU_dD, lambdaU_dupD, vetU_dD, vetU_dupD, vetU_dDD, betU_dupD, cf_dD,
cf_dupD, cf_dDD, alpha_dD, alpha_dupD, alpha_dDD, trK_dD, trK_dupD) and the
hatted reference-metric quantities; so the same code is checked against the
reference's trusted values (symbol values in, expression values out) and
driven on grids (symbols from finite differences).

Restated from (zachetienne/nrpytutorial):
  BSSN/BSSN_quantities.py:84-534   gammabar, Abar, Christoffels, Ricci, beta and phi derivatives
  BSSN/BSSN_RHSs.py:28-328         gammabar, Abar, cf (W), trK, Lambdabar RHSs + rescaling
  BSSN/BSSN_gauge_RHSs.py:33-293   1+log lapse, GammaDriving2ndOrder_Covariant shift
  BSSN/Enforce_Detgammabar_Constraint.py:16-75
  BSSN/BSSN_constraints.py:19-74   Hamiltonian constraint
"""
import numpy as np

from .fd import Stencils
from .grid import CART, hatted_grid

EVOL = ["aDD00", "aDD01", "aDD02", "aDD11", "aDD12", "aDD22", "alpha", "betU0", "betU1", "betU2", "cf",
        "hDD00", "hDD01", "hDD02", "hDD11", "hDD12", "hDD22", "lambdaU0", "lambdaU1", "lambdaU2", "trK",
        "vetU0", "vetU1", "vetU2"]
GF = {n: i for i, n in enumerate(EVOL)}
SYM = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
R3 = range(3)


def inv3(g):
    """indexedexp.py:331 symm_matrix_inverter3x3."""
    det = (-g[0, 2] ** 2 * g[1, 1] + 2 * g[0, 1] * g[0, 2] * g[1, 2] - g[0, 0] * g[1, 2] ** 2
           - g[0, 1] ** 2 * g[2, 2] + g[0, 0] * g[1, 1] * g[2, 2])
    inv = np.empty_like(g)
    inv[0, 0] = (-g[1, 2] ** 2 + g[1, 1] * g[2, 2]) / det
    inv[0, 1] = inv[1, 0] = (g[0, 2] * g[1, 2] - g[0, 1] * g[2, 2]) / det
    inv[0, 2] = inv[2, 0] = (-g[0, 2] * g[1, 1] + g[0, 1] * g[1, 2]) / det
    inv[1, 1] = (-g[0, 2] ** 2 + g[0, 0] * g[2, 2]) / det
    inv[1, 2] = inv[2, 1] = (g[0, 1] * g[0, 2] - g[0, 0] * g[1, 2]) / det
    inv[2, 2] = (-g[0, 1] ** 2 + g[0, 0] * g[1, 1]) / det
    return inv, det


class _Q:
    """Basic tensors shared by the RHS, Ricci and constraint expressions."""

    def __init__(self, v, q):
        self.v, self.q = v, q
        h, ReDD = v["hDD"], q["ReDD"]
        # BSSN_quantities.py:84-104
        self.gammabarDD = h * ReDD + q["ghatDD"]
        self.AbarDD = v["aDD"] * ReDD
        self.LambdabarU = v["lambdaU"] * q["ReU"]
        self.betaU = v["vetU"] * q["ReU"]
        self.BU = v["betU"] * q["ReU"]
        # :118-132
        self.gammabarUU, _ = inv3(self.gammabarDD)
        hd = v["hDD_dD"]
        self.gammabarDD_dD = q["ghatDDdD"] + hd * ReDD[:, :, None] + h[:, :, None] * q["ReDDdD"]
        # :153-158
        gUU, gd = self.gammabarUU, self.gammabarDD_dD
        G = np.zeros((3, 3, 3) + h.shape[2:])
        for i in R3:
            for k in R3:
                for l in R3:
                    for m in R3:
                        G[i, k, l] += 0.5 * gUU[i, m] * (gd[m, k, l] + gd[m, l, k] - gd[k, l, m])
        self.GammabarUDD = G
        # :349-363
        self.DGammaUDD = G - q["GammahatUDD"]
        self.DGammaU = np.einsum("jk...,ijk...->i...", gUU, self.DGammaUDD)


def ricci(v, q, Q=None):
    """RbarDD of BSSN_quantities.py:260-425 (Rbar_ij, all 9 components)."""
    Q = Q or _Q(v, q)
    h, hd, hdd = v["hDD"], v["hDD_dD"], v["hDD_dDD"]
    ReDD, ReDDdD, ReDDdDD = q["ReDD"], q["ReDDdD"], q["ReDDdDD"]
    G, GdD = q["GammahatUDD"], q["GammahatUDDdD"]
    shp = h.shape[2:]
    eps = h * ReDD
    epsd = hd * ReDD[:, :, None] + h[:, :, None] * ReDDdD
    epsdd = (hdd * ReDD[:, :, None, None] + hd[:, :, :, None] * ReDDdD[:, :, None, :]
             + hd[:, :, None, :] * ReDDdD[:, :, :, None] + h[:, :, None, None] * ReDDdDD)
    # gammabarDD_dHatD [i][j][l]
    dH = epsd.copy()
    for i in R3:
        for j in R3:
            for l in R3:
                for m in R3:
                    dH[i, j, l] += -G[m, i, l] * eps[m, j] - G[m, j, l] * eps[i, m]
    # gammabarDD_dHatD_dD [i][j][l][k]
    dHd = epsdd.copy()
    for i in R3:
        for j in R3:
            for l in R3:
                for k in R3:
                    for m in R3:
                        dHd[i, j, l, k] += (-GdD[m, i, l, k] * eps[m, j] - G[m, i, l] * epsd[m, j, k]
                                            - GdD[m, j, l, k] * eps[i, m] - G[m, j, l] * epsd[i, m, k])
    # gammabarDD_dHatDD [i][j][l][k]
    dHH = dHd.copy()
    for i in R3:
        for j in R3:
            for l in R3:
                for k in R3:
                    for m in R3:
                        dHH[i, j, l, k] += (-G[m, l, k] * dH[i, j, m] - G[m, i, k] * dH[m, j, l]
                                            - G[m, j, k] * dH[i, m, l])
    # LambarU_dHatD [k][j]
    lam, lamd, ReU, ReUdD = v["lambdaU"], v["lambdaU_dD"], q["ReU"], q["ReUdD"]
    LdH = lamd * ReU[:, None] + lam[:, None] * ReUdD
    for k in R3:
        for j in R3:
            for m in R3:
                LdH[k, j] += G[k, m, j] * lam[m] * ReU[m]
    gbar, gUU, DG, DGU = Q.gammabarDD, Q.gammabarUU, Q.DGammaUDD, Q.DGammaU
    DGD = np.einsum("im...,mjk...->ijk...", gbar, DG)
    Rbar = np.zeros((3, 3) + shp)
    for i in R3:
        for j in R3:
            for k in R3:
                for l in R3:
                    Rbar[i, j] += -0.5 * gUU[k, l] * dHH[i, j, l, k]
    for i in R3:
        for j in R3:
            for k in R3:
                Rbar[i, j] += 0.5 * (gbar[k, i] * LdH[k, j] + gbar[k, j] * LdH[k, i])
                Rbar[i, j] += 0.5 * DGU[k] * (DGD[i, j, k] + DGD[j, i, k])
    for i in R3:
        for j in R3:
            for k in R3:
                for l in R3:
                    for m in R3:
                        Rbar[i, j] += gUU[k, l] * (DG[m, k, i] * DGD[j, m, l] + DG[m, k, j] * DGD[i, m, l]
                                                   + DG[m, i, k] * DGD[m, j, l])
    return Rbar


def rhs(v, q, eta, RbarDD=None):
    """All BSSN + gauge RHSs (rescaled), dict keyed by gridfunction name."""
    Q = _Q(v, q)
    if RbarDD is None:
        RbarDD = ricci(v, q, Q)
    ReU, ReUdD, ReUdDD, ReDD, ReDDdD = q["ReU"], q["ReUdD"], q["ReUdDD"], q["ReDD"], q["ReDDdD"]
    G, GdD = q["GammahatUDD"], q["GammahatUDDdD"]
    alpha, cf, trK = v["alpha"], v["cf"], v["trK"]
    gbar, gUU, Gbar = Q.gammabarDD, Q.gammabarUU, Q.GammabarUDD
    betaU, BU, Lbar = Q.betaU, Q.BU, Q.LambdabarU
    shp = alpha.shape
    # betaU derivatives (BSSN_quantities.py:431-456)
    vet, vetd, vetdup, vetdd = v["vetU"], v["vetU_dD"], v["vetU_dupD"], v["vetU_dDD"]
    betad = vetd * ReU[:, None] + vet[:, None] * ReUdD
    betadup = vetdup * ReU[:, None] + vet[:, None] * ReUdD
    betadd = (vetdd * ReU[:, None, None] + vetd[:, :, None] * ReUdD[:, None, :]
              + vetd[:, None, :] * ReUdD[:, :, None] + vet[:, None, None] * ReUdDD)
    gbar_dup = q["ghatDDdD"] + v["hDD_dupD"] * ReDD[:, :, None] + v["hDD"][:, :, None] * ReDDdD
    # gammabar RHS (BSSN_RHSs.py:69-96)
    detg, detgd, detgdd = q["detgammahat"], q["detgammahatdD"], q["detgammahatdDD"]
    Dbb = np.zeros(shp)
    for k in R3:
        Dbb = Dbb + betad[k, k] + betaU[k] * detgd[k] / (2 * detg)
    AbarDD = Q.AbarDD
    AUU = np.einsum("ik...,jl...,kl...->ij...", gUU, gUU, AbarDD)
    AUD = np.einsum("ik...,kj...->ij...", gUU, AbarDD)
    trAbar = np.einsum("kj...,jk...->...", gUU, AbarDD)
    grhs = np.zeros((3, 3) + shp)
    for i in R3:
        for j in R3:
            for k in R3:
                grhs[i, j] += betaU[k] * gbar_dup[i, j, k] + betad[k, i] * gbar[k, j] + betad[k, j] * gbar[i, k]
            grhs[i, j] += 2.0 / 3.0 * gbar[i, j] * (alpha * trAbar - Dbb)
            grhs[i, j] += -2 * alpha * AbarDD[i, j]
    # Abar RHS (BSSN_RHSs.py:98-165)
    Adup = ReDDdD * v["aDD"][:, :, None] + ReDD[:, :, None] * v["aDD_dupD"]
    arhs = np.zeros((3, 3) + shp)
    for i in R3:
        for j in R3:
            for k in R3:
                arhs[i, j] += betaU[k] * Adup[i, j, k] + betad[k, i] * AbarDD[k, j] + betad[k, j] * AbarDD[i, k]
            arhs[i, j] += -2.0 / 3.0 * AbarDD[i, j] * Dbb + alpha * AbarDD[i, j] * trK
            for k in R3:
                arhs[i, j] += -2 * alpha * AbarDD[i, k] * AUD[k, j]
    # phi (W) derivatives (BSSN_quantities.py:496-508, 527-534)
    cfd, cfdup, cfdd = v["cf_dD"], v["cf_dupD"], v["cf_dDD"]
    phid = -cfd / (2 * cf)
    phidup = -cfdup / (2 * cf)
    phidd = (-cfdd + cfd[:, None] * cfd[None, :] / cf) / (2 * cf)
    exp_m4phi = cf * cf
    phidBarDD = phidd - np.einsum("kij...,k...->ij...", Gbar, phid)
    ad, add = v["alpha_dD"], v["alpha_dDD"]
    adBarDD = add - np.einsum("kij...,k...->ij...", Gbar, ad)
    curly = np.zeros((3, 3) + shp)
    for i in R3:
        for j in R3:
            curly[i, j] = (-2 * alpha * phidBarDD[i, j] + 4 * alpha * phid[i] * phid[j] + 2 * ad[i] * phid[j]
                           + 2 * ad[j] * phid[i] - adBarDD[i, j] + alpha * RbarDD[i, j])
    curly_tr = np.einsum("ij...,ij...->...", gUU, curly)
    for i in R3:
        for j in R3:
            arhs[i, j] += exp_m4phi * (curly[i, j] - gbar[i, j] * curly_tr / 3.0)
    # cf RHS (BSSN_RHSs.py:167-194)
    cf_rhs = (Dbb - alpha * trK) / 6.0
    for k in R3:
        cf_rhs = cf_rhs + betaU[k] * phidup[k]
    cf_rhs = cf_rhs * (-2 * cf)
    # trK RHS (BSSN_RHSs.py:196-223)
    trK_rhs = alpha * trK * trK / 3.0
    for i in R3:
        trK_rhs = trK_rhs + betaU[i] * v["trK_dupD"][i]
    for i in R3:
        for j in R3:
            trK_rhs = trK_rhs - exp_m4phi * gUU[i, j] * (adBarDD[i, j] + 2 * ad[j] * phid[i])
    trK_rhs = trK_rhs + alpha * np.einsum("ij...,ij...->...", AbarDD, AUU)
    # Lambdabar RHS (BSSN_RHSs.py:225-318)
    lam = v["lambdaU"]
    Ldup = v["lambdaU_dupD"] * ReU[:, None] + lam[:, None] * ReUdD
    Lrhs = np.zeros((3,) + shp)
    for i in R3:
        for k in R3:
            Lrhs[i] += betaU[k] * Ldup[i, k] - betad[i, k] * Lbar[k]
    for i in R3:
        for j in R3:
            for k in R3:
                t = betadd[i, k, j].copy()
                for m in R3:
                    t += GdD[i, m, k, j] * betaU[m] + G[i, m, k] * betad[m, j] + G[i, m, j] * betad[m, k] \
                        - G[m, k, j] * betad[i, m]
                    for d in R3:
                        t += (G[i, d, j] * G[d, m, k] - G[d, k, j] * G[i, m, d]) * betaU[m]
                Lrhs[i] += gUU[j, k] * t
    DGU = Q.DGammaU
    for i in R3:
        Lrhs[i] += 2.0 / 3.0 * DGU[i] * Dbb
    DbbdBar = np.zeros((3,) + shp)
    for k in R3:
        for m in R3:
            DbbdBar[m] += betadd[k, k, m] + (betad[k, m] * detgd[k] + betaU[k] * detgdd[k, m]) / (2 * detg) \
                - betaU[k] * detgd[k] * detgd[m] / (2 * detg * detg)
    for i in R3:
        for m in R3:
            Lrhs[i] += gUU[i, m] * DbbdBar[m] / 3.0
        for j in R3:
            Lrhs[i] += -2 * AUU[i, j] * (ad[j] - 6 * alpha * phid[j])
            for k in R3:
                Lrhs[i] += 2 * alpha * AUU[j, k] * Q.DGammaUDD[i, j, k]
            Lrhs[i] += -4.0 / 3.0 * alpha * gUU[i, j] * v["trK_dD"][j]
    # gauge (BSSN_gauge_RHSs.py:61-67, 191-255)
    alpha_rhs = -2 * alpha * trK
    for i in R3:
        alpha_rhs = alpha_rhs + betaU[i] * v["alpha_dupD"][i]
    BUdup = v["betU_dupD"] * ReU[:, None] + v["betU"][:, None] * ReUdD
    beta_rhs = np.zeros((3,) + shp)
    B_rhs = np.zeros((3,) + shp)
    for i in R3:
        for j in R3:
            beta_rhs[i] += betaU[j] * betadup[i, j]
            for m in R3:
                beta_rhs[i] += betaU[j] * Gbar[i, m, j] * betaU[m]
        beta_rhs[i] += BU[i]
        for j in R3:
            B_rhs[i] += betaU[j] * BUdup[i, j]
            for m in R3:
                B_rhs[i] += betaU[j] * Gbar[i, m, j] * BU[m]
        B_rhs[i] += 0.75 * Lrhs[i]
        for j in R3:
            B_rhs[i] += -0.75 * betaU[j] * Ldup[i, j]
            for m in R3:
                B_rhs[i] += -0.75 * betaU[j] * Gbar[i, m, j] * Lbar[m]
        B_rhs[i] += -eta * BU[i]
    out = {"alpha": alpha_rhs, "cf": cf_rhs, "trK": trK_rhs}
    for i in R3:
        out["lambdaU%d" % i] = Lrhs[i] / ReU[i]
        out["vetU%d" % i] = beta_rhs[i] / ReU[i]
        out["betU%d" % i] = B_rhs[i] / ReU[i]
    for (i, j) in SYM:
        out["hDD%d%d" % (i, j)] = grhs[i, j] / ReDD[i, j]
        out["aDD%d%d" % (i, j)] = arhs[i, j] / ReDD[i, j]
    return out


def hamiltonian(v, q):
    """BSSN_constraints.py:36-74 (H; Ricci evaluated inline)."""
    Q = _Q(v, q)
    Rbar = ricci(v, q, Q)
    gUU, AbarDD, cf, trK = Q.gammabarUU, Q.AbarDD, v["cf"], v["trK"]
    AUU = np.einsum("ik...,jl...,kl...->ij...", gUU, gUU, AbarDD)
    H = 2.0 / 3.0 * trK ** 2 - np.einsum("ij...,ij...->...", AbarDD, AUU)
    cfd, cfdd = v["cf_dD"], v["cf_dDD"]
    phid = -cfd / (2 * cf)
    phidd = (-cfdd + cfd[:, None] * cfd[None, :] / cf) / (2 * cf)
    phidBarDD = phidd - np.einsum("kij...,k...->ij...", Q.GammabarUDD, phid)
    Rtr = np.einsum("ij...,ij...->...", gUU, Rbar)
    pp = np.einsum("ij...,i...,j...->...", gUU, phid, phid)
    pdd = np.einsum("ij...,ij...->...", gUU, phidBarDD)
    return H + cf * cf * (Rtr - 8 * (pp + pdd))


def momentum(v, q):
    """BSSN_constraints.py:76-126: M^i = e^{-4 phi}/ReU^i [gammabar^ik gammabar^jl
    Dbar_j Abar_kl + 6 Abar^ij d_j phi - 2/3 gammabar^ij d_j K], with
    AbarDD_dD from BSSN_quantities.py:247-255 and d_j phi = -d_j W/(2 W)."""
    Q = _Q(v, q)
    gUU, Abar, G = Q.gammabarUU, Q.AbarDD, Q.GammabarUDD
    cf = v["cf"]
    AUU = np.einsum("ik...,jl...,kl...->ij...", gUU, gUU, Abar)
    phid = -v["cf_dD"] / (2 * cf)
    AdD = q["ReDDdD"] * v["aDD"][:, :, None] + q["ReDD"][:, :, None] * v["aDD_dD"]
    AdBar = (AdD - np.einsum("lki...,lj...->ijk...", G, Abar)
             - np.einsum("lkj...,il...->ijk...", G, Abar))
    MU = (6 * np.einsum("ij...,j...->i...", AUU, phid)
          - 2.0 / 3.0 * np.einsum("ij...,j...->i...", gUU, v["trK_dD"])
          + np.einsum("ik...,jl...,klj...->i...", gUU, gUU, AdBar))
    return MU * cf * cf / q["ReU"]


# ----------------------------------------------------- T^{mu nu} sources
T4 = [(0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3)]


def t4uu_full(T10):
    """(10, ...) T4UU00, 01, 02, 03, 11, 12, 13, 22, 23, 33 -> (4, 4, ...)."""
    T = np.empty((4, 4) + np.shape(T10)[1:])
    for n, (a, b) in enumerate(T4):
        T[a, b] = T[b, a] = T10[n]
    return T


def stress_energy(v, q, T):
    """BSSN_stress_energy_source_terms.py:24-85 (inputvars "BSSN") with
    ADMBSSN_tofrom_4metric.py:38-68: S_ij, S_i, S, rho from T^{mu nu} (4, 4,
    ...), with gamma_ij = gammabar_ij / W^2, beta^i = vet^i ReU^i and the
    spatial projector gamma4_{mu nu} = g4_{mu nu} + n_mu n_nu, n_mu = (-alpha, 0, 0, 0)."""
    alpha = v["alpha"]
    gbar = v["hDD"] * q["ReDD"] + q["ghatDD"]
    g = gbar / v["cf"] ** 2
    beta = v["vetU"] * q["ReU"]
    betaD = np.einsum("ij...,j...->i...", g, beta)
    # gamma4[i+1][0] = beta_i, gamma4[i+1][k+1] = gamma_ik
    P = np.empty((3, 4) + np.shape(alpha))
    P[:, 0] = betaD
    P[:, 1:] = g
    SDD = np.einsum("im...,jn...,mn...->ij...", P, P, T)
    SD = alpha * np.einsum("im...,m...->i...", P, T[:, 0])
    gUU, _ = inv3(g)
    S = np.einsum("ij...,ij...->...", gUU, SDD)
    rho = alpha * alpha * T[0, 0]
    return SDD, SD, S, rho


def source_terms(v, q, T, PI=np.pi):
    """BSSN_stress_energy_source_terms.py:88-131 added to the RHSs as the
    BaikalETK drivers add them (BaikalETK_C_kernels_codegen.py:133-145,
    before the gauge RHSs, so the Gamma-driver's B picks up 3/4 of the
    Lambdabar source): returns {gf name: term}."""
    SDD, SD, S, rho = stress_energy(v, q, T)
    alpha, cf = v["alpha"], v["cf"]
    gbar = v["hDD"] * q["ReDD"] + q["ghatDD"]
    gbUU, _ = inv3(gbar)
    trS = np.einsum("km...,km...->...", gbUU, SDD)
    out = {"trK": 4 * PI * alpha * (rho + S)}
    for (i, j) in SYM:
        tf = SDD[i, j] - gbar[i, j] * trS / 3.0
        out["aDD%d%d" % (i, j)] = -8 * PI * alpha * cf * cf * tf / q["ReDD"][i, j]
    LamU = -16 * PI * alpha * np.einsum("ij...,j...->i...", gbUU, SD)
    for i in R3:
        out["lambdaU%d" % i] = LamU[i] / q["ReU"][i]
        out["betU%d" % i] = 0.75 * LamU[i] / q["ReU"][i]
    return out, LamU


def constraint_source_terms(v, q, T, PI=np.pi):
    """BSSN_stress_energy_source_terms.py:134-161: (-16 pi rho, -8 pi S^i / ReU^i)."""
    SDD, SD, S, rho = stress_energy(v, q, T)
    gbar = v["hDD"] * q["ReDD"] + q["ghatDD"]
    gUU, _ = inv3(gbar / v["cf"] ** 2)
    SU = np.einsum("ij...,j...->i...", gUU, SD)
    return -16 * PI * rho, -8 * PI * SU / q["ReU"]


# ------------------------------------------------------------------ grids
def grid_symbols(gp, gfs, need_ricci=True):
    """Symbol values at interior points from FD of a (24, n2, n1, n0) array."""
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    f = {n: gfs[GF[n]] for n in EVOL}
    g = gp.NGHOSTS
    # hatted arrays broadcast over the interior (an i2 or i1 axis of length 1)
    q = hatted_grid(gp, interior=True)
    v = {}

    def t2(base):
        a = np.empty((3, 3) + (gp.Nxx[2], gp.Nxx[1], gp.Nxx[0]))
        for (i, j) in SYM:
            a[i, j] = a[j, i] = S.interior(f[base + "%d%d" % (i, j)])
        return a

    v["hDD"], v["aDD"] = t2("hDD"), t2("aDD")
    for b in ("lambdaU", "vetU", "betU"):
        v[b] = np.array([S.interior(f[b + str(i)]) for i in R3])
    for b in ("alpha", "cf", "trK"):
        v[b] = S.interior(f[b])
    betaU = v["vetU"] * q["ReU"]
    ctrl = [betaU[d] for d in R3]

    def d1(a, d):
        return S.d1(a, d)

    def dup(a, d):
        return S.dupwind(a, d, ctrl[d])

    v["hDD_dD"] = np.empty((3, 3, 3) + v["cf"].shape)
    v["hDD_dupD"] = np.empty_like(v["hDD_dD"])
    v["aDD_dupD"] = np.empty_like(v["hDD_dD"])
    for (i, j) in SYM:
        for k in R3:
            v["hDD_dD"][i, j, k] = v["hDD_dD"][j, i, k] = d1(f["hDD%d%d" % (i, j)], k)
            v["hDD_dupD"][i, j, k] = v["hDD_dupD"][j, i, k] = dup(f["hDD%d%d" % (i, j)], k)
            v["aDD_dupD"][i, j, k] = v["aDD_dupD"][j, i, k] = dup(f["aDD%d%d" % (i, j)], k)
    if need_ricci:
        v["hDD_dDD"] = np.empty((3, 3, 3, 3) + v["cf"].shape)
        for (i, j) in SYM:
            for (k, l) in SYM:
                d = S.d11(f["hDD%d%d" % (i, j)], k, l)
                for a, b in ((i, j), (j, i)):
                    v["hDD_dDD"][a, b, k, l] = v["hDD_dDD"][a, b, l, k] = d
    for b in ("lambdaU", "vetU", "betU"):
        v[b + "_dD"] = np.array([[d1(f[b + str(i)], j) for j in R3] for i in R3])
        v[b + "_dupD"] = np.array([[dup(f[b + str(i)], j) for j in R3] for i in R3])
    v["vetU_dDD"] = np.empty((3, 3, 3) + v["cf"].shape)
    for i in R3:
        for (j, k) in SYM:
            v["vetU_dDD"][i, j, k] = v["vetU_dDD"][i, k, j] = S.d11(f["vetU%d" % i], j, k)
    for b in ("alpha", "cf", "trK"):
        v[b + "_dD"] = np.array([d1(f[b], j) for j in R3])
        v[b + "_dupD"] = np.array([dup(f[b], j) for j in R3])
    for b in ("alpha", "cf"):
        a = np.empty((3, 3) + v["cf"].shape)
        for (j, k) in SYM:
            a[j, k] = a[k, j] = S.d11(f[b], j, k)
        v[b + "_dDD"] = a
    return v, q


def ricci_grid(gp, gfs):
    """Ricci_eval: RbarDD (6, n2, n1, n0) at interior points, zero elsewhere."""
    v, q = grid_symbols(gp, gfs)
    R = ricci(v, q)
    out = np.zeros((6,) + gp.shape)
    for n, (i, j) in enumerate(SYM):
        gp.interior(out[n])[...] = R[i, j]
    return out


def rhs_grid(gp, gfs, RbarDD6=None, diss_strength=0.0, T4UU10=None):
    """rhs_eval: 24 RHSs at interior points (zero elsewhere).  RbarDD6, if
    given, is the (6, n2, n1, n0) auxevol array (LeaveRicciSymbolic form).
    diss_strength != 0 adds Kreiss-Oliger dissipation to every RHS,
    diss_strength * sum_k f_dKOD[k] * ReU[k]
    (BaikalETK/BaikalETK_C_kernels_codegen.py:147-171).  T4UU10, if given,
    is the (10, n2, n1, n0) stress-energy tensor (T4UU00, 01, 02, 03, 11,
    12, 13, 22, 23, 33) whose source terms are added (source_terms)."""
    v, q = grid_symbols(gp, gfs, need_ricci=RbarDD6 is None)
    Rbar = None
    if RbarDD6 is not None:
        Rbar = np.empty((3, 3) + v["cf"].shape)
        for n, (i, j) in enumerate(SYM):
            Rbar[i, j] = Rbar[j, i] = gp.interior(RbarDD6[n])
    r = rhs(v, q, gp.eta, Rbar)
    if T4UU10 is not None:
        src, _ = source_terms(v, q, t4uu_full(np.array([gp.interior(t) for t in T4UU10])))
        r = dict(r)
        for k, val in src.items():
            r[k] = r[k] + val
    out = np.zeros((24,) + gp.shape)
    if diss_strength != 0.0:
        S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
        ReU = q["ReU"]
    for n, name in enumerate(EVOL):
        val = r[name]
        if diss_strength != 0.0:
            ko = sum(S.dko(gfs[GF[name]], k) * ReU[k] for k in R3)
            val = val + diss_strength * ko
        gp.interior(out[n])[...] = val
    return out


def hamiltonian_grid(gp, gfs, T4UU10=None):
    v, q = grid_symbols(gp, gfs)
    out = np.zeros(gp.shape)
    H = hamiltonian(v, q)
    if T4UU10 is not None:
        H = H + constraint_source_terms(v, q, t4uu_full(np.array([gp.interior(t) for t in T4UU10])))[0]
    gp.interior(out)[...] = H
    return out


def momentum_grid(gp, gfs, T4UU10=None):
    """M^i (3, n2, n1, n0) at interior points, zero elsewhere (with the
    -8 pi S^i / ReU^i matter term when T4UU10 is given)."""
    v, q = grid_symbols(gp, gfs, need_ricci=False)
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    f = {n: gfs[GF[n]] for n in EVOL}
    a = np.empty((3, 3, 3) + v["cf"].shape)
    for (i, j) in SYM:
        for k in R3:
            a[i, j, k] = a[j, i, k] = S.d1(f["aDD%d%d" % (i, j)], k)
    v["aDD_dD"] = a
    M = momentum(v, q)
    if T4UU10 is not None:
        M = M + constraint_source_terms(v, q, t4uu_full(np.array([gp.interior(t) for t in T4UU10])))[1]
    out = np.zeros((3,) + gp.shape)
    for i in R3:
        gp.interior(out[i])[...] = M[i]
    return out


def enforce_detgammabar(gp, gfs):
    """Enforce_Detgammabar_Constraint.py:42-50 at ALL points (in place copy)."""
    qf = hatted_grid(gp)
    out = gfs.copy()
    h = np.empty((3, 3) + gp.shape)
    for (i, j) in SYM:
        h[i, j] = h[j, i] = gfs[GF["hDD%d%d" % (i, j)]]
    gbar = h * qf["ReDD"] + qf["ghatDD"]
    _, det = inv3(gbar)
    fac = np.cbrt(np.abs(qf["detgammahat"]) / det)
    for (i, j) in SYM:
        d = 1.0 if i == j else 0.0
        out[GF["hDD%d%d" % (i, j)]] = fac * (d + h[i, j]) - d
    return out
