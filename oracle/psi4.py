"""psi_4 from the BSSN variables, the quasi-Kinnersley tetrad, and the
spin-weight -2 spherical-harmonic decomposition on an extraction shell (numpy).

TEST INFRASTRUCTURE (see oracle/__init__.py).

Restated from (zachetienne/nrpytutorial):
  BSSN/ADM_in_terms_of_BSSN.py:20-170   physical metric, its first and second
                                        derivatives, Christoffels, K_ij and its
                                        derivative from the BSSN variables (W = cf)
  BSSN/BSSN_quantities.py:118-155, 250-255  gammabar and Abar derivatives
  BSSN/Psi4.py:14-193                   3+1 Riemann tensor and the three terms
                                        of Baker, Campanelli & Lousto (2002) eq. 5.1
  BSSN/Psi4_tetrads.py:25-193           quasi-Kinnersley tetrad (Gram-Schmidt of
                                        phi-hat, r-hat and their cross product
                                        in the physical metric; u = (1,0,0,0))
  SpinWeight_minus2_SphHarmonics/SpinWeight_minus2_SphHarmonics.py:22-48
                                        Goldberg's formula for sY_lm, s = -2
  Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide-Psi4.ipynb
    (driver_psi4_spinweightm2_decomposition, lowlevel_decompose_psi4_into_swm2_modes):
                                        psi4_lm = sum over the shell's (theta, phi)
                                        cells of psi4 conj(Y) sin(theta) dtheta dphi

Arrays keep tensor indices first and point axes last, as in oracle/bssn.py.
Functions accept complex inputs (the reference's trusted-value test feeds
random symbol values for which the tetrad normalisation is imaginary).
"""
from math import comb, factorial, pi

import numpy as np

from .bssn import GF, R3, SYM, inv3
from .fd import Stencils
from .grid import CART, SPH, cylinder_maps, cylindrical, hatted_grid, radial

ISQRT2 = 0.707106781186547524400844362104849039


def _csqrt(x):
    x = np.asarray(x)
    if np.iscomplexobj(x) or np.any(x < 0):
        return np.sqrt(x.astype(complex))
    return np.sqrt(x)


def adm_from_bssn(v, q):
    """ADM quantities of ADM_in_terms_of_BSSN.py from symbol values v
    (hDD, hDD_dD, hDD_dDD, aDD, aDD_dD, cf, cf_dD, cf_dDD, trK, trK_dD) and
    hatted quantities q (ghatDD, ghatDDdD, ghatDDdDD, ReDD, ReDDdD, ReDDdDD).
    The evolved conformal factor is W: exp(4 phi) = 1 / cf^2."""
    h, hd, hdd = v["hDD"], v["hDD_dD"], v["hDD_dDD"]
    ReDD, ReDDdD, ReDDdDD = q["ReDD"], q["ReDDdD"], q["ReDDdDD"]
    gbar = h * ReDD + q["ghatDD"]
    gbar_d = q["ghatDDdD"] + hd * ReDD[:, :, None] + h[:, :, None] * ReDDdD
    gbar_dd = (q["ghatDDdDD"] + hdd * ReDD[:, :, None, None] + hd[:, :, :, None] * ReDDdD[:, :, None, :]
               + hd[:, :, None, :] * ReDDdD[:, :, :, None] + h[:, :, None, None] * ReDDdDD)
    Abar = v["aDD"] * ReDD
    Abar_d = ReDDdD * v["aDD"][:, :, None] + ReDD[:, :, None] * v["aDD_dD"]
    cf, cfd, cfdd = v["cf"], v["cf_dD"], v["cf_dDD"]
    e4 = 1.0 / cf ** 2
    e2 = 1.0 / cf
    phid = -0.5 * e2 * cfd
    phidd = 0.5 * (e4 * cfd[:, None] * cfd[None, :] - e2 * cfdd)
    e4d = 4.0 * e4 * phid
    e4dd = 16.0 * e4 * phid[:, None] * phid[None, :] + 4.0 * e4 * phidd
    g = e4 * gbar
    gd = e4d[None, None, :] * gbar[:, :, None] + e4 * gbar_d
    gdd = (e4dd[None, None] * gbar[:, :, None, None] + e4d[None, None, :, None] * gbar_d[:, :, None, :]
           + e4d[None, None, None, :] * gbar_d[:, :, :, None] + e4 * gbar_dd)
    gUU, detg = inv3(g)
    G = np.zeros((3, 3, 3) + np.shape(cf), dtype=np.result_type(g, gd))
    for i in R3:
        for j in R3:
            for k in R3:
                for l in R3:
                    G[i, j, k] = G[i, j, k] + 0.5 * gUU[i, l] * (gd[l, j, k] + gd[l, k, j] - gd[j, k, l])
    trK, trKd = v["trK"], v["trK_dD"]
    K = e4 * Abar + g * trK / 3.0
    Kd = (e4d[None, None, :] * Abar[:, :, None] + e4 * Abar_d
          + (gd * trK + g[:, :, None] * trKd[None, None, :]) / 3.0)
    return dict(gammaDD=g, gammaDDdD=gd, gammaDDdDD=gdd, gammaUU=gUU, detgamma=detg, GammaUDD=G, KDD=K,
                KDDdD=Kd)


def psi4_parts(adm, n4U, mre4U, mim4U):
    """Psi4.py:50-193: the real and imaginary parts of psi_4 in three pieces
    each, given the tetrad vectors n, Re(m), Im(m) (4-vectors, index 0 = t)."""
    g, gdd, gUU, G, K, Kd = (adm[k] for k in ("gammaDD", "gammaDDdDD", "gammaUU", "GammaUDD", "KDD", "KDDdD"))
    # Riemann R_iklm of the 3-metric (:50-72)
    R = np.zeros((3, 3, 3, 3) + g.shape[2:], dtype=np.result_type(g, gdd, G))
    for i in R3:
        for k in R3:
            for l in R3:
                for m in R3:
                    r = 0.5 * (gdd[i, m, k, l] + gdd[k, l, i, m] - gdd[i, l, k, m] - gdd[k, m, i, l])
                    for n in R3:
                        for p in R3:
                            r = r + g[n, p] * (G[n, k, l] * G[p, i, m] - G[n, k, m] * G[p, i, l])
                    R[i, k, l, m] = r
    # term 1 (:76-85), term 2 (:89-110), term 3 (:114-144)
    t1 = np.zeros_like(R, dtype=np.result_type(R, K))
    for i in R3:
        for j in R3:
            for k in R3:
                for l in R3:
                    t1[i, j, k, l] = R[i, j, k, l] + K[i, k] * K[l, j] - K[i, l] * K[k, j]
    t2 = np.zeros((3, 3, 3) + g.shape[2:], dtype=np.result_type(Kd, G, K))
    for j in R3:
        for k in R3:
            for l in R3:
                a = 0.5 * (Kd[j, k, l] - Kd[j, l, k])
                for p in R3:
                    a = a + 0.5 * (G[p, j, k] * K[l, p] - G[p, j, l] * K[k, p])
                t2[j, k, l] = -8.0 * a
    RDD = np.einsum("im...,ijml...->jl...", gUU, R)
    KUD = np.einsum("pi...,il...->pl...", gUU, K)
    trK = np.einsum("ij...,ij...->...", gUU, K)
    t3 = np.zeros((3, 3) + g.shape[2:], dtype=np.result_type(RDD, K))
    for j in R3:
        for l in R3:
            a = RDD[j, l] + trK * K[j, l]
            for p in R3:
                a = a - K[j, p] * KUD[p, l]
            t3[j, l] = 4.0 * a
    n, Mr, Mi = n4U, mre4U, mim4U

    def T_re(mu, nu, eta, de):
        return n[mu] * Mr[nu] * n[eta] * Mr[de] - n[mu] * Mi[nu] * n[eta] * Mi[de]

    def T_im(mu, nu, eta, de):
        return -n[mu] * Mr[nu] * n[eta] * Mi[de] - n[mu] * Mi[nu] * n[eta] * Mr[de]

    re, im = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    for i in R3:
        for j in R3:
            for k in R3:
                for l in R3:
                    re[0] = re[0] + t1[i, j, k, l] * T_re(i + 1, j + 1, k + 1, l + 1)
                    im[0] = im[0] + t1[i, j, k, l] * T_im(i + 1, j + 1, k + 1, l + 1)
    for j in R3:
        for k in R3:
            for l in R3:
                re[1] = re[1] + t2[j, k, l] * 0.5 * (T_re(0, j + 1, k + 1, l + 1) - T_re(j + 1, 0, k + 1, l + 1))
                im[1] = im[1] + t2[j, k, l] * 0.5 * (T_im(0, j + 1, k + 1, l + 1) - T_im(j + 1, 0, k + 1, l + 1))
    for j in R3:
        for l in R3:
            re[2] = re[2] + t3[j, l] * 0.25 * (T_re(0, j + 1, 0, l + 1) - T_re(j + 1, 0, 0, l + 1)
                                               - T_re(0, j + 1, l + 1, 0) + T_re(j + 1, 0, l + 1, 0))
            im[2] = im[2] + t3[j, l] * 0.25 * (T_im(0, j + 1, 0, l + 1) - T_im(j + 1, 0, 0, l + 1)
                                               - T_im(0, j + 1, l + 1, 0) + T_im(j + 1, 0, l + 1, 0))
    return re, im


def cart_and_jacobian(cs, xx0, xx1, xx2, AMPL=10.0, SINHW=0.2, const_dr=0.0625, cyl=None):
    """xx_to_Cart (reference_metric.py: Spherical :159-161, SinhSpherical
    and SinhSphericalv2 :210-212 with their r(xx0), the Cylindrical family
    :296-298 (cyl: a GridParams carrying its parameters), Cartesian identity)
    and the Jacobian d x_Cart^i / d xx^j."""
    xx0, xx1, xx2 = np.broadcast_arrays(*(np.asarray(a, dtype=float) for a in (xx0, xx1, xx2)))
    if cs == CART:
        one, zero = np.ones_like(xx0), np.zeros_like(xx0)
        J = np.array([[one, zero, zero], [zero, one, zero], [zero, zero, one]])
        return np.array([xx0, xx1, xx2]), J
    if cs in (7, 8):  # SymTP family, reference_metric.py:334-336
        b = cyl.bScale
        if cs == 8:
            from .grid import sinh_map
            A, dA = sinh_map(cyl.AMAX, cyl.SINHWAA, xx0)
        else:
            A, dA = xx0, np.ones_like(xx0)
        st, ct, sp_, cp = np.sin(xx1), np.cos(xx1), np.sin(xx2), np.cos(xx2)
        v2 = np.sqrt(A * A + b * b)
        zero = np.zeros_like(A)
        x = np.array([A * st * cp, A * st * sp_, v2 * ct])
        J = np.array([[dA * st * cp, A * ct * cp, -A * st * sp_], [dA * st * sp_, A * ct * sp_, A * st * cp],
                      [A * dA / v2 * ct, -v2 * st, zero]])
        return x, J
    if cylindrical(cs):  # (rho cos phi, rho sin phi, z), reference_metric.py:296-298
        (rho, drho), (z, dz) = cylinder_maps(cyl, xx0, xx2)
        sp_, cp = np.sin(xx1), np.cos(xx1)
        zero = np.zeros_like(rho)
        x = np.array([rho * cp, rho * sp_, z])
        J = np.array([[drho * cp, -rho * sp_, zero], [drho * sp_, rho * cp, zero], [zero, zero, dz]])
        return x, J
    r, drdx = radial(cs, xx0, AMPL, SINHW, const_dr)
    st, ct, sp_, cp = np.sin(xx1), np.cos(xx1), np.sin(xx2), np.cos(xx2)
    x = np.array([r * st * cp, r * st * sp_, r * ct])
    J = np.array([[drdx * st * cp, r * ct * cp, -r * st * sp_],
                  [drdx * st * sp_, r * ct * sp_, r * st * cp],
                  [drdx * ct, -r * st, np.zeros_like(r)]])
    return x, J


def _inv_general(J):
    """3x3 inverse by cofactors (indexedexp.py generic_matrix_inverter3x3)."""
    c = np.empty_like(J)
    c[0, 0] = J[1, 1] * J[2, 2] - J[1, 2] * J[2, 1]
    c[0, 1] = J[0, 2] * J[2, 1] - J[0, 1] * J[2, 2]
    c[0, 2] = J[0, 1] * J[1, 2] - J[0, 2] * J[1, 1]
    c[1, 0] = J[1, 2] * J[2, 0] - J[1, 0] * J[2, 2]
    c[1, 1] = J[0, 0] * J[2, 2] - J[0, 2] * J[2, 0]
    c[1, 2] = J[0, 2] * J[1, 0] - J[0, 0] * J[1, 2]
    c[2, 0] = J[1, 0] * J[2, 1] - J[1, 1] * J[2, 0]
    c[2, 1] = J[0, 1] * J[2, 0] - J[0, 0] * J[2, 1]
    c[2, 2] = J[0, 0] * J[1, 1] - J[0, 1] * J[1, 0]
    det = J[0, 0] * c[0, 0] + J[0, 1] * c[1, 0] + J[0, 2] * c[2, 0]
    return c / det


def tetrad(gammaDD, cs, xx0, xx1, xx2, AMPL=10.0, SINHW=0.2, const_dr=0.0625, cyl=None):
    """Psi4_tetrads.py:50-193 (QuasiKinnersley, UseCorrectUnitNormal False):
    returns l4U, n4U, mre4U, mim4U (lists of 4 arrays)."""
    x, J = cart_and_jacobian(cs, xx0, xx1, xx2, AMPL, SINHW, const_dr, cyl)
    Ji = _inv_general(J)
    gUU, detg = inv3(gammaDD)
    v1C = [-x[1], x[0], np.zeros_like(x[0])]
    v2C = [x[0], x[1], x[2]]
    v1 = [sum(Ji[i, j] * v1C[j] for j in R3) for i in R3]
    v2 = [sum(Ji[i, j] * v2C[j] for j in R3) for i in R3]
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1.0
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1.0
    sq = _csqrt(detg)
    v3 = [0.0, 0.0, 0.0]
    for a in R3:
        for b in R3:
            for c in R3:
                for d in R3:
                    if eps[d, b, c] != 0.0:
                        v3[a] = v3[a] + sq * gUU[a, d] * eps[d, b, c] * v1[b] * v2[c]

    def om(u, w):
        return sum(u[a] * w[b] * gammaDD[a, b] for a in R3 for b in R3)

    e1 = [v1[a] / _csqrt(om(v1, v1)) for a in R3]
    w01 = om(e1, v2)
    e2 = [v2[a] - w01 * e1[a] for a in R3]
    n2 = _csqrt(om(e2, e2))
    e2 = [e2[a] / n2 for a in R3]
    w02, w12 = om(e1, v3), om(e2, v3)
    e3 = [v3[a] - w02 * e1[a] - w12 * e2[a] for a in R3]
    n3 = _csqrt(om(e3, e3))
    e3 = [e3[a] / n3 for a in R3]
    zero = np.zeros_like(np.asarray(x[0]))
    u4 = [zero + 1.0, zero, zero, zero]
    r4 = [zero] + e2
    th4 = [zero] + e3
    ph4 = [zero] + e1
    l4 = [ISQRT2 * (u4[m] + r4[m]) for m in range(4)]
    n4 = [ISQRT2 * (u4[m] - r4[m]) for m in range(4)]
    mre = [ISQRT2 * th4[m] for m in range(4)]
    mim = [ISQRT2 * ph4[m] for m in range(4)]
    return l4, n4, mre, mim


# ------------------------------------------------------------------ grids
def psi4_grid(gp, gfs, i0_range=None):
    """psi_4 (real, imaginary) at interior points of a (24, n2, n1, n0)
    BSSN state (zero elsewhere), optionally only for i0 in i0_range
    (a radial shell of a spherical-like grid).  Second-order-accurate
    centred FD of gp.FD_order for every derivative, as FD_outputC writes
    them for the psi4 expressions."""
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    g = gp.NGHOSTS
    f = {n: gfs[GF[n]] for n in GF}
    q = hatted_grid(gp, interior=True)
    shp = (gp.Nxx[2], gp.Nxx[1], gp.Nxx[0])
    v = {}

    def t2(base):
        a = np.empty((3, 3) + shp)
        for (i, j) in SYM:
            a[i, j] = a[j, i] = S.interior(f[base + "%d%d" % (i, j)])
        return a

    v["hDD"], v["aDD"] = t2("hDD"), t2("aDD")
    v["cf"], v["trK"] = S.interior(f["cf"]), S.interior(f["trK"])
    v["hDD_dD"] = np.empty((3, 3, 3) + shp)
    v["aDD_dD"] = np.empty((3, 3, 3) + shp)
    v["hDD_dDD"] = np.empty((3, 3, 3, 3) + shp)
    for (i, j) in SYM:
        for k in R3:
            v["hDD_dD"][i, j, k] = v["hDD_dD"][j, i, k] = S.d1(f["hDD%d%d" % (i, j)], k)
            v["aDD_dD"][i, j, k] = v["aDD_dD"][j, i, k] = S.d1(f["aDD%d%d" % (i, j)], k)
        for (k, l) in SYM:
            d = S.d11(f["hDD%d%d" % (i, j)], k, l)
            for a, b in ((i, j), (j, i)):
                v["hDD_dDD"][a, b, k, l] = v["hDD_dDD"][a, b, l, k] = d
    v["cf_dD"] = np.array([S.d1(f["cf"], k) for k in R3])
    v["trK_dD"] = np.array([S.d1(f["trK"], k) for k in R3])
    v["cf_dDD"] = np.empty((3, 3) + shp)
    for (k, l) in SYM:
        v["cf_dDD"][k, l] = v["cf_dDD"][l, k] = S.d11(f["cf"], k, l)
    adm = adm_from_bssn(v, q)
    X2, X1, X0 = np.meshgrid(gp.xx[2][g:-g], gp.xx[1][g:-g], gp.xx[0][g:-g], indexing="ij")
    _, n4, mre, mim = tetrad(adm["gammaDD"], gp.CoordSystem, X0, X1, X2, gp.AMPL, gp.SINHW, gp.const_dr, gp)
    re, im = psi4_parts(adm, n4, mre, mim)
    out = np.zeros((2,) + gp.shape)
    gp.interior(out[0])[...] = re[0] + re[1] + re[2]
    gp.interior(out[1])[...] = im[0] + im[1] + im[2]
    if i0_range is not None:
        keep = np.zeros(gp.shape[2], dtype=bool)
        keep[i0_range[0]:i0_range[1]] = True
        out[:, :, :, ~keep] = 0.0
    return out


# ------------------------------------------- spin-weight -2 harmonics
def swsh_m2(l, m, th, ph):
    """Goldberg's formula (SpinWeight_minus2_SphHarmonics.py:31-43) for
    s = -2: returns (Re, Im) of sY_lm(th, ph).  sin^{2l}(th/2) cot^k(th/2)
    is evaluated as sin^{2l-k}(th/2) cos^k(th/2) (k = 2r + s - m lies in
    [0, 2l] wherever the binomials are nonzero)."""
    s = -2
    th, ph = np.asarray(th, dtype=float), np.asarray(ph, dtype=float)
    acc = np.zeros(np.broadcast(th, ph).shape)
    if l < -s:
        return acc, acc.copy()  # no spin-weight -2 harmonics below l = 2 (the reference's C writes 0)
    sh, ch = np.sin(th / 2), np.cos(th / 2)
    for r in range(l - s + 1):
        b2 = r + s - m
        if b2 < 0 or b2 > l + s:
            continue
        k = 2 * r + s - m
        acc = acc + comb(l - s, r) * comb(l + s, b2) * (-1.0) ** (l - r - s) * sh ** (2 * l - k) * ch ** k
    norm = (-1.0) ** m * np.sqrt(factorial(l + m) * factorial(l - m) * (2 * l + 1)
                                 / (4 * pi * factorial(l + s) * factorial(l - s)))
    return norm * acc * np.cos(m * ph), norm * acc * np.sin(m * ph)


def swm2_modes(gp, psi4, i0, l_max=8):
    """Mode coefficients psi4_lm (l = 2..l_max, m = -l..l) on the shell of
    radial index i0: sum over interior (i1, i2) of psi4 conj(Y) sin(th)
    dxx1 dxx2 (midpoint rule in th, ph), as lowlevel_decompose_psi4_into_swm2_modes
    integrates.  Returns {(l, m): (re, im)}."""
    g = gp.NGHOSTS
    th = np.asarray(gp.xx[1][g:-g])[:, None]
    ph = np.asarray(gp.xx[2][g:-g])[None, :]
    a = psi4[0][g:-g, g:-g, i0].T  # (i1, i2)
    b = psi4[1][g:-g, g:-g, i0].T
    w = np.sin(th) * gp.dxx[1] * gp.dxx[2]
    out = {}
    for l in range(2, l_max + 1):
        for m in range(-l, l + 1):
            c, d = swsh_m2(l, m, th, ph)
            out[(l, m)] = (float(np.sum((a * c + b * d) * w)), float(np.sum((b * c - a * d) * w)))
    return out
