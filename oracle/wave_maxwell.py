"""ScalarWave and vacuum-Maxwell RHSs, initial data and exact solutions (numpy).

TEST INFRASTRUCTURE (see oracle/__init__.py).

  ScalarWave/ScalarWave_RHSs.py:46-71              uu_rhs = vv, vv_rhs = c^2 sum_i uu_dDii
  ScalarWave/ScalarWaveCurvilinear_RHSs.py:43-98    vv_rhs = c^2 (ghat^ij uu_dDij - ghat^ij Gammahat^k_ij uu_dDk)
  Maxwell/VacuumMaxwell_Flat_Evol_Cartesian.py:49-74  System I RHSs and C = d_i E^i
  Maxwell/InitialData.py:26-117                      toroidal dipole A, E = -d_t A, psi = 0
"""
import numpy as np

from .fd import Stencils
from .grid import CART, hatted_grid, radial


def scalarwave_rhs_grid(gp, gfs):
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    uu, vv = gfs[0], gfs[1]
    out = np.zeros((2,) + gp.shape)
    c2 = gp.wavespeed ** 2
    if gp.CoordSystem == CART:
        lap = S.d2(uu, 0) + S.d2(uu, 1) + S.d2(uu, 2)
        rhs_v = c2 * lap
    else:
        g = gp.NGHOSTS
        q = hatted_grid(gp, interior=True)
        gUU, G = q["ghatUU"], q["GammahatUDD"]
        contracted = np.einsum("ij...,kij...->k...", gUU, G)
        acc = 0.0
        for i in range(3):
            acc = acc - contracted[i] * S.d1(uu, i)
            for j in range(3):
                if i == j:
                    acc = acc + gUU[i, j] * S.d2(uu, i)
        rhs_v = acc * c2
    gp.interior(out[0])[...] = S.interior(vv)
    gp.interior(out[1])[...] = rhs_v
    return out


def scalarwave_pointwise(v, q, c, cartesian):
    """uu_rhs, vv_rhs from symbol values (uu, vv, uu_dD[3], uu_dDD[3][3])."""
    if cartesian:
        return v["vv"], c * c * (v["uu_dDD"][0, 0] + v["uu_dDD"][1, 1] + v["uu_dDD"][2, 2])
    gUU, G = q["ghatUU"], q["GammahatUDD"]
    contracted = np.einsum("ij...,kij...->k...", gUU, G)
    acc = 0.0
    for i in range(3):
        acc = acc - contracted[i] * v["uu_dD"][i]
        for j in range(3):
            acc = acc + gUU[i, j] * v["uu_dDD"][i, j]
    return v["vv"], acc * c * c


def maxwell_pointwise(v):
    """System I RHSs and C from symbol values (VacuumMaxwell_Flat_Evol_Cartesian.py:49-74)."""
    E, AdD, AdDD, psid = v["EU"], v["AU_dD"], v["AU_dDD"], v["psi_dD"]
    Arhs = [-E[i] - psid[i] for i in range(3)]
    Erhs = []
    for i in range(3):
        acc = 0.0
        for j in range(3):
            if j != i:
                acc = acc - AdDD[i, j, j] + AdDD[j, j, i]
        Erhs.append(acc)
    psi_rhs = -(AdD[0, 0] + AdD[1, 1] + AdD[2, 2])
    C = v["EU_dD"][0, 0] + v["EU_dD"][1, 1] + v["EU_dD"][2, 2]
    return Arhs, Erhs, psi_rhs, C


def plane_wave(gp, t, kvec=(2 * np.pi / 20,) * 3, c=1.0):
    """Plane wave u = sin(k.x - |k| c t), v = d_t u at every point (Cartesian)."""
    x = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")  # (i2, i1, i0)
    z, y, xx = x
    k = np.asarray(kvec, dtype=float)
    kn = np.sqrt((k ** 2).sum())
    ph = k[0] * xx + k[1] * y + k[2] * z - kn * c * t
    return np.array([np.sin(ph), -kn * c * np.cos(ph)])


def maxwell_rhs_grid(gp, gfs):
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    A, E, psi = gfs[0:3], gfs[3:6], gfs[6]
    out = np.zeros((7,) + gp.shape)
    for i in range(3):
        gp.interior(out[i])[...] = -S.interior(E[i]) - S.d1(psi, i)
    for i in range(3):
        acc = 0.0
        for j in range(3):
            if j == i:
                continue  # -A^i_{,jj} + A^j_{,ji} cancels symbolically for j == i
            acc = acc - S.d2(A[i], j) + S.d11(A[j], j, i)
        gp.interior(out[3 + i])[...] = acc
    gp.interior(out[6])[...] = -(S.d1(A[0], 0) + S.d1(A[1], 1) + S.d1(A[2], 2))
    return out


def maxwell_constraint_grid(gp, gfs):
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    out = np.zeros(gp.shape)
    gp.interior(out)[...] = S.d1(gfs[3], 0) + S.d1(gfs[4], 1) + S.d1(gfs[5], 2)
    return out


def toroidal_dipole(gp, t, amp=1.0, lam=1.0):
    """Exact toroidal-dipole solution (Maxwell/InitialData.py:41-104) at all
    points of a Cartesian grid: A^i, E^i = -d_t A^i, psi = 0.

    The reference sets A_phi = A_phi-hat / (r sin_theta) with its
    sin_theta = z/r and A_phi-hat = amp sin_theta [(e^{-lam v^2} -
    e^{-lam u^2})/r^2 - 2 lam (v e^{-lam v^2} + u e^{-lam u^2})/r],
    u = t + r, v = t - r, then maps A^i_Cart = (dx^i/dphi) A_phi with
    dx/dphi = (-y, x, 0).  The z/r factors cancel, leaving
    A = F(r,t) (-y, x, 0) with F = amp/r [ ... ].
    """
    z, y, x = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
    r = np.sqrt(x * x + y * y + z * z)
    u, v = t + r, t - r
    eu, ev = np.exp(-lam * u ** 2), np.exp(-lam * v ** 2)
    deu, dev = -2 * lam * u * eu, -2 * lam * v * ev
    F = amp / r * ((ev - eu) / r ** 2 - 2 * lam * (v * ev + u * eu) / r)
    dF = amp / r * ((dev - deu) / r ** 2 - 2 * lam * (ev + v * dev + eu + u * deu) / r)
    out = np.zeros((7,) + gp.shape)
    out[0], out[1] = -y * F, x * F
    out[3], out[4] = y * dF, -x * dF
    return out


def scalarwave_id_pointwise(kind, x, y, z, t, c, k=(1.0, 1.0, 1.0), sigma=3.0):
    """ScalarWave/InitialData.py:27-88 at Cartesian points.
    PlaneWave: uu = sin(khat.x - c t) + 2, vv = -c cos(khat.x - c t), khat = k/|k|.
    SphericalGaussian: uu = (r-ct)/r e^{-(r-ct)^2/(2 s^2)} + (r+ct)/r e^{-(r+ct)^2/(2 s^2)} + 1,
    vv = d uu/dt = c/r [e_a ((r-ct)^2/s^2 - 1) + e_b (1 - (r+ct)^2/s^2)]."""
    if kind == "PlaneWave":
        kn = np.sqrt(k[0] ** 2 + k[1] ** 2 + k[2] ** 2)
        ph = (k[0] * x + k[1] * y + k[2] * z) / kn - c * t
        return np.sin(ph) + 2.0, -c * np.cos(ph)
    r = np.sqrt(x * x + y * y + z * z)
    a, b = r - c * t, r + c * t
    ea, eb = np.exp(-a * a / (2 * sigma ** 2)), np.exp(-b * b / (2 * sigma ** 2))
    uu = a / r * ea + b / r * eb + 1.0
    vv = c / r * (ea * (a * a / sigma ** 2 - 1.0) + eb * (1.0 - b * b / sigma ** 2))
    return uu, vv


def scalarwave_id_grid(gp, kind, t=0.0, k=(1.0, 1.0, 1.0), sigma=3.0):
    """(2, n2, n1, n0) initial data at every point of a grid (Cartesian
    coordinates from xx_to_Cart of the grid's CoordSystem)."""
    X2, X1, X0 = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
    if gp.CoordSystem == 0:
        x, y, z = X0, X1, X2
    elif gp.CoordSystem in (4, 5, 6, 7, 8):  # Cylindrical and SymTP families
        from .psi4 import cart_and_jacobian
        (x, y, z), _ = cart_and_jacobian(gp.CoordSystem, X0, X1, X2, cyl=gp)
    else:
        r, _ = radial(gp.CoordSystem, X0, gp.AMPL, gp.SINHW, gp.const_dr)
        x, y, z = r * np.sin(X1) * np.cos(X2), r * np.sin(X1) * np.sin(X2), r * np.cos(X1)
    uu, vv = scalarwave_id_pointwise(kind, x, y, z, t, gp.wavespeed, k, sigma)
    return np.stack([uu, vv])


# ------------------------------------------------ curvilinear Maxwell (System II)
MC_GFS = ["Gamma", "aU0", "aU1", "aU2", "eU0", "eU1", "eU2", "psi"]  # alphabetical (uppercase first)


def maxwell_curvi_pointwise(v, q):
    """Maxwell/VacuumMaxwell_Flat_Evol_Curvilinear_rescaled.py:22-190 (System II,
    rescaled a^i = A^i / ReU^i, e^i = E^i / ReU^i, auxiliary Gamma):
      d_t a^i = -e^i - ghat^ij psi_,j / ReU^i
      d_t e^i = [ ghat^ij Gamma_,j - ghat^jk (A^i_,kj + d_j Gammahat^i_mk A^m
                 + Gammahat^i_mk A^m_,j + Gammahat^i_mj A^m_,k - Gammahat^m_kj A^i_,m
                 + (Gammahat^i_dj Gammahat^d_mk - Gammahat^d_kj Gammahat^i_md) A^m) ] / ReU^i
      d_t psi = -Gamma
      d_t Gamma = -ghat^ij psi_,ij + ghat^ij Gammahat^k_ji psi_,k
      C = E^i_,i + Gammahat^i_ji E^j,   G = Gamma - A^i_,i + Gammahat^i_ji A^j.
    v: aU, aU_dD, aU_dDD, eU, eU_dD, psi_dD, psi_dDD, Gamma, Gamma_dD (tensor indices
    first); q: hatted quantities.  Returns (arhsU, erhsU, psi_rhs, Gamma_rhs, C, G)."""
    R = range(3)
    gUU, G, GdD = q["ghatUU"], q["GammahatUDD"], q["GammahatUDDdD"]  # GdD[i,k,l,n] = d_n Gammahat^i_kl
    ReU, ReUdD, ReUdDD = q["ReU"], q["ReUdD"], q["ReUdDD"]
    a, ad, add = v["aU"], v["aU_dD"], v["aU_dDD"]
    A = a * ReU
    Ad = ad * ReU[:, None] + a[:, None] * ReUdD
    Add = (add * ReU[:, None, None] + ad[:, :, None] * ReUdD[:, None, :] + ad[:, None, :] * ReUdD[:, :, None]
           + a[:, None, None] * ReUdDD)
    arhs = [-v["eU"][i] - sum(gUU[i, j] * v["psi_dD"][j] for j in R) / ReU[i] for i in R]
    erhs = []
    for i in R:
        E = sum(gUU[i, j] * v["Gamma_dD"][j] for j in R)
        for j in R:
            for k in R:
                t = Add[i, k, j]
                for m in R:
                    t = t + GdD[i, m, k, j] * A[m] + G[i, m, k] * Ad[m, j] + G[i, m, j] * Ad[m, k] - G[m, k, j] * Ad[i, m]
                    for d in R:
                        t = t + (G[i, d, j] * G[d, m, k] - G[d, k, j] * G[i, m, d]) * A[m]
                E = E - gUU[j, k] * t
        erhs.append(E / ReU[i])
    Grhs = 0.0
    for i in R:
        for j in R:
            Grhs = Grhs - gUU[i, j] * v["psi_dDD"][i, j]
            for k in R:
                Grhs = Grhs + gUU[i, j] * G[k, j, i] * v["psi_dD"][k]
    psi_rhs = -v["Gamma"]
    Gc = v["Gamma"] - sum(Ad[i, i] for i in R) + sum(G[i, j, i] * A[j] for i in R for j in R)
    e = v["eU"]
    Ed = v["eU_dD"] * ReU[:, None] + e[:, None] * ReUdD
    Cc = sum(Ed[i, i] for i in R) + sum(G[i, j, i] * e[j] * ReU[j] for i in R for j in R)
    return arhs, erhs, psi_rhs, Grhs, Cc, Gc


def _mc_symbols(gp, gfs):
    S = Stencils(gp.FD_order, gp.NGHOSTS, gp.invdx)
    g = gp.NGHOSTS
    q = hatted_grid(gp, interior=True)
    f = {n: gfs[i] for i, n in enumerate(MC_GFS)}
    v = {"aU": np.array([S.interior(f["aU%d" % i]) for i in range(3)]),
         "eU": np.array([S.interior(f["eU%d" % i]) for i in range(3)]),
         "Gamma": S.interior(f["Gamma"])}
    v["aU_dD"] = np.array([[S.d1(f["aU%d" % i], j) for j in range(3)] for i in range(3)])
    v["eU_dD"] = np.array([[S.d1(f["eU%d" % i], j) for j in range(3)] for i in range(3)])
    v["aU_dDD"] = np.array([[[S.d11(f["aU%d" % i], j, k) for k in range(3)] for j in range(3)] for i in range(3)])
    v["psi_dD"] = np.array([S.d1(f["psi"], j) for j in range(3)])
    v["psi_dDD"] = np.array([[S.d11(f["psi"], j, k) for k in range(3)] for j in range(3)])
    v["Gamma_dD"] = np.array([S.d1(f["Gamma"], j) for j in range(3)])
    return v, q


def maxwell_curvi_rhs_grid(gp, gfs):
    """rhs_eval of the 8 gridfunctions (MC_GFS order) at interior points."""
    v, q = _mc_symbols(gp, gfs)
    arhs, erhs, psi_rhs, Grhs, _, _ = maxwell_curvi_pointwise(v, q)
    out = np.zeros((8,) + gp.shape)
    for i in range(3):
        gp.interior(out[1 + i])[...] = arhs[i]
        gp.interior(out[4 + i])[...] = erhs[i]
    gp.interior(out[7])[...] = psi_rhs
    gp.interior(out[0])[...] = Grhs
    return out


def maxwell_curvi_constraints_grid(gp, gfs):
    """(C, G) at interior points."""
    v, q = _mc_symbols(gp, gfs)
    _, _, _, _, Cc, Gc = maxwell_curvi_pointwise(v, q)
    out = np.zeros((2,) + gp.shape)
    gp.interior(out[0])[...] = Cc
    gp.interior(out[1])[...] = Gc
    return out


def maxwell_curvi_toroidal_dipole(gp, t, amp=1.0, lam=1.0):
    """Toroidal dipole of Maxwell/InitialData.py:26-117 for System II in the
    grid's basis (the Tutorial-Start_to_Finish-...-Curvilinear driver stores
    AidU/ReU, EidU/ReU, psi = Gamma = 0): the Cartesian vectors of
    toroidal_dipole are carried to the xx basis by the inverse Jacobian of
    xx_to_Cart and divided by ReU."""
    from .psi4 import _inv_general, cart_and_jacobian
    X2, X1, X0 = np.meshgrid(gp.xx[2], gp.xx[1], gp.xx[0], indexing="ij")
    xyz, J = cart_and_jacobian(gp.CoordSystem, X0, X1, X2, gp.AMPL, gp.SINHW, gp.const_dr, gp)
    x, y, z = xyz
    r = np.sqrt(x * x + y * y + z * z)
    u, vv = t + r, t - r
    eu, ev = np.exp(-lam * u ** 2), np.exp(-lam * vv ** 2)
    deu, dev = -2 * lam * u * eu, -2 * lam * vv * ev
    F = amp / r * ((ev - eu) / r ** 2 - 2 * lam * (vv * ev + u * eu) / r)
    dF = amp / r * ((dev - deu) / r ** 2 - 2 * lam * (ev + vv * dev + eu + u * deu) / r)
    Ac = [-y * F, x * F, 0.0 * x]
    Ec = [y * dF, -x * dF, 0.0 * x]
    Ji = _inv_general(J)
    ReU = hatted_grid(gp)["ReU"]  # (3, 1, n1, n0), or (3, n2, 1, n0) for the Cylindrical family
    out = np.zeros((8,) + gp.shape)
    for i in range(3):
        out[1 + i] = sum(Ji[i, j] * Ac[j] for j in range(3)) / ReU[i]
        out[4 + i] = sum(Ji[i, j] * Ec[j] for j in range(3)) / ReU[i]
    return out
