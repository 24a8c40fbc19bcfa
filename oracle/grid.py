"""Grid set-up and reference metric for the CPU oracle (numpy, FP64).

TEST INFRASTRUCTURE (see oracle/__init__.py).

- `GridParams` restates reference_metric.py:1330-1395
  (set_Nxx_dxx_invdx_params__and__xx): domain per CoordSystem
  (Spherical :106-108, SinhSpherical :118-120, SinhSphericalv2 :137-138,
  Cylindrical :233-234, SinhCylindrical :246-247, Cartesian :400-403),
  dxx = (xxmax - xxmin)/Nxx, cell-centred xx[j] = xxmin + (j - NGHOSTS + 1/2) dxx.
- `hatted` restates reference_metric.py:487-601: for orthogonal scale factors
  s_i (reference_metric.py:168-175: s0 = dr/dxx0, s1 = r, s2 = r sin(xx1);
  r(xx0) of :111, :125-126 and :142-143; :289-291 for the Cylindrical family:
  s0 = drho/dxx0, s1 = rho, s2 = dz/dxx2 with rho(xx0), z(xx2) of :237-239,
  :255-258; Cartesian s_i = 1) it returns ReU, ReDD, ghat and their first and second
  derivatives, GammahatUDD and its derivatives, det(ghat) and derivatives.
  Where the reference differentiates symbolically, here the derivatives of
  s_i are written in closed form and propagated by the product/quotient
  rules, all as numpy arrays.
- `find_timestep` restates reference_metric.py:1412-1439.
"""
import numpy as np

CART, SPH, SINHSPH, SINHSPHV2, CYL, SINHCYL, SINHCYLV2, SYMTP, SINHSYMTP = 0, 1, 2, 3, 4, 5, 6, 7, 8
NAMES = {"Cartesian": CART, "Spherical": SPH, "SinhSpherical": SINHSPH, "SinhSphericalv2": SINHSPHV2,
         "Cylindrical": CYL, "SinhCylindrical": SINHCYL, "SinhCylindricalv2": SINHCYLV2, "SymTP": SYMTP,
         "SinhSymTP": SINHSYMTP}


def symtp(cs):
    return cs in (SYMTP, SINHSYMTP)


def symtp_scale_factors(gp, x0, x1):
    """SymTP family (reference_metric.py:306-383): AA(xx0) (xx0, or the sinh
    map of AMAX/SINHWAA), var1 = sqrt(AA^2 + (bScale sin xx1)^2), var2 =
    sqrt(AA^2 + bScale^2); s0 = AA' var1/var2, s1 = var1, s2 = AA sin xx1,
    with first and second derivatives in xx0, xx1 by the chain rule."""
    b = gp.bScale
    z = np.zeros_like(x0)
    if gp.CoordSystem == SINHSYMTP:
        A, A1 = sinh_map(gp.AMAX, gp.SINHWAA, x0)
        A2, A3 = A / gp.SINHWAA ** 2, A1 / gp.SINHWAA ** 2
    else:
        A, A1, A2, A3 = x0, np.ones_like(x0), z, z
    S, Cs = np.sin(x1), np.cos(x1)
    u = A * A + b * b * S * S
    v1 = np.sqrt(u)
    du = [2 * A * A1, 2 * b * b * S * Cs]
    ddu = [[2 * (A1 * A1 + A * A2), z], [z, 2 * b * b * (Cs * Cs - S * S)]]
    dv1 = [du[k] / (2 * v1) for k in range(2)]
    ddv1 = [[ddu[k][l] / (2 * v1) - du[k] * du[l] / (4 * v1 ** 3) for l in range(2)] for k in range(2)]
    w = A * A + b * b
    v2 = np.sqrt(w)
    dv2 = [2 * A * A1 / (2 * v2), z]
    ddv2 = [[2 * (A1 * A1 + A * A2) / (2 * v2) - (2 * A * A1) ** 2 / (4 * v2 ** 3), z], [z, z]]
    q = v1 / v2
    dq = [dv1[k] / v2 - v1 * dv2[k] / v2 ** 2 for k in range(2)]
    ddq = [[ddv1[k][l] / v2 - (dv1[k] * dv2[l] + dv1[l] * dv2[k]) / v2 ** 2 - v1 * ddv2[k][l] / v2 ** 2
            + 2 * v1 * dv2[k] * dv2[l] / v2 ** 3 for l in range(2)] for k in range(2)]
    dA1 = [A2, z]
    ddA1 = [[A3, z], [z, z]]
    s = [A1 * q, v1, A * S]
    ds = [[z.copy() for _ in range(3)] for _ in range(3)]
    dds = [[[z.copy() for _ in range(3)] for _ in range(3)] for _ in range(3)]
    ds2 = [A1 * S, A * Cs]
    dds2 = [[A2 * S, A1 * Cs], [A1 * Cs, -A * S]]
    for k in range(2):
        ds[0][k] = dA1[k] * q + A1 * dq[k]
        ds[1][k] = dv1[k]
        ds[2][k] = ds2[k]
        for l in range(2):
            dds[0][k][l] = ddA1[k][l] * q + dA1[k] * dq[l] + dA1[l] * dq[k] + A1 * ddq[k][l]
            dds[1][k][l] = ddv1[k][l]
            dds[2][k][l] = dds2[k][l]
    return s, ds, dds


def cylindrical(cs):
    return cs in (CYL, SINHCYL, SINHCYLV2)


def sinh_map(A, w, x):
    """A sinh(x/w) / sinh(1/w) and its derivative, with exponentials as
    reference_metric.py:125-126, 255-258 write them."""
    x = np.asarray(x, dtype=float)
    den = np.exp(1.0 / w) - np.exp(-1.0 / w)
    return A * (np.exp(x / w) - np.exp(-x / w)) / den, A * (np.exp(x / w) + np.exp(-x / w)) / (w * den)


def cylinder_maps(gp, x0, x2):
    """(rho, drho/dxx0), (z, dz/dxx2) of the Cylindrical family
    (SinhCylindricalv2 adds AMPLRHO const_drho xx0 and AMPLZ const_dz xx2,
    reference_metric.py:273-275)."""
    if gp.CoordSystem in (SINHCYL, SINHCYLV2):
        (r, dr), (z, dz) = sinh_map(gp.AMPLRHO, gp.SINHWRHO, x0), sinh_map(gp.AMPLZ, gp.SINHWZ, x2)
        if gp.CoordSystem == SINHCYLV2:
            r, dr = r + gp.AMPLRHO * gp.const_drho * np.asarray(x0), dr + gp.AMPLRHO * gp.const_drho
            z, dz = z + gp.AMPLZ * gp.const_dz * np.asarray(x2), dz + gp.AMPLZ * gp.const_dz
        return (r, dr), (z, dz)
    x0, x2 = np.asarray(x0, dtype=float), np.asarray(x2, dtype=float)
    return (x0, np.ones_like(x0)), (x2, np.ones_like(x2))


def radial(cs, x0, AMPL=10.0, SINHW=0.2, const_dr=0.0625):
    """r(xx0) and dr/dxx0 of the Spherical family: Spherical r = xx0
    (reference_metric.py:111); SinhSpherical r = AMPL sinh(xx0/SINHW) /
    sinh(1/SINHW) (:125-126); SinhSphericalv2 adds AMPL const_dr xx0
    (:142-143)."""
    x0 = np.asarray(x0, dtype=float)
    if cs == SPH:
        return x0, np.ones_like(x0)
    den = np.exp(1.0 / SINHW) - np.exp(-1.0 / SINHW)
    r = AMPL * (np.exp(x0 / SINHW) - np.exp(-x0 / SINHW)) / den
    drdx = AMPL * (np.exp(x0 / SINHW) + np.exp(-x0 / SINHW)) / (SINHW * den)
    if cs == SINHSPHV2:
        r = r + AMPL * const_dr * x0
        drdx = drdx + AMPL * const_dr
    elif cs != SINHSPH:
        raise ValueError(cs)
    return r, drdx


class GridParams:
    def __init__(self, CoordSystem, Nxx, NGHOSTS, FD_order=4, AMPL=10.0, SINHW=0.2, RMAX=10.0,
                 domain=(-10.0, 10.0), eta=2.0, wavespeed=1.0, EigenCoord=0, const_dr=0.0625, RHOMAX=10.0,
                 ZMIN=-10.0, ZMAX=10.0, AMPLRHO=10.0, SINHWRHO=0.2, AMPLZ=10.0, SINHWZ=0.2, const_drho=0.0625,
                 const_dz=0.0625, bScale=0.5, SINHWAA=0.2, AMAX=10.0):
        cs = NAMES[CoordSystem] if isinstance(CoordSystem, str) else int(CoordSystem)
        self.CoordSystem = cs
        self.FD_order = FD_order
        self.NGHOSTS = NGHOSTS
        self.AMPL, self.SINHW, self.RMAX = AMPL, SINHW, RMAX
        self.const_dr = const_dr
        self.RHOMAX, self.ZMIN, self.ZMAX = RHOMAX, ZMIN, ZMAX
        self.AMPLRHO, self.SINHWRHO, self.AMPLZ, self.SINHWZ = AMPLRHO, SINHWRHO, AMPLZ, SINHWZ
        self.const_drho, self.const_dz = const_drho, const_dz
        self.bScale, self.SINHWAA, self.AMAX = bScale, SINHWAA, AMAX
        self.eta, self.wavespeed = eta, wavespeed
        self.Nxx = [int(n) for n in Nxx]
        self.np = [n + 2 * NGHOSTS for n in self.Nxx]
        ecs = SPH if (EigenCoord and cs in (SINHSPH, SINHSPHV2)) else cs
        ecs = CYL if (EigenCoord and cs in (SINHCYL, SINHCYLV2)) else ecs
        ecs = SYMTP if (EigenCoord and cs == SINHSYMTP) else ecs
        if ecs == CART:
            ext = [tuple(d) for d in domain] if np.ndim(domain) == 2 else [tuple(domain)] * 3
            self.xxmin, self.xxmax = [e[0] for e in ext], [e[1] for e in ext]
        elif ecs == CYL:
            self.xxmin, self.xxmax = [0.0, -np.pi, ZMIN], [RHOMAX, np.pi, ZMAX]
        elif symtp(ecs):  # :317-322
            self.xxmin, self.xxmax = [0.0, 0.0, -np.pi], [AMAX if ecs == SYMTP else 1.0, np.pi, np.pi]
        elif ecs in (SINHCYL, SINHCYLV2):
            self.xxmin, self.xxmax = [0.0, -np.pi, -1.0], [1.0, np.pi, 1.0]
        else:
            self.xxmin = [0.0, 0.0, -np.pi]
            self.xxmax = [RMAX if ecs == SPH else 1.0, np.pi, np.pi]
        self.dxx = [(self.xxmax[d] - self.xxmin[d]) / float(self.Nxx[d]) for d in range(3)]
        self.invdx = [1.0 / v for v in self.dxx]
        self.xx = [self.xxmin[d] + ((np.arange(self.np[d]) - NGHOSTS) + 0.5) * self.dxx[d] for d in range(3)]

    @property
    def shape(self):
        return (self.np[2], self.np[1], self.np[0])

    def interior(self, f):
        g = self.NGHOSTS
        return f[..., g:-g, g:-g, g:-g]


def scale_factors(gp, xx0, xxB):
    """s[i], ds[i][k], dds[i][k][l] as arrays broadcast over (xxB, xx0), xxB
    the second coordinate the metric depends on: xx1 (Spherical family) or
    xx2 (Cylindrical family)."""
    x0, x1 = np.meshgrid(xx0, xxB)  # shape (nB, n0)
    z = np.zeros_like(x0)
    one = np.ones_like(x0)
    s = [one.copy(), one.copy(), one.copy()]
    ds = [[z.copy() for _ in range(3)] for _ in range(3)]
    dds = [[[z.copy() for _ in range(3)] for _ in range(3)] for _ in range(3)]
    if gp.CoordSystem == CART:
        return s, ds, dds
    if symtp(gp.CoordSystem):
        return symtp_scale_factors(gp, x0, x1)
    if cylindrical(gp.CoordSystem):
        (rho, rho1), (zz, z1) = cylinder_maps(gp, x0, x1)
        if gp.CoordSystem in (SINHCYL, SINHCYLV2):
            # second and third derivatives come from the sinh part alone
            (sh, ch), (shz, chz) = sinh_map(gp.AMPLRHO, gp.SINHWRHO, x0), sinh_map(gp.AMPLZ, gp.SINHWZ, x1)
            rho2, rho3 = sh / gp.SINHWRHO ** 2, ch / gp.SINHWRHO ** 2
            z2, z3 = shz / gp.SINHWZ ** 2, chz / gp.SINHWZ ** 2
        else:
            rho2 = rho3 = z2 = z3 = z
        s = [rho1, rho, z1]
        ds[0][0], ds[1][0], ds[2][2] = rho2, rho1, z2
        dds[0][0][0], dds[1][0][0], dds[2][2][2] = rho3, rho2, z3
        return s, ds, dds
    if gp.CoordSystem in (SINHSPH, SINHSPHV2):
        A, w = gp.AMPL, gp.SINHW
        den = np.exp(1.0 / w) - np.exp(-1.0 / w)
        sh = A * (np.exp(x0 / w) - np.exp(-x0 / w)) / den
        ch = A * (np.exp(x0 / w) + np.exp(-x0 / w)) / (w * den)
        lin = A * gp.const_dr if gp.CoordSystem == SINHSPHV2 else 0.0
        r = sh + lin * x0
        r1 = ch + lin
        r2 = sh / w ** 2
        r3 = ch / w ** 2
    else:
        r, r1, r2, r3 = x0, one, z, z
    st, ct = np.sin(x1), np.cos(x1)
    s = [r1, r, r * st]
    ds[0][0] = r2
    ds[1][0] = r1
    ds[2][0] = r1 * st
    ds[2][1] = r * ct
    dds[0][0][0] = r3
    dds[1][0][0] = r2
    dds[2][0][0] = r2 * st
    dds[2][0][1] = dds[2][1][0] = r1 * ct
    dds[2][1][1] = -r * st
    return s, ds, dds


def hatted(gp):
    """Hatted quantities on the (nB, n0) plane of the metric's coordinates
    (nB = n1, or n2 for the Cylindrical family); tensors indexed first."""
    xxB = gp.xx[2] if cylindrical(gp.CoordSystem) else gp.xx[1]
    return hatted_from_scale_factors(*scale_factors(gp, gp.xx[0], xxB))


def hatted_grid(gp, interior=False):
    """Hatted quantities broadcastable over (n2, n1, n0) grid arrays (or,
    with interior=True, over interior arrays): shape (tensor..., 1, n1, n0),
    or (tensor..., n2, 1, n0) for the Cylindrical family."""
    g = gp.NGHOSTS
    cyl = cylindrical(gp.CoordSystem)
    out = {}
    for k, a in hatted(gp).items():
        a = a[..., :, None, :] if cyl else a[..., None, :, :]
        if interior:
            a = a[..., g:-g, :, g:-g] if cyl else a[..., :, g:-g, g:-g]
        out[k] = a
    return out


class _PointParams:
    def __init__(self, cs, **kw):
        self.CoordSystem = cs
        for k, v in dict(AMPL=10.0, SINHW=0.2, const_dr=0.0625, AMPLRHO=10.0, SINHWRHO=0.2, AMPLZ=10.0,
                         SINHWZ=0.2, const_drho=0.0625, const_dz=0.0625, bScale=0.5, SINHWAA=0.2,
                         AMAX=10.0).items():
            setattr(self, k, kw.get(k, v))


def hatted_at(CoordSystem, xx0, xx1, AMPL=10.0, SINHW=0.2, const_dr=0.0625, xx2=0.0, **cyl):
    """Hatted quantities at one point (xx0, xx1, xx2): arrays with point shape
    (1, 1).  cyl: AMPLRHO, SINHWRHO, AMPLZ, SINHWZ of SinhCylindrical."""
    cs = NAMES[CoordSystem] if isinstance(CoordSystem, str) else CoordSystem
    xxB = xx2 if cylindrical(cs) else xx1
    return hatted_from_scale_factors(*scale_factors(_PointParams(cs, AMPL=AMPL, SINHW=SINHW, const_dr=const_dr,
                                                                 **cyl), np.array([xx0]), np.array([xxB])))


def hatted_from_scale_factors(s, ds, dds):
    # the formulas hold wherever asked; on a coordinate singularity (r = 0)
    # they give inf/nan entries as the reference's expressions do
    with np.errstate(divide="ignore", invalid="ignore"):
        return _hatted(s, ds, dds)


def _hatted(s, ds, dds):
    s = np.array(s)
    ds = np.array(ds)
    dds = np.array(dds)
    shp = s.shape[1:]
    q = {}
    q["ReU"] = 1.0 / s
    q["ReUdD"] = -ds / s[:, None] ** 2
    q["ReUdDD"] = -dds / s[:, None, None] ** 2 + 2.0 * ds[:, :, None] * ds[:, None, :] / s[:, None, None] ** 3
    q["ReDD"] = s[:, None] * s[None, :]
    q["ReDDdD"] = ds[:, None, :] * s[None, :, None] + s[:, None, None] * ds[None, :, :]
    q["ReDDdDD"] = (dds[:, None] * s[None, :, None, None] + ds[:, None, :, None] * ds[None, :, None, :]
                    + ds[:, None, None, :] * ds[None, :, :, None] + s[:, None, None, None] * dds[None, :])
    g = s ** 2
    dg = 2.0 * s[:, None] * ds
    ddg = 2.0 * (ds[:, :, None] * ds[:, None, :] + s[:, None, None] * dds)
    eye = np.eye(3)
    q["ghatDD"] = eye[:, :, None, None] * g[:, None]
    q["ghatUU"] = eye[:, :, None, None] / g[:, None]
    ghatDDdD = np.zeros((3, 3, 3) + shp)
    ghatDDdDD = np.zeros((3, 3, 3, 3) + shp)
    for i in range(3):
        ghatDDdD[i, i] = dg[i]
        ghatDDdDD[i, i] = ddg[i]
    q["ghatDDdD"] = ghatDDdD
    q["ghatDDdDD"] = ghatDDdDD
    # Christoffels of the diagonal metric: (1/2) g^ii (g_ik,l + g_il,k - g_kl,i)
    G = np.zeros((3, 3, 3) + shp)
    GdD = np.zeros((3, 3, 3, 3) + shp)
    for i in range(3):
        for k in range(3):
            for l in range(3):
                br = ghatDDdD[i, k, l] + ghatDDdD[i, l, k] - ghatDDdD[k, l, i]
                G[i, k, l] = 0.5 * br / g[i]
                for n in range(3):
                    dbr = ghatDDdDD[i, k, l, n] + ghatDDdDD[i, l, k, n] - ghatDDdDD[k, l, i, n]
                    GdD[i, k, l, n] = 0.5 * dbr / g[i] - 0.5 * br * dg[i, n] / g[i] ** 2
    q["GammahatUDD"] = G
    q["GammahatUDDdD"] = GdD
    det = g[0] * g[1] * g[2]
    q["detgammahat"] = det
    ddet = np.zeros((3,) + shp)
    dddet = np.zeros((3, 3) + shp)
    for k in range(3):
        ddet[k] = dg[0, k] * g[1] * g[2] + g[0] * dg[1, k] * g[2] + g[0] * g[1] * dg[2, k]
        for l in range(3):
            dddet[k, l] = (ddg[0, k, l] * g[1] * g[2] + g[0] * ddg[1, k, l] * g[2] + g[0] * g[1] * ddg[2, k, l]
                           + dg[0, k] * dg[1, l] * g[2] + dg[0, l] * dg[1, k] * g[2]
                           + dg[0, k] * g[1] * dg[2, l] + dg[0, l] * g[1] * dg[2, k]
                           + g[0] * dg[1, k] * dg[2, l] + g[0] * dg[1, l] * dg[2, k])
    q["detgammahatdD"] = ddet
    q["detgammahatdDD"] = dddet
    return q


def find_timestep(gp, CFL_FACTOR):
    """CFL * min over interior points of dxx_i * s_i / wavespeed."""
    g = gp.NGHOSTS
    xxB = gp.xx[2] if cylindrical(gp.CoordSystem) else gp.xx[1]
    s, _, _ = scale_factors(gp, gp.xx[0][g:-g], xxB[g:-g])
    dsmin = min(float(np.min(gp.dxx[d] * s[d])) for d in range(3))
    return dsmin * CFL_FACTOR / gp.wavespeed
