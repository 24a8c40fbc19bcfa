"""Curvilinear boundary conditions and the RK4 MoL step (numpy).

TEST INFRASTRUCTURE (see oracle/__init__.py).

Boundary maps restate CurviBoundaryConditions/boundary_conditions/
set_up__bc_gz_map_and_parity_condns.h:7-113 (map every eigen-grid point to
Cartesian and back; a different index means an inner parity point; parities
from unit-vector dot products, CurviBoundaryConditions.py:80-113) and
set_bcstruct.h:32-124 (per ghost layer, faces i0min, i0max, i1min, i1max,
i2min, i2max with the box widened after each face).  apply_bcs restates
apply_bcs_curvilinear.h:7-64: per layer, every outer point gets
3 f1 - 3 f2 + f3 along its face normal, in list order, then every inner
point gets parity * f(src).

The RK4 step restates the diagonal low-storage RK_MoL.h that
MoLtimestepping/C_Code_Generation.py:266-329 emits for "RK4": RHS into the
stage buffer at interior points, LOOP_ALL_GFS_GPS update of every point,
then the post-RHS calls (BCs, then the det(gammabar) rescale for BSSN).
"""
import numpy as np

from .grid import CART, GridParams, cylinder_maps, cylindrical, radial, symtp


def build_bcstruct(gp):
    """Returns a list over ghost layers of (outer, inner):
    outer = list of (idx3, step) in application order (grouped per face dir:
    list of 3 arrays), inner = (dest idx3, src idx3, parity (n,10) ints)."""
    eg = GridParams(gp.CoordSystem, gp.Nxx, gp.NGHOSTS, gp.FD_order, gp.AMPL, gp.SINHW, gp.RMAX,
                    EigenCoord=1, RHOMAX=gp.RHOMAX, ZMIN=gp.ZMIN, ZMAX=gp.ZMAX, bScale=gp.bScale, AMAX=gp.AMAX)
    n0, n1, n2 = eg.np
    ng = gp.NGHOSTS
    cart = gp.CoordSystem == CART
    cyl = cylindrical(gp.CoordSystem)
    stp = symtp(gp.CoordSystem)
    b = gp.bScale
    X2, X1, X0 = np.meshgrid(eg.xx[2], eg.xx[1], eg.xx[0], indexing="ij")
    if cart:
        xc = [X0, X1, X2]
        xin = [X0, X1, X2]
    elif stp:
        # SymTP eigen-coordinates (reference_metric.py:334-336, 348-366)
        xc = [X0 * np.sin(X1) * np.cos(X2), X0 * np.sin(X1) * np.sin(X2), np.sqrt(X0 ** 2 + b * b) * np.cos(X1)]
        r = np.sqrt(xc[0] ** 2 + xc[1] ** 2 + xc[2] ** 2)
        cth = xc[2] / r
        root = np.sqrt(b ** 4 + 2 * b * b * r * r + r ** 4 - 4 * b * b * r * r * cth * cth)
        xin = [np.sqrt(-b * b + r * r + root) * np.sqrt(0.5),
               np.arccos(np.sign(xc[2]) * np.sqrt(1 + r * r / (b * b) - root / (b * b)) * np.sqrt(0.5)),
               np.arctan2(xc[1], xc[0])]
    elif cyl:
        # Cylindrical eigen-coordinates (reference_metric.py:240-242, 296-298)
        xc = [X0 * np.cos(X1), X0 * np.sin(X1), X2]
        xin = [np.sqrt(xc[0] ** 2 + xc[1] ** 2), np.arctan2(xc[1], xc[0]), X2]
    else:
        xc = [X0 * np.sin(X1) * np.cos(X2), X0 * np.sin(X1) * np.sin(X2), X0 * np.cos(X1)]
        r = np.sqrt(xc[0] ** 2 + xc[1] ** 2 + xc[2] ** 2)
        xin = [r, np.arccos(xc[2] / r), np.arctan2(xc[1], xc[0])]
    xxmin = [eg.xx[d][0] - ((0 - ng) + 0.5) * eg.dxx[d] for d in range(3)]
    ib = [np.trunc((xin[d] - xxmin[d] - 0.5 * eg.dxx[d] + ng * eg.dxx[d]) / eg.dxx[d] + 0.5).astype(int)
          for d in range(3)]
    I2, I1, I0 = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    inner = (ib[0] != I0) | (ib[1] != I1) | (ib[2] != I2)

    def unit(x1, x2, x0=None):
        if cart:
            e = np.zeros((3, 3) + np.shape(x1))
            for i in range(3):
                e[i, i] = 1.0
            return e
        if stp:  # reference_metric.py:373-379
            st, ct, sp, cp = np.sin(x1), np.cos(x1), np.sin(x2), np.cos(x2)
            v1, v2 = np.sqrt(x0 ** 2 + b * b * st * st), np.sqrt(x0 ** 2 + b * b)
            return np.array([[st * cp * v2 / v1, st * sp * v2 / v1, x0 * ct / v1],
                             [x0 * ct * cp / v1, x0 * ct * sp / v1, -st * v2 / v1], [-sp, cp, 0 * st]])
        if cyl:  # reference_metric.py:300-302, phi = xx1
            sp, cp, z0 = np.sin(x1), np.cos(x1), 0 * np.asarray(x1, dtype=float)
            return np.array([[cp, sp, z0], [-sp, cp, z0], [z0, z0, z0 + 1.0]])
        st, ct, sp, cp = np.sin(x1), np.cos(x1), np.sin(x2), np.cos(x2)
        return np.array([[st * cp, st * sp, ct], [ct * cp, ct * sp, -st], [-sp, cp, 0 * st]])

    U = unit(X1, X2, X0)
    ibc = [np.clip(ib[d], 0, eg.np[d] - 1) for d in range(3)]
    Ui = unit(eg.xx[1][ibc[1]], eg.xx[2][ibc[2]], eg.xx[0][ibc[0]])
    par = np.ones((10,) + X0.shape)
    for t in range(1, 4):
        par[t] = (U[t - 1] * Ui[t - 1]).sum(axis=0)
    c = 4
    for i in range(3):
        for j in range(i, 3):
            par[c] = par[i + 1] * par[j + 1]
            c += 1
    parity = np.where(par < 0, -1, 1).astype(int)
    src = ibc[0] + n0 * (ibc[1] + n1 * ibc[2])

    layers = []
    imin, imax = [ng, ng, ng], [n0 - ng, n1 - ng, n2 - ng]
    stride = [1, n0, n0 * n1]
    for g in range(ng):
        lo, hi = list(imin), list(imax)
        faces = []
        for d in range(3):
            for side in (0, 1):
                rng = [[lo[e], hi[e]] for e in range(3)]
                if side == 0:
                    rng[d] = [lo[d] - 1, lo[d]]
                    lo[d] -= 1
                else:
                    rng[d] = [hi[d], hi[d] + 1]
                    hi[d] += 1
                faces.append((d, side, rng))
        outer_dirs = [[], [], []]
        idst, isrc, ipar = [], [], []
        for d, side, rng in faces:
            for i2 in range(rng[2][0], rng[2][1]):
                for i1 in range(rng[1][0], rng[1][1]):
                    for i0 in range(rng[0][0], rng[0][1]):
                        idx = i0 + n0 * (i1 + n1 * i2)
                        if not inner[i2, i1, i0]:
                            outer_dirs[d].append((idx, (1 if side == 0 else -1) * stride[d]))
        for d, side, rng in faces:
            for i2 in range(rng[2][0], rng[2][1]):
                for i1 in range(rng[1][0], rng[1][1]):
                    for i0 in range(rng[0][0], rng[0][1]):
                        if inner[i2, i1, i0]:
                            idst.append(i0 + n0 * (i1 + n1 * i2))
                            isrc.append(int(src[i2, i1, i0]))
                            ipar.append(parity[:, i2, i1, i0])
        layers.append(([np.array(o, dtype=np.int64).reshape(-1, 2) for o in outer_dirs],
                       (np.array(idst, dtype=np.int64), np.array(isrc, dtype=np.int64),
                        np.array(ipar, dtype=np.int64).reshape(-1, 10))))
        imin = [v - 1 for v in imin]
        imax = [v + 1 for v in imax]
    return layers


def parity_type(name):
    """Parity type of a DIM-3 gridfunction from the digits its name ends in,
    as set_parity_types of CurviBoundaryConditions.py:122-160 assigns it:
    no index -> 0 (scalar); one index i -> 1 + i; two indices (symmetric)
    -> 4..9 for 00, 01, 02, 11, 12, 22."""
    digits = ""
    for ch in reversed(name):
        if not ch.isdigit():
            break
        digits = ch + digits
    if len(digits) == 0:
        return 0
    if len(digits) == 1:
        return 1 + int(digits)
    i, j = sorted((int(digits[-2]), int(digits[-1])))
    return 4 + {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 1): 3, (1, 2): 4, (2, 2): 5}[(i, j)]


def apply_bcs(layers, gfs, parity_types):
    """In place on gfs (ngf, n2, n1, n0), sequentially as the reference does."""
    ngf = gfs.shape[0]
    flat = gfs.reshape(ngf, -1)
    for outer_dirs, (idst, isrc, ipar) in layers:
        for arr in outer_dirs:
            for idx, st in arr:
                flat[:, idx] = 3.0 * flat[:, idx + st] - 3.0 * flat[:, idx + 2 * st] + 1.0 * flat[:, idx + 3 * st]
        if len(idst):
            for g in range(ngf):
                flat[g, idst] = ipar[:, parity_types[g]] * flat[g, isrc]
    return gfs


def rk4_step(y_n, dt, rhs_fn, post_fn, ng, k_odd=None, k_even=None):
    """One RK4 step.  rhs_fn(gfs) returns the RHS (only its interior is
    used: rhs_eval writes interior points); post_fn(gfs) applies BCs (and the
    rescale) in place.  Stage-buffer ghost values are whatever the previous
    use left, as in the reference; they start at zero here.  Returns
    (y_n at t+dt, k_odd, k_even)."""
    k_odd = np.zeros_like(y_n) if k_odd is None else k_odd.copy()
    k_even = np.zeros_like(y_n) if k_even is None else k_even.copy()
    I = (Ellipsis, slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))

    def rhs_into(buf, inp):
        buf[I] = rhs_fn(inp)[I]

    rhs_into(k_odd, y_n)                                   # RHS(y_n) -> k_odd
    rt = k_odd * dt * (1.0 / 6.0)
    k_odd = y_n + k_odd * dt * (1.0 / 2.0)
    post_fn(k_odd)
    rhs_into(k_even, k_odd)                                # RHS(k_odd) -> k_even
    rt = rt + k_even * dt * (1.0 / 3.0)
    k_even = y_n + k_even * dt * (1.0 / 2.0)
    post_fn(k_even)
    rhs_into(k_odd, k_even)                                # RHS(k_even) -> k_odd
    rt = rt + k_odd * dt * (1.0 / 3.0)
    k_odd = y_n + k_odd * dt
    post_fn(k_odd)
    rhs_into(k_even, k_odd)                                # RHS(k_odd) -> k_even
    y_new = y_n + rt + k_even * dt * (1.0 / 6.0)
    post_fn(y_new)
    return y_new, k_odd, k_even


# ------------------------------------------------------------ Sommerfeld
# CurviBoundaryConditions.py:259-658 (sommerfeld_boundary_condition_class):
# at every outer ghost point the RHS becomes the radiation condition
#   rhs = -c (d_r f + (f - f_inf)/r)
# plus, for a radial falloff power n > 0, the correction
#   (rhs(o) + c (d_r f(o) + (f(o) - f_inf)/r(o))) (r(o)/r)^n
# from the point o one step inward along the face normal; d_r f =
# sum_i d_i f dx^i/dr, with d_i f one-sided (stencil shifted into the grid
# along the face normal, or near an edge of the array) or centred.  Inner
# points copy the RHS with parity.  Per gridfunction, per ghost layer: outer
# points in list order, then inner points.
SOMMERFELD_FD = {
    2: ((-1.5, 2.0, -0.5), (0.5,)),
    4: ((-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -1.0 / 4.0), (2.0 / 3.0, -1.0 / 12.0)),
    6: ((-49.0 / 20.0, 6.0, -15.0 / 2.0, 20.0 / 3.0, -15.0 / 4.0, 6.0 / 5.0, -1.0 / 6.0),
        (3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0)),
}


def _radial_geometry(gp, i0, i1, i2):
    """(r, dx^i/dr) at a grid point (CoordSystem's xxSph[0] and Jacobian)."""
    x0, x1, x2 = gp.xx[0][i0], gp.xx[1][i1], gp.xx[2][i2]
    if gp.CoordSystem == CART:
        r = np.sqrt(x0 * x0 + x1 * x1 + x2 * x2)
        return r, (x0 / r, x1 / r, x2 / r)
    if gp.CoordSystem == 1:  # Spherical: xx0 = r
        return x0, (1.0, 0.0, 0.0)
    if symtp(gp.CoordSystem):  # dxx^i/dr = (J^-1 x / r)^i
        from .psi4 import _inv_general, cart_and_jacobian
        x, Jm = cart_and_jacobian(gp.CoordSystem, x0, x1, x2, cyl=gp)
        r = float(np.sqrt((np.asarray(x) ** 2).sum()))
        Ji = _inv_general(np.asarray(Jm, dtype=float))
        return r, tuple(float(sum(Ji[i, j] * x[j] for j in range(3)) / r) for i in range(3))
    if cylindrical(gp.CoordSystem):  # r = sqrt(rho^2 + z^2)
        (rho, drho), (z, dz) = cylinder_maps(gp, x0, x2)
        r = float(np.sqrt(rho * rho + z * z))
        return r, (float(rho / r / drho), 0.0, float(z / r / dz))
    r, drdx = radial(gp.CoordSystem, x0, gp.AMPL, gp.SINHW, gp.const_dr)
    return r, (1.0 / float(drdx), 0.0, 0.0)


def _sommerfeld_dr(gp, f, idx3, face, fd_order):
    n = gp.np
    ng = gp.NGHOSTS
    up, cen = SOMMERFELD_FD[fd_order]
    r, J = _radial_geometry(gp, *idx3)
    acc = 0.0
    for d in range(3):
        if J[d] == 0.0:
            continue
        i = idx3[d]
        if abs(face[d]) == 1 or i + ng >= n[d] or i - ng <= 0:
            shift = face[d]
            if i + ng >= n[d]:
                shift = -1
            if i - ng <= 0:
                shift = 1
            s = 0.0
            for k, c in enumerate(up):
                j = list(idx3)
                j[d] += k * shift
                s += c * f[j[2], j[1], j[0]]
            fd = shift * s * gp.invdx[d]
        else:
            s = 0.0
            for k, c in enumerate(cen, start=1):
                jp, jm = list(idx3), list(idx3)
                jp[d] += k
                jm[d] -= k
                s += c * (f[jp[2], jp[1], jp[0]] - f[jm[2], jm[1], jm[0]])
            fd = s * gp.invdx[d]
        acc += fd * J[d]
    return r, acc


def apply_sommerfeld(gp, layers, gfs, rhs, parity_types, fd_order=2, speed=None, f_inf=None, falloff=None):
    """In place on rhs (ngf, n2, n1, n0), from the state gfs."""
    ngf = gfs.shape[0]
    speed = [1.0] * ngf if speed is None else speed
    f_inf = [0.0] * ngf if f_inf is None else f_inf
    falloff = [3.0] * ngf if falloff is None else falloff
    n0, n1, _ = gp.np
    stride = [1, n0, n0 * n1]
    for g in range(ngf):
        f, R = gfs[g], rhs[g]
        Rf = R.reshape(-1)
        for outer_dirs, (idst, isrc, ipar) in layers:
            for d, arr in enumerate(outer_dirs):
                for idx, st in arr:
                    i0, i1, i2 = idx % n0, (idx // n0) % n1, idx // (n0 * n1)
                    face = [0, 0, 0]
                    face[d] = 1 if st > 0 else -1
                    r, pif = _sommerfeld_dr(gp, f, (i0, i1, i2), face, fd_order)
                    val = -speed[g] * (pif + (f[i2, i1, i0] - f_inf[g]) / r)
                    if falloff[g] > 0:
                        o = [i0, i1, i2]
                        o[d] += face[d]
                        ro, pifo = _sommerfeld_dr(gp, f, tuple(o), face, fd_order)
                        extrap = speed[g] * (pifo + (f[o[2], o[1], o[0]] - f_inf[g]) / ro)
                        val += (R[o[2], o[1], o[0]] + extrap) * (ro / r) ** falloff[g]
                    Rf[idx] = val
            if len(idst):
                Rf[idst] = ipar[:, parity_types[g]] * Rf[isrc]
    return rhs


def rk4_step_sommerfeld(y_n, dt, rhs_fn, ng):
    """RK4 step whose RHS function returns the full array (interior RHS plus
    the Sommerfeld ghost RHS); the update runs over every point, with no
    post-RHS boundary step (the reference's Sommerfeld driver)."""
    k1 = rhs_fn(y_n)
    rt = k1 * dt * (1.0 / 6.0)
    y1 = y_n + k1 * dt * (1.0 / 2.0)
    k2 = rhs_fn(y1)
    rt = rt + k2 * dt * (1.0 / 3.0)
    y2 = y_n + k2 * dt * (1.0 / 2.0)
    k3 = rhs_fn(y2)
    rt = rt + k3 * dt * (1.0 / 3.0)
    y3 = y_n + k3 * dt
    k4 = rhs_fn(y3)
    return y_n + rt + k4 * dt * (1.0 / 6.0)
