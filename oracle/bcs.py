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

from .grid import CART, GridParams


def build_bcstruct(gp):
    """Returns a list over ghost layers of (outer, inner):
    outer = list of (idx3, step) in application order (grouped per face dir:
    list of 3 arrays), inner = (dest idx3, src idx3, parity (n,10) ints)."""
    eg = GridParams(gp.CoordSystem, gp.Nxx, gp.NGHOSTS, gp.FD_order, gp.AMPL, gp.SINHW, gp.RMAX,
                    EigenCoord=1)
    n0, n1, n2 = eg.np
    ng = gp.NGHOSTS
    cart = gp.CoordSystem == CART
    X2, X1, X0 = np.meshgrid(eg.xx[2], eg.xx[1], eg.xx[0], indexing="ij")
    if cart:
        xc = [X0, X1, X2]
        xin = [X0, X1, X2]
    else:
        xc = [X0 * np.sin(X1) * np.cos(X2), X0 * np.sin(X1) * np.sin(X2), X0 * np.cos(X1)]
        r = np.sqrt(xc[0] ** 2 + xc[1] ** 2 + xc[2] ** 2)
        xin = [r, np.arccos(xc[2] / r), np.arctan2(xc[1], xc[0])]
    xxmin = [eg.xx[d][0] - ((0 - ng) + 0.5) * eg.dxx[d] for d in range(3)]
    ib = [np.trunc((xin[d] - xxmin[d] - 0.5 * eg.dxx[d] + ng * eg.dxx[d]) / eg.dxx[d] + 0.5).astype(int)
          for d in range(3)]
    I2, I1, I0 = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    inner = (ib[0] != I0) | (ib[1] != I1) | (ib[2] != I2)

    def unit(x1, x2):
        if cart:
            e = np.zeros((3, 3) + np.shape(x1))
            for i in range(3):
                e[i, i] = 1.0
            return e
        st, ct, sp, cp = np.sin(x1), np.cos(x1), np.sin(x2), np.cos(x2)
        return np.array([[st * cp, st * sp, ct], [ct * cp, ct * sp, -st], [-sp, cp, 0 * st]])

    U = unit(X1, X2)
    ibc = [np.clip(ib[d], 0, eg.np[d] - 1) for d in range(3)]
    Ui = unit(eg.xx[1][ibc[1]], eg.xx[2][ibc[2]])
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
