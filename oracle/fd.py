"""Finite-difference stencil coefficients and stencil application (CPU oracle).

TEST INFRASTRUCTURE: this module is part of the CPU oracle.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import it.

Restates finite_difference.py:252-369 (compute_fdcoeffs_fdstencl): the
coefficients of an order-N first or second derivative on an (N+1)-point
stencil come from the inverse of the Vandermonde matrix
M[i][j] = (j - N/2 + shift)**i  (with 0**0 = 1 and 0**i = 0 for i > 0),
row `m` of the inverse times m! giving the m-th derivative weights.
"dupD" shifts the stencil by +1 and "ddnD" by -1 (finite_difference.py:260-270);
mixed second derivatives are products of two first-derivative stencils
(finite_difference.py:343-368).  Exact rational arithmetic (fractions).
"""
from fractions import Fraction
from math import factorial

import numpy as np


def _solve_exact(M, b):
    """Gauss-Jordan elimination over Fractions: returns x with M x = b."""
    n = len(M)
    A = [list(M[i]) + [b[i]] for i in range(n)]
    for c in range(n):
        p = next(r for r in range(c, n) if A[r][c] != 0)
        A[c], A[p] = A[p], A[c]
        piv = A[c][c]
        A[c] = [v / piv for v in A[c]]
        for r in range(n):
            if r != c and A[r][c] != 0:
                f = A[r][c]
                A[r] = [vr - f * vc for vr, vc in zip(A[r], A[c])]
    return [A[i][n] for i in range(n)]


def fd_weights(order, deriv, shift=0):
    """Weights w[j] for points x_j = j - order/2 + shift, j = 0..order.

    deriv = 1 (first derivative) or 2 (second derivative).  Returns
    (offsets, weights) as lists of int and Fraction; the derivative is
    sum_j w[j] f(x_j) / dx**deriv.
    """
    n = order + 1
    offs = [j - order // 2 + shift for j in range(n)]
    # Row i of M holds offs**i; w solves M w = deriv! e_deriv, which is the
    # transpose statement of "row `deriv` of M^-1 times deriv!".
    M = [[Fraction(o) ** i if not (o == 0 and i > 0) else Fraction(0) for o in offs]
         for i in range(n)]
    M[0] = [Fraction(1)] * n
    rhs = [Fraction(0)] * n
    rhs[deriv] = Fraction(factorial(deriv))
    w = _solve_exact(M, rhs)
    return offs, w


def ko_weights(order):
    """Kreiss-Oliger dissipation weights for FD order `order`
    (finite_difference.py:252-258, 310-313, 331-334): the (order+2)-th
    derivative on order+3 points (FD_KO_ORDER__CENTDERIVS_PLUS = 2) times
    (-1)**((order+4)/2) / 2**(order+2).  Offsets -(order/2+1) .. order/2+1;
    the stencil is multiplied by invdx once (finite_difference_helpers.py:486)."""
    n = order + 2
    offs, w = fd_weights(n, n)
    sign = -1 if ((n + 2) // 2) % 2 else 1
    return offs, [sign * x / Fraction(2) ** n for x in w]


def coeff_table(order):
    """Float coefficient table used by both the oracle and the C-ABI check."""
    c1 = fd_weights(order, 1)[1]
    c2 = fd_weights(order, 2)[1]
    up = fd_weights(order, 1, +1)[1]
    return ([float(x) for x in c1], [float(x) for x in c2], [float(x) for x in up])


# ----------------------------------------------------------------- stencils
class Stencils:
    """Applies FD stencils to arrays of shape (..., n2, n1, n0) (IDX4S order:
    axis -1 is i0).  Results are defined on the interior [ng:-ng] in every
    direction; `interior` trims to that block.
    """

    def __init__(self, order, ng, invdx):
        self.order = order
        self.ng = ng
        self.invdx = [float(v) for v in invdx]
        self.r = order // 2
        self.c1 = [float(v) for v in fd_weights(order, 1)[1]]
        self.c2 = [float(v) for v in fd_weights(order, 2)[1]]
        self.up = [float(v) for v in fd_weights(order, 1, +1)[1]]
        self.dn = [float(v) for v in fd_weights(order, 1, -1)[1]]

    def _shift(self, f, offs):
        """f shifted so that element [interior idx] reads f[idx + offs]."""
        ng = self.ng
        n2, n1, n0 = f.shape[-3:]
        o0, o1, o2 = offs
        return f[..., ng + o2:n2 - ng + o2, ng + o1:n1 - ng + o1, ng + o0:n0 - ng + o0]

    def _off(self, d, k):
        o = [0, 0, 0]
        o[d] = k
        return o

    def interior(self, f):
        return self._shift(f, (0, 0, 0))

    def d1(self, f, d):
        acc = 0.0
        for j, w in enumerate(self.c1):
            k = j - self.r
            if w != 0.0:
                acc = acc + w * self._shift(f, self._off(d, k))
        return acc * self.invdx[d]

    def d2(self, f, d):
        acc = 0.0
        for j, w in enumerate(self.c2):
            k = j - self.r
            if w != 0.0:
                acc = acc + w * self._shift(f, self._off(d, k))
        return acc * self.invdx[d] ** 2

    def d11(self, f, d, e):
        """Mixed second derivative d_d d_e f, d != e."""
        if d == e:
            return self.d2(f, d)
        acc = 0.0
        for a, wa in enumerate(self.c1):
            if wa == 0.0:
                continue
            for b, wb in enumerate(self.c1):
                if wb == 0.0:
                    continue
                o = [0, 0, 0]
                o[d] = a - self.r
                o[e] = b - self.r
                acc = acc + (wa * wb) * self._shift(f, o)
        return acc * (self.invdx[d] * self.invdx[e])

    def dup(self, f, d):
        acc = 0.0
        for j, w in enumerate(self.up):
            k = j - self.r + 1
            if w != 0.0:
                acc = acc + w * self._shift(f, self._off(d, k))
        return acc * self.invdx[d]

    def ddn(self, f, d):
        acc = 0.0
        for j, w in enumerate(self.dn):
            k = j - self.r - 1
            if w != 0.0:
                acc = acc + w * self._shift(f, self._off(d, k))
        return acc * self.invdx[d]

    def dko(self, f, d):
        """Kreiss-Oliger derivative ("_dKOD" symbols) along direction d."""
        acc = 0.0
        for k, w in zip(*ko_weights(self.order)):
            acc = acc + float(w) * self._shift(f, self._off(d, k))
        return acc * self.invdx[d]

    def dupwind(self, f, d, control):
        """Control-vector upwinding of finite_difference_helpers.py:790-820:
        UpWind = (control > 0); result = UpWind*(dupD - ddnD) + ddnD."""
        up = self.dup(f, d)
        dn = self.ddn(f, d)
        w = (control > 0.0).astype(np.float64)
        return w * (up - dn) + dn


if __name__ == "__main__":
    for order in (2, 4, 6, 8):
        c1, c2, up = coeff_table(order)
        print(order, "c1", fd_weights(order, 1)[1])
        print(order, "c2", fd_weights(order, 2)[1])
        print(order, "up", fd_weights(order, 1, 1)[1])
