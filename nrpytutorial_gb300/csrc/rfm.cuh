// rfm.cuh -- reference metric ("hatted" quantities) for orthogonal,
// diagonal coordinate systems: Cartesian, Spherical, SinhSpherical,
// SinhSphericalv2, Cylindrical, SinhCylindrical.
//
// reference_metric.py:487-601 derives, from the orthogonal scale factors
// s_i(xx) (ghat_ii = s_i^2, ReU_i = 1/s_i, ReDD_ij = s_i s_j), the first and
// second derivatives of ReU, ReDD and ghat, the Christoffel symbols
// GammahatUDD and their derivatives, and det(ghat) with derivatives.  Here
// the same quantities are evaluated numerically in FP64 from closed-form
// s_i, ds_i, d2s_i, once per (i0,iB) column of the grid (the Spherical family
// depends on xx0 and xx1 only, iB = i1; the Cylindrical family on xx0 and xx2
// only, iB = i2), and stored as dense tables -- the analogue of the
// rfm_precompute arrays of reference_metric.py:603-886.
//
// Which entries can be non-zero follows from which coordinates each s_i
// depends on (the `dep` matrix).  Kernels test those masks with constexpr
// functions of the (unrolled, hence constant) tensor indices, so structural
// zeros cost no arithmetic and no loads; on Cartesian grids every hatted
// quantity is a literal 0 or 1.
#pragma once
#include "common.cuh"

namespace nrgpu {

// ------------------------------------------------------ table slot layout
namespace rq {
constexpr int ReU = 0;          // [3]
constexpr int ReUdD = 3;        // [3][3]      d_j ReU_i
constexpr int ReUdDD = 12;      // [3][3][3]   d_j d_k ReU_i
constexpr int ReDD = 39;        // [3][3]
constexpr int ReDDdD = 48;      // [3][3][3]
constexpr int ReDDdDD = 75;     // [3][3][3][3]
constexpr int ghatDD = 156;     // [3][3]
constexpr int ghatUU = 165;     // [3][3]
constexpr int ghatDDdD = 174;   // [3][3][3]
constexpr int ghatDDdDD = 201;  // [3][3][3][3]
constexpr int GammahatUDD = 282;    // [3][3][3]
constexpr int GammahatUDDdD = 309;  // [3][3][3][3]  d_l Gammahat^i_jk
constexpr int detgammahat = 390;    // [1]
constexpr int detgammahatdD = 391;  // [3]
constexpr int detgammahatdDD = 394; // [3][3]
constexpr int NQ = 403;
}  // namespace rq

// ------------------------------------------------------- dependency masks
__host__ __device__ constexpr bool cylindrical_family(int cs) {
  return cs == NRGPU_COORD_CYLINDRICAL || cs == NRGPU_COORD_SINHCYLINDRICAL || cs == NRGPU_COORD_SINHCYLINDRICALV2;
}

__host__ __device__ constexpr bool symtp_family(int cs) {
  return cs == NRGPU_COORD_SYMTP || cs == NRGPU_COORD_SINHSYMTP;
}

// dep(CS, i, k): does scale factor s_i depend on xx_k?
__host__ __device__ constexpr bool dep(int cs, int i, int k) {
  return cs == NRGPU_COORD_CARTESIAN ? false
         // SymTP family: s0 = AA' var1/var2, s1 = var1, s2 = AA sin(xx1), all of (xx0, xx1)
         : symtp_family(cs) ? k <= 1
         // Cylindrical family: s0 = drho/dxx0, s1 = rho(xx0), s2 = dz/dxx2
         : cylindrical_family(cs) ? ((k == 0 && i <= 1) || (k == 2 && i == 2))
         // Spherical family: s0 = dr/dxx0, s1 = r(xx0), s2 = r(xx0) sin(xx1)
         : (k == 0) ? true : (k == 1 ? i == 2 : false);
}

template <int CS> struct RfmMask {
  static constexpr bool trivial = (CS == NRGPU_COORD_CARTESIAN);
  static constexpr bool ReUdD(int i, int j) { return dep(CS, i, j); }
  static constexpr bool ReUdDD(int i, int j, int k) { return dep(CS, i, j) && dep(CS, i, k); }
  static constexpr bool ReDDdD(int i, int j, int k) { return dep(CS, i, k) || dep(CS, j, k); }
  static constexpr bool ReDDdDD(int i, int j, int k, int l) {
    return (dep(CS, i, k) && dep(CS, i, l)) || (dep(CS, j, k) && dep(CS, j, l)) ||
           (dep(CS, i, k) && dep(CS, j, l)) || (dep(CS, i, l) && dep(CS, j, k));
  }
  static constexpr bool ghatDDdD(int i, int j, int k) { return i == j && dep(CS, i, k); }
  static constexpr bool ghatDDdDD(int i, int j, int k, int l) {
    return i == j && dep(CS, i, k) && dep(CS, i, l);
  }
  // Gammahat^i_kl = (1/2) ghat^ii (d_l ghat_ik + d_k ghat_il - d_i ghat_kl)
  static constexpr bool Gammahat(int i, int k, int l) {
    return (i == k && dep(CS, i, l)) || (i == l && dep(CS, i, k)) || (k == l && dep(CS, k, i));
  }
  static constexpr bool GammahatdD(int i, int k, int l, int n) {
    return Gammahat(i, k, l) && (dep(CS, i, n) || (k == l && dep(CS, k, n)) ||
                                 (i == k && dep(CS, i, n)) || (i == l && dep(CS, i, n)));
  }
  static constexpr bool detgdD(int k) { return dep(CS, 0, k) || dep(CS, 1, k) || dep(CS, 2, k); }
  static constexpr bool detgdDD(int k, int l) {
    return (dep(CS, 0, k) || dep(CS, 1, k) || dep(CS, 2, k)) &&
           (dep(CS, 0, l) || dep(CS, 1, l) || dep(CS, 2, l));
  }
};

// ------------------------------------------------------- point accessor
// Reads hatted quantities at one (i0,iB) column.  R is the arithmetic type
// of the caller; tables are FP64 (tab64) with an FP32 copy (tab32).
// MODE RFM_TABLE: base = table + iB*N0 + i0, plane = N0*NB.
// MODE RFM_LOCAL: base points at this thread's own NQ values (plane 1),
//   computed from the caller's coordinates instead of read from the table.
enum RfmMode { RFM_TABLE = 0, RFM_LOCAL = 1 };

template <int CS, typename R, int MODE = RFM_TABLE> struct Rfm {
  using M = RfmMask<CS>;
  const R *__restrict__ base;
  long long plane;

  __device__ __forceinline__ R q(int slot) const {
    if constexpr (MODE == RFM_LOCAL) return base[slot];
    else return __ldg(base + slot * plane);
  }

  __device__ __forceinline__ R ReU(int i) const { return M::trivial ? (R)1 : q(rq::ReU + i); }
  __device__ __forceinline__ R ReUdD(int i, int j) const { return q(rq::ReUdD + 3 * i + j); }
  __device__ __forceinline__ R ReUdDD(int i, int j, int k) const {
    return q(rq::ReUdDD + 9 * i + 3 * j + k);
  }
  __device__ __forceinline__ R ReDD(int i, int j) const {
    return M::trivial ? (R)1 : q(rq::ReDD + 3 * i + j);
  }
  __device__ __forceinline__ R ReDDdD(int i, int j, int k) const {
    return q(rq::ReDDdD + 9 * i + 3 * j + k);
  }
  __device__ __forceinline__ R ReDDdDD(int i, int j, int k, int l) const {
    return q(rq::ReDDdDD + 27 * i + 9 * j + 3 * k + l);
  }
  // ghatDD/ghatUU are only read where i == j.
  __device__ __forceinline__ R ghatDD(int i) const {
    return M::trivial ? (R)1 : q(rq::ghatDD + 4 * i);
  }
  __device__ __forceinline__ R ghatUU(int i) const {
    return M::trivial ? (R)1 : q(rq::ghatUU + 4 * i);
  }
  __device__ __forceinline__ R ghatDDdD(int i, int j, int k) const {
    return q(rq::ghatDDdD + 9 * i + 3 * j + k);
  }
  __device__ __forceinline__ R ghatDDdDD(int i, int j, int k, int l) const {
    return q(rq::ghatDDdDD + 27 * i + 9 * j + 3 * k + l);
  }
  __device__ __forceinline__ R G(int i, int k, int l) const {
    return q(rq::GammahatUDD + 9 * i + 3 * k + l);
  }
  __device__ __forceinline__ R GdD(int i, int k, int l, int n) const {
    return q(rq::GammahatUDDdD + 27 * i + 9 * k + 3 * l + n);
  }
  __device__ __forceinline__ R detg() const { return M::trivial ? (R)1 : q(rq::detgammahat); }
  __device__ __forceinline__ R detgdD(int k) const { return q(rq::detgammahatdD + k); }
  __device__ __forceinline__ R detgdDD(int k, int l) const { return q(rq::detgammahatdDD + 3 * k + l); }
};

// Extent of the table's second coordinate, and whether tables fit a grid.
inline int rfm_second_extent(const paramstruct *p) {
  return cylindrical_family(p->CoordSystem) ? p->Nxx_plus_2NGHOSTS2 : p->Nxx_plus_2NGHOSTS1;
}
inline bool rfm_matches(const rfm_struct *rfm, const paramstruct *p) {
  return rfm && rfm->table64 && rfm->CoordSystem == p->CoordSystem && rfm->N0 == p->Nxx_plus_2NGHOSTS0 &&
         rfm->N1 == rfm_second_extent(p);
}

template <int CS, typename R>
__device__ __forceinline__ Rfm<CS, R> rfm_at(const R *tab, const Grid &g, int i0, int i1, int i2) {
  constexpr bool cyl = cylindrical_family(CS);
  const int nB = cyl ? g.n2 : g.n1, iB = cyl ? i2 : i1;
  Rfm<CS, R> r;
  r.base = tab ? tab + (long long)iB * g.n0 + i0 : nullptr;
  r.plane = (long long)g.n0 * nB;
  return r;
}

// --------------------------------------------------- scale-factor closed forms
// The coordinate parameters of a paramstruct that the maps below read.
struct CoordParams {
  int cs;
  double AMPL, SINHW, const_dr;             // Spherical family
  double AMPLRHO, SINHWRHO, AMPLZ, SINHWZ;  // SinhCylindrical
  double const_drho, const_dz;              // SinhCylindricalv2
  double bScale, SINHWAA, AMAX;             // SymTP family
};

__host__ __device__ inline CoordParams coord_params(const paramstruct &p) {
  return CoordParams{p.CoordSystem, p.AMPL,      p.SINHW,    p.const_dr, p.AMPLRHO, p.SINHWRHO, p.AMPLZ,
                     p.SINHWZ,      p.const_drho, p.const_dz, p.bScale,   p.SINHWAA, p.AMAX};
}

__host__ __device__ inline bool spherical_family(int cs) {
  return cs == NRGPU_COORD_SPHERICAL || cs == NRGPU_COORD_SINHSPHERICAL || cs == NRGPU_COORD_SINHSPHERICALV2;
}

// f(x) = A sinh(x/w) / sinh(1/w) + A c x and its first three derivatives,
// with the exponentials written as reference_metric.py:125-126, 255-258 does.
__host__ __device__ inline void sinh_map(double A, double w, double c, double x, double f[4]) {
  const double ep = exp(x / w), em = exp(-x / w);
  const double den = exp(1.0 / w) - exp(-1.0 / w);
  const double sh = A * (ep - em) / den, ch = A * (ep + em) / (w * den);
  f[0] = sh + A * c * x;
  f[1] = ch + A * c;
  f[2] = sh / (w * w);
  f[3] = ch / (w * w);
}

// Spherical family: r(xx0) and three derivatives.  Spherical: r = xx0;
// SinhSpherical: the sinh map (reference_metric.py:125-126); SinhSphericalv2
// adds AMPL const_dr xx0 (:142-143).
__host__ __device__ inline void radial_map(const CoordParams &c, double x, double r[4]) {
  if (c.cs == NRGPU_COORD_SINHSPHERICAL || c.cs == NRGPU_COORD_SINHSPHERICALV2) {
    sinh_map(c.AMPL, c.SINHW, c.cs == NRGPU_COORD_SINHSPHERICALV2 ? c.const_dr : 0.0, x, r);
  } else {
    r[0] = x;
    r[1] = 1.0;
    r[2] = r[3] = 0.0;
  }
}

// Cylindrical family: rho(xx0) and z(xx2) with three derivatives each
// (Cylindrical: the identity, reference_metric.py:237-239; SinhCylindrical:
// sinh maps, :255-258; SinhCylindricalv2 adds the linear terms, :273-275).
__host__ __device__ inline void cylinder_maps(const CoordParams &c, double x0, double x2, double rho[4],
                                              double z[4]) {
  if (c.cs == NRGPU_COORD_SINHCYLINDRICAL || c.cs == NRGPU_COORD_SINHCYLINDRICALV2) {
    const bool v2 = c.cs == NRGPU_COORD_SINHCYLINDRICALV2;
    sinh_map(c.AMPLRHO, c.SINHWRHO, v2 ? c.const_drho : 0.0, x0, rho);
    sinh_map(c.AMPLZ, c.SINHWZ, v2 ? c.const_dz : 0.0, x2, z);
  } else {
    rho[0] = x0; rho[1] = 1.0; rho[2] = rho[3] = 0.0;
    z[0] = x2; z[1] = 1.0; z[2] = z[3] = 0.0;
  }
}

// SymTP family (reference_metric.py:320-383): AA(xx0) with three derivatives
// (SymTP: AA = xx0; SinhSymTP: the sinh map of AMAX, SINHWAA), var1 =
// sqrt(AA^2 + (bScale sin xx1)^2), var2 = sqrt(AA^2 + bScale^2).
__host__ __device__ inline void symtp_aa(const CoordParams &c, double x0, double A[4]) {
  if (c.cs == NRGPU_COORD_SINHSYMTP) {
    sinh_map(c.AMAX, c.SINHWAA, 0.0, x0, A);
  } else {
    A[0] = x0;
    A[1] = 1.0;
    A[2] = A[3] = 0.0;
  }
}

// s[i], ds[i][k] = d s_i / d xx_k, dds[i][k][l] at uniform coordinates
// (xx0, xx1, xx2) (reference_metric.py:168-175 Spherical family: s0 = dr/dxx0,
// s1 = r, s2 = r sin(xx1); :289-291 Cylindrical family: s0 = drho/dxx0,
// s1 = rho, s2 = dz/dxx2; Cartesian: 1).
struct ScaleFactors {
  double s[3], ds[3][3], dds[3][3][3];
};

__host__ __device__ inline void scale_factors(const CoordParams &c, double xx0, double xx1, double xx2,
                                              ScaleFactors *S) {
  for (int i = 0; i < 3; i++) {
    S->s[i] = 1.0;
    for (int k = 0; k < 3; k++) {
      S->ds[i][k] = 0.0;
      for (int l = 0; l < 3; l++) S->dds[i][k][l] = 0.0;
    }
  }
  if (c.cs == NRGPU_COORD_CARTESIAN) return;
  if (symtp_family(c.cs)) {
    // s0 = AA' q with q = var1/var2, s1 = var1, s2 = AA sin(xx1); derivatives
    // in (xx0, xx1) by the chain rule (none depends on xx2)
    double A[4];
    symtp_aa(c, xx0, A);
    const double b2 = c.bScale * c.bScale, sn = sin(xx1), cn = cos(xx1);
    const double v1 = sqrt(A[0] * A[0] + b2 * sn * sn), v2 = sqrt(A[0] * A[0] + b2);
    const double du[2] = {2.0 * A[0] * A[1], 2.0 * b2 * sn * cn};
    const double ddu[2][2] = {{2.0 * (A[1] * A[1] + A[0] * A[2]), 0.0}, {0.0, 2.0 * b2 * (cn * cn - sn * sn)}};
    double dv1[2], ddv1[2][2], dv2[2] = {du[0] / (2.0 * v2), 0.0}, ddv2[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    ddv2[0][0] = ddu[0][0] / (2.0 * v2) - du[0] * du[0] / (4.0 * v2 * v2 * v2);
    for (int k = 0; k < 2; k++) {
      dv1[k] = du[k] / (2.0 * v1);
      for (int l = 0; l < 2; l++) ddv1[k][l] = ddu[k][l] / (2.0 * v1) - du[k] * du[l] / (4.0 * v1 * v1 * v1);
    }
    const double q = v1 / v2;
    double dq[2], ddq[2][2];
    for (int k = 0; k < 2; k++) dq[k] = dv1[k] / v2 - v1 * dv2[k] / (v2 * v2);
    for (int k = 0; k < 2; k++)
      for (int l = 0; l < 2; l++)
        ddq[k][l] = ddv1[k][l] / v2 - (dv1[k] * dv2[l] + dv1[l] * dv2[k]) / (v2 * v2) -
                    v1 * ddv2[k][l] / (v2 * v2) + 2.0 * v1 * dv2[k] * dv2[l] / (v2 * v2 * v2);
    const double dA1[2] = {A[2], 0.0}, ddA1[2][2] = {{A[3], 0.0}, {0.0, 0.0}};
    const double ds2[2] = {A[1] * sn, A[0] * cn}, dds2[2][2] = {{A[2] * sn, A[1] * cn}, {A[1] * cn, -A[0] * sn}};
    S->s[0] = A[1] * q;
    S->s[1] = v1;
    S->s[2] = A[0] * sn;
    for (int k = 0; k < 2; k++) {
      S->ds[0][k] = dA1[k] * q + A[1] * dq[k];
      S->ds[1][k] = dv1[k];
      S->ds[2][k] = ds2[k];
      for (int l = 0; l < 2; l++) {
        S->dds[0][k][l] = ddA1[k][l] * q + dA1[k] * dq[l] + dA1[l] * dq[k] + A[1] * ddq[k][l];
        S->dds[1][k][l] = ddv1[k][l];
        S->dds[2][k][l] = dds2[k][l];
      }
    }
    return;
  }
  if (cylindrical_family(c.cs)) {
    double rho[4], z[4];
    cylinder_maps(c, xx0, xx2, rho, z);
    S->s[0] = rho[1];
    S->s[1] = rho[0];
    S->s[2] = z[1];
    S->ds[0][0] = rho[2];
    S->ds[1][0] = rho[1];
    S->ds[2][2] = z[2];
    S->dds[0][0][0] = rho[3];
    S->dds[1][0][0] = rho[2];
    S->dds[2][2][2] = z[3];
    return;
  }
  double r[4];
  radial_map(c, xx0, r);
  const double sn = sin(xx1), cs1 = cos(xx1);
  S->s[0] = r[1];
  S->s[1] = r[0];
  S->s[2] = r[0] * sn;
  S->ds[0][0] = r[2];
  S->ds[1][0] = r[1];
  S->ds[2][0] = r[1] * sn;
  S->ds[2][1] = r[0] * cs1;
  S->dds[0][0][0] = r[3];
  S->dds[1][0][0] = r[2];
  S->dds[2][0][0] = r[2] * sn;
  S->dds[2][0][1] = S->dds[2][1][0] = r[1] * cs1;
  S->dds[2][1][1] = -r[0] * sn;
}

// Fills all rq::NQ derived quantities from scale factors (dense, FP64).
__host__ __device__ inline void hatted_quantities(const ScaleFactors &S, double *out /*[rq::NQ]*/) {
  const double *s = S.s;
  for (int q = 0; q < rq::NQ; q++) out[q] = 0.0;
  double g[3], dg[3][3], ddg[3][3][3];
  for (int i = 0; i < 3; i++) {
    g[i] = s[i] * s[i];
    for (int k = 0; k < 3; k++) {
      dg[i][k] = 2.0 * s[i] * S.ds[i][k];
      for (int l = 0; l < 3; l++)
        ddg[i][k][l] = 2.0 * (S.ds[i][k] * S.ds[i][l] + s[i] * S.dds[i][k][l]);
    }
  }
  for (int i = 0; i < 3; i++) {
    out[rq::ReU + i] = 1.0 / s[i];
    out[rq::ghatDD + 4 * i] = g[i];
    out[rq::ghatUU + 4 * i] = 1.0 / g[i];
    for (int j = 0; j < 3; j++) {
      out[rq::ReUdD + 3 * i + j] = -S.ds[i][j] / (s[i] * s[i]);
      for (int k = 0; k < 3; k++)
        out[rq::ReUdDD + 9 * i + 3 * j + k] =
            -S.dds[i][j][k] / (s[i] * s[i]) + 2.0 * S.ds[i][j] * S.ds[i][k] / (s[i] * s[i] * s[i]);
      out[rq::ReDD + 3 * i + j] = s[i] * s[j];
      for (int k = 0; k < 3; k++) {
        out[rq::ReDDdD + 9 * i + 3 * j + k] = S.ds[i][k] * s[j] + s[i] * S.ds[j][k];
        for (int l = 0; l < 3; l++)
          out[rq::ReDDdDD + 27 * i + 9 * j + 3 * k + l] =
              S.dds[i][k][l] * s[j] + S.ds[i][k] * S.ds[j][l] + S.ds[i][l] * S.ds[j][k] +
              s[i] * S.dds[j][k][l];
      }
    }
    for (int k = 0; k < 3; k++) {
      out[rq::ghatDDdD + 9 * i + 3 * i + k] = dg[i][k];
      for (int l = 0; l < 3; l++) out[rq::ghatDDdDD + 27 * i + 9 * i + 3 * k + l] = ddg[i][k][l];
    }
  }
  // Christoffel symbols of the diagonal metric and their derivatives:
  // Gamma^i_kl = (1/2) ghat^ii (d_l g_ik + d_k g_il - d_i g_kl)
  auto dgDD = [&](int a, int b, int k) { return a == b ? dg[a][k] : 0.0; };
  auto ddgDD = [&](int a, int b, int k, int l) { return a == b ? ddg[a][k][l] : 0.0; };
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++)
      for (int l = 0; l < 3; l++) {
        const double bracket = dgDD(i, k, l) + dgDD(i, l, k) - dgDD(k, l, i);
        out[rq::GammahatUDD + 9 * i + 3 * k + l] = 0.5 / g[i] * bracket;
        for (int n = 0; n < 3; n++) {
          const double dbracket = ddgDD(i, k, l, n) + ddgDD(i, l, k, n) - ddgDD(k, l, i, n);
          const double dginv = -dg[i][n] / (g[i] * g[i]);
          out[rq::GammahatUDDdD + 27 * i + 9 * k + 3 * l + n] =
              0.5 * dginv * bracket + 0.5 / g[i] * dbracket;
        }
      }
  // det(ghat) = g0 g1 g2 and derivatives.
  out[rq::detgammahat] = g[0] * g[1] * g[2];
  for (int k = 0; k < 3; k++) {
    out[rq::detgammahatdD + k] = dg[0][k] * g[1] * g[2] + g[0] * dg[1][k] * g[2] + g[0] * g[1] * dg[2][k];
    for (int l = 0; l < 3; l++)
      out[rq::detgammahatdDD + 3 * k + l] =
          ddg[0][k][l] * g[1] * g[2] + g[0] * ddg[1][k][l] * g[2] + g[0] * g[1] * ddg[2][k][l] +
          dg[0][k] * dg[1][l] * g[2] + dg[0][l] * dg[1][k] * g[2] + dg[0][k] * g[1] * dg[2][l] +
          dg[0][l] * g[1] * dg[2][k] + g[0] * dg[1][k] * dg[2][l] + g[0] * dg[1][l] * dg[2][k];
  }
}

// xx -> Cartesian and d x_Cart^i / d xx^j (reference_metric.py xx_to_Cart:
// Spherical family :159-161, Cylindrical family :296-298).
__host__ __device__ inline void cart_jacobian(const CoordParams &c, double xx0, double xx1, double xx2,
                                              double x[3], double J[3][3]) {
  if (c.cs == NRGPU_COORD_CARTESIAN) {
    x[0] = xx0;
    x[1] = xx1;
    x[2] = xx2;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) J[i][j] = i == j ? 1.0 : 0.0;
  } else if (symtp_family(c.cs)) {
    // (AA sin xx1 cos xx2, AA sin xx1 sin xx2, var2 cos xx1) (reference_metric.py:334-336)
    double A[4];
    symtp_aa(c, xx0, A);
    const double b2 = c.bScale * c.bScale, v2 = sqrt(A[0] * A[0] + b2), dv2 = A[0] * A[1] / v2;
    const double st = sin(xx1), ct = cos(xx1), sp = sin(xx2), cp = cos(xx2);
    x[0] = A[0] * st * cp;
    x[1] = A[0] * st * sp;
    x[2] = v2 * ct;
    J[0][0] = A[1] * st * cp;
    J[0][1] = A[0] * ct * cp;
    J[0][2] = -A[0] * st * sp;
    J[1][0] = A[1] * st * sp;
    J[1][1] = A[0] * ct * sp;
    J[1][2] = A[0] * st * cp;
    J[2][0] = dv2 * ct;
    J[2][1] = -v2 * st;
    J[2][2] = 0.0;
  } else if (cylindrical_family(c.cs)) {
    double rho[4], z[4];
    cylinder_maps(c, xx0, xx2, rho, z);
    const double sp = sin(xx1), cp = cos(xx1);
    x[0] = rho[0] * cp;
    x[1] = rho[0] * sp;
    x[2] = z[0];
    J[0][0] = rho[1] * cp;
    J[0][1] = -rho[0] * sp;
    J[0][2] = 0.0;
    J[1][0] = rho[1] * sp;
    J[1][1] = rho[0] * cp;
    J[1][2] = 0.0;
    J[2][0] = 0.0;
    J[2][1] = 0.0;
    J[2][2] = z[1];
  } else {
    double r[4];
    radial_map(c, xx0, r);
    const double st = sin(xx1), ct = cos(xx1), sp = sin(xx2), cp = cos(xx2);
    x[0] = r[0] * st * cp;
    x[1] = r[0] * st * sp;
    x[2] = r[0] * ct;
    J[0][0] = r[1] * st * cp;
    J[0][1] = r[0] * ct * cp;
    J[0][2] = -r[0] * st * sp;
    J[1][0] = r[1] * st * sp;
    J[1][1] = r[0] * ct * sp;
    J[1][2] = r[0] * st * cp;
    J[2][0] = r[1] * ct;
    J[2][1] = -r[0] * st;
    J[2][2] = 0.0;
  }
}

// General 3x3 inverse by cofactors (indexedexp.py generic_matrix_inverter3x3).
__host__ __device__ inline void inverse3(const double J[3][3], double Ji[3][3]) {
  Ji[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  Ji[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  Ji[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  Ji[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  Ji[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  Ji[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  Ji[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  Ji[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  Ji[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const double det = J[0][0] * Ji[0][0] + J[0][1] * Ji[1][0] + J[0][2] * Ji[2][0];
  const double id = 1.0 / det;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Ji[i][j] *= id;
}

// Cell-centred uniform coordinate of index j (reference_metric.py:1001-1006).
// Evaluated without FMA contraction, so device and host agree bit for bit
// with the reference's `xxmin + ((REAL)(j-NGHOSTS) + (1.0/2.0))*dxx`.
__host__ __device__ inline double xx_of(double xxmin, double dxx, int j, int ng) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(xxmin, __dmul_rn((double)(j - ng) + 0.5, dxx));
#else
  volatile double t = ((double)(j - ng) + 0.5) * dxx;
  return xxmin + t;
#endif
}

}  // namespace nrgpu
