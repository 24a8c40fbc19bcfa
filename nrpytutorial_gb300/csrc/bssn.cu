// bssn.cu -- BSSN dispatch, det(gammabar) = det(gammahat) rescale,
// Hamiltonian constraint, Brill-Lindquist initial data, and the C ABI.
#include <math.h>

#include "bssn_kernels.cuh"
#include "bssn_staged.cuh"

namespace nrgpu {
namespace bssn {

NRGPU_BSSN_DECLARE(NRGPU_COORD_CARTESIAN, 2)
NRGPU_BSSN_DECLARE(NRGPU_COORD_CARTESIAN, 4)
NRGPU_BSSN_DECLARE(NRGPU_COORD_CARTESIAN, 6)
NRGPU_BSSN_DECLARE(NRGPU_COORD_CARTESIAN, 8)
NRGPU_BSSN_DECLARE(NRGPU_COORD_SINHSPHERICAL, 4)
NRGPU_BSSN_DECLARE(NRGPU_COORD_SINHCYLINDRICAL, 4)
NRGPU_BSSN_DECLARE(NRGPU_COORD_SINHSYMTP, 4)
NRGPU_BSSN_DECLARE(NRGPU_COORD_SPHERICAL, 4)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_CARTESIAN, 2)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_CARTESIAN, 4)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_CARTESIAN, 6)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_CARTESIAN, 8)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_SINHSPHERICAL, 4)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_SINHCYLINDRICAL, 4)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_SINHSYMTP, 4)
NRGPU_BSSN_STAGED_DECLARE(NRGPU_COORD_SPHERICAL, 4)

// Which BSSN Ricci/RHS kernels run (nrgpu_set_bssn_kernels).
static int g_kernels = NRGPU_BSSN_KERNELS_AUTO;
// The family a grid and precision run on.  AUTO: the fastest whole step
// measured on GB300 with the split RK update (graph replay, one call; ms per
// step, 128^3 Cartesian and 128x64x16 curvilinear grids):
//   pairs, Cartesian FD2 / 4 / 6 / 8:  point 5.40 / 8.30 / 13.36 / 19.28,
//     staged 6.17 / 7.80 / 9.94 / 15.50, fused 5.73 / 7.47 / 10.78 / 15.77;
//   pairs, SinhSpherical / SinhCylindrical / SinhSymTP FD4:  point 0.938 /
//     0.934 / 1.020, staged 0.831 / 0.851 / 0.849, fused 0.802 / 0.804 / 0.882;
//   plain FP32, Cartesian FD2 / FD6:  point 4.13 / 8.35, staged 5.03 / 8.42,
//     fused 5.02 / 7.69 (grids whose FP32 rows are not a multiple of 16 bytes,
//     e.g. 134 points, run the point kernels whatever the selection).
// FP64 is FP64-pipe bound and keeps the point kernels.
static int family(const paramstruct *p, int prec) {
  if (g_kernels != NRGPU_BSSN_KERNELS_AUTO) return g_kernels;
  const int cs = dispatch_cs(p->CoordSystem);
  if (prec == NRGPU_PREC_FP64) return NRGPU_BSSN_KERNELS_POINT;
  if (cs == NRGPU_COORD_CARTESIAN) {
    if (p->FD_order <= 2) return NRGPU_BSSN_KERNELS_POINT;
    if (pair_precision(prec)) return p->FD_order >= 6 ? NRGPU_BSSN_KERNELS_STAGED : NRGPU_BSSN_KERNELS_FUSED;
    return p->FD_order >= 6 ? NRGPU_BSSN_KERNELS_FUSED : NRGPU_BSSN_KERNELS_POINT;
  }
  if (pair_precision(prec)) return cs == NRGPU_COORD_SINHSYMTP ? NRGPU_BSSN_KERNELS_STAGED : NRGPU_BSSN_KERNELS_FUSED;
  return NRGPU_BSSN_KERNELS_STAGED;
}
static bool staged_for(const paramstruct *p, int prec) { return family(p, prec) != NRGPU_BSSN_KERNELS_POINT; }

#define NRGPU_BSSN_SWITCH(CALL)                                                               \
  switch (dispatch_cs(p->CoordSystem) * 16 + p->FD_order) {                                   \
    case NRGPU_COORD_CARTESIAN * 16 + 2: return CALL(NRGPU_COORD_CARTESIAN, 2);               \
    case NRGPU_COORD_CARTESIAN * 16 + 4: return CALL(NRGPU_COORD_CARTESIAN, 4);               \
    case NRGPU_COORD_CARTESIAN * 16 + 6: return CALL(NRGPU_COORD_CARTESIAN, 6);               \
    case NRGPU_COORD_CARTESIAN * 16 + 8: return CALL(NRGPU_COORD_CARTESIAN, 8);               \
    case NRGPU_COORD_SINHSPHERICAL * 16 + 4: return CALL(NRGPU_COORD_SINHSPHERICAL, 4);       \
    case NRGPU_COORD_SINHCYLINDRICAL * 16 + 4: return CALL(NRGPU_COORD_SINHCYLINDRICAL, 4);   \
    case NRGPU_COORD_SINHSYMTP * 16 + 4: return CALL(NRGPU_COORD_SINHSYMTP, 4);               \
    case NRGPU_COORD_SPHERICAL * 16 + 4: return CALL(NRGPU_COORD_SPHERICAL, 4);               \
  }                                                                                           \
  set_error("BSSN: CoordSystem %d with FD_order %d not built", p->CoordSystem, p->FD_order); \
  return NRGPU_ERR_UNSUPPORTED;

static int check_bssn(const rfm_struct *rfm, const paramstruct *p) {
  int st = check_params(p);
  if (st) return st;
  // The upwinded stencils reach FD_order/2 + 1 points (NGHOSTS rule of
  // Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide.ipynb:835).
  NRGPU_REQUIRE(p->NGHOSTS >= p->FD_order / 2 + 1, "BSSN needs NGHOSTS >= FD_order/2+1 (have %d)", p->NGHOSTS);
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN || rfm_matches(rfm, p),
                "curvilinear BSSN needs an rfm_struct defined for this grid");
  return NRGPU_OK;
}

// ---------------------------------------------------- det(gammabar) rescale
// h'_ij = (|det ghat| / det gammabar)^(1/3) (delta_ij + h_ij) - delta_ij at
// all points (Enforce_Detgammabar_Constraint.py:42-50), FP64 arithmetic on
// FP64 data (FP32 data: enforce_ff_kernel below).
template <int CS, typename T>
__global__ void enforce_kernel(Grid g, const double *__restrict__ tab, T *__restrict__ gfs) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  if (i0 >= g.n0) return;
  const long long idx = (long long)i0 + (long long)g.n0 * ((long long)i1 + (long long)g.n1 * i2);
  const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
  double h[3][3], gb[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const long long k = (long long)(HDD00 + S6(i, j)) * g.ntot + idx;
      if constexpr (std::is_same<T, float2>::value) h[i][j] = h[j][i] = pair_value(gfs[k]);
      else h[i][j] = h[j][i] = (double)gfs[k];
      double v = RfmMask<CS>::trivial ? h[i][j] : h[i][j] * rf.ReDD(i, j);
      if (i == j) v += rf.ghatDD(i);
      gb[i][j] = gb[j][i] = v;
    }
  const double det = -gb[0][2] * gb[0][2] * gb[1][1] + 2.0 * gb[0][1] * gb[0][2] * gb[1][2] -
                     gb[0][0] * gb[1][2] * gb[1][2] - gb[0][1] * gb[0][1] * gb[2][2] +
                     gb[0][0] * gb[1][1] * gb[2][2];
  // f = (|det ghat| / det gammabar)^{1/3} = s^{-1/3}, s = det gammabar / |det ghat|:
  // Newton-Raphson on w^{-3} = s (w <- w (4 - s w^3) / 3, quadratic
  // convergence) from the FP32 reciprocal cube root, two steps to FP64
  // accuracy, in place of the FP64 cube root (several times the FP64
  // instructions on this FP64-light GPU).
  const double sdet = det / fabs(rf.detg());
  double f = (double)rcbrtf((float)sdet);
#pragma unroll
  for (int it = 0; it < 2; it++) f = f * (4.0 - sdet * f * f * f) * (1.0 / 3.0);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const double d = (i == j) ? 1.0 : 0.0;
      const long long k = (long long)(HDD00 + S6(i, j)) * g.ntot + idx;
      const double v = f * (d + h[i][j]) - d;
      if constexpr (std::is_same<T, float2>::value) gfs[k] = split_pair(v);
      else gfs[k] = (T)v;
    }
}

// The same rescale for FP32 storage (pairs or plain FP32), and for the FP64
// state of the FP32-stage steps (which carry it at float-float precision),
// in float-float arithmetic on the FP32 pipe.  For the orthogonal reference metrics
// (gammahat_ij = s_i^2 delta_ij, ReDD_ij = s_i s_j) det gammabar / det ghat =
// det(I + h), so f = det(I + h)^{-1/3}: the FP32 reciprocal cube root, then
// two Newton steps w <- w + w (1 - D w^3)/3 with the residual in float-float;
// h'_ij = (f - 1) delta_ij + f h_ij.  About 48 significant bits.
template <typename T>
__global__ void enforce_ff_kernel(Grid g, T *__restrict__ gfs) {
  // pointwise and coordinate-free: one thread per point of the flat grid
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.ntot) return;
  float2 h[6];
#pragma unroll
  for (int s = 0; s < 6; s++) {
    const long long k = (long long)(HDD00 + s) * g.ntot + idx;
    if constexpr (std::is_same<T, float2>::value) h[s] = gfs[k];
    else if constexpr (std::is_same<T, double>::value) h[s] = split_pair_fast(gfs[k]);
    else h[s] = make_float2(gfs[k], 0.f);
  }
  const float2 one = make_float2(1.f, 0.f);
  const float2 a = ff_add(one, h[S6(0, 0)]), b = ff_add(one, h[S6(1, 1)]), c = ff_add(one, h[S6(2, 2)]);
  const float2 h01 = h[S6(0, 1)], h02 = h[S6(0, 2)], h12 = h[S6(1, 2)];
  float2 D = ff_mul_ff(ff_mul_ff(a, b), c);
  const float2 t = ff_mul_ff(ff_mul_ff(h01, h02), h12);
  D = ff_add(D, ff_add(t, t));
  D = ff_add(D, ff_neg(ff_mul_ff(a, ff_mul_ff(h12, h12))));
  D = ff_add(D, ff_neg(ff_mul_ff(b, ff_mul_ff(h02, h02))));
  D = ff_add(D, ff_neg(ff_mul_ff(c, ff_mul_ff(h01, h01))));
  float2 w = make_float2(rcbrtf(D.x), 0.f);
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const float2 r = ff_add(one, ff_neg(ff_mul_ff(D, ff_mul_ff(ff_mul_ff(w, w), w))));
    w = ff_add(w, make_float2(__fmul_rn(w.x, r.x) * (1.0f / 3.0f), 0.f));
  }
  const float2 fm1 = ff_add(w, ff_neg(one));
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const int s = S6(i, j);
      float2 v = ff_mul_ff(w, h[s]);
      if (i == j) v = ff_add(fm1, v);
      const long long k = (long long)(HDD00 + s) * g.ntot + idx;
      if constexpr (std::is_same<T, float2>::value) gfs[k] = v;
      else if constexpr (std::is_same<T, double>::value) gfs[k] = f2d_bits(v.x) + f2d_bits(v.y);
      else gfs[k] = v.x;
    }
}

// ------------------------------------------------------ momentum constraint
template <int CS, int ORDER>
__global__ void __launch_bounds__(kBlockX *kBlockY)
    momentum_kernel(Grid g, const double *__restrict__ in, const double *__restrict__ tab, double *__restrict__ aux) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
  double MU[3];
  momentum_point<ORDER, CS, double>(P, rf, inv, MU);
#pragma unroll
  for (int k = 0; k < 3; k++) aux[(long long)k * g.ntot + idx] = MU[k];
}

// --------------------------------------------------- Hamiltonian constraint
template <int CS, int ORDER>
__global__ void __launch_bounds__(kBlockX *kBlockY)
    hamiltonian_kernel(Grid g, const double *__restrict__ in, const double *__restrict__ tab,
                       double *__restrict__ aux) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  using R = double;
  using M = RfmMask<CS>;
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const R inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g, i0, i1, i2);
  Metric<CS, R> m;
  metric_point<ORDER, CS, R>(P, rf, inv, m);
  R Rbar[6];
  ricci_point<ORDER, CS, R>(P, rf, inv, m, Rbar);
  const R cf = __ldg(P.gf(CF)), trK = __ldg(P.gf(TRK));
  R Abar[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const R a = __ldg(P.gf(ADD00 + S6(i, j)));
      Abar[i][j] = Abar[j][i] = M::trivial ? a : a * rf.ReDD(i, j);
    }
  R H = (R)(2.0 / 3.0) * trK * trK;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R auu = 0.0;
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = 0; l < 3; l++) auu += m.gUU[i][k] * m.gUU[j][l] * Abar[k][l];
      H -= Abar[i][j] * auu;
    }
  R cfd[3], phid[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    cfd[i] = D1<ORDER, R>(P, CF, i, inv);
    phid[i] = -cfd[i] / (2.0 * cf);
  }
  R Rtr = 0.0, pp = 0.0, pdd = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Rtr += m.gUU[i][j] * Rbar[S6(i, j)];
      pp += m.gUU[i][j] * phid[i] * phid[j];
      R v = (-D2<ORDER, R>(P, CF, i, j, inv) + cfd[i] * cfd[j] / cf) / (2.0 * cf);
#pragma unroll
      for (int k = 0; k < 3; k++) v -= m.Gbar[k][i][j] * phid[k];
      pdd += m.gUU[i][j] * v;
    }
  H += cf * cf * (Rtr - 8.0 * (pp + pdd));
  aux[idx] = H;
}

// ------------------------------------------------- Brill-Lindquist data
// Forward-mode dual numbers over (xx0, xx1, xx2): the initial Lambdabar^i
// needs exact first derivatives of gammabar_ij (BSSN_in_terms_of_ADM.py:78-117).
struct Dual {
  double v, d[3];
};
__device__ __forceinline__ Dual dconst(double c) { return Dual{c, {0.0, 0.0, 0.0}}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) {
  return Dual{a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}};
}
__device__ __forceinline__ Dual operator-(Dual a, Dual b) {
  return Dual{a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}};
}
__device__ __forceinline__ Dual operator-(Dual a) { return Dual{-a.v, {-a.d[0], -a.d[1], -a.d[2]}}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
  Dual r;
  r.v = a.v * b.v;
  for (int k = 0; k < 3; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
__device__ __forceinline__ Dual operator*(double c, Dual a) { return Dual{c * a.v, {c * a.d[0], c * a.d[1], c * a.d[2]}}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  Dual r;
  r.v = a.v / b.v;
  for (int k = 0; k < 3; k++) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
__device__ __forceinline__ Dual chain(Dual a, double f, double df) {
  return Dual{f, {df * a.d[0], df * a.d[1], df * a.d[2]}};
}
__device__ __forceinline__ Dual dexp(Dual a) { const double e = exp(a.v); return chain(a, e, e); }
__device__ __forceinline__ Dual dsin(Dual a) { return chain(a, sin(a.v), cos(a.v)); }
__device__ __forceinline__ Dual dcos(Dual a) { return chain(a, cos(a.v), -sin(a.v)); }
__device__ __forceinline__ Dual dsqrt(Dual a) { const double s = sqrt(a.v); return chain(a, s, 0.5 / s); }
__device__ __forceinline__ Dual dcbrt(Dual a) {
  const double c = cbrt(a.v);
  return chain(a, c, c / (3.0 * a.v));
}

struct BLParams {
  double m1, x1[3], m2, x2[3];
};

template <int CS>
__global__ void bl_id_kernel(paramstruct p, BLParams bl, double *__restrict__ gfs) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  const int n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1, n2 = p.Nxx_plus_2NGHOSTS2;
  if (i0 >= n0) return;
  const long long ntot = (long long)n0 * n1 * n2;
  const long long idx = (long long)i0 + (long long)n0 * ((long long)i1 + (long long)n1 * i2);
  const Dual X0{xx_of(p.xxmin0, p.dxx0, i0, p.NGHOSTS), {1.0, 0.0, 0.0}};
  const Dual X1{xx_of(p.xxmin1, p.dxx1, i1, p.NGHOSTS), {0.0, 1.0, 0.0}};
  const Dual X2{xx_of(p.xxmin2, p.dxx2, i2, p.NGHOSTS), {0.0, 0.0, 1.0}};
  Dual xc[3], J[3][3], s[3];
  // sinh map A sinh(x/w)/sinh(1/w) (+ A c x) as a dual number, and its derivative
  auto dsinh_map = [](double A, double w, double c, const Dual &x, Dual &f, Dual &df) {
    const double den = exp(1.0 / w) - exp(-1.0 / w);
    const Dual ep = dexp((1.0 / w) * x), em = dexp((-1.0 / w) * x);
    f = (A / den) * (ep - em) + (A * c) * x;
    df = (A / (w * den)) * (ep + em) + dconst(A * c);
  };
  if (CS == NRGPU_COORD_CARTESIAN) {
    xc[0] = X0; xc[1] = X1; xc[2] = X2;
    for (int a = 0; a < 3; a++) {
      s[a] = dconst(1.0);
      for (int b = 0; b < 3; b++) J[a][b] = dconst(a == b ? 1.0 : 0.0);
    }
  } else if (symtp_family(p.CoordSystem)) {
    // (AA sin xx1 cos xx2, AA sin xx1 sin xx2, var2 cos xx1) (reference_metric.py:334-336)
    Dual A = X0, dA = dconst(1.0);
    if (p.CoordSystem == NRGPU_COORD_SINHSYMTP) dsinh_map(p.AMAX, p.SINHWAA, 0.0, X0, A, dA);
    const Dual st = dsin(X1), ct = dcos(X1), sp = dsin(X2), cp = dcos(X2);
    const Dual b2 = dconst(p.bScale * p.bScale);
    const Dual v1 = dsqrt(A * A + b2 * st * st), v2 = dsqrt(A * A + b2);
    const Dual dv2 = (A * dA) / v2;
    xc[0] = A * st * cp; xc[1] = A * st * sp; xc[2] = v2 * ct;
    J[0][0] = dA * st * cp; J[0][1] = A * ct * cp; J[0][2] = -(A * st * sp);
    J[1][0] = dA * st * sp; J[1][1] = A * ct * sp; J[1][2] = A * st * cp;
    J[2][0] = dv2 * ct;     J[2][1] = -(v2 * st);  J[2][2] = dconst(0.0);
    s[0] = dA * v1 / v2; s[1] = v1; s[2] = A * st;
  } else if (cylindrical_family(p.CoordSystem)) {
    // (rho cos phi, rho sin phi, z) (reference_metric.py:296-298)
    Dual rho = X0, drho = dconst(1.0), z = X2, dz = dconst(1.0);
    if (p.CoordSystem != NRGPU_COORD_CYLINDRICAL) {
      const bool v2 = p.CoordSystem == NRGPU_COORD_SINHCYLINDRICALV2;
      dsinh_map(p.AMPLRHO, p.SINHWRHO, v2 ? p.const_drho : 0.0, X0, rho, drho);
      dsinh_map(p.AMPLZ, p.SINHWZ, v2 ? p.const_dz : 0.0, X2, z, dz);
    }
    const Dual sp = dsin(X1), cp = dcos(X1);
    xc[0] = rho * cp; xc[1] = rho * sp; xc[2] = z;
    J[0][0] = drho * cp; J[0][1] = -(rho * sp); J[0][2] = dconst(0.0);
    J[1][0] = drho * sp; J[1][1] = rho * cp;    J[1][2] = dconst(0.0);
    J[2][0] = dconst(0.0); J[2][1] = dconst(0.0); J[2][2] = dz;
    s[0] = drho; s[1] = rho; s[2] = dz;
  } else {
    Dual r = X0, dr = dconst(1.0);
    if (p.CoordSystem == NRGPU_COORD_SINHSPHERICAL || p.CoordSystem == NRGPU_COORD_SINHSPHERICALV2)
      dsinh_map(p.AMPL, p.SINHW, p.CoordSystem == NRGPU_COORD_SINHSPHERICALV2 ? p.const_dr : 0.0, X0, r, dr);
    const Dual st = dsin(X1), ct = dcos(X1), sp = dsin(X2), cp = dcos(X2);
    xc[0] = r * st * cp; xc[1] = r * st * sp; xc[2] = r * ct;
    J[0][0] = dr * st * cp; J[0][1] = r * ct * cp; J[0][2] = -(r * st * sp);
    J[1][0] = dr * st * sp; J[1][1] = r * ct * sp; J[1][2] = r * st * cp;
    J[2][0] = dr * ct;      J[2][1] = -(r * st);   J[2][2] = dconst(0.0);
    s[0] = dr; s[1] = r; s[2] = r * st;
  }
  // psi = 1 + sum m/(2|x - x_BH|) (BrillLindquist.py:58-61)
  Dual psi = dconst(1.0);
  {
    Dual dx = xc[0] - dconst(bl.x1[0]), dy = xc[1] - dconst(bl.x1[1]), dz = xc[2] - dconst(bl.x1[2]);
    psi = psi + dconst(bl.m1) / (2.0 * dsqrt(dx * dx + dy * dy + dz * dz));
    dx = xc[0] - dconst(bl.x2[0]); dy = xc[1] - dconst(bl.x2[1]); dz = xc[2] - dconst(bl.x2[2]);
    psi = psi + dconst(bl.m2) / (2.0 * dsqrt(dx * dx + dy * dy + dz * dz));
  }
  const Dual psi2 = psi * psi, psi4 = psi2 * psi2;
  // gamma_ij in the grid basis: psi^4 J^k_i J^k_j
  Dual gam[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++) {
      Dual acc = dconst(0.0);
      for (int k = 0; k < 3; k++) acc = acc + J[k][i] * J[k][j];
      gam[i][j] = gam[j][i] = psi4 * acc;
    }
  auto det3 = [](Dual a[3][3]) {
    return -(a[0][2] * a[0][2] * a[1][1]) + 2.0 * (a[0][1] * a[0][2] * a[1][2]) - a[0][0] * a[1][2] * a[1][2] -
           a[0][1] * a[0][1] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
  };
  const Dual detgam = det3(gam);
  const Dual detghat = (s[0] * s[0]) * (s[1] * s[1]) * (s[2] * s[2]);
  const Dual fac = dcbrt(detghat / detgam);
  Dual gb[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) gb[i][j] = fac * gam[i][j];
  const Dual detgb = det3(gb);
  // inverse of gammabar (values) and of ghat
  double g[3][3], gUU[3][3], dtmp;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) g[i][j] = gb[i][j].v;
  sym_inverse<double>(g, gUU, dtmp);
  double out[NUM_EVOL_GFS];
  for (int k = 0; k < NUM_EVOL_GFS; k++) out[k] = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++) {
      const double ghat = (i == j) ? s[i].v * s[i].v : 0.0;
      out[HDD00 + S6(i, j)] = (gb[i][j].v - ghat) / (s[i].v * s[j].v);
    }
  // W = (gamma / gammabar)^(-1/6)  (BSSN_in_terms_of_ADM.py:141-144)
  out[CF] = pow(detgam.v / detgb.v, -1.0 / 6.0);
  out[ALPHA] = 1.0 / psi2.v;
  // Lambdabar^i = gammabar^jk (Gammabar^i_jk - Gammahat^i_jk), lambda^i = Lambdabar^i s_i
  for (int i = 0; i < 3; i++) {
    double Lb = 0.0;
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) {
        double Gb = 0.0;
        for (int l = 0; l < 3; l++)
          Gb += 0.5 * gUU[i][l] * (gb[l][j].d[k] + gb[l][k].d[j] - gb[j][k].d[l]);
        // diagonal ghat: Gammahat^i_jk = (d_k g_ij + d_j g_ik - d_i g_jk)/(2 g_ii)
        const double gii = s[i].v * s[i].v;
        auto dg = [&](int a, int b, int c) { return a == b ? 2.0 * s[a].v * s[a].d[c] : 0.0; };
        const double Gh = (dg(i, j, k) + dg(i, k, j) - dg(j, k, i)) / (2.0 * gii);
        Lb += gUU[j][k] * (Gb - Gh);
      }
    out[LAMBDAU0 + i] = Lb * s[i].v;
  }
  for (int k = 0; k < NUM_EVOL_GFS; k++) gfs[(long long)k * ntot + idx] = out[k];
}

// Matter terms of the constraints (BSSN_stress_energy_source_terms.py:134-161,
// BSSN_source_terms_for_BSSN_constraints): H += -16 pi rho, M^i += -8 pi S^i / ReU^i
// with rho = alpha^2 T^{00}, S_i = alpha gamma4_{i mu} T^{mu 0}, S^i = gamma^ij S_j.
template <int CS>
__global__ void constraint_sources_kernel(Grid g, const double *__restrict__ in, const double *__restrict__ tab,
                                          const double *__restrict__ T4, double *__restrict__ H,
                                          double *__restrict__ MU) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  using M = RfmMask<CS>;
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
  const double pi = 3.14159265358979323846;
  const double alpha = __ldg(P.gf(ALPHA)), cf = __ldg(P.gf(CF));
  const double T00 = __ldg(T4 + idx);
  if (H) H[idx] += -16.0 * pi * alpha * alpha * T00;
  if (!MU) return;
  double gbar[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++) {
      const double h = __ldg(P.gf(HDD00 + S6(i, j)));
      gbar[i][j] = gbar[j][i] = (M::trivial ? h : h * rf.ReDD(i, j)) + (i == j ? rf.ghatDD(i) : 0.0);
    }
  double gbUU[3][3], det;
  sym_inverse(gbar, gbUU, det);
  const double e4 = 1.0 / (cf * cf);
  double beta[3], T0[4];
  for (int j = 0; j < 3; j++) {
    const double vet = __ldg(P.gf(VETU0 + j));
    beta[j] = M::trivial ? vet : vet * rf.ReU(j);
  }
  for (int m = 0; m < 4; m++) T0[m] = __ldg(T4 + (long long)m * g.ntot + idx);  // T4UU00, 01, 02, 03
  double SD[3];
  for (int i = 0; i < 3; i++) {
    double bD = 0.0, s = 0.0;
    for (int j = 0; j < 3; j++) {
      bD += e4 * gbar[i][j] * beta[j];
      s += e4 * gbar[i][j] * T0[j + 1];
    }
    SD[i] = alpha * (bD * T0[0] + s);
  }
  for (int i = 0; i < 3; i++) {
    const double SU = cf * cf * (gbUU[i][0] * SD[0] + gbUU[i][1] * SD[1] + gbUU[i][2] * SD[2]);
    MU[(long long)i * g.ntot + idx] += -8.0 * pi * (M::trivial ? SU : SU / rf.ReU(i));
  }
}

}  // namespace bssn

using namespace bssn;

#define RICCI_CALL(CS, ORD) ricci_launch_t<CS, ORD>(rfm, p, in, in_is_f64, prec, auxevol)
#define STAGED_RICCI_CALL(CS, ORD) staged_ricci_launch_t<CS, ORD>(rfm, p, in, in_is_f64, prec, auxevol)
static int staged_ricci(const rfm_struct *rfm, const paramstruct *p, const void *in, bool in_is_f64, int prec,
                        void *auxevol) {
  NRGPU_BSSN_SWITCH(STAGED_RICCI_CALL)
}
int bssn_ricci_launch(const rfm_struct *rfm, const paramstruct *p, const void *in, bool in_is_f64, int prec,
                      void *auxevol) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(in && auxevol, "NULL gridfunctions");
  if (staged_for(p, prec)) {
    st = staged_ricci(rfm, p, in, in_is_f64, prec, auxevol);
    if (st != NRGPU_ERR_UNSUPPORTED) return st;
  }
  NRGPU_BSSN_SWITCH(RICCI_CALL)
}
static bool extras_on(const paramstruct *p) {
  return p->diss_strength != 0.0 || p->enable_stress_energy_source_terms;
}
#define RHS_CALL(CS, ORD) \
  (extras_on(p) ? rhs_launch_t<CS, ORD, true>(rfm, p, a) : rhs_launch_t<CS, ORD, false>(rfm, p, a))
#define STAGED_RHS_CALL(CS, ORD) staged_rhs_launch_t<CS, ORD>(rfm, p, a, fused)
static int staged_rhs(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a, bool fused) {
  NRGPU_BSSN_SWITCH(STAGED_RHS_CALL)
}
int bssn_rhs_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(a.in && a.auxevol, "NULL gridfunctions");
  // Kreiss-Oliger dissipation and T^{mu nu} sources run on the point kernels.
  if (staged_for(p, a.prec) && !extras_on(p)) {
    st = staged_rhs(rfm, p, a, false);
    if (st != NRGPU_ERR_UNSUPPORTED) return st;
  }
  NRGPU_BSSN_SWITCH(RHS_CALL)
}
// The staged and fused kernels run 8 warps per SM, too few to hide the
// latency of the epilogue's y_n and running-total loads: on SinhSpherical
// 128x64x16 (compensated) the RK update costs ~60 us of the fused kernel's
// ~210 us, while storing k (the kernel then takes 142 us) and updating in a
// separate high-occupancy kernel (29 us) takes the step from 0.97 to
// 0.82 ms (graph replay; mixed: 0.82 to 0.72 ms).  With the update in FP64
// arithmetic (COMPENSATED_FP64RK) the separate kernel is FP64-pipe bound
// (70 us a substep) and the split gains less: 1.12 to 1.10 ms.  The point
// kernels gain with plain FP32 stages (128^3 Cartesian FD4 mixed: 6.10 ms
// fused, 5.69 with a separate all-points update) and lose with pairs
// (compensated: 8.62 vs 8.79 ms), so there they keep their epilogue.
// Kreiss-Oliger and source-term runs keep the fused epilogue (not measured
// split).
int bssn_kernels_mode() { return g_kernels; }

bool bssn_split_update(const paramstruct *p, int prec) {
  if (extras_on(p)) return false;
  if (prec == NRGPU_PREC_MIXED) return true;
  return (prec == NRGPU_PREC_COMPENSATED || prec == NRGPU_PREC_COMPENSATED_FP64RK) && staged_for(p, prec);
}

// One MoL substep's Ricci + RHS: the fused staged kernel when selected,
// else Ricci_eval then rhs_eval.
int bssn_stage_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(a.in && a.auxevol, "NULL gridfunctions");
  if (family(p, a.prec) == NRGPU_BSSN_KERNELS_FUSED && !extras_on(p)) {
    st = staged_rhs(rfm, p, a, true);
    if (st != NRGPU_ERR_UNSUPPORTED) return st;
  }
  st = bssn_ricci_launch(rfm, p, a.in, a.in_is_f64, a.prec, a.auxevol);
  if (st) return st;
  return bssn_rhs_launch(rfm, p, a);
}

int bssn_enforce_launch(const rfm_struct *rfm, const paramstruct *p, void *gfs, bool is_f64, bool pair, bool ff_f64,
                        bool f64_pair) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(gfs != nullptr, "NULL gridfunctions");
  Grid g = make_grid(p);
  dim3 block(64), grid((g.n0 + 63) / 64, g.n1, g.n2);
  if ((!is_f64 || ff_f64) && !(pair && f64_pair)) {  // FP32 storage (or the FP32-stage steps' FP64 state): float-float rescale
    const dim3 fb(256), fg((unsigned)((g.ntot + 255) / 256));
    if (is_f64) enforce_ff_kernel<double><<<fg, fb, 0, stream()>>>(g, (double *)gfs);
    else if (pair) enforce_ff_kernel<float2><<<fg, fb, 0, stream()>>>(g, (float2 *)gfs);
    else enforce_ff_kernel<float><<<fg, fb, 0, stream()>>>(g, (float *)gfs);
    NRGPU_LAUNCH_CHECK();
    return NRGPU_OK;
  }
  const double *tab = rfm ? rfm->table64 : nullptr;
  const bool cart = p->CoordSystem == NRGPU_COORD_CARTESIAN;
#define ENF(T)                                                                                           \
  if (cart) enforce_kernel<NRGPU_COORD_CARTESIAN, T><<<grid, block, 0, stream()>>>(g, tab, (T *)gfs);     \
  else if (p->CoordSystem == NRGPU_COORD_SPHERICAL)                                                      \
    enforce_kernel<NRGPU_COORD_SPHERICAL, T><<<grid, block, 0, stream()>>>(g, tab, (T *)gfs);            \
  else if (cylindrical_family(p->CoordSystem))                                                            \
    enforce_kernel<NRGPU_COORD_SINHCYLINDRICAL, T><<<grid, block, 0, stream()>>>(g, tab, (T *)gfs);      \
  else if (symtp_family(p->CoordSystem))                                                                  \
    enforce_kernel<NRGPU_COORD_SINHSYMTP, T><<<grid, block, 0, stream()>>>(g, tab, (T *)gfs);            \
  else enforce_kernel<NRGPU_COORD_SINHSPHERICAL, T><<<grid, block, 0, stream()>>>(g, tab, (T *)gfs);
  if (pair) {  // pair stage buffers, FP64 arithmetic (COMPENSATED_FP64RK)
    ENF(float2)
  } else {
    ENF(double)
  }
#undef ENF
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

}  // namespace nrgpu

using namespace nrgpu;

static int bssn_plain(const rfm_struct *rfm, const paramstruct *p, const void *aux, const void *in, void *rhs,
                      int prec) {
  NRGPU_REQUIRE(p && aux && in && rhs, "NULL argument");
  StageArgs a{};
  a.stage = -1;
  a.prec = prec;
  a.in = in;
  a.in_is_f64 = (prec == NRGPU_PREC_FP64);
  a.out = rhs;
  a.auxevol = (void *)aux;
  return bssn_rhs_launch(rfm, p, a);
}

extern "C" {
int nrgpu_set_bssn_kernels(int mode) {
  NRGPU_REQUIRE(mode >= NRGPU_BSSN_KERNELS_AUTO && mode <= NRGPU_BSSN_KERNELS_FUSED, "unknown BSSN kernel mode %d",
                mode);
  g_kernels = mode;
  return NRGPU_OK;
}
int nrgpu_get_bssn_kernels(void) { return g_kernels; }
int BSSN_Ricci_eval(const rfm_struct *rfm, const paramstruct *p, const double *in, double *aux) {
  return bssn_ricci_launch(rfm, p, in, true, NRGPU_PREC_FP64, aux);
}
int BSSN_Ricci_eval_f32(const rfm_struct *rfm, const paramstruct *p, const float *in, float *aux) {
  return bssn_ricci_launch(rfm, p, in, false, NRGPU_PREC_MIXED, aux);
}
int BSSN_rhs_eval(const rfm_struct *rfm, const paramstruct *p, const double *aux, const double *in, double *rhs) {
  return bssn_plain(rfm, p, aux, in, rhs, NRGPU_PREC_FP64);
}
int BSSN_rhs_eval_f32(const rfm_struct *rfm, const paramstruct *p, const float *aux, const float *in, float *rhs) {
  return bssn_plain(rfm, p, aux, in, rhs, NRGPU_PREC_MIXED);
}
int BSSN_enforce_detgammabar_constraint(const rfm_struct *rfm, const paramstruct *p, double *gfs) {
  return bssn_enforce_launch(rfm, p, gfs, true);
}
int BSSN_enforce_detgammabar_constraint_f32(const rfm_struct *rfm, const paramstruct *p, float *gfs) {
  return bssn_enforce_launch(rfm, p, gfs, false);
}
int BSSN_Hamiltonian_constraint(const rfm_struct *rfm, const paramstruct *p, const double *in, double *aux) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(in && aux, "NULL argument");
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  const double *tab = rfm ? rfm->table64 : nullptr;
  switch (dispatch_cs(p->CoordSystem) * 16 + p->FD_order) {
    case NRGPU_COORD_CARTESIAN * 16 + 2:
      hamiltonian_kernel<NRGPU_COORD_CARTESIAN, 2><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_CARTESIAN * 16 + 4:
      hamiltonian_kernel<NRGPU_COORD_CARTESIAN, 4><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_CARTESIAN * 16 + 6:
      hamiltonian_kernel<NRGPU_COORD_CARTESIAN, 6><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_CARTESIAN * 16 + 8:
      hamiltonian_kernel<NRGPU_COORD_CARTESIAN, 8><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_SINHSPHERICAL * 16 + 4:
      hamiltonian_kernel<NRGPU_COORD_SINHSPHERICAL, 4><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_SINHCYLINDRICAL * 16 + 4:
      hamiltonian_kernel<NRGPU_COORD_SINHCYLINDRICAL, 4><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_SINHSYMTP * 16 + 4:
      hamiltonian_kernel<NRGPU_COORD_SINHSYMTP, 4><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    case NRGPU_COORD_SPHERICAL * 16 + 4:
      hamiltonian_kernel<NRGPU_COORD_SPHERICAL, 4><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux); break;
    default:
      set_error("Hamiltonian: CoordSystem %d FD_order %d not built", p->CoordSystem, p->FD_order);
      return NRGPU_ERR_UNSUPPORTED;
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
int BSSN_Ricci_eval_xx(const paramstruct *p, double *xx[3], const double *in, double *aux) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(xx && xx[0] && xx[1] && xx[2] && in && aux, "NULL argument");
  NRGPU_REQUIRE(p->NGHOSTS >= p->FD_order / 2 + 1, "BSSN needs NGHOSTS >= FD_order/2 + 1");
  const XXArgs xa{xx[0], xx[1], xx[2], coord_params(*p)};
#define RXX(CS, ORD) ricci_xx_launch_t<CS, ORD>(p, xa, in, aux)
  NRGPU_BSSN_SWITCH(RXX)
#undef RXX
}

int BSSN_rhs_eval_xx(const paramstruct *p, double *xx[3], const double *aux, const double *in, double *rhs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(xx && xx[0] && xx[1] && xx[2] && aux && in && rhs, "NULL argument");
  NRGPU_REQUIRE(p->NGHOSTS >= p->FD_order / 2 + 1, "BSSN needs NGHOSTS >= FD_order/2 + 1");
  const XXArgs xa{xx[0], xx[1], xx[2], coord_params(*p)};
#define HXX(CS, ORD)                                                                 \
  (extras_on(p) ? rhs_xx_launch_t<CS, ORD, true>(p, xa, aux, in, rhs) \
                : rhs_xx_launch_t<CS, ORD, false>(p, xa, aux, in, rhs))
  NRGPU_BSSN_SWITCH(HXX)
#undef HXX
}

int BSSN_momentum_constraint(const rfm_struct *rfm, const paramstruct *p, const double *in, double *aux) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(in && aux, "NULL argument");
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  const double *tab = rfm ? rfm->table64 : nullptr;
#define MOM(CS, ORD) momentum_kernel<CS, ORD><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux)
  switch (dispatch_cs(p->CoordSystem) * 16 + p->FD_order) {
    case NRGPU_COORD_CARTESIAN * 16 + 2: MOM(NRGPU_COORD_CARTESIAN, 2); break;
    case NRGPU_COORD_CARTESIAN * 16 + 4: MOM(NRGPU_COORD_CARTESIAN, 4); break;
    case NRGPU_COORD_CARTESIAN * 16 + 6: MOM(NRGPU_COORD_CARTESIAN, 6); break;
    case NRGPU_COORD_CARTESIAN * 16 + 8: MOM(NRGPU_COORD_CARTESIAN, 8); break;
    case NRGPU_COORD_SINHSPHERICAL * 16 + 4: MOM(NRGPU_COORD_SINHSPHERICAL, 4); break;
    case NRGPU_COORD_SINHCYLINDRICAL * 16 + 4: MOM(NRGPU_COORD_SINHCYLINDRICAL, 4); break;
    case NRGPU_COORD_SINHSYMTP * 16 + 4: MOM(NRGPU_COORD_SINHSYMTP, 4); break;
    case NRGPU_COORD_SPHERICAL * 16 + 4: MOM(NRGPU_COORD_SPHERICAL, 4); break;
    default:
      set_error("momentum constraint: CoordSystem %d FD_order %d not built", p->CoordSystem, p->FD_order);
      return NRGPU_ERR_UNSUPPORTED;
  }
#undef MOM
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
int BSSN_constraints_add_source_terms(const rfm_struct *rfm, const paramstruct *p, const double *in,
                                      const double *T4UU, double *H, double *MU) {
  int st = check_bssn(rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(in && T4UU && (H || MU), "NULL argument");
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  const double *tab = rfm ? rfm->table64 : nullptr;
  switch (p->CoordSystem) {
    case NRGPU_COORD_CARTESIAN:
      constraint_sources_kernel<NRGPU_COORD_CARTESIAN><<<L.grid, L.block, 0, stream()>>>(g, in, tab, T4UU, H, MU);
      break;
    case NRGPU_COORD_SPHERICAL:
      constraint_sources_kernel<NRGPU_COORD_SPHERICAL><<<L.grid, L.block, 0, stream()>>>(g, in, tab, T4UU, H, MU);
      break;
    case NRGPU_COORD_CYLINDRICAL:
    case NRGPU_COORD_SINHCYLINDRICAL:
    case NRGPU_COORD_SINHCYLINDRICALV2:
      constraint_sources_kernel<NRGPU_COORD_SINHCYLINDRICAL><<<L.grid, L.block, 0, stream()>>>(g, in, tab, T4UU,
                                                                                              H, MU);
      break;
    case NRGPU_COORD_SYMTP:
    case NRGPU_COORD_SINHSYMTP:
      constraint_sources_kernel<NRGPU_COORD_SINHSYMTP><<<L.grid, L.block, 0, stream()>>>(g, in, tab, T4UU, H, MU);
      break;
    default:
      constraint_sources_kernel<NRGPU_COORD_SINHSPHERICAL><<<L.grid, L.block, 0, stream()>>>(g, in, tab, T4UU, H,
                                                                                              MU);
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
int BSSN_initial_data_BrillLindquist(const paramstruct *p, double m1, const double x1[3], double m2,
                                     const double x2[3], double *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(x1 && x2 && gfs, "NULL argument");
  BLParams bl{m1, {x1[0], x1[1], x1[2]}, m2, {x2[0], x2[1], x2[2]}};
  dim3 block(64), grid((p->Nxx_plus_2NGHOSTS0 + 63) / 64, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2);
  if (p->CoordSystem == NRGPU_COORD_CARTESIAN)
    bl_id_kernel<NRGPU_COORD_CARTESIAN><<<grid, block, 0, stream()>>>(*p, bl, gfs);
  else if (p->CoordSystem == NRGPU_COORD_SPHERICAL)
    bl_id_kernel<NRGPU_COORD_SPHERICAL><<<grid, block, 0, stream()>>>(*p, bl, gfs);
  else
    bl_id_kernel<NRGPU_COORD_SINHSPHERICAL><<<grid, block, 0, stream()>>>(*p, bl, gfs);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
}
