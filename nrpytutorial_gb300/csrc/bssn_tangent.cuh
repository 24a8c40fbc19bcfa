// bssn_tangent.cuh -- forward-mode (tangent-linear) BSSN: the FP64 RHS of a
// state together with the RHS's derivative along N tangent states.
//
// The BSSN evolution is nonlinear, so the derivative of an observable with
// respect to initial-data parameters (Brill-Lindquist masses and positions)
// needs the Jacobian of the whole discrete evolution.  With few parameters,
// forward mode is the direct route: the state y and N tangent states
// t_k = dy/dp_k evolve together, t_k by the linearisation of every step.
// The algebra of bssn.cuh is generic in its arithmetic type and uses only
// + - * / on it, so instantiating it with DualN<N> (dualn.cuh) gives, in
// one pass per point, the RHS value and its N directional derivatives
// exactly (no finite-difference error); the finite-difference stencils are
// linear, so a tangent's derivative is the stencil of the tangent.
//
// Layout: a "tangent state" is (N+1) consecutive IDX4S state arrays -- the
// value, then t_1..t_N -- at component stride ts (24 * Nxx_plus_2NGHOSTS_tot
// for the evolved gridfunctions, 6 * ... for RbarDD).
#pragma once
#include "bssn.cuh"
#include "dualn.cuh"
#include "epilogue.cuh"
#include "systems.cuh"

namespace nrgpu {
namespace bssn {
namespace tangent {

// ----------------------------------------------------------- input access
// Stage-input tag of a tangent state with N tangents, and its pointer: the
// value at p, tangent k at p + (k+1) ts.
template <int N> struct DualTag {};
template <int N> struct DualPtr {
  const double *p;
  long long ts;
  __device__ __forceinline__ DualPtr operator+(long long o) const { return DualPtr{p + o, ts}; }
};

// Value and stencils of a tangent state: the plain FP64 stencil of the
// value and of each tangent array (found by argument-dependent lookup from
// the generic accessors of bssn.cuh).
template <typename R, int N> __device__ __forceinline__ R val(DualPtr<N> q) {
  R r(__ldg(q.p));
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = __ldg(q.p + (k + 1) * q.ts);
  return r;
}
template <int ORDER, typename R, int N>
__device__ __forceinline__ R fd_d1(DualPtr<N> q, long long s) {
  R r(nrgpu::fd_d1<ORDER, double>(q.p, s));
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = nrgpu::fd_d1<ORDER, double>(q.p + (k + 1) * q.ts, s);
  return r;
}
template <int ORDER, typename R, int N>
__device__ __forceinline__ R fd_d2(DualPtr<N> q, long long s) {
  R r(nrgpu::fd_d2<ORDER, double>(q.p, s));
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = nrgpu::fd_d2<ORDER, double>(q.p + (k + 1) * q.ts, s);
  return r;
}
template <int ORDER, typename R, int N>
__device__ __forceinline__ R fd_d11(DualPtr<N> q, long long s, long long t) {
  R r(nrgpu::fd_d11<ORDER, double>(q.p, s, t));
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = nrgpu::fd_d11<ORDER, double>(q.p + (k + 1) * q.ts, s, t);
  return r;
}
// The upwind direction follows the value of the shift (UPWIND_ALG), the
// same stencil for the tangents.
template <int ORDER, typename R, int N>
__device__ __forceinline__ R fd_dupwind(DualPtr<N> q, long long s, bool positive) {
  R r(nrgpu::fd_dupwind<ORDER, double>(q.p, s, positive));
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = nrgpu::fd_dupwind<ORDER, double>(q.p + (k + 1) * q.ts, s, positive);
  return r;
}


}  // namespace tangent
}  // namespace bssn

template <int N> struct InRef<bssn::tangent::DualTag<N>> {
  using type = bssn::tangent::DualPtr<N>;
};

// The reference metric is parameter-independent: its DualN accessor wraps
// the FP64 table and returns constants.
template <int CS, int N> struct Rfm<CS, DualN<N>, RFM_TABLE> {
  using M = RfmMask<CS>;
  using D = DualN<N>;
  Rfm<CS, double, RFM_TABLE> t;
  __device__ __forceinline__ D ReU(int i) const { return D(t.ReU(i)); }
  __device__ __forceinline__ D ReUdD(int i, int j) const { return D(t.ReUdD(i, j)); }
  __device__ __forceinline__ D ReUdDD(int i, int j, int k) const { return D(t.ReUdDD(i, j, k)); }
  __device__ __forceinline__ D ReDD(int i, int j) const { return D(t.ReDD(i, j)); }
  __device__ __forceinline__ D ReDDdD(int i, int j, int k) const { return D(t.ReDDdD(i, j, k)); }
  __device__ __forceinline__ D ReDDdDD(int i, int j, int k, int l) const { return D(t.ReDDdDD(i, j, k, l)); }
  __device__ __forceinline__ D ghatDD(int i) const { return D(t.ghatDD(i)); }
  __device__ __forceinline__ D ghatUU(int i) const { return D(t.ghatUU(i)); }
  __device__ __forceinline__ D ghatDDdD(int i, int j, int k) const { return D(t.ghatDDdD(i, j, k)); }
  __device__ __forceinline__ D ghatDDdDD(int i, int j, int k, int l) const { return D(t.ghatDDdDD(i, j, k, l)); }
  __device__ __forceinline__ D G(int i, int k, int l) const { return D(t.G(i, k, l)); }
  __device__ __forceinline__ D GdD(int i, int k, int l, int n) const { return D(t.GdD(i, k, l, n)); }
  __device__ __forceinline__ D detg() const { return D(t.detg()); }
  __device__ __forceinline__ D detgdD(int k) const { return D(t.detgdD(k)); }
  __device__ __forceinline__ D detgdDD(int k, int l) const { return D(t.detgdDD(k, l)); }
};

namespace bssn {
namespace tangent {

// Arithmetic type, stage-input tag and reference-metric accessor for N
// tangents (N = 0: plain FP64).
template <int N> struct Types {
  using R = DualN<N>;
  using Tin = DualTag<N>;
  static __device__ __forceinline__ typename InRef<Tin>::type in(const double *p, long long ts) {
    return DualPtr<N>{p, ts};
  }
  template <int CS> static __device__ __forceinline__ Rfm<CS, R> rfm(const Rfm<CS, double> &t) {
    return Rfm<CS, R>{t};
  }
  static __device__ __forceinline__ R load(const double *p, long long ts) {
    R r(__ldg(p));
#pragma unroll
    for (int k = 0; k < N; k++) r.d[k] = __ldg(p + (k + 1) * ts);
    return r;
  }
  static __device__ __forceinline__ void store(double *p, long long ts, const R &v) {
    p[0] = v.v;
#pragma unroll
    for (int k = 0; k < N; k++) p[(k + 1) * ts] = v.d[k];
  }
};
template <> struct Types<0> {
  using R = double;
  using Tin = double;
  static __device__ __forceinline__ const double *in(const double *p, long long) { return p; }
  template <int CS> static __device__ __forceinline__ Rfm<CS, double> rfm(const Rfm<CS, double> &t) { return t; }
  static __device__ __forceinline__ double load(const double *p, long long) { return __ldg(p); }
  static __device__ __forceinline__ void store(double *p, long long, double v) { p[0] = v; }
};

// Both kernels declare a minimum of one block per SM: without it ptxas keeps
// the dual-number kernels at 32 registers and spills their whole state
// (38 KB of stack per thread for 4 tangents, against 12 KB at 255 registers).

// RbarDD (value and tangents) at interior points: aux at stride ats.
template <int CS, int ORDER, int N>
__global__ void __launch_bounds__(128, 1) ricci_kernel(Grid g, const double *__restrict__ in, long long ts,
                                                    const double *__restrict__ tab, double *__restrict__ aux,
                                                    long long ats) {
  using TY = Types<N>;
  using R = typename TY::R;
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  Point<typename TY::Tin> P{TY::in(in, ts) + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const R inv[3] = {R(g.invdx0), R(g.invdx1), R(g.invdx2)};
  const auto rf = TY::template rfm<CS>(rfm_at<CS, double>(tab, g, i0, i1, i2));
  Metric<CS, R> m;
  metric_point<ORDER, CS, R>(P, rf, inv, m);
  R Rbar[6];
  ricci_point<ORDER, CS, R>(P, rf, inv, m, Rbar);
#pragma unroll
  for (int k = 0; k < 6; k++) TY::store(aux + (long long)k * g.ntot + idx, ats, Rbar[k]);
}

// The 24 RHSs (value and tangents) at interior points into out (stride ts).
template <int CS, int ORDER, int N>
__global__ void __launch_bounds__(128, 1) rhs_kernel(Grid g, const double *__restrict__ in, long long ts,
                                                  const double *__restrict__ aux, long long ats,
                                                  const double *__restrict__ tab, double eta,
                                                  double *__restrict__ out) {
  using TY = Types<N>;
  using R = typename TY::R;
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  Point<typename TY::Tin> P{TY::in(in, ts) + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const R inv[3] = {R(g.invdx0), R(g.invdx1), R(g.invdx2)};
  const auto rf = TY::template rfm<CS>(rfm_at<CS, double>(tab, g, i0, i1, i2));
  R Rbar[6];
#pragma unroll
  for (int k = 0; k < 6; k++) Rbar[k] = TY::load(aux + (long long)k * g.ntot + idx, ats);
  R o[NUM_EVOL_GFS];
  rhs_point<ORDER, CS, R>(P, rf, inv, Rbar, R(eta), o);
#pragma unroll 1
  for (int gf = 0; gf < NUM_EVOL_GFS; gf++) TY::store(out + (long long)gf * g.ntot + idx, ts, o[gf]);
}

// Ricci then RHS of a tangent state (in, stride ts) into out (stride ts),
// RbarDD into aux (stride ats).
template <int CS, int ORDER, int N>
int rhs_launch(const rfm_struct *rfm, const Grid &g, const double *in, long long ts, double *aux, long long ats,
               double eta, double *out) {
  const double *tab = rfm ? rfm->table64 : nullptr;
  InteriorLaunch L = interior_launch(g, 32, 4);
  ricci_kernel<CS, ORDER, N><<<L.grid, L.block, 0, stream()>>>(g, in, ts, tab, aux, ats);
  NRGPU_LAUNCH_CHECK();
  rhs_kernel<CS, ORDER, N><<<L.grid, L.block, 0, stream()>>>(g, in, ts, aux, ats, tab, eta, out);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

#define NRGPU_TANGENT_DECLARE(CS, ORDER, N)                                                                   \
  extern template int rhs_launch<CS, ORDER, N>(const rfm_struct *, const Grid &, const double *, long long, \
                                               double *, long long, double, double *);
#define NRGPU_TANGENT_INSTANTIATE(CS, ORDER, N)                                                               \
  template int rhs_launch<CS, ORDER, N>(const rfm_struct *, const Grid &, const double *, long long, double *, \
                                        long long, double, double *);

}  // namespace tangent
}  // namespace bssn
}  // namespace nrgpu
