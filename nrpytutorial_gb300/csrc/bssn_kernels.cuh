// bssn_kernels.cuh -- BSSN Ricci / RHS kernels and their launchers,
// templated on coordinate system and FD order.  Each (CS, ORDER) pair is
// instantiated in its own translation unit (bssn_inst_*.cu) so the heavy
// kernels compile in parallel.
#pragma once
#include "bssn.cuh"
#include "epilogue.cuh"
#include "systems.cuh"

namespace nrgpu {
namespace bssn {

constexpr int kBlockX = 32, kBlockY = 4;
// Resident blocks per SM the compiler must allow (caps registers per thread):
// measured on GB300, the rhs kernel runs fastest at 4 blocks of 128 threads
// (128 registers, spilling to L1), the Ricci kernel at 1 (255 registers).
#ifndef NRGPU_BSSN_RICCI_MIN_BLOCKS
#define NRGPU_BSSN_RICCI_MIN_BLOCKS 1
#endif
#ifndef NRGPU_BSSN_RHS_MIN_BLOCKS
#define NRGPU_BSSN_RHS_MIN_BLOCKS 4
#endif

template <typename R, typename Tin, int CS, int ORDER, typename TAux>
__global__ void __launch_bounds__(kBlockX *kBlockY, NRGPU_BSSN_RICCI_MIN_BLOCKS)
    ricci_kernel(Grid g, typename InRef<Tin>::type in, const R *__restrict__ tab, TAux *__restrict__ aux) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  Point<Tin> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g.n0, g.n1, i0, i1);
  Metric<CS, R> m;
  metric_point<ORDER, CS, R>(P, rf, inv, m);
  R Rbar[6];
  ricci_point<ORDER, CS, R>(P, rf, inv, m, Rbar);
#pragma unroll
  for (int k = 0; k < 6; k++) aux[(long long)k * g.ntot + idx] = (TAux)Rbar[k];
}

// Kreiss-Oliger dissipation of gridfunction gf at the point:
// sum_k f_dKOD[k] ReU[k] (BaikalETK/BaikalETK_C_kernels_codegen.py:147-171).
template <int ORDER, int CS, typename R, typename Tin, bool LOC>
__device__ __forceinline__ R ko_point(const Point<Tin> &P, int gf, const Rfm<CS, R, LOC> &rf, const R *inv) {
  R acc = (R)0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const R d = fd_ko<ORDER, R>(P.gf(gf), P.st[k]) * inv[k];
    acc += RfmMask<CS>::trivial ? d : d * rf.ReU(k);
  }
  return acc;
}

// KO: add diss * ko_point to every RHS (diss_strength != 0); a separate
// instantiation, so the default kernel carries no dissipation code.
template <typename R, typename Tin, int CS, int ORDER, typename TStage, bool KO>
__global__ void __launch_bounds__(kBlockX *kBlockY, NRGPU_BSSN_RHS_MIN_BLOCKS)
    rhs_kernel(Grid g, typename InRef<Tin>::type in, const R *__restrict__ aux, const R *__restrict__ tab,
               R eta, R diss, RKEpilogue<TStage> epi) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  Point<Tin> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g.n0, g.n1, i0, i1);
  R Rbar[6];
#pragma unroll
  for (int k = 0; k < 6; k++) Rbar[k] = (R)__ldg(aux + (long long)k * g.ntot + idx);
  R out[NUM_EVOL_GFS];
  rhs_point<ORDER, CS, R>(P, rf, inv, Rbar, eta, out);
#pragma unroll
  for (int gf = 0; gf < NUM_EVOL_GFS; gf++) {
    R v = out[gf];
    if constexpr (KO) v += diss * ko_point<ORDER, CS, R>(P, gf, rf, inv);
    epi(gf, idx, v);
  }
}

// The same kernels with the reference metric evaluated at each point from the
// caller's coordinate arrays xx0[i0], xx1[i1] (FP64), as the reference's
// no-precompute rhs_eval(params, xx, auxevol_gfs, in_gfs, rhs_gfs) does.
struct XXArgs {
  const double *xx0, *xx1;
  double AMPL, SINHW;
};

template <int CS>
__device__ __forceinline__ void hatted_at_point(const XXArgs &xa, int i0, int i1, double *q) {
  if constexpr (CS != NRGPU_COORD_CARTESIAN) {
    ScaleFactors S;
    scale_factors(CS, xa.AMPL, xa.SINHW, xa.xx0[i0], xa.xx1[i1], &S);
    hatted_quantities(S, q);
  }
}

template <int CS, int ORDER>
__global__ void __launch_bounds__(kBlockX *kBlockY, NRGPU_BSSN_RICCI_MIN_BLOCKS)
    ricci_xx_kernel(Grid g, const double *__restrict__ in, XXArgs xa, double *__restrict__ aux) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  double q[rq::NQ];
  hatted_at_point<CS>(xa, i0, i1, q);
  const Rfm<CS, double, true> rf{q, 1};
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  Metric<CS, double> m;
  metric_point<ORDER, CS, double>(P, rf, inv, m);
  double Rbar[6];
  ricci_point<ORDER, CS, double>(P, rf, inv, m, Rbar);
#pragma unroll
  for (int k = 0; k < 6; k++) aux[(long long)k * g.ntot + idx] = Rbar[k];
}

template <int CS, int ORDER, bool KO>
__global__ void __launch_bounds__(kBlockX *kBlockY, NRGPU_BSSN_RHS_MIN_BLOCKS)
    rhs_xx_kernel(Grid g, const double *__restrict__ in, const double *__restrict__ aux, XXArgs xa, double eta,
                  double diss, double *__restrict__ out) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  double q[rq::NQ];
  hatted_at_point<CS>(xa, i0, i1, q);
  const Rfm<CS, double, true> rf{q, 1};
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  double Rbar[6];
#pragma unroll
  for (int k = 0; k < 6; k++) Rbar[k] = __ldg(aux + (long long)k * g.ntot + idx);
  double r[NUM_EVOL_GFS];
  rhs_point<ORDER, CS, double>(P, rf, inv, Rbar, eta, r);
#pragma unroll
  for (int gf = 0; gf < NUM_EVOL_GFS; gf++) {
    double v = r[gf];
    if constexpr (KO) v += diss * ko_point<ORDER, CS, double>(P, gf, rf, inv);
    out[(long long)gf * g.ntot + idx] = v;
  }
}

template <int CS, int ORDER>
int ricci_xx_launch_t(const paramstruct *p, const XXArgs &xa, const double *in, double *aux) {
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  ricci_xx_kernel<CS, ORDER><<<L.grid, L.block, 0, stream()>>>(g, in, xa, aux);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <int CS, int ORDER, bool KO>
int rhs_xx_launch_t(const paramstruct *p, const XXArgs &xa, const double *aux, const double *in, double *out) {
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  rhs_xx_kernel<CS, ORDER, KO><<<L.grid, L.block, 0, stream()>>>(g, in, aux, xa, p->eta, p->diss_strength, out);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <typename R> inline const R *table_of(const rfm_struct *rfm) {
  if (!rfm) return nullptr;
  if constexpr (sizeof(R) == 8) return (const R *)rfm->table64;
  else return (const R *)rfm->table32;
}

template <int CS, int ORDER>
int ricci_launch_t(const rfm_struct *rfm, const paramstruct *p, const void *in, bool in_is_f64, int prec,
                   void *aux) {
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  if (prec == NRGPU_PREC_COMPENSATED) {
    ricci_kernel<float, Pair32, CS, ORDER, float><<<L.grid, L.block, 0, stream()>>>(
        g, (const float2 *)in, table_of<float>(rfm), (float *)aux);
  } else if (prec == NRGPU_PREC_FP64) {
    ricci_kernel<double, double, CS, ORDER, double>
        <<<L.grid, L.block, 0, stream()>>>(g, (const double *)in, table_of<double>(rfm), (double *)aux);
  } else if (in_is_f64) {
    ricci_kernel<float, double, CS, ORDER, float>
        <<<L.grid, L.block, 0, stream()>>>(g, (const double *)in, table_of<float>(rfm), (float *)aux);
  } else {
    ricci_kernel<float, float, CS, ORDER, float>
        <<<L.grid, L.block, 0, stream()>>>(g, (const float *)in, table_of<float>(rfm), (float *)aux);
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <int CS, int ORDER, bool KO>
int rhs_launch_t(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  const float eta32 = (float)p->eta, diss32 = (float)p->diss_strength;
  if (a.prec == NRGPU_PREC_FP64) {
    RKEpilogue<double> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (double *)a.out};
    rhs_kernel<double, double, CS, ORDER, double, KO><<<L.grid, L.block, 0, stream()>>>(
        g, (const double *)a.in, (const double *)a.auxevol, table_of<double>(rfm), p->eta, p->diss_strength, epi);
  } else if (a.prec == NRGPU_PREC_COMPENSATED) {
    RKEpilogue<float2> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float2 *)a.out};
    rhs_kernel<float, Pair32, CS, ORDER, float2, KO><<<L.grid, L.block, 0, stream()>>>(
        g, stage_input<Pair32>(a), (const float *)a.auxevol, table_of<float>(rfm), eta32, diss32, epi);
  } else {
    RKEpilogue<float> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float *)a.out};
    if (a.in_is_f64)
      rhs_kernel<float, double, CS, ORDER, float, KO><<<L.grid, L.block, 0, stream()>>>(
          g, (const double *)a.in, (const float *)a.auxevol, table_of<float>(rfm), eta32, diss32, epi);
    else
      rhs_kernel<float, float, CS, ORDER, float, KO><<<L.grid, L.block, 0, stream()>>>(
          g, (const float *)a.in, (const float *)a.auxevol, table_of<float>(rfm), eta32, diss32, epi);
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

#define NRGPU_BSSN_DECLARE(CS, ORDER)                                                                    \
  extern template int ricci_launch_t<CS, ORDER>(const rfm_struct *, const paramstruct *, const void *,    \
                                                bool, int, void *);                                       \
  extern template int rhs_launch_t<CS, ORDER, false>(const rfm_struct *, const paramstruct *,             \
                                                     const StageArgs &);                                  \
  extern template int rhs_launch_t<CS, ORDER, true>(const rfm_struct *, const paramstruct *,              \
                                                    const StageArgs &);                                   \
  extern template int ricci_xx_launch_t<CS, ORDER>(const paramstruct *, const XXArgs &, const double *,   \
                                                   double *);                                             \
  extern template int rhs_xx_launch_t<CS, ORDER, false>(const paramstruct *, const XXArgs &,              \
                                                        const double *, const double *, double *);        \
  extern template int rhs_xx_launch_t<CS, ORDER, true>(const paramstruct *, const XXArgs &,               \
                                                       const double *, const double *, double *);
#define NRGPU_BSSN_INSTANTIATE(CS, ORDER)                                                             \
  template int ricci_launch_t<CS, ORDER>(const rfm_struct *, const paramstruct *, const void *,     \
                                         bool, int, void *);                                        \
  template int rhs_launch_t<CS, ORDER, false>(const rfm_struct *, const paramstruct *, const StageArgs &); \
  template int ricci_xx_launch_t<CS, ORDER>(const paramstruct *, const XXArgs &, const double *, double *); \
  template int rhs_xx_launch_t<CS, ORDER, false>(const paramstruct *, const XXArgs &, const double *,     \
                                                 const double *, double *);
// The Kreiss-Oliger instantiations, in their own translation units.
#define NRGPU_BSSN_INSTANTIATE_KO(CS, ORDER)                                                          \
  template int rhs_launch_t<CS, ORDER, true>(const rfm_struct *, const paramstruct *, const StageArgs &); \
  template int rhs_xx_launch_t<CS, ORDER, true>(const paramstruct *, const XXArgs &, const double *,      \
                                                const double *, double *);

}  // namespace bssn
}  // namespace nrgpu
