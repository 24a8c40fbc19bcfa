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

// Block shape of the BSSN point kernels: 32 x 4, 64 x 2, 128 x 1 and 32 x 2
// (8 blocks) measure alike on GB300 (within 1%); 16 x 8 is 3% slower.
#ifndef NRGPU_BSSN_BLOCK_X
#define NRGPU_BSSN_BLOCK_X 32
#endif
#ifndef NRGPU_BSSN_BLOCK_Y
#define NRGPU_BSSN_BLOCK_Y 4
#endif
constexpr int kBlockX = NRGPU_BSSN_BLOCK_X, kBlockY = NRGPU_BSSN_BLOCK_Y;
// Resident blocks per SM the compiler must allow (caps registers per thread):
// measured on GB300, the rhs kernel runs fastest at 4 blocks of 128 threads
// (128 registers, spilling), the Ricci kernel at 1 (255 registers).
// NRGPU_BSSN_SMEM_SPILL lets ptxas place part of the rhs kernel's register
// spills in shared memory (CUDA 13's enable_smem_spilling pragma; about
// 100 B per thread here) instead of local memory, which at this frame size
// misses L1: 3.5% faster rhs kernel on GB300.
#ifndef NRGPU_BSSN_RICCI_MIN_BLOCKS
#define NRGPU_BSSN_RICCI_MIN_BLOCKS 1
#endif
#ifndef NRGPU_BSSN_SMEM_SPILL
#define NRGPU_BSSN_SMEM_SPILL 1
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
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g, i0, i1, i2);
  Metric<CS, R> m;
  metric_point<ORDER, CS, R>(P, rf, inv, m);
  R Rbar[6];
  ricci_point<ORDER, CS, R>(P, rf, inv, m, Rbar);
#pragma unroll
  for (int k = 0; k < 6; k++) aux[(long long)k * g.ntot + idx] = (TAux)Rbar[k];
}

// Kreiss-Oliger dissipation of gridfunction gf at the point:
// sum_k f_dKOD[k] ReU[k] (BaikalETK/BaikalETK_C_kernels_codegen.py:147-171).
template <int ORDER, int CS, typename R, typename Tin, int LOC>
__device__ __forceinline__ R ko_point(const Point<Tin> &P, int gf, const Rfm<CS, R, LOC> &rf, const R *inv) {
  R acc = (R)0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const R d = fd_ko<ORDER, R>(P.gf(gf), P.st[k]) * inv[k];
    acc += RfmMask<CS>::trivial ? d : d * rf.ReU(k);
  }
  return acc;
}

// T^{mu nu} source terms of the BSSN RHSs at the point, added to out[]
// (BSSN_stress_energy_source_terms.py:24-131 with ADMBSSN_tofrom_4metric.py:38-68,
// added as BaikalETK_C_kernels_codegen.py:133-145 adds them):
//   gamma4_{i mu} = (beta_i, gamma_ij), S_ij = gamma4_{i mu} gamma4_{j nu} T^{mu nu},
//   S_i = alpha gamma4_{i mu} T^{mu 0}, S = gamma^ij S_ij, rho = alpha^2 T^{00};
//   trK += 4 pi alpha (rho + S);  a_ij += -8 pi alpha W^2 (S_ij - gammabar_ij S^bar/3) / ReDD_ij;
//   Lambdabar source L^i = -16 pi alpha gammabar^ij S_j: lambda^i += L^i / ReU^i and,
//   through the Gamma-driver's 3/4 d_t Lambdabar^i, B^i += (3/4) L^i / ReU^i.
// T4: the ten T4UU gridfunctions at this point (stride ntot).
template <int CS, typename R, typename Tin, int LOC>
__device__ __forceinline__ void source_point(const Point<Tin> &P, const Rfm<CS, R, LOC> &rf,
                                             const R *__restrict__ T4, long long ntot, R *out) {
  using M = RfmMask<CS>;
  const R alpha = pval<R>(P, ALPHA), cf = pval<R>(P, CF);
  R gbar[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const R h = pval<R>(P, HDD00 + S6(i, j));
      R v = M::trivial ? h : h * rf.ReDD(i, j);
      if (i == j) v += rf.ghatDD(i);
      gbar[i][j] = gbar[j][i] = v;
    }
  R gbUU[3][3], detgb;
  sym_inverse(gbar, gbUU, detgb);
  const R e4 = (R)1 / (cf * cf), cf2 = cf * cf;
  R P4[3][4];  // gamma4_{i+1, mu}
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R bD = (R)0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const R vet = pval<R>(P, VETU0 + j);
      bD += e4 * gbar[i][j] * (M::trivial ? vet : vet * rf.ReU(j));
      P4[i][j + 1] = e4 * gbar[i][j];
    }
    P4[i][0] = bD;
  }
  R T[4][4];
  {
    int n = 0;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = a; b < 4; b++) {
        const R t = (R)__ldg(T4 + (long long)n * ntot);
        T[a][b] = T[b][a] = t;
        n++;
      }
  }
  R SDD[3][3], SD[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R s = (R)0;
#pragma unroll
    for (int m = 0; m < 4; m++) s += P4[i][m] * T[m][0];
    SD[i] = alpha * s;
#pragma unroll
    for (int j = i; j < 3; j++) {
      R acc = (R)0;
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) acc += P4[i][m] * P4[j][n] * T[m][n];
      SDD[i][j] = SDD[j][i] = acc;
    }
  }
  R trSbar = (R)0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) trSbar += gbUU[i][j] * SDD[i][j];
  const R S = cf2 * trSbar;  // gamma^ij = W^2 gammabar^ij
  const R rho = alpha * alpha * T[0][0];
  const R pi = (R)3.14159265358979323846;
  out[TRK] += (R)4 * pi * alpha * (rho + S);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const R a = (R)(-8) * pi * alpha * cf2 * (SDD[i][j] - gbar[i][j] * trSbar * (R)(1.0 / 3.0));
      out[ADD00 + S6(i, j)] += M::trivial ? a : a / rf.ReDD(i, j);
    }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const R L = (R)(-16) * pi * alpha * (gbUU[i][0] * SD[0] + gbUU[i][1] * SD[1] + gbUU[i][2] * SD[2]);
    const R Lr = M::trivial ? L : L / rf.ReU(i);
    out[LAMBDAU0 + i] += Lr;
    out[BETU0 + i] += (R)0.75 * Lr;
  }
}

// EXTRA: the instantiation that adds Kreiss-Oliger dissipation (diss != 0)
// and/or the T^{mu nu} source terms (T4 != nullptr) to every RHS; both are
// uniform branches.  The default instantiation carries neither.
template <typename R, typename Tin, int CS, int ORDER, typename TStage, bool EXTRA>
__global__ void __launch_bounds__(kBlockX *kBlockY, NRGPU_BSSN_RHS_MIN_BLOCKS)
    rhs_kernel(Grid g, typename InRef<Tin>::type in, const R *__restrict__ aux, const R *__restrict__ tab,
               R eta, R diss, const R *__restrict__ T4, RKEpilogue<TStage> epi) {
#if NRGPU_BSSN_SMEM_SPILL
  asm volatile(".pragma \"enable_smem_spilling\";");
#endif
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  Point<Tin> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g, i0, i1, i2);
  R Rbar[6];
#pragma unroll
  for (int k = 0; k < 6; k++) Rbar[k] = (R)__ldg(aux + (long long)k * g.ntot + idx);
  R out[NUM_EVOL_GFS];
  rhs_point<ORDER, CS, R>(P, rf, inv, Rbar, eta, out);
  if constexpr (EXTRA) {
    if (T4) source_point<CS, R>(P, rf, T4 + idx, g.ntot, out);
  }
  // Not unrolled: one copy of the RK update (and of the dissipation stencil)
  // serves the 24 gridfunctions, keeping its temporaries off the registers
  // the RHS algebra needs.
#pragma unroll 1
  for (int gf = 0; gf < NUM_EVOL_GFS; gf++) {
    R v = out[gf];
    if constexpr (EXTRA) {
      if (diss != (R)0) v += diss * ko_point<ORDER, CS, R>(P, gf, rf, inv);
    }
    epi(gf, idx, v);
  }
}

// The same kernels with the reference metric evaluated at each point from the
// caller's coordinate arrays xx0[i0], xx1[i1], xx2[i2] (FP64), as the reference's
// no-precompute rhs_eval(params, xx, auxevol_gfs, in_gfs, rhs_gfs) does.
struct XXArgs {
  const double *xx0, *xx1, *xx2;
  CoordParams c;  // the runtime CoordSystem and its parameters
};

template <int CS>
__device__ __forceinline__ void hatted_at_point(const XXArgs &xa, int i0, int i1, int i2, double *q) {
  if constexpr (CS != NRGPU_COORD_CARTESIAN) {
    ScaleFactors S;
    scale_factors(xa.c, xa.xx0[i0], xa.xx1[i1], xa.xx2[i2], &S);
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
  hatted_at_point<CS>(xa, i0, i1, i2, q);
  const Rfm<CS, double, RFM_LOCAL> rf{q, 1};
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  Metric<CS, double> m;
  metric_point<ORDER, CS, double>(P, rf, inv, m);
  double Rbar[6];
  ricci_point<ORDER, CS, double>(P, rf, inv, m, Rbar);
#pragma unroll
  for (int k = 0; k < 6; k++) aux[(long long)k * g.ntot + idx] = Rbar[k];
}

template <int CS, int ORDER, bool EXTRA>
__global__ void __launch_bounds__(kBlockX *kBlockY, NRGPU_BSSN_RHS_MIN_BLOCKS)
    rhs_xx_kernel(Grid g, const double *__restrict__ in, const double *__restrict__ aux, XXArgs xa, double eta,
                  double diss, const double *__restrict__ T4, double *__restrict__ out) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  double q[rq::NQ];
  hatted_at_point<CS>(xa, i0, i1, i2, q);
  const Rfm<CS, double, RFM_LOCAL> rf{q, 1};
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  double Rbar[6];
#pragma unroll
  for (int k = 0; k < 6; k++) Rbar[k] = __ldg(aux + (long long)k * g.ntot + idx);
  double r[NUM_EVOL_GFS];
  rhs_point<ORDER, CS, double>(P, rf, inv, Rbar, eta, r);
  if constexpr (EXTRA) {
    if (T4) source_point<CS, double>(P, rf, T4 + idx, g.ntot, r);
  }
#pragma unroll
  for (int gf = 0; gf < NUM_EVOL_GFS; gf++) {
    double v = r[gf];
    if constexpr (EXTRA) {
      if (diss != 0.0) v += diss * ko_point<ORDER, CS, double>(P, gf, rf, inv);
    }
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

// The ten T4UU gridfunctions follow the six RbarDD ones in auxevol.
template <typename R> inline const R *t4uu_of(const paramstruct *p, const void *aux, long long ntot) {
  return p->enable_stress_energy_source_terms ? (const R *)aux + 6 * ntot : nullptr;
}

template <int CS, int ORDER, bool EXTRA>
int rhs_xx_launch_t(const paramstruct *p, const XXArgs &xa, const double *aux, const double *in, double *out) {
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  rhs_xx_kernel<CS, ORDER, EXTRA><<<L.grid, L.block, 0, stream()>>>(g, in, aux, xa, p->eta, p->diss_strength,
                                                                     t4uu_of<double>(p, aux, g.ntot), out);
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
  if (pair_precision(prec)) {
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

template <int CS, int ORDER, bool EXTRA>
int rhs_launch_t(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, kBlockX, kBlockY);
  const float eta32 = (float)p->eta, diss32 = (float)p->diss_strength;
  if (a.prec == NRGPU_PREC_FP64) {
    RKEpilogue<double> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (double *)a.out};
    rhs_kernel<double, double, CS, ORDER, double, EXTRA><<<L.grid, L.block, 0, stream()>>>(
        g, (const double *)a.in, (const double *)a.auxevol, table_of<double>(rfm), p->eta, p->diss_strength,
        t4uu_of<double>(p, a.auxevol, g.ntot), epi);
  } else if (pair_precision(a.prec)) {
    RKEpilogue<float2> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float2 *)a.out, stage_consts(a.dt),
                           a.prec == NRGPU_PREC_COMPENSATED_FP64RK};
    rhs_kernel<float, Pair32, CS, ORDER, float2, EXTRA><<<L.grid, L.block, 0, stream()>>>(
        g, stage_input<Pair32>(a), (const float *)a.auxevol, table_of<float>(rfm), eta32, diss32,
        t4uu_of<float>(p, a.auxevol, g.ntot), epi);
  } else {
    RKEpilogue<float> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float *)a.out, stage_consts(a.dt)};
    if (a.in_is_f64)
      rhs_kernel<float, double, CS, ORDER, float, EXTRA><<<L.grid, L.block, 0, stream()>>>(
          g, (const double *)a.in, (const float *)a.auxevol, table_of<float>(rfm), eta32, diss32,
          t4uu_of<float>(p, a.auxevol, g.ntot), epi);
    else
      rhs_kernel<float, float, CS, ORDER, float, EXTRA><<<L.grid, L.block, 0, stream()>>>(
          g, (const float *)a.in, (const float *)a.auxevol, table_of<float>(rfm), eta32, diss32,
          t4uu_of<float>(p, a.auxevol, g.ntot), epi);
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
// The instantiations with Kreiss-Oliger dissipation and T^{mu nu} source
// terms, in their own translation units.
#define NRGPU_BSSN_INSTANTIATE_EXTRA(CS, ORDER)                                                          \
  template int rhs_launch_t<CS, ORDER, true>(const rfm_struct *, const paramstruct *, const StageArgs &); \
  template int rhs_xx_launch_t<CS, ORDER, true>(const paramstruct *, const XXArgs &, const double *,      \
                                                const double *, double *);

}  // namespace bssn
}  // namespace nrgpu
