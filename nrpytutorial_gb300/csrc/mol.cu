// mol.cu -- RK4 method-of-lines step (MoLtimestepping/RK_MoL.h for "RK4"),
// fused and unfused, the host-buffer evolve loop, per-system gridfunction
// tables, and the interior L2-norm reduction used by constraint diagnostics.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>

#include "epilogue.cuh"
#include "systems.cuh"

namespace nrgpu {

// ---------------------------------------------------------- system tables
// Alphabetical gf order (grid.py:226-243); parity types per
// CurviBoundaryConditions.py:122-213 (0 scalar, 1..3 vector component,
// 4..9 rank-2 components 00,01,02,11,12,22).
static const int8_t kParitySW[2] = {0, 0};                           // uu vv
static const int8_t kParityMaxwell[7] = {1, 2, 3, 1, 2, 3, 0};       // AU0-2 EU0-2 psi
static const int8_t kParityMaxwellCurvi[8] = {0, 1, 2, 3, 1, 2, 3, 0};  // Gamma aU0-2 eU0-2 psi
static const int8_t kParityBSSN[24] = {4, 5, 6, 7, 8, 9,             // aDD00..aDD22
                                       0,                            // alpha
                                       1, 2, 3,                      // betU0..2
                                       0,                            // cf
                                       4, 5, 6, 7, 8, 9,             // hDD00..hDD22
                                       1, 2, 3,                      // lambdaU0..2
                                       0,                            // trK
                                       1, 2, 3};                     // vetU0..2

int system_num_gfs(int system) {
  switch (system) {
    case NRGPU_SYS_SCALARWAVE: return 2;
    case NRGPU_SYS_MAXWELL: return 7;
    case NRGPU_SYS_BSSN: return 24;
    case NRGPU_SYS_MAXWELL_CURVILINEAR: return 8;
  }
  return -1;
}
const int8_t *system_parity(int system) {
  switch (system) {
    case NRGPU_SYS_SCALARWAVE: return kParitySW;
    case NRGPU_SYS_MAXWELL: return kParityMaxwell;
    case NRGPU_SYS_BSSN: return kParityBSSN;
    case NRGPU_SYS_MAXWELL_CURVILINEAR: return kParityMaxwellCurvi;
  }
  return nullptr;
}

template <typename T>
int apply_bcs_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity, T *gfs);

// ------------------------------------------------------- unfused update
// LOOP_ALL_GFS_GPS RK update over all points of all gfs, reading the RHS the
// RHS kernel stored in `k` (C_Code_Generation.py:159 and :277-329).
// float2 stage buffers hold FP32 (hi, lo) pairs: the RHS is read as their
// sum and the stage value is stored back as a pair.
template <typename TStage> __device__ __forceinline__ double as_double(TStage v) {
  if constexpr (std::is_same<TStage, float2>::value) return pair_value(v);
  else return (double)v;
}
template <typename TStage> __device__ __forceinline__ TStage from_double(double v) {
  if constexpr (std::is_same<TStage, float2>::value) return split_pair(v);
  else return (TStage)v;
}

// f64_update: FP32 stage buffers with the update in FP64 arithmetic on the
// FP64 y_n and running total (NRGPU_PREC_COMPENSATED_FP64RK).
template <typename TStage>
__global__ void rk4_update_kernel(int stage, double dt, StageConsts kc, long long n, double *__restrict__ y_n,
                                  double *__restrict__ rt, TStage *__restrict__ k, bool f64_update = false) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (!std::is_same<TStage, double>::value && !f64_update) {
      // FP32 stages: the fused epilogue's float-float update (y_n, rt hold pairs)
      float kv;
      if constexpr (std::is_same<TStage, float2>::value) kv = k[i].x;  // rhs_eval stored (k, 0)
      else kv = k[i];
      const float2 v = ff_rk4_update(stage, kv, kc, y_n, rt, i);
      if (stage < 3) {
        if constexpr (std::is_same<TStage, float2>::value) k[i] = v;
        else k[i] = v.x;
      }
      continue;
    }
    const double kdt = __dmul_rn(as_double(k[i]), dt);
    switch (stage) {
      case 0:
        rt[i] = __dmul_rn(kdt, 1.0 / 6.0);
        k[i] = from_double<TStage>(__dadd_rn(y_n[i], __dmul_rn(kdt, 1.0 / 2.0)));
        break;
      case 1:
        rt[i] = __dadd_rn(rt[i], __dmul_rn(kdt, 1.0 / 3.0));
        k[i] = from_double<TStage>(__dadd_rn(y_n[i], __dmul_rn(kdt, 1.0 / 2.0)));
        break;
      case 2:
        rt[i] = __dadd_rn(rt[i], __dmul_rn(kdt, 1.0 / 3.0));
        k[i] = from_double<TStage>(__dadd_rn(y_n[i], kdt));
        break;
      default:
        y_n[i] = __dadd_rn(__dadd_rn(y_n[i], rt[i]), __dmul_rn(kdt, 1.0 / 6.0));
        break;
    }
  }
}

// RK update of a split step (FP32 stages, float-float update) at the
// interior points, where the RHS kernel stored k (as (k, 0) pairs, or FP32
// values): ff_rk4_pairs, exactly as the fused epilogue applies it, with the
// stage value written over k (substeps 0..2) or y_n written as FP64
// (substep 3).  Ghost points are left to the boundary conditions, as in the
// fused step.  One thread per point of a 128-point row along i0; each thread
// walks the gfs in groups of 6 whose loads are issued together.  At most 64
// registers, so 8 blocks fit an SM: the 1024 rows of a 128x64x16 grid run in
// one wave (at 77 registers, 6 blocks per SM, they took two).
template <typename TStage, int STAGE>
__global__ void __launch_bounds__(128, 8) rk4_update_interior_kernel(Grid g, int ngf, StageConsts kc, double *y_n,
                                                                  double *rt, TStage *k) {
  const int i0 = g.ng + blockIdx.x * 128 + threadIdx.x;
  if (i0 >= g.n0 - g.ng) return;
  const long long idx =
      (long long)i0 + (long long)g.n0 * ((long long)(g.ng + blockIdx.y) + (long long)g.n1 * (g.ng + blockIdx.z));
  float2 *y2 = (float2 *)y_n, *r2 = (float2 *)rt;
  constexpr int GRP = 6;
  for (int g0 = 0; g0 < ngf; g0 += GRP) {
    float kv[GRP];
    float2 yv[GRP], rv[GRP];
#pragma unroll
    for (int j = 0; j < GRP; j++) {
      if (g0 + j < ngf) {
        const long long i = (long long)(g0 + j) * g.ntot + idx;
        if constexpr (std::is_same<TStage, float2>::value) kv[j] = k[i].x;
        else kv[j] = k[i];
        yv[j] = y2[i];
        rv[j] = (STAGE > 0) ? r2[i] : make_float2(0.f, 0.f);
      }
    }
#pragma unroll
    for (int j = 0; j < GRP; j++) {
      if (g0 + j < ngf) {
        const long long i = (long long)(g0 + j) * g.ntot + idx;
        const float2 v = ff_rk4_pairs(STAGE, kv[j], kc, yv[j], rv[j]);
        if (STAGE < 3) {
          r2[i] = rv[j];
          if constexpr (std::is_same<TStage, float2>::value) k[i] = v;
          else k[i] = v.x;
        } else {
          y_n[i] = f2d_bits(v.x) + f2d_bits(v.y);
        }
      }
    }
  }
}

// The same for pair stages with the update in FP64 arithmetic on the FP64
// y_n and running total (NRGPU_PREC_COMPENSATED_FP64RK): the FP64 branch of
// RKEpilogue::apply on k = the stored FP32 RHS, so it gives the fused
// epilogue's bits.
template <int STAGE>
__global__ void __launch_bounds__(128, 8) rk4_update_interior_f64_kernel(Grid g, int ngf, double dt, double *y_n,
                                                                      double *rt, float2 *k) {
  const int i0 = g.ng + blockIdx.x * 128 + threadIdx.x;
  if (i0 >= g.n0 - g.ng) return;
  const long long idx =
      (long long)i0 + (long long)g.n0 * ((long long)(g.ng + blockIdx.y) + (long long)g.n1 * (g.ng + blockIdx.z));
  constexpr int GRP = 6;
  for (int g0 = 0; g0 < ngf; g0 += GRP) {
    float kv[GRP];
    double yv[GRP], rv[GRP];
#pragma unroll
    for (int j = 0; j < GRP; j++) {
      if (g0 + j < ngf) {
        const long long i = (long long)(g0 + j) * g.ntot + idx;
        kv[j] = k[i].x;
        yv[j] = y_n[i];
        rv[j] = (STAGE > 0) ? rt[i] : 0.0;
      }
    }
#pragma unroll
    for (int j = 0; j < GRP; j++) {
      if (g0 + j < ngf) {
        const long long i = (long long)(g0 + j) * g.ntot + idx;
        const double kdt = dmul((double)kv[j], dt);
        switch (STAGE) {
          case 0:
            rt[i] = dmul(kdt, 1.0 / 6.0);
            k[i] = split_pair(dadd(yv[j], dmul(kdt, 1.0 / 2.0)));
            break;
          case 1:
            rt[i] = dadd(rv[j], dmul(kdt, 1.0 / 3.0));
            k[i] = split_pair(dadd(yv[j], dmul(kdt, 1.0 / 2.0)));
            break;
          case 2:
            rt[i] = dadd(rv[j], dmul(kdt, 1.0 / 3.0));
            k[i] = split_pair(dadd(yv[j], kdt));
            break;
          default:
            y_n[i] = dadd(dadd(yv[j], rv[j]), dmul(kdt, 1.0 / 6.0));
            break;
        }
      }
    }
  }
}

template <typename TStage>
static int update_interior_t(const paramstruct *p, int ngf, int stage, StageConsts kc, double *y_n, double *rt,
                             TStage *k) {
  const Grid g = make_grid(p);
  NRGPU_REQUIRE(p->Nxx1 <= 65535 && p->Nxx2 <= 65535, "Nxx1, Nxx2 above the launch's grid limit");
  const dim3 grid((unsigned)((p->Nxx0 + 127) / 128), (unsigned)p->Nxx1, (unsigned)p->Nxx2);
  switch (stage) {
    case 0: rk4_update_interior_kernel<TStage, 0><<<grid, 128, 0, stream()>>>(g, ngf, kc, y_n, rt, k); break;
    case 1: rk4_update_interior_kernel<TStage, 1><<<grid, 128, 0, stream()>>>(g, ngf, kc, y_n, rt, k); break;
    case 2: rk4_update_interior_kernel<TStage, 2><<<grid, 128, 0, stream()>>>(g, ngf, kc, y_n, rt, k); break;
    default: rk4_update_interior_kernel<TStage, 3><<<grid, 128, 0, stream()>>>(g, ngf, kc, y_n, rt, k); break;
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

static int update_interior_f64(const paramstruct *p, int ngf, int stage, double dt, double *y_n, double *rt,
                               float2 *k) {
  const Grid g = make_grid(p);
  NRGPU_REQUIRE(p->Nxx1 <= 65535 && p->Nxx2 <= 65535, "Nxx1, Nxx2 above the launch's grid limit");
  const dim3 grid((unsigned)((p->Nxx0 + 127) / 128), (unsigned)p->Nxx1, (unsigned)p->Nxx2);
  switch (stage) {
    case 0: rk4_update_interior_f64_kernel<0><<<grid, 128, 0, stream()>>>(g, ngf, dt, y_n, rt, k); break;
    case 1: rk4_update_interior_f64_kernel<1><<<grid, 128, 0, stream()>>>(g, ngf, dt, y_n, rt, k); break;
    case 2: rk4_update_interior_f64_kernel<2><<<grid, 128, 0, stream()>>>(g, ngf, dt, y_n, rt, k); break;
    default: rk4_update_interior_f64_kernel<3><<<grid, 128, 0, stream()>>>(g, ngf, dt, y_n, rt, k); break;
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

// SM count of the current device, cached per device ordinal (grid sizes of
// the reductions and update loops depend on the device they run on).
static int sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  if (dev >= 0 && dev < 64) {
    const int c = cached[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = 152;
  }
  if (dev >= 0 && dev < 64) cached[dev].store(n, std::memory_order_relaxed);
  return n;
}

static int rhs_stage(int system, const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  switch (system) {
    case NRGPU_SYS_SCALARWAVE: return scalarwave_launch(rfm, p, a);
    case NRGPU_SYS_MAXWELL: return maxwell_launch(p, a);
    case NRGPU_SYS_MAXWELL_CURVILINEAR: return maxwell_curvi_launch(rfm, p, a);
    case NRGPU_SYS_BSSN: {
      return bssn_stage_launch(rfm, p, a);
    }
  }
  set_error("unknown system %d", system);
  return NRGPU_ERR_ARG;
}

// Boundary conditions, then (BSSN) the det(gammabar) rescale, on `gfs`
// (double, float, or float2 pairs when `pair`).
// reduced: an FP32-stage step (its FP64 y_n is rescaled in float-float arithmetic)
// f64_rescale: pair stage buffers rescaled in FP64 arithmetic (COMPENSATED_FP64RK)
static int post_rhs(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc, void *gfs,
                    bool is_f64, bool pair = false, bool reduced = false, bool f64_rescale = false) {
  const int ngf = system_num_gfs(system);
  int st;
  if (pair) st = apply_bcs_pair_impl(p, bc, ngf, system_parity(system), (float2 *)gfs);
  else if (is_f64) st = apply_bcs_impl<double>(p, bc, ngf, system_parity(system), (double *)gfs);
  else st = apply_bcs_impl<float>(p, bc, ngf, system_parity(system), (float *)gfs);
  if (st) return st;
  if (system == NRGPU_SYS_BSSN)
    return bssn_enforce_launch(rfm, p, gfs, is_f64, pair, reduced && is_f64, f64_rescale && pair);
  return NRGPU_OK;
}

static long long state_len(int system, const paramstruct *p) {
  return (long long)system_num_gfs(system) * p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 *
         p->Nxx_plus_2NGHOSTS2;
}

// Start of an NRGPU_PREC_COMPENSATED_FP64RK step: the FP64 y_n stays as it is
// and its (hi, lo) pairs go to `out`, substep 0's stencil input.
__global__ void pair_copy_kernel(long long n, const double *__restrict__ y, float2 *__restrict__ out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
    double v[4];
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (i0 + j * stride < n) v[j] = y[i0 + j * stride];
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (i0 + j * stride < n) out[i0 + j * stride] = split_pair(v[j]);
  }
}

// Blocks of a grid-stride loop over n items: as many as the SMs hold at once
// (one wave; a fixed multiple of the SM count can leave a partial second
// wave), fewer when n is small.
template <typename K> static int one_wave_blocks(K kernel, int threads, long long n) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads,
                                                         (long long)sm_count() * per_sm));
}

static int prep_state(int system, const paramstruct *p, MoL_gridfunctions *gfs) {
  const long long n = state_len(system, p);
  const int threads = 256;
  if (gfs->precision == NRGPU_PREC_COMPENSATED_FP64RK) {
    const int blocks = one_wave_blocks(pair_copy_kernel, threads, n);
    pair_copy_kernel<<<blocks, threads, 0, stream()>>>(n, gfs->y_n_gfs, (float2 *)gfs->k_even_gfs);
  } else if (gfs->precision == NRGPU_PREC_COMPENSATED) {
    const int blocks = one_wave_blocks(split_state_kernel<false>, threads, n);
    split_state_kernel<false><<<blocks, threads, 0, stream()>>>(n, gfs->y_n_gfs, nullptr);
  } else {
    const int blocks = one_wave_blocks(split_state_kernel<true>, threads, n);
    split_state_kernel<true><<<blocks, threads, 0, stream()>>>(n, gfs->y_n_gfs, (float *)gfs->k_even_gfs);
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

// A split step (bssn_split_update): the RHS kernel stores k and the RK
// update runs as rk4_update_interior_kernel (float-float) or
// rk4_update_interior_f64_kernel (FP64-accumulation form); the arithmetic is
// the fused epilogue's, so both forms give the same bits.
static bool split_step(int system, const paramstruct *p, int prec) {
  return system == NRGPU_SYS_BSSN && bssn_split_update(p, prec);
}
static int update_interior(int system, const paramstruct *p, MoL_gridfunctions *gfs, int stage, StageConsts kc,
                           void *k, double dt) {
  const int ngf = system_num_gfs(system);
  if (gfs->precision == NRGPU_PREC_COMPENSATED_FP64RK)
    return update_interior_f64(p, ngf, stage, dt, gfs->y_n_gfs, gfs->y_nplus1_running_total_gfs, (float2 *)k);
  if (pair_precision(gfs->precision))
    return update_interior_t<float2>(p, ngf, stage, kc, gfs->y_n_gfs, gfs->y_nplus1_running_total_gfs, (float2 *)k);
  return update_interior_t<float>(p, ngf, stage, kc, gfs->y_n_gfs, gfs->y_nplus1_running_total_gfs, (float *)k);
}

static int check_step_args(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc,
                           const MoL_gridfunctions *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(system_num_gfs(system) > 0, "unknown system %d", system);
  NRGPU_REQUIRE(bc != nullptr && gfs != nullptr, "NULL bcstruct or gridfunctions");
  NRGPU_REQUIRE(gfs->precision == NRGPU_PREC_FP64 || gfs->precision == NRGPU_PREC_MIXED ||
                    pair_precision(gfs->precision),
                "unknown precision %d", gfs->precision);
  NRGPU_REQUIRE(gfs->y_n_gfs && gfs->y_nplus1_running_total_gfs && gfs->k_odd_gfs && gfs->k_even_gfs,
                "MoL gridfunction buffer is NULL");
  NRGPU_REQUIRE(system != NRGPU_SYS_BSSN || gfs->auxevol_gfs, "BSSN needs auxevol_gfs");
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN || rfm != nullptr,
                "curvilinear grids need an rfm_struct");
  return NRGPU_OK;
}

}  // namespace nrgpu

using namespace nrgpu;

extern "C" {

int MoL_step_forward_in_time(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc,
                             MoL_gridfunctions *gfs, double dt) {
  int st = check_step_args(system, rfm, p, bc, gfs);
  if (st) return st;
  const bool f64 = gfs->precision == NRGPU_PREC_FP64;
  const bool pair = pair_precision(gfs->precision);
  const bool acc64 = gfs->precision == NRGPU_PREC_COMPENSATED_FP64RK;
  const bool split = split_step(system, p, gfs->precision);
  void *kbuf[2] = {gfs->k_odd_gfs, gfs->k_even_gfs};
  if (!f64 && (st = prep_state(system, p, gfs))) return st;
  const StageConsts kc = stage_consts(dt);
  for (int s = 0; s < 4; s++) {
    StageArgs a{};
    a.stage = split ? -1 : s;
    a.dt = dt;
    a.prec = gfs->precision;
    // substep 0 reads y_n: itself in FP64, its pairs in place when compensated,
    // its pair copy (COMPENSATED_FP64RK) or FP32 copy (plain FP32 stages) in k_even
    a.in = (s == 0) ? (f64 || (pair && !acc64) ? (const void *)gfs->y_n_gfs : (const void *)gfs->k_even_gfs)
                    : (const void *)kbuf[(s + 1) % 2];
    a.in_is_f64 = f64;
    a.y_n = gfs->y_n_gfs;
    a.rt = gfs->y_nplus1_running_total_gfs;
    // fused: the stage value (substeps 0..2; substep 3 writes y_n); split: k
    a.out = (s == 3 && !split) ? nullptr : kbuf[s % 2];
    a.auxevol = gfs->auxevol_gfs;
    if ((st = rhs_stage(system, rfm, p, a))) return st;
    if (split && (st = update_interior(system, p, gfs, s, kc, kbuf[s % 2], dt))) return st;
    void *post = (s == 3) ? (void *)gfs->y_n_gfs : kbuf[s % 2];
    const bool post_f64 = (s == 3) || f64;
    if ((st = post_rhs(system, rfm, p, bc, post, post_f64, pair && s < 3, !f64 && !acc64, acc64))) return st;
  }
  return NRGPU_OK;
}

int MoL_substep_rhs(int system, const rfm_struct *rfm, const paramstruct *p, MoL_gridfunctions *gfs, int stage,
                    double dt, int which) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(system_num_gfs(system) > 0 && gfs, "bad arguments");
  NRGPU_REQUIRE(stage >= 0 && stage <= 3, "stage %d not in 0..3", stage);
  NRGPU_REQUIRE(which >= 0 && which <= 4, "which %d not in 0..4", which);
  NRGPU_REQUIRE(which == 0 || which == 3 || system == NRGPU_SYS_BSSN, "which = 1, 2 select BSSN's two kernels");
  const bool f64 = gfs->precision == NRGPU_PREC_FP64;
  const bool pair = pair_precision(gfs->precision);
  const bool split = split_step(system, p, gfs->precision);
  NRGPU_REQUIRE(which != 4 || split, "which = 4: this step updates in the RHS kernel's epilogue");
  void *kbuf[2] = {gfs->k_odd_gfs, gfs->k_even_gfs};
  if (which == 4) return update_interior(system, p, gfs, stage, stage_consts(dt), kbuf[stage % 2], dt);
  StageArgs a{};
  a.stage = split ? -1 : stage;
  a.dt = dt;
  a.prec = gfs->precision;
  a.in = (stage == 0) ? (pair ? (const void *)gfs->k_even_gfs : (const void *)gfs->y_n_gfs)
                      : (const void *)kbuf[(stage + 1) % 2];
  a.in_is_f64 = !pair && ((stage == 0) || f64);
  a.y_n = gfs->y_n_gfs;
  a.rt = gfs->y_nplus1_running_total_gfs;
  a.out = (stage == 3 && !split) ? nullptr : kbuf[stage % 2];
  a.auxevol = gfs->auxevol_gfs;
  if (which == 1) return bssn_ricci_launch(rfm, p, a.in, a.in_is_f64, a.prec, a.auxevol);
  if (which == 2) return bssn_rhs_launch(rfm, p, a);
  if ((st = rhs_stage(system, rfm, p, a)) || which == 3 || !split) return st;
  return update_interior(system, p, gfs, stage, stage_consts(dt), kbuf[stage % 2], dt);
}

int MoL_step_forward_in_time_sommerfeld(int system, const rfm_struct *rfm, const paramstruct *p,
                                        const bc_struct *bc, MoL_gridfunctions *gfs, double dt) {
  int st = check_step_args(system, rfm, p, bc, gfs);
  if (st) return st;
  NRGPU_REQUIRE(gfs->precision == NRGPU_PREC_FP64, "the Sommerfeld step is FP64");
  void *kbuf[2] = {gfs->k_odd_gfs, gfs->k_even_gfs};
  const int ngf = system_num_gfs(system);
  const long long n = state_len(system, p);
  const int threads = 256;
  const int blocks = (int)std::min<long long>((n + threads - 1) / threads, (long long)sm_count() * 16);
  for (int s = 0; s < 4; s++) {
    StageArgs a{};
    a.stage = -1;
    a.dt = dt;
    a.prec = gfs->precision;
    a.in = (s == 0) ? (const void *)gfs->y_n_gfs : (const void *)kbuf[(s + 1) % 2];
    a.in_is_f64 = true;
    a.out = kbuf[s % 2];  // RHS_output: k_odd, k_even, k_odd, k_even
    a.auxevol = gfs->auxevol_gfs;
    if ((st = rhs_stage(system, rfm, p, a))) return st;
    // radiation condition on the RHS at the ghost points (RHS_string), then the
    // update over every point; no post-RHS boundary step
    if ((st = apply_sommerfeld_impl(p, nullptr, bc, ngf, system_parity(system), (const double *)a.in,
                                    (double *)kbuf[s % 2])))
      return st;
    rk4_update_kernel<double><<<blocks, threads, 0, stream()>>>(s, dt, StageConsts{}, n, gfs->y_n_gfs,
                                                                gfs->y_nplus1_running_total_gfs,
                                                                (double *)kbuf[s % 2]);
    NRGPU_LAUNCH_CHECK();
    if (system == NRGPU_SYS_BSSN &&
        (st = bssn_enforce_launch(rfm, p, s == 3 ? (void *)gfs->y_n_gfs : kbuf[s % 2], true)))
      return st;
  }
  return NRGPU_OK;
}

int MoL_step_forward_in_time_unfused(int system, const rfm_struct *rfm, const paramstruct *p,
                                     const bc_struct *bc, MoL_gridfunctions *gfs, double dt) {
  int st = check_step_args(system, rfm, p, bc, gfs);
  if (st) return st;
  const bool f64 = gfs->precision == NRGPU_PREC_FP64;
  const bool pair = pair_precision(gfs->precision);
  const bool acc64 = gfs->precision == NRGPU_PREC_COMPENSATED_FP64RK;
  void *kbuf[2] = {gfs->k_odd_gfs, gfs->k_even_gfs};
  const long long n = state_len(system, p);
  const int threads = 256;
  const int blocks = (int)std::min<long long>((n + threads - 1) / threads, (long long)sm_count() * 16);
  if (!f64 && (st = prep_state(system, p, gfs))) return st;
  const StageConsts kc = stage_consts(dt);
  for (int s = 0; s < 4; s++) {
    StageArgs a{};
    a.stage = -1;
    a.dt = dt;
    a.prec = gfs->precision;
    a.in = (s == 0) ? (f64 || (pair && !acc64) ? (const void *)gfs->y_n_gfs : (const void *)gfs->k_even_gfs)
                    : (const void *)kbuf[(s + 1) % 2];
    a.in_is_f64 = f64;
    a.out = kbuf[s % 2];  // RHS_output: k_odd, k_even, k_odd, k_even
    a.auxevol = gfs->auxevol_gfs;
    if ((st = rhs_stage(system, rfm, p, a))) return st;
    if (pair)
      rk4_update_kernel<float2><<<blocks, threads, 0, stream()>>>(s, dt, kc, n, gfs->y_n_gfs,
                                                                  gfs->y_nplus1_running_total_gfs,
                                                                  (float2 *)kbuf[s % 2], acc64);
    else if (!f64)
      rk4_update_kernel<float><<<blocks, threads, 0, stream()>>>(s, dt, kc, n, gfs->y_n_gfs,
                                                                 gfs->y_nplus1_running_total_gfs,
                                                                 (float *)kbuf[s % 2]);
    else
      rk4_update_kernel<double><<<blocks, threads, 0, stream()>>>(s, dt, StageConsts{}, n, gfs->y_n_gfs,
                                                                  gfs->y_nplus1_running_total_gfs,
                                                                  (double *)kbuf[s % 2]);
    NRGPU_LAUNCH_CHECK();
    void *post = (s == 3) ? (void *)gfs->y_n_gfs : kbuf[s % 2];
    const bool post_f64 = (s == 3) || f64;
    if ((st = post_rhs(system, rfm, p, bc, post, post_f64, pair && s < 3, !f64 && !acc64, acc64))) return st;
  }
  return NRGPU_OK;
}

// The host-buffer evolution's work on the library stream: copy in, n_steps
// steps, copy out (no synchronisation).
static int evolve_host_enqueue(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc,
                               MoL_gridfunctions *gfs, double dt, int n_steps, double *y_host) {
  const size_t bytes = sizeof(double) * (size_t)system_num_gfs(system) * p->Nxx_plus_2NGHOSTS0 *
                       p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  int st;
  NRGPU_CUDA_CHECK(cudaMemcpyAsync(gfs->y_n_gfs, y_host, bytes, cudaMemcpyHostToDevice, stream()));
  for (int n = 0; n < n_steps; n++)
    if ((st = MoL_step_forward_in_time(system, rfm, p, bc, gfs, dt))) return st;
  NRGPU_CUDA_CHECK(cudaMemcpyAsync(y_host, gfs->y_n_gfs, bytes, cudaMemcpyDeviceToHost, stream()));
  return NRGPU_OK;
}

// A call that repeats the previous one exactly (system, the bytes of the
// parameter, reference-metric, boundary and gridfunction structures, dt,
// step count, host array, device, BSSN kernel selection) with a pinned host
// array replays a CUDA graph of its copies and steps, captured on the
// second such call: one graph launch instead of ~21 kernel launches per
// step removes their launch gaps.  Other calls return NRGPU_ERR_UNSUPPORTED
// and run eagerly.  One graph is cached per process, for the last
// configuration seen.
constexpr int kEvolveGraphMaxSteps = 16;
struct EvolveKey {
  int system, n_steps, dev, kernels, has_rfm, pad;
  double dt;
  const double *y_host;
  paramstruct p;
  rfm_struct rfm;
  bc_struct bc;
  MoL_gridfunctions gfs;
};
static std::mutex g_evolve_mutex;
static bool g_evolve_have_key = false;
static EvolveKey g_evolve_key;
static cudaGraphExec_t g_evolve_exec = nullptr;

static int evolve_host_graph(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc,
                             MoL_gridfunctions *gfs, double dt, int n_steps, double *y_host) {
  if (n_steps < 1 || n_steps > kEvolveGraphMaxSteps) return NRGPU_ERR_UNSUPPORTED;
  cudaPointerAttributes pa;
  memset(&pa, 0, sizeof(pa));
  if (cudaPointerGetAttributes(&pa, y_host) != cudaSuccess || pa.type != cudaMemoryTypeHost) {
    cudaGetLastError();
    return NRGPU_ERR_UNSUPPORTED;
  }
  EvolveKey k;
  memset(&k, 0, sizeof(k));
  k.system = system;
  k.n_steps = n_steps;
  if (cudaGetDevice(&k.dev) != cudaSuccess) {
    cudaGetLastError();
    return NRGPU_ERR_UNSUPPORTED;
  }
  k.kernels = bssn_kernels_mode();
  k.dt = dt;
  k.y_host = y_host;
  k.p = *p;
  if (rfm) {
    k.has_rfm = 1;
    k.rfm = *rfm;
  }
  k.bc = *bc;
  k.gfs = *gfs;
  std::lock_guard<std::mutex> lock(g_evolve_mutex);
  if (!g_evolve_have_key || memcmp(&g_evolve_key, &k, sizeof(k)) != 0) {
    if (g_evolve_exec) cudaGraphExecDestroy(g_evolve_exec);
    g_evolve_exec = nullptr;
    g_evolve_key = k;
    g_evolve_have_key = true;
    return NRGPU_ERR_UNSUPPORTED;  // first call of this configuration: eager
  }
  if (!g_evolve_exec) {
    cudaStream_t cs = nullptr, saved = stream();
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      return NRGPU_ERR_UNSUPPORTED;
    }
    cudaGraph_t graph = nullptr;
    int st = NRGPU_ERR_CUDA;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      nrgpu_set_stream(cs);
      st = evolve_host_enqueue(system, rfm, p, bc, gfs, dt, n_steps, y_host);
      nrgpu_set_stream(saved);
      if (cudaStreamEndCapture(cs, &graph) != cudaSuccess) st = NRGPU_ERR_CUDA;
    }
    if (st == NRGPU_OK && graph && cudaGraphInstantiate(&g_evolve_exec, graph, 0) != cudaSuccess)
      g_evolve_exec = nullptr;
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    cudaGetLastError();
    if (!g_evolve_exec) {
      g_evolve_have_key = false;
      return NRGPU_ERR_UNSUPPORTED;  // capture failed: this call runs eagerly
    }
  }
  NRGPU_CUDA_CHECK(cudaGraphLaunch(g_evolve_exec, stream()));
  NRGPU_CUDA_CHECK(cudaStreamSynchronize(stream()));
  return NRGPU_OK;
}

int MoL_evolve_host(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc,
                    MoL_gridfunctions *gfs, double dt, int n_steps, double *y_host) {
  int st = check_step_args(system, rfm, p, bc, gfs);
  if (st) return st;
  NRGPU_REQUIRE(y_host != nullptr && n_steps >= 0, "bad host buffer or step count");
  if ((st = evolve_host_graph(system, rfm, p, bc, gfs, dt, n_steps, y_host)) != NRGPU_ERR_UNSUPPORTED) return st;
  if ((st = evolve_host_enqueue(system, rfm, p, bc, gfs, dt, n_steps, y_host))) return st;
  NRGPU_CUDA_CHECK(cudaStreamSynchronize(stream()));
  return NRGPU_OK;
}

}  // extern "C"

// ------------------------------------------------------------ L2 norms
namespace nrgpu {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Pass 1: each block sums f^2 over a grid-stride share of the interior
// points and writes one partial to scratch[blockIdx.x].
__global__ void l2_partial_kernel(Grid g, const double *__restrict__ f, double *__restrict__ partial) {
  const int nx = g.n0 - 2 * g.ng, ny = g.n1 - 2 * g.ng, nz = g.n2 - 2 * g.ng;
  const long long n = (long long)nx * ny * nz;
  double acc = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(t % nx) + g.ng;
    const int i1 = (int)((t / nx) % ny) + g.ng;
    const int i2 = (int)(t / ((long long)nx * ny)) + g.ng;
    const double v = f[i0 + (long long)g.n0 * (i1 + (long long)g.n1 * i2)];
    acc += v * v;
  }
  __shared__ double sh[32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}

// Pass 2: one block adds the partials in a fixed order (deterministic).
__global__ void l2_final_kernel(const double *__restrict__ partial, int nparts, double count,
                                double *__restrict__ result) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partial[i];
  __shared__ double sh[32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) {
      result[0] = v;
      result[1] = count;
    }
  }
}

int l2_norm_sq_impl(const paramstruct *p, const double *gfs, int gf, double *scratch, int scratch_len,
                    double *result) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(gfs && scratch && result, "NULL argument");
  NRGPU_REQUIRE(gf >= 0, "negative gridfunction index");
  NRGPU_REQUIRE(scratch_len >= 1, "scratch_len must be >= 1");
  Grid g = make_grid(p);
  const long long n = (long long)p->Nxx0 * p->Nxx1 * p->Nxx2;
  const int threads = 256;
  int blocks = (int)std::min<long long>((n + threads - 1) / threads, (long long)sm_count() * 4);
  blocks = std::max(1, std::min(blocks, scratch_len));
  l2_partial_kernel<<<blocks, threads, 0, stream()>>>(g, gfs + (long long)gf * g.ntot, scratch);
  NRGPU_LAUNCH_CHECK();
  l2_final_kernel<<<1, 256, 0, stream()>>>(scratch, blocks, (double)n, result);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

}  // namespace nrgpu

extern "C" int nrgpu_l2_norm_sq(const paramstruct *p, const double *gfs, int gf, double *scratch,
                                int scratch_len, double *result) {
  return nrgpu::l2_norm_sq_impl(p, gfs, gf, scratch, scratch_len, result);
}

// ------------------------------------------- allocation-free L2 norm
// Some callers cannot allocate device memory: host codes that hand this
// library only the state arrays they own and forbid any allocation during
// their time loop (arena-managed frameworks, drivers whose device memory is
// fixed at start-up), and plain C/Fortran drivers that have no device
// allocator of their own.  For them the per-block partial sums of the L2
// reduction live in this fixed file-scope array instead of a caller-supplied
// scratch buffer.  Every GPU that loads the library holds these 16 KB until
// the process exits.
#define NRGPU_L2_STATIC_MAX_PARTIALS 2048
static __device__ __align__(256) double g_l2_static_partials[NRGPU_L2_STATIC_MAX_PARTIALS];

namespace nrgpu {
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_l2_static_mutex;
double *g_l2_static_ptr[kMaxDevices] = {nullptr};
}  // namespace
}  // namespace nrgpu

extern "C" int nrgpu_l2_norm_sq_static(const paramstruct *p, const double *gfs, int gf, double *result) {
  using namespace nrgpu;
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(gfs && result, "NULL argument");
  NRGPU_REQUIRE(gf >= 0, "negative gridfunction index");
  int dev = 0;
  NRGPU_CUDA_CHECK(cudaGetDevice(&dev));
  NRGPU_REQUIRE(dev >= 0 && dev < kMaxDevices, "device %d beyond the %d this entry point tracks", dev, kMaxDevices);
  double *partials;
  {
    // One-time set-up per device, with that device current: the host-side
    // name of the array is not a device address, so look the address up.
    // The cached address belongs to the device's current context: after a
    // cudaDeviceReset (or any teardown of the primary context) the library
    // module is loaded again, possibly elsewhere, and this cached address
    // is stale -- callers that reset a device must not use this entry point
    // afterwards in the same process.
    std::lock_guard<std::mutex> lock(g_l2_static_mutex);
    if (!g_l2_static_ptr[dev]) {
      void *addr = nullptr;
      NRGPU_CUDA_CHECK(cudaGetSymbolAddress(&addr, g_l2_static_partials));
      g_l2_static_ptr[dev] = (double *)addr;
    }
    partials = g_l2_static_ptr[dev];
  }
  Grid g = make_grid(p);
  const long long n = (long long)p->Nxx0 * p->Nxx1 * p->Nxx2;
  const int threads = 256;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads,
                                                                      (long long)sm_count() * 4));
  if (blocks > NRGPU_L2_STATIC_MAX_PARTIALS) {
    set_error("nrgpu_l2_norm_sq_static: needs %d partial sums, the static scratch holds %d", blocks,
              NRGPU_L2_STATIC_MAX_PARTIALS);
    return NRGPU_ERR_SIZE;
  }
  // Every partial the final pass reads is written by this call's first pass,
  // so the array needs no clearing between calls.
  l2_partial_kernel<<<blocks, threads, 0, stream()>>>(g, gfs + (long long)gf * g.ntot, partials);
  NRGPU_LAUNCH_CHECK();
  l2_final_kernel<<<1, 256, 0, stream()>>>(partials, blocks, (double)n, result);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
