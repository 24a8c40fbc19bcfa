// batch.cu -- many independent small ScalarWave evolutions (curvilinear,
// ragged grid sizes) advanced together: one persistent launch per RK4
// substep covers every instance, and one launch per boundary-condition
// application covers every instance's ghost zones.
//
// Physics per instance is exactly the single-grid path: the curvilinear
// ScalarWave RHS (ScalarWave/ScalarWaveCurvilinear_RHSs.py:43-98), FD4, the
// RK4 low-storage step (MoLtimestepping/C_Code_Generation.py:266-329) and
// apply_bcs_curvilinear (boundary_conditions/apply_bcs_curvilinear.h:19-64).
//
// Layout: instance-major packed arrays, [instance][gf][i2][i1][i0]; a table of
// BatchInstance records gives each instance's extents and offsets.  Work is a
// list of (instance, i2, i1-block) items; a persistent grid walks the list
// with a fixed stride, so instances of any size share one launch.  The item
// shape (TX threads along i0, TY rows of i1) is chosen by a timing autotuner.
// Boundary conditions: one launch per application, one block per instance,
// which walks that instance's ghost-layer phases in the reference's order
// with a block barrier between phases (instances do not depend on each other).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "epilogue.cuh"
#include "fd.cuh"
#include "rfm.cuh"

namespace nrgpu {

template <typename T>
int apply_bcs_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity, T *gfs);

struct BatchInstance {
  int n0, n1, n2;          // Nxx_plus_2NGHOSTS0..2
  int pad;
  long long base;          // offset of (gf 0, point 0) in packed state arrays
  long long ntot;          // points per gridfunction
  long long tab;           // offset of this instance's [6][n1][n0] metric table
  double invdx0, invdx1, invdx2;
  double dxx0, dxx1;       // uniform spacings, for the coordinates xx0, xx1
  double dt;               // this instance's time step
  StageConsts kc;          // dt/6, dt/3, dt/2, dt as FP32 pairs (FP32 stage modes)
};

constexpr int kBatchNG = 2;     // FD4 ScalarWave ghost zones
constexpr int kBatchPhases = 4 * kBatchNG;  // per layer: outer i0, i1, i2, inner
constexpr int kBatchTab = 6;    // ghatUU0..2, contracted Gammahat^0..2

struct BatchWork {
  int inst, i2, i1;
};

// vv_rhs = c^2 (ghat^ii d_i d_i uu - ghat^ij Gammahat^k_ij d_k uu), per point.
// At most 64 registers (1024 threads' worth of blocks per SM): the kernel is
// bound by load latency, and 32 warps per SM instead of the ~16 that 96
// registers allow took the 512-instance step from 2.00 to 1.60 ms (plain
// FP32 stages) and 2.18 to 1.91 ms (pairs), despite a few spilled bytes.
template <typename R, typename Tin, typename TStage, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, 1024 / (TX * TY))
    sw_batch_rhs_kernel(const BatchInstance *__restrict__ insts, const BatchWork *__restrict__ work, int nwork,
                        typename InRef<Tin>::type in, const R *__restrict__ tab, R c2, RKEpilogue<TStage> epi) {
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const BatchWork it = work[w];
    const BatchInstance I = insts[it.inst];
    const int i1 = it.i1 + threadIdx.y;
    if (i1 >= I.n1 - kBatchNG) continue;
    const int i2 = it.i2;
    const long long st[3] = {1, I.n0, (long long)I.n0 * I.n1};
    const R inv[3] = {(R)I.invdx0, (R)I.invdx1, (R)I.invdx2};
    const long long plane = (long long)I.n0 * I.n1;
    // the epilogue indexes gf g at base + g*ntot + idx of this instance
    RKEpilogue<TStage> e = epi;
    e.ntot = I.ntot;
    e.dt = I.dt;
    e.kc = I.kc;
    e.y_n = epi.y_n ? epi.y_n + I.base : nullptr;
    e.rt = epi.rt ? epi.rt + I.base : nullptr;
    e.out = epi.out ? epi.out + I.base : nullptr;
    for (int i0 = kBatchNG + threadIdx.x; i0 < I.n0 - kBatchNG; i0 += TX) {
      const long long idx = i0 + I.n0 * ((long long)i1 + (long long)I.n1 * i2);
      // the update's y_n and running-total loads go out with the stencil loads
      const typename RKEpilogue<TStage>::Operands o0 = e.fetch(0, idx), o1 = e.fetch(1, idx);
      const auto uu = in + I.base + idx;
      const R vv = val<R>(in + I.base + I.ntot + idx);
      const R *t = tab + I.tab + (long long)i1 * I.n0 + i0;
      R lap = (R)0;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        lap += __ldg(t + d * plane) * (fd_d2<4, R>(uu, st[d]) * (inv[d] * inv[d]));
        if (d < 2) lap -= __ldg(t + (3 + d) * plane) * (fd_d1<4, R>(uu, st[d]) * inv[d]);
      }
      e.apply(0, idx, vv, o0);
      e.apply(1, idx, c2 * lap, o1);
    }
  }
}

// Metric table of every instance: ghatUU (diagonal) and the contracted
// Christoffels ghat^ij Gammahat^k_ij, from the FP64 hatted quantities.
__global__ void sw_batch_table_kernel(const BatchInstance *__restrict__ insts, int ninst, int cs, double xxmin0,
                                      double xxmin1, double AMPL, double SINHW, double *tab64, float *tab32) {
  const int inst = blockIdx.y;
  if (inst >= ninst) return;
  const BatchInstance I = insts[inst];
  const long long plane = (long long)I.n0 * I.n1;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < plane; c += gridDim.x * (long long)blockDim.x) {
    const int i0 = (int)(c % I.n0), i1 = (int)(c / I.n0);
    const double xx0 = xx_of(xxmin0, I.dxx0, i0, kBatchNG);
    const double xx1 = xx_of(xxmin1, I.dxx1, i1, kBatchNG);
    ScaleFactors S;
    CoordParams cp{};
    cp.cs = cs, cp.AMPL = AMPL, cp.SINHW = SINHW;
    scale_factors(cp, xx0, xx1, 0.0, &S);
    double q[rq::NQ];
    hatted_quantities(S, q);
    double v[kBatchTab];
    for (int i = 0; i < 3; i++) v[i] = q[rq::ghatUU + 4 * i];
    for (int k = 0; k < 3; k++) {
      double s = 0.0;
      for (int i = 0; i < 3; i++) s += q[rq::ghatUU + 4 * i] * q[rq::GammahatUDD + 9 * k + 4 * i];
      v[3 + k] = s;
    }
    for (int j = 0; j < kBatchTab; j++) {
      tab64[I.tab + j * plane + c] = v[j];
      tab32[I.tab + j * plane + c] = (float)v[j];
    }
  }
}

// Gaussian pulse u = A exp(-(r - r0)^2 / w^2), v = 0 at every point.
__global__ void sw_batch_gaussian_kernel(const BatchInstance *__restrict__ insts, int ninst, int cs,
                                         double xxmin0, double AMPL, double SINHW, const double *__restrict__ A,
                                         const double *__restrict__ r0, const double *__restrict__ w,
                                         double *__restrict__ y) {
  const int inst = blockIdx.y;
  if (inst >= ninst) return;
  const BatchInstance I = insts[inst];
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < I.ntot; c += gridDim.x * (long long)blockDim.x) {
    const int i0 = (int)(c % I.n0);
    const double xx0 = xx_of(xxmin0, I.dxx0, i0, kBatchNG);
    CoordParams cp{};
    cp.cs = cs, cp.AMPL = AMPL, cp.SINHW = SINHW;
    double r[4];
    radial_map(cp, xx0, r);
    const double x = (r[0] - r0[inst]) / w[inst];
    y[I.base + c] = A[inst] * exp(-x * x);
    y[I.base + I.ntot + c] = 0.0;
  }
}

// Batched boundary conditions: block `inst` applies instance inst's ghost
// phases (per layer: outer faces along i0, i1, i2, then inner points) in
// order.  Offsets a (dest) and b (outer: signed step; inner: src) are
// relative to the instance's first point; both gridfunctions per thread.
template <typename T> __device__ __forceinline__ T bc_extrapolate3(T f1, T f2, T f3) {
  if constexpr (std::is_same<T, double>::value)
    return __dadd_rn(__dsub_rn(__dmul_rn(3.0, f1), __dmul_rn(3.0, f2)), f3);
  else if constexpr (std::is_same<T, float>::value)
    return __fadd_rn(__fsub_rn(__fmul_rn(3.0f, f1), __fmul_rn(3.0f, f2)), f3);
  else  // FP32 pairs: the rule on the FP64 values, re-split
    return split_pair(__dadd_rn(__dsub_rn(__dmul_rn(3.0, pair_value(f1)), __dmul_rn(3.0, pair_value(f2))),
                                pair_value(f3)));
}
template <typename T> __device__ __forceinline__ T bc_extrapolate(const T *f, long long s) {
  return bc_extrapolate3(f[s], f[2 * s], f[3 * s]);
}

template <typename T>
__global__ void sw_batch_bc_kernel(const BatchInstance *__restrict__ insts, const int *__restrict__ phases,
                                   const int *__restrict__ a, const int *__restrict__ b, T *gfs) {
  const BatchInstance I = insts[blockIdx.x];
  T *f = gfs + I.base;
  const int *ph = phases + (long long)blockIdx.x * (kBatchPhases + 1);
  for (int q = 0; q < kBatchPhases; q++) {
    const bool inner = (q % 4) == 3;
    for (int p = ph[q] + threadIdx.x; p < ph[q + 1]; p += blockDim.x) {
      const long long d = a[p], e = b[p];
#pragma unroll
      for (int g = 0; g < 2; g++) {
        T *fg = f + g * I.ntot;
        fg[d] = inner ? fg[e] : bc_extrapolate(fg + d, e);  // scalars: parity +1
      }
    }
    __syncthreads();
  }
}

// Level-scheduled boundary conditions.  A ghost point's level is 1 + the
// largest level among the points it reads (interior points: 0), following
// the reference's sequential order (layers inner to outer; per layer outer
// faces i0, i1, i2, then inner points).  When no point is read before the
// sequence writes it (checked on the host), every point of one level can be
// filled at once, from the same final source values and with the same
// arithmetic as the sequential application, so the result is bit-identical.
// Per distinct instance shape one template holds the entries sorted by
// level, outer before inner within a level; tpl_off[lvl][0 / 1] are the
// starts of a level's outer / inner entries (lvl = 1..kBcMaxLevels + 1).
constexpr int kBcMaxLevels = 8;
constexpr int kBcOffStride = 2 * (kBcMaxLevels + 2);

// Both gridfunctions' source values are loaded before either store (within
// a level no entry reads another entry's destination).
template <typename T>
__device__ __forceinline__ void bc_apply_entry(T *f, long long ntot, long long d, long long e, bool inner) {
  T *f1 = f + ntot;
  if (inner) {  // scalars: parity +1
    const T a = f[e], b = f1[e];
    f[d] = a;
    f1[d] = b;
  } else {
    const T a1 = f[d + e], a2 = f[d + 2 * e], a3 = f[d + 3 * e];
    const T b1 = f1[d + e], b2 = f1[d + 2 * e], b3 = f1[d + 3 * e];
    f[d] = bc_extrapolate3(a1, a2, a3);
    f1[d] = bc_extrapolate3(b1, b2, b3);
  }
}

// Level 1 of every instance: grid (chunks, instances), grid-stride within
// the instance's template.
template <typename T>
__global__ void sw_batch_bc_level1_kernel(const BatchInstance *__restrict__ insts, const int *__restrict__ tpl_off,
                                          const int *__restrict__ ta, const int *__restrict__ tb, T *gfs) {
  const BatchInstance I = insts[blockIdx.y];
  const int *o = tpl_off + I.pad * kBcOffStride;
  const int si = o[3], e = o[4];
  T *f = gfs + I.base;
  for (int p = o[2] + blockIdx.x * blockDim.x + threadIdx.x; p < e; p += gridDim.x * blockDim.x)
    bc_apply_entry(f, I.ntot, ta[p], tb[p], p >= si);
}

// Levels 2..nlev of one instance per block, a block barrier between levels.
template <typename T>
__global__ void sw_batch_bc_levels_kernel(const BatchInstance *__restrict__ insts, const int *__restrict__ tpl_off,
                                          const int *__restrict__ ta, const int *__restrict__ tb, int nlev, T *gfs) {
  const BatchInstance I = insts[blockIdx.x];
  const int *o = tpl_off + I.pad * kBcOffStride;
  T *f = gfs + I.base;
  for (int lv = 2; lv <= nlev; lv++) {
    const int si = o[2 * lv + 1], e = o[2 * lv + 2];
    for (int p = o[2 * lv] + threadIdx.x; p < e; p += blockDim.x) bc_apply_entry(f, I.ntot, ta[p], tb[p], p >= si);
    __syncthreads();
  }
}

}  // namespace nrgpu

using namespace nrgpu;

// Opaque batch state (host handle).
struct nrgpu_batch {
  int ninst, cs, N1, N2, prec;
  double RMAX, AMPL, SINHW, xxmin0, xxmin1, c2;
  long long total_points;   // per gridfunction-set: sum of 2*ntot
  std::vector<BatchInstance> h_insts;
  BatchInstance *d_insts = nullptr;
  BatchWork *d_work[4] = {nullptr, nullptr, nullptr, nullptr};  // for TY = 1, 2, 4, 8
  int nwork[4] = {0, 0, 0, 0};
  double *d_tab64 = nullptr;
  float *d_tab32 = nullptr;
  // boundary phases: per instance, kBatchPhases+1 offsets into a/b
  int *d_bc_phases = nullptr, *d_bc_a = nullptr, *d_bc_b = nullptr;
  // level-scheduled boundary templates (one per distinct instance shape)
  bool bc_levels = false;
  int bc_nlev = 0, bc_l1_max = 0;
  int *d_tpl_off = nullptr, *d_tpl_a = nullptr, *d_tpl_b = nullptr;
  // tuned launch shape
  int tx = 64, tyi = 1, grid = 0;
  int bc_threads = 256;  // block size of the boundary-condition kernel
};

static void batch_destroy(nrgpu_batch *b) {
  if (!b) return;
  cudaFree(b->d_insts);
  for (int t = 0; t < 4; t++) cudaFree(b->d_work[t]);
  cudaFree(b->d_bc_phases);
  cudaFree(b->d_bc_a);
  cudaFree(b->d_bc_b);
  cudaFree(b->d_tpl_off);
  cudaFree(b->d_tpl_a);
  cudaFree(b->d_tpl_b);
  cudaFree(b->d_tab64);
  cudaFree(b->d_tab32);
  delete b;
}

static int batch_launch_rhs(nrgpu_batch *b, const void *in, bool in_f64, int stage, double *y_n,
                            double *rt, void *out) {
  const int TYs[4] = {1, 2, 4, 8};
  const int ty = TYs[b->tyi];
  const int grid = b->grid > 0 ? b->grid : 152 * 8;
  const BatchWork *work = b->d_work[b->tyi];
  const int nwork = b->nwork[b->tyi];
#define LAUNCH(R, Tin, TS, TX, TY)                                                                          \
  sw_batch_rhs_kernel<R, Tin, TS, TX, TY><<<grid, dim3(TX, TY), 0, stream()>>>(                            \
      b->d_insts, work, nwork, (typename InRef<Tin>::type)in,                                               \
      (const R *)(sizeof(R) == 8 ? (const void *)b->d_tab64                                                 \
                                                                            : (const void *)b->d_tab32),    \
      (R)b->c2, RKEpilogue<TS>{stage, 0.0, 0, y_n, rt, (TS *)out})
#define SHAPES(R, Tin, TS)                                                   \
  switch (b->tx * 16 + ty) {                                                 \
    case 32 * 16 + 1: LAUNCH(R, Tin, TS, 32, 1); break;                      \
    case 32 * 16 + 2: LAUNCH(R, Tin, TS, 32, 2); break;                      \
    case 32 * 16 + 4: LAUNCH(R, Tin, TS, 32, 4); break;                      \
    case 32 * 16 + 8: LAUNCH(R, Tin, TS, 32, 8); break;                      \
    case 64 * 16 + 1: LAUNCH(R, Tin, TS, 64, 1); break;                      \
    case 64 * 16 + 2: LAUNCH(R, Tin, TS, 64, 2); break;                      \
    case 64 * 16 + 4: LAUNCH(R, Tin, TS, 64, 4); break;                      \
    case 128 * 16 + 1: LAUNCH(R, Tin, TS, 128, 1); break;                    \
    case 128 * 16 + 2: LAUNCH(R, Tin, TS, 128, 2); break;                    \
    default: set_error("unsupported batch tile %dx%d", b->tx, ty); return NRGPU_ERR_ARG; \
  }
  if (b->prec == NRGPU_PREC_FP64) {
    SHAPES(double, double, double)
  } else if (b->prec == NRGPU_PREC_COMPENSATED) {
    SHAPES(float, Pair32, float2)
  } else if (in_f64) {
    SHAPES(float, double, float)
  } else {
    SHAPES(float, float, float)
  }
#undef SHAPES
#undef LAUNCH
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <typename T> static int batch_bcs(nrgpu_batch *b, T *gfs) {
  if (b->bc_levels) {
    const int t = b->bc_threads;
    const int chunks = std::max(1, std::min(64, (b->bc_l1_max + 4 * t - 1) / (4 * t)));
    sw_batch_bc_level1_kernel<T><<<dim3(chunks, b->ninst), t, 0, stream()>>>(b->d_insts, b->d_tpl_off, b->d_tpl_a,
                                                                             b->d_tpl_b, gfs);
    NRGPU_LAUNCH_CHECK();
    if (b->bc_nlev >= 2) {
      sw_batch_bc_levels_kernel<T><<<b->ninst, t, 0, stream()>>>(b->d_insts, b->d_tpl_off, b->d_tpl_a, b->d_tpl_b,
                                                                 b->bc_nlev, gfs);
      NRGPU_LAUNCH_CHECK();
    }
    return NRGPU_OK;
  }
  sw_batch_bc_kernel<T><<<b->ninst, b->bc_threads, 0, stream()>>>(b->d_insts, b->d_bc_phases, b->d_bc_a, b->d_bc_b,
                                                                  gfs);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

extern "C" {

int nrgpu_batch_create(int ninst, const int *Nr, int Ntheta, int Nphi, int CoordSystem, double RMAX, double AMPL,
                       double SINHW, double wavespeed, double CFL_FACTOR, int precision, nrgpu_batch **out) {
  NRGPU_REQUIRE(out && Nr && ninst >= 1, "bad arguments");
  NRGPU_REQUIRE(CoordSystem == NRGPU_COORD_SPHERICAL || CoordSystem == NRGPU_COORD_SINHSPHERICAL,
                "batched ScalarWave needs a Spherical-family CoordSystem");
  NRGPU_REQUIRE(precision == NRGPU_PREC_FP64 || precision == NRGPU_PREC_MIXED ||
                    precision == NRGPU_PREC_COMPENSATED,
                "bad precision");
  NRGPU_REQUIRE(ninst <= 65535, "at most 65535 instances (grid y dimension)");
  nrgpu_batch *b = new nrgpu_batch();
  b->ninst = ninst;
  b->cs = CoordSystem;
  b->N1 = Ntheta;
  b->N2 = Nphi;
  b->prec = precision;
  b->RMAX = RMAX;
  b->AMPL = AMPL;
  b->SINHW = SINHW;
  b->c2 = wavespeed * wavespeed;
  long long base = 0, tab = 0;
  std::vector<BatchWork> work[4];
  const int TYs[4] = {1, 2, 4, 8};
  std::vector<int> bphase, ba, bb;  // per-instance phase offsets; dest; step or src
  // level templates, one per distinct (n0, n1, n2)
  std::vector<long long> tpl_key;
  std::vector<int> tpl_off, tpl_a, tpl_b;
  bool levels_ok = true;
  int nlev_all = 1, l1_max = 0;
  for (int i = 0; i < ninst; i++) {
    paramstruct p{};
    p.CoordSystem = CoordSystem;
    p.FD_order = 4;
    p.NGHOSTS = kBatchNG;
    p.RMAX = RMAX;
    p.AMPL = AMPL;
    p.SINHW = SINHW;
    p.wavespeed = wavespeed;
    const int Nxx[3] = {Nr[i], Ntheta, Nphi};
    int st = set_Nxx_dxx_invdx_params__and__xx(0, Nxx, &p, nullptr);
    if (st) {
      batch_destroy(b);
      return st;
    }
    if (i == 0) {
      b->xxmin0 = p.xxmin0;
      b->xxmin1 = p.xxmin1;
    }
    BatchInstance I{};
    I.n0 = p.Nxx_plus_2NGHOSTS0;
    I.n1 = p.Nxx_plus_2NGHOSTS1;
    I.n2 = p.Nxx_plus_2NGHOSTS2;
    I.ntot = (long long)I.n0 * I.n1 * I.n2;
    I.base = base;
    I.tab = tab;
    I.invdx0 = p.invdx0;
    I.invdx1 = p.invdx1;
    I.invdx2 = p.invdx2;
    I.dxx0 = p.dxx0;
    I.dt = find_timestep(&p, CFL_FACTOR);
    I.kc = stage_consts(I.dt);
    I.dxx1 = p.dxx1;
    base += 2 * I.ntot;
    tab += (long long)kBatchTab * I.n0 * I.n1;
    b->h_insts.push_back(I);
    for (int t = 0; t < 4; t++)
      for (int i2 = kBatchNG; i2 < I.n2 - kBatchNG; i2++)
        for (int i1 = kBatchNG; i1 < I.n1 - kBatchNG; i1 += TYs[t]) work[t].push_back(BatchWork{i, i2, i1});
    // this instance's boundary map, offset into the packed arrays
    bc_struct bc;
    st = driver_bcstruct(&p, &bc);
    if (st) {
      batch_destroy(b);
      return st;
    }
    std::vector<int> od(bc.total_outer), os(bc.total_outer), id_(bc.total_inner), is(bc.total_inner),
        ip(bc.total_inner);
    st = bcstruct_download(&bc, od.data(), os.data(), id_.data(), is.data(), ip.data());
    bcstruct_freemem(&bc);
    if (st) {
      batch_destroy(b);
      return st;
    }
    if (I.ntot > 0x7fffffffLL) {
      batch_destroy(b);
      set_error("instance %d has more than 2^31 points", i);
      return NRGPU_ERR_SIZE;
    }
    for (int g = 0; g < kBatchNG; g++) {
      for (int d = 0; d < 3; d++) {
        bphase.push_back((int)ba.size());
        for (int k = bc.ob_dir_start[g][d]; k < bc.ob_dir_start[g][d + 1]; k++) {
          ba.push_back(od[k]);
          bb.push_back(os[k]);
        }
      }
      bphase.push_back((int)ba.size());
      for (int k = bc.ib_start[g]; k < bc.ib_start[g] + bc.num_ib_gz_pts[g]; k++) {
        ba.push_back(id_[k]);
        bb.push_back(is[k]);
      }
    }
    bphase.push_back((int)ba.size());  // end of this instance's last phase
    // level template of this shape (built once per distinct shape)
    const long long key = ((long long)I.n0 * 4096 + I.n1) * 4096 + I.n2;
    int tid = (int)(std::find(tpl_key.begin(), tpl_key.end(), key) - tpl_key.begin());
    if (tid == (int)tpl_key.size() && levels_ok) {
      // the sequential order: per layer, outer faces i0, i1, i2, then inner points
      struct Ent {
        int d, e;
        bool inner;
      };
      std::vector<Ent> seq;
      for (int g = 0; g < kBatchNG; g++) {
        for (int k = bc.ob_dir_start[g][0]; k < bc.ob_dir_start[g][3]; k++) seq.push_back({od[k], os[k], false});
        for (int k = bc.ib_start[g]; k < bc.ib_start[g] + bc.num_ib_gz_pts[g]; k++)
          seq.push_back({id_[k], is[k], true});
      }
      std::vector<int> worder(I.ntot, -1), lvl(I.ntot, 0);
      for (int k = 0; k < (int)seq.size(); k++) {
        if (worder[seq[k].d] >= 0) levels_ok = false;  // written twice
        worder[seq[k].d] = k;
      }
      int L = 0;
      for (int k = 0; k < (int)seq.size() && levels_ok; k++) {
        const Ent &en = seq[k];
        int lv = 0;
        const int nsrc = en.inner ? 1 : 3;
        for (int j = 0; j < nsrc; j++) {
          const long long x = en.inner ? en.e : (long long)en.d + (long long)(j + 1) * en.e;
          if (x < 0 || x >= I.ntot) {
            levels_ok = false;
            break;
          }
          if (worder[x] > k) levels_ok = false;        // read before it is written: keep the phases
          else if (worder[x] >= 0) lv = std::max(lv, lvl[x]);
        }
        lvl[en.d] = lv + 1;
        L = std::max(L, lv + 1);
      }
      if (L > kBcMaxLevels) levels_ok = false;
      if (levels_ok) {
        tpl_key.push_back(key);
        std::vector<int> off(kBcOffStride, 0);
        for (int lv = 1; lv <= kBcMaxLevels + 1; lv++) {
          for (int inner = 0; inner < 2; inner++) {
            off[2 * lv + inner] = (int)tpl_a.size();
            if (lv > L) continue;
            for (const Ent &en : seq)
              if (lvl[en.d] == lv && (int)en.inner == inner) {
                tpl_a.push_back(en.d);
                tpl_b.push_back(en.e);
              }
          }
        }
        l1_max = std::max(l1_max, off[4] - off[2]);
        nlev_all = std::max(nlev_all, L);
        tpl_off.insert(tpl_off.end(), off.begin(), off.end());
      }
    }
    b->h_insts.back().pad = tid;
  }
  b->bc_levels = levels_ok && !tpl_key.empty();
  b->bc_nlev = nlev_all;
  b->bc_l1_max = l1_max;
  b->total_points = base;
  auto up = [&](void **dst, const void *src, size_t bytes) -> int {
    *dst = nullptr;
    if (!bytes) return NRGPU_OK;
    NRGPU_CUDA_CHECK(cudaMalloc(dst, bytes));
    NRGPU_CUDA_CHECK(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    return NRGPU_OK;
  };
  int st;
#define NRGPU_BATCH_TRY(x)  \
  if ((st = (x))) {         \
    batch_destroy(b);       \
    return st;              \
  }
  NRGPU_BATCH_TRY(up((void **)&b->d_insts, b->h_insts.data(), b->h_insts.size() * sizeof(BatchInstance)))
  for (int t = 0; t < 4; t++) {
    b->nwork[t] = (int)work[t].size();
    NRGPU_BATCH_TRY(up((void **)&b->d_work[t], work[t].data(), work[t].size() * sizeof(BatchWork)))
  }
  NRGPU_BATCH_TRY(up((void **)&b->d_bc_phases, bphase.data(), bphase.size() * sizeof(int)))
  NRGPU_BATCH_TRY(up((void **)&b->d_bc_a, ba.data(), ba.size() * sizeof(int)))
  NRGPU_BATCH_TRY(up((void **)&b->d_bc_b, bb.data(), bb.size() * sizeof(int)))
  if (b->bc_levels) {
    NRGPU_BATCH_TRY(up((void **)&b->d_tpl_off, tpl_off.data(), tpl_off.size() * sizeof(int)))
    NRGPU_BATCH_TRY(up((void **)&b->d_tpl_a, tpl_a.data(), tpl_a.size() * sizeof(int)))
    NRGPU_BATCH_TRY(up((void **)&b->d_tpl_b, tpl_b.data(), tpl_b.size() * sizeof(int)))
  }
  NRGPU_BATCH_TRY(cudaMalloc(&b->d_tab64, tab * sizeof(double)) == cudaSuccess ? NRGPU_OK : NRGPU_ERR_CUDA)
  NRGPU_BATCH_TRY(cudaMalloc(&b->d_tab32, tab * sizeof(float)) == cudaSuccess ? NRGPU_OK : NRGPU_ERR_CUDA)
#undef NRGPU_BATCH_TRY
  sw_batch_table_kernel<<<dim3(64, ninst), 128, 0, stream()>>>(b->d_insts, ninst, CoordSystem, b->xxmin0, b->xxmin1,
                                                                AMPL, SINHW, b->d_tab64, b->d_tab32);
  if (cudaGetLastError() != cudaSuccess) {
    set_error("batch metric table launch failed");
    batch_destroy(b);
    return NRGPU_ERR_CUDA;
  }
  count_launch();
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->grid = sms * 8;
  *out = b;
  return NRGPU_OK;
}

long long nrgpu_batch_total_points(const nrgpu_batch *b) { return b ? b->total_points : -1; }

int nrgpu_batch_offsets(const nrgpu_batch *b, long long *base, long long *ntot, int *n0n1n2) {
  NRGPU_REQUIRE(b && base && ntot, "NULL argument");
  for (int i = 0; i < b->ninst; i++) {
    base[i] = b->h_insts[i].base;
    ntot[i] = b->h_insts[i].ntot;
    if (n0n1n2) {
      n0n1n2[3 * i] = b->h_insts[i].n0;
      n0n1n2[3 * i + 1] = b->h_insts[i].n1;
      n0n1n2[3 * i + 2] = b->h_insts[i].n2;
    }
  }
  return NRGPU_OK;
}

int nrgpu_batch_set_tile(nrgpu_batch *b, int tx, int ty, int grid) {
  NRGPU_REQUIRE(b, "NULL batch");
  int tyi = ty == 1 ? 0 : ty == 2 ? 1 : ty == 4 ? 2 : ty == 8 ? 3 : -1;
  NRGPU_REQUIRE(tyi >= 0, "TY must be 1, 2, 4 or 8");
  NRGPU_REQUIRE((tx == 32 && ty <= 8) || (tx == 64 && ty <= 4) || (tx == 128 && ty <= 2),
                "tile %dx%d not built (TX in {32,64,128}, TX*TY <= 256)", tx, ty);
  NRGPU_REQUIRE(grid >= 1, "grid must be positive");
  b->tx = tx;
  b->tyi = tyi;
  b->grid = grid;
  return NRGPU_OK;
}

int nrgpu_batch_get_tile(const nrgpu_batch *b, int *tx, int *ty, int *grid) {
  NRGPU_REQUIRE(b && tx && ty && grid, "NULL argument");
  const int TYs[4] = {1, 2, 4, 8};
  *tx = b->tx;
  *ty = TYs[b->tyi];
  *grid = b->grid;
  return NRGPU_OK;
}

int nrgpu_batch_timesteps(const nrgpu_batch *b, double *dt) {
  NRGPU_REQUIRE(b && dt, "NULL argument");
  for (int i = 0; i < b->ninst; i++) dt[i] = b->h_insts[i].dt;
  return NRGPU_OK;
}

int nrgpu_batch_set_timesteps(nrgpu_batch *b, const double *dt) {
  NRGPU_REQUIRE(b && dt, "NULL argument");
  for (int i = 0; i < b->ninst; i++) {
    NRGPU_REQUIRE(dt[i] > 0.0 && isfinite(dt[i]), "time step of instance %d is not positive", i);
    b->h_insts[i].dt = dt[i];
  }
  NRGPU_CUDA_CHECK(cudaMemcpy(b->d_insts, b->h_insts.data(), b->h_insts.size() * sizeof(BatchInstance),
                              cudaMemcpyHostToDevice));
  return NRGPU_OK;
}

// Times the RHS launch (plain store into rhs_scratch) for every built tile
// shape and several persistent grid sizes; keeps the fastest.
int nrgpu_batch_autotune(nrgpu_batch *b, const void *in, void *rhs_scratch, int reps, float *best_ms) {
  NRGPU_REQUIRE(b && in && rhs_scratch && reps >= 1, "bad arguments");
  const int shapes[][2] = {{32, 1}, {32, 2}, {32, 4}, {32, 8}, {64, 1}, {64, 2}, {64, 4}, {128, 1}, {128, 2}};
  const int mult[] = {2, 4, 8, 16, 32};
  int dev = 0, sms = 152;
  NRGPU_CUDA_CHECK(cudaGetDevice(&dev));
  NRGPU_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaEvent_t e0, e1;
  NRGPU_CUDA_CHECK(cudaEventCreate(&e0));
  NRGPU_CUDA_CHECK(cudaEventCreate(&e1));
  const bool f64 = b->prec == NRGPU_PREC_FP64;
  float best = 1e30f;
  int btx = b->tx, btyi = b->tyi, bgrid = b->grid, st = NRGPU_OK;
  for (const auto &sh : shapes) {
    for (int m : mult) {
      if ((st = nrgpu_batch_set_tile(b, sh[0], sh[1], m * sms))) break;
      if ((st = batch_launch_rhs(b, in, f64, -1, nullptr, nullptr, rhs_scratch))) break;  // warm-up
      cudaEventRecord(e0, stream());
      for (int r = 0; r < reps && st == NRGPU_OK; r++)
        st = batch_launch_rhs(b, in, f64, -1, nullptr, nullptr, rhs_scratch);
      cudaEventRecord(e1, stream());
      if (st) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) { st = NRGPU_ERR_CUDA; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      if (ms < best) {
        best = ms;
        btx = b->tx;
        btyi = b->tyi;
        bgrid = b->grid;
      }
    }
    if (st) break;
  }
  // boundary-condition block size, timed on the scratch buffer's ghost points
  float best_bc = 1e30f;
  int bthreads = b->bc_threads;
  for (int threads : {128, 256, 512, 1024}) {
    if (st) break;
    b->bc_threads = threads;
    auto bcs = [&]() {
      if (b->prec == NRGPU_PREC_FP64) return batch_bcs<double>(b, (double *)rhs_scratch);
      if (b->prec == NRGPU_PREC_COMPENSATED) return batch_bcs<float2>(b, (float2 *)rhs_scratch);
      return batch_bcs<float>(b, (float *)rhs_scratch);
    };
    if ((st = bcs())) break;
    cudaEventRecord(e0, stream());
    for (int r = 0; r < reps && st == NRGPU_OK; r++) st = bcs();
    cudaEventRecord(e1, stream());
    if (st) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) { st = NRGPU_ERR_CUDA; break; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms / reps < best_bc) {
      best_bc = ms / reps;
      bthreads = threads;
    }
  }
  b->bc_threads = bthreads;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->tx = btx;
  b->tyi = btyi;
  b->grid = bgrid;
  if (st) return st;
  if (best_ms) *best_ms = best;
  return NRGPU_OK;
}

int nrgpu_batch_initial_data_gaussian(nrgpu_batch *b, const double *A, const double *r0, const double *w,
                                      double *y_n) {
  NRGPU_REQUIRE(b && A && r0 && w && y_n, "NULL argument");
  double *d = nullptr;
  const size_t n = (size_t)b->ninst;
  NRGPU_CUDA_CHECK(cudaMalloc(&d, 3 * n * sizeof(double)));
  NRGPU_CUDA_CHECK(cudaMemcpy(d, A, n * sizeof(double), cudaMemcpyHostToDevice));
  NRGPU_CUDA_CHECK(cudaMemcpy(d + n, r0, n * sizeof(double), cudaMemcpyHostToDevice));
  NRGPU_CUDA_CHECK(cudaMemcpy(d + 2 * n, w, n * sizeof(double), cudaMemcpyHostToDevice));
  sw_batch_gaussian_kernel<<<dim3(64, b->ninst), 128, 0, stream()>>>(b->d_insts, b->ninst, b->cs, b->xxmin0, b->AMPL,
                                                                     b->SINHW, d, d + n, d + 2 * n, y_n);
  cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(stream());
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error("gaussian initial data: %s", cudaGetErrorString(e));
    return NRGPU_ERR_CUDA;
  }
  count_launch();
  return NRGPU_OK;
}

int nrgpu_batch_rhs_eval(nrgpu_batch *b, const void *in, void *rhs) {
  NRGPU_REQUIRE(b && in && rhs, "NULL argument");
  return batch_launch_rhs(b, in, b->prec == NRGPU_PREC_FP64, -1, nullptr, nullptr, rhs);  // compensated: pairs
}

int nrgpu_batch_apply_bcs(nrgpu_batch *b, void *gfs, int kind) {
  NRGPU_REQUIRE(b && gfs, "NULL argument");
  NRGPU_REQUIRE(kind >= 0 && kind <= 2, "kind must be 0 (float), 1 (double) or 2 (float2 pairs)");
  if (kind == 1) return batch_bcs<double>(b, (double *)gfs);
  if (kind == 2) return batch_bcs<float2>(b, (float2 *)gfs);
  return batch_bcs<float>(b, (float *)gfs);
}

int nrgpu_batch_step(nrgpu_batch *b, MoL_gridfunctions *gfs) {
  NRGPU_REQUIRE(b && gfs && gfs->y_n_gfs && gfs->y_nplus1_running_total_gfs && gfs->k_odd_gfs && gfs->k_even_gfs,
                "NULL argument");
  NRGPU_REQUIRE(gfs->precision == b->prec, "buffers' precision differs from the batch's");
  const bool f64 = b->prec == NRGPU_PREC_FP64, pair = b->prec == NRGPU_PREC_COMPENSATED;
  void *kbuf[2] = {gfs->k_odd_gfs, gfs->k_even_gfs};
  int st;
  if (!f64) {  // y_n -> pairs in place (+ FP32 copy in k_even for plain FP32 stages)
    const int blocks = (int)std::min<long long>((b->total_points + 255) / 256, 152LL * 16);
    if (pair)
      split_state_kernel<false><<<blocks, 256, 0, stream()>>>(b->total_points, gfs->y_n_gfs, nullptr);
    else
      split_state_kernel<true><<<blocks, 256, 0, stream()>>>(b->total_points, gfs->y_n_gfs,
                                                               (float *)gfs->k_even_gfs);
    NRGPU_LAUNCH_CHECK();
  }
  for (int s = 0; s < 4; s++) {
    // substep 0 input: y_n (FP64), its pairs in place (compensated), its FP32 copy (mixed)
    const void *in = (s == 0) ? (f64 || pair ? (const void *)gfs->y_n_gfs : gfs->k_even_gfs) : kbuf[(s + 1) % 2];
    const bool in_f64 = f64;
    void *out = (s == 3) ? nullptr : kbuf[s % 2];
    if ((st = batch_launch_rhs(b, in, in_f64, s, gfs->y_n_gfs, gfs->y_nplus1_running_total_gfs, out))) return st;
    void *post = (s == 3) ? (void *)gfs->y_n_gfs : kbuf[s % 2];
    if (s == 3 || f64) st = batch_bcs<double>(b, (double *)post);
    else if (pair) st = batch_bcs<float2>(b, (float2 *)post);
    else st = batch_bcs<float>(b, (float *)post);
    if (st) return st;
  }
  return NRGPU_OK;
}

int nrgpu_batch_free(nrgpu_batch *b) {
  batch_destroy(b);
  return NRGPU_OK;
}

}  // extern "C"
