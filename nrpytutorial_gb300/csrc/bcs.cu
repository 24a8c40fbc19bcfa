// bcs.cu -- curvilinear boundary conditions.
//
// Map construction (host, once per grid) follows
// CurviBoundaryConditions/boundary_conditions/set_up__bc_gz_map_and_parity_condns.h:7-113
// and set_bcstruct.h:32-124:
//  * every point of the eigen-coordinate grid is mapped to Cartesian and back
//    (EigenCoord_xx_to_Cart / EigenCoord_Cart_to_xx); if the returned index
//    differs from the point's own, the point is an inner (parity) boundary
//    point that copies from that interior index, else an outer point (or
//    interior);
//  * parities are dot products of the unit vectors at the two points
//    (CurviBoundaryConditions.py:80-113), rank-2 types as products;
//  * ghost layers are visited innermost first; within a layer the outer
//    points are listed face by face (i0 min, i0 max, i1 min, i1 max, i2 min,
//    i2 max) with the box widened after each face, then the inner points in
//    the same face order.
// Application (apply_bcs_curvilinear.h:7-64) runs per layer: the i0 faces,
// then the i1 faces (which read the i0 ghost columns just written), then the
// i2 faces, then the inner points.  Each of those four phases is one launch
// covering all gridfunctions; inside a phase no point reads another's output.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "fd.cuh"
#include "rfm.cuh"

namespace nrgpu {

// b: bScale of the SymTP eigen-coordinates (unused by the others).
static void eigen_xx_to_cart(int cs, double b, double x0, double x1, double x2, double out[3]) {
  if (cs == NRGPU_COORD_CARTESIAN) {
    out[0] = x0; out[1] = x1; out[2] = x2;
    return;
  }
  if (cs == NRGPU_COORD_SYMTP) {  // reference_metric.py:334-336 with AA = xx0
    out[0] = x0 * sin(x1) * cos(x2);
    out[1] = x0 * sin(x1) * sin(x2);
    out[2] = sqrt(x0 * x0 + b * b) * cos(x1);
    return;
  }
  if (cs == NRGPU_COORD_CYLINDRICAL) {  // reference_metric.py:296-298
    out[0] = x0 * cos(x1);
    out[1] = x0 * sin(x1);
    out[2] = x2;
    return;
  }
  // Spherical eigen-coordinates (reference_metric.py:163-166)
  out[0] = x0 * sin(x1) * cos(x2);
  out[1] = x0 * sin(x1) * sin(x2);
  out[2] = x0 * cos(x1);
}

static void eigen_cart_to_xx(int cs, double b, const double c[3], double out[3]) {
  if (cs == NRGPU_COORD_CARTESIAN) {
    out[0] = c[0]; out[1] = c[1]; out[2] = c[2];
    return;
  }
  if (cs == NRGPU_COORD_SYMTP) {  // reference_metric.py:348-366
    const double r = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    const double cth = c[2] / r, b2 = b * b, r2 = r * r;
    const double root = sqrt(b2 * b2 + 2.0 * b2 * r2 + r2 * r2 - 4.0 * b2 * r2 * cth * cth);
    const double sgn = c[2] > 0.0 ? 1.0 : (c[2] < 0.0 ? -1.0 : 0.0);
    out[0] = sqrt(-b2 + r2 + root) * M_SQRT1_2;
    out[1] = acos(sgn * sqrt(1.0 + r2 / b2 - root / b2) * M_SQRT1_2);
    out[2] = atan2(c[1], c[0]);
    return;
  }
  if (cs == NRGPU_COORD_CYLINDRICAL) {  // reference_metric.py:240-242
    out[0] = sqrt(c[0] * c[0] + c[1] * c[1]);
    out[1] = atan2(c[1], c[0]);
    out[2] = c[2];
    return;
  }
  // reference_metric.py:113-115
  const double r = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  out[0] = r;
  out[1] = acos(c[2] / r);
  out[2] = atan2(c[1], c[0]);
}

// Unit vectors (rows) of the eigen-coordinate basis at (x0,x1,x2)
// (reference_metric.py:180-182 for the Spherical family, :300-302 for the
// Cylindrical family with phi = x1, :373-379 for SymTP; identity otherwise).
static void unit_vectors(int cs, double b, double x0, double x1, double x2, double U[3][3]) {
  if (cs == NRGPU_COORD_CARTESIAN) {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) U[i][j] = (i == j) ? 1.0 : 0.0;
    return;
  }
  if (cs == NRGPU_COORD_SYMTP) {
    const double st = sin(x1), ct = cos(x1), sp = sin(x2), cp = cos(x2);
    const double v1 = sqrt(x0 * x0 + b * b * st * st), v2 = sqrt(x0 * x0 + b * b);
    U[0][0] = st * cp * v2 / v1; U[0][1] = st * sp * v2 / v1; U[0][2] = x0 * ct / v1;
    U[1][0] = x0 * ct * cp / v1; U[1][1] = x0 * ct * sp / v1; U[1][2] = -st * v2 / v1;
    U[2][0] = -sp;               U[2][1] = cp;               U[2][2] = 0.0;
    return;
  }
  if (cs == NRGPU_COORD_CYLINDRICAL) {
    const double sp = sin(x1), cp = cos(x1);
    U[0][0] = cp;  U[0][1] = sp;  U[0][2] = 0.0;
    U[1][0] = -sp; U[1][1] = cp;  U[1][2] = 0.0;
    U[2][0] = 0.0; U[2][1] = 0.0; U[2][2] = 1.0;
    return;
  }
  const double st = sin(x1), ct = cos(x1), sp = sin(x2), cp = cos(x2);
  U[0][0] = st * cp; U[0][1] = st * sp; U[0][2] = ct;
  U[1][0] = ct * cp; U[1][1] = ct * sp; U[1][2] = -st;
  U[2][0] = -sp;     U[2][1] = cp;      U[2][2] = 0.0;
}

struct GzMap {
  int i0, i1, i2;    // -1 => not an inner boundary point
  int parity_bits;   // bit t set <=> parity type t is -1
};

static int build_gz_map(const paramstruct *p, std::vector<GzMap> &map) {
  // Eigen-coordinate grid: same Nxx and NGHOSTS, eigen domain.
  paramstruct e = *p;
  const int Nxx[3] = {p->Nxx0, p->Nxx1, p->Nxx2};
  std::vector<double> xs[3];
  const int np[3] = {p->Nxx_plus_2NGHOSTS0, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2};
  double *xxp[3];
  for (int d = 0; d < 3; d++) {
    xs[d].resize(np[d]);
    xxp[d] = xs[d].data();
  }
  // The map is invariant under the eigen grid's radial / z extent; a
  // zero-initialised extent parameter (not read by this CoordSystem itself)
  // gets a unit extent instead of a degenerate grid.
  if (!(e.RMAX > 0.0)) e.RMAX = 1.0;
  if (!(e.RHOMAX > 0.0)) e.RHOMAX = 1.0;
  if (!(e.ZMAX > e.ZMIN)) e.ZMIN = -1.0, e.ZMAX = 1.0;
  if (!(e.AMAX > 0.0)) e.AMAX = 1.0;
  int st = set_Nxx_dxx_invdx_params__and__xx(1, Nxx, &e, xxp);
  if (st) return st;
  const int cs = p->CoordSystem == NRGPU_COORD_CARTESIAN     ? NRGPU_COORD_CARTESIAN
                 : cylindrical_family(p->CoordSystem) ? NRGPU_COORD_CYLINDRICAL
                 : symtp_family(p->CoordSystem)       ? NRGPU_COORD_SYMTP
                                                      : NRGPU_COORD_SPHERICAL;
  const int ng = p->NGHOSTS;
  const double dxx[3] = {e.dxx0, e.dxx1, e.dxx2};
  // set_up__bc_gz_map_and_parity_condns.h:17-19 recovers xxmin from xx[d][0].
  double xxmin[3];
  for (int d = 0; d < 3; d++) xxmin[d] = xs[d][0] - ((double)(0 - ng) + (1.0 / 2.0)) * dxx[d];
  map.assign((size_t)np[0] * np[1] * np[2], GzMap{-1, -1, -1, 0});
  for (int i2 = 0; i2 < np[2]; i2++)
    for (int i1 = 0; i1 < np[1]; i1++)
      for (int i0 = 0; i0 < np[0]; i0++) {
        double c[3], xin[3], c2[3];
        eigen_xx_to_cart(cs, e.bScale, xs[0][i0], xs[1][i1], xs[2][i2], c);
        eigen_cart_to_xx(cs, e.bScale, c, xin);
        int ib[3];
        for (int d = 0; d < 3; d++)
          ib[d] = (int)((xin[d] - xxmin[d] - (1.0 / 2.0) * dxx[d] + ((double)ng) * dxx[d]) / dxx[d] + 0.5);
        for (int d = 0; d < 3; d++)
          if (ib[d] < 0 || ib[d] >= np[d]) {
            set_error("ghost-zone map: point (%d,%d,%d) maps outside the grid", i0, i1, i2);
            return NRGPU_ERR_BCMAP;
          }
        eigen_xx_to_cart(cs, e.bScale, xs[0][ib[0]], xs[1][ib[1]], xs[2][ib[2]], c2);
        for (int d = 0; d < 3; d++)
          if (fabs(c[d] - c2[d]) > 1e-8) {
            set_error("Cartesian disagreement at (%d,%d,%d): (%.15e %.15e %.15e) != (%.15e %.15e %.15e)",
                      i0, i1, i2, c[0], c[1], c[2], c2[0], c2[1], c2[2]);
            return NRGPU_ERR_BCMAP;
          }
        const size_t idx = (size_t)i0 + (size_t)np[0] * ((size_t)i1 + (size_t)np[1] * i2);
        if (ib[0] == i0 && ib[1] == i1 && ib[2] == i2) continue;
        double U[3][3], Ui[3][3], par[10];
        unit_vectors(cs, e.bScale, xs[0][i0], xs[1][i1], xs[2][i2], U);
        unit_vectors(cs, e.bScale, xs[0][ib[0]], xs[1][ib[1]], xs[2][ib[2]], Ui);
        par[0] = 1.0;
        for (int t = 1; t <= 3; t++) {
          par[t] = 0.0;
          for (int i = 0; i < 3; i++) par[t] += U[t - 1][i] * Ui[t - 1][i];
        }
        int cnt = 4;
        for (int i = 0; i < 3; i++)
          for (int j = i; j < 3; j++) par[cnt++] = par[i + 1] * par[j + 1];
        int bits = 0;
        for (int t = 0; t < 10; t++) {
          if ((par[t] > 0 && fabs(par[t] - 1.0) > 1e-8) || (par[t] <= 0 && fabs(par[t] + 1.0) > 1e-8)) {
            set_error("parity %d evaluated to %e at (%d,%d,%d), not +-1", t, par[t], i0, i1, i2);
            return NRGPU_ERR_BCMAP;
          }
          if (par[t] < 0.0) bits |= (1 << t);
        }
        map[idx] = GzMap{ib[0], ib[1], ib[2], bits};
      }
  return NRGPU_OK;
}

// ------------------------------------------------------------------ kernels
struct ParityTypes {
  int8_t t[64];
};

template <typename T>
__global__ void bc_outer_kernel(const int *__restrict__ dest, const int *__restrict__ step, int npts,
                                int ngfs, long long ntot, T *gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  T *f = gfs + (long long)gf * ntot;
  const long long d = dest[p], s = step[p];
  // +3 f1 - 3 f2 + 1 f3, left to right without contraction (BC_UPDATE_OUTER).
  const T a = f[d + s], b = f[d + 2 * s], c = f[d + 3 * s];
  T v;
  if constexpr (sizeof(T) == 8) {
    v = __dadd_rn(__dsub_rn(__dmul_rn(3.0, a), __dmul_rn(3.0, b)), c);
  } else {
    v = __fadd_rn(__fsub_rn(__fmul_rn(3.0f, a), __fmul_rn(3.0f, b)), c);
  }
  f[d] = v;
}

template <typename T>
__global__ void bc_inner_kernel(const int *__restrict__ dest, const int *__restrict__ src,
                                const int *__restrict__ parity, int npts, int ngfs, long long ntot,
                                ParityTypes types, T *gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  T *f = gfs + (long long)gf * ntot;
  const bool neg = (parity[p] >> types.t[gf]) & 1;
  const T v = f[src[p]];
  f[dest[p]] = neg ? -v : v;
}

// Point-major exchange buffers of the slab path: buf[j * ngfs + gf].
__global__ void bc_gather_kernel(const int *__restrict__ src, int npts, int ngfs, long long ntot,
                                 const double *__restrict__ gfs, double *__restrict__ buf) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  buf[(long long)p * ngfs + gf] = gfs[(long long)gf * ntot + src[p]];
}

__global__ void bc_scatter_parity_kernel(const int *__restrict__ dest, const int *__restrict__ parity, int npts,
                                         int ngfs, long long ntot, ParityTypes types,
                                         const double *__restrict__ buf, double *__restrict__ gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  const bool neg = (parity[p] >> types.t[gf]) & 1;
  const double v = buf[(long long)p * ngfs + gf];
  gfs[(long long)gf * ntot + dest[p]] = neg ? -v : v;
}

// FP32 pair gridfunctions (value = hi + lo): the outer rule evaluated in
// FP64 on the values and re-split; the parity copy moves (or negates) both
// parts, which is exact.
__global__ void bc_outer_pair_kernel(const int *__restrict__ dest, const int *__restrict__ step, int npts,
                                     int ngfs, long long ntot, float2 *gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  float2 *f = gfs + (long long)gf * ntot;
  const long long d = dest[p], s = step[p];
  // 3 f1 - 3 f2 + f3 in float-float arithmetic (FP32 pipe; ~48 significant bits)
  const float2 a = ff_mul(3.0f, f[d + s]), b = ff_mul(3.0f, f[d + 2 * s]);
  f[d] = ff_add(ff_add(a, ff_neg(b)), f[d + 3 * s]);
}

__global__ void bc_inner_pair_kernel(const int *__restrict__ dest, const int *__restrict__ src,
                                     const int *__restrict__ parity, int npts, int ngfs, long long ntot,
                                     ParityTypes types, float2 *gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  float2 *f = gfs + (long long)gf * ntot;
  const bool neg = (parity[p] >> types.t[gf]) & 1;
  const float2 v = f[src[p]];
  f[dest[p]] = neg ? make_float2(-v.x, -v.y) : v;
}

// ------------------------------------------------- level-scheduled application
// One entry of the schedule: an outer point (3 f1 - 3 f2 + f3 along its step,
// the same arithmetic as bc_outer_kernel / bc_outer_pair_kernel) or an inner
// point (parity copy).
template <typename T> __device__ __forceinline__ T bc_outer_value(T f1, T f2, T f3) {
  if constexpr (std::is_same<T, double>::value) {
    return __dadd_rn(__dsub_rn(__dmul_rn(3.0, f1), __dmul_rn(3.0, f2)), f3);
  } else if constexpr (std::is_same<T, float>::value) {
    return __fadd_rn(__fsub_rn(__fmul_rn(3.0f, f1), __fmul_rn(3.0f, f2)), f3);
  } else {
    const float2 x = ff_mul(3.0f, f1), y = ff_mul(3.0f, f2);
    return ff_add(ff_add(x, ff_neg(y)), f3);
  }
}
template <typename T> __device__ __forceinline__ T bc_parity_value(T v, bool neg) {
  if constexpr (std::is_same<T, float2>::value) return neg ? make_float2(-v.x, -v.y) : v;
  else return neg ? -v : v;
}
template <typename T>
__device__ __forceinline__ void bc_entry(T *f, long long d, long long a, int bits, bool inner, int type) {
  if (inner) f[d] = bc_parity_value(f[a], (bits >> type) & 1);
  else f[d] = bc_outer_value(f[d + a], f[d + 2 * a], f[d + 3 * a]);
}

// One level: one thread per entry over a chunk of gridfunctions (the entry's
// indices are read once).  Within a level no entry reads another's
// destination, so the chunk's loads are all issued before its stores.
constexpr int kBcGfChunk = 6;  // gridfunctions per thread (blockIdx.y picks the chunk)
template <typename T>
__global__ void bc_level_kernel(const int *__restrict__ dest, const int *__restrict__ arg,
                                const int *__restrict__ par, int start, int inner_start, int end, int ngfs,
                                long long ntot, ParityTypes types, T *gfs) {
  const int p = start + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= end) return;
  const long long d = dest[p], a = arg[p];
  const int bits = par[p];
  const int g0 = blockIdx.y * kBcGfChunk, n = min(ngfs - g0, kBcGfChunk);
  T *f0 = gfs + (long long)g0 * ntot;
  if (p >= inner_start) {
    T v[kBcGfChunk];
#pragma unroll
    for (int k = 0; k < kBcGfChunk; k++)
      if (k < n) v[k] = f0[(long long)k * ntot + a];
#pragma unroll
    for (int k = 0; k < kBcGfChunk; k++)
      if (k < n) f0[(long long)k * ntot + d] = bc_parity_value(v[k], (bits >> types.t[g0 + k]) & 1);
  } else {
    T v1[kBcGfChunk], v2[kBcGfChunk], v3[kBcGfChunk];
#pragma unroll
    for (int k = 0; k < kBcGfChunk; k++) {
      if (k < n) {
        const T *f = f0 + (long long)k * ntot + d;
        v1[k] = f[a];
        v2[k] = f[2 * a];
        v3[k] = f[3 * a];
      }
    }
#pragma unroll
    for (int k = 0; k < kBcGfChunk; k++)
      if (k < n) f0[(long long)k * ntot + d] = bc_outer_value(v1[k], v2[k], v3[k]);
  }
}

// The small trailing levels: one block per gridfunction, a block barrier
// between levels.
struct LevelTable {
  int start[NRGPU_MAX_BC_LEVELS + 1], inner[NRGPU_MAX_BC_LEVELS];
};
template <typename T>
__global__ void bc_tail_kernel(const int *__restrict__ dest, const int *__restrict__ arg,
                               const int *__restrict__ par, LevelTable lt, int l0, int nlev, long long ntot,
                               ParityTypes types, T *gfs) {
  const int gf = blockIdx.x;
  T *f = gfs + (long long)gf * ntot;
  for (int l = l0; l < nlev; l++) {
    for (int p = lt.start[l] + threadIdx.x; p < lt.start[l + 1]; p += blockDim.x)
      bc_entry(f, dest[p], arg[p], par[p], p >= lt.inner[l], types.t[gf]);
    __syncthreads();
  }
}

template <typename T>
static int apply_bcs_levels(const bc_struct *bc, int NUM_GFS, long long ntot, const ParityTypes &types, T *gfs) {
  const int B = 128;
  for (int l = 0; l < bc->lev_tail; l++) {
    const int n = bc->lev_start[l + 1] - bc->lev_start[l];
    if (n <= 0) continue;
    dim3 grid((n + B - 1) / B, (NUM_GFS + kBcGfChunk - 1) / kBcGfChunk);
    bc_level_kernel<T><<<grid, B, 0, stream()>>>(bc->lev_dest, bc->lev_arg, bc->lev_parity, bc->lev_start[l],
                                                 bc->lev_inner[l], bc->lev_start[l + 1], NUM_GFS, ntot, types, gfs);
    NRGPU_LAUNCH_CHECK();
  }
  if (bc->lev_tail < bc->nlev) {
    LevelTable lt;
    memcpy(lt.start, bc->lev_start, sizeof(lt.start));
    memcpy(lt.inner, bc->lev_inner, sizeof(lt.inner));
    bc_tail_kernel<T><<<NUM_GFS, 1024, 0, stream()>>>(bc->lev_dest, bc->lev_arg, bc->lev_parity, lt, bc->lev_tail,
                                                     bc->nlev, ntot, types, gfs);
    NRGPU_LAUNCH_CHECK();
  }
  return NRGPU_OK;
}

template <typename T>
int apply_bcs_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS,
                          const int8_t *gfs_parity, T *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(bc != nullptr && gfs != nullptr, "NULL argument");
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64, "NUM_GFS %d out of range", NUM_GFS);
  NRGPU_REQUIRE(bc->NGHOSTS == p->NGHOSTS, "bcstruct built for NGHOSTS=%d, params say %d", bc->NGHOSTS,
                p->NGHOSTS);
  ParityTypes types;
  memset(&types, 0, sizeof(types));
  for (int g = 0; g < NUM_GFS; g++) {
    const int t = gfs_parity ? gfs_parity[g] : 0;
    NRGPU_REQUIRE(t >= 0 && t <= 9, "parity type %d of gf %d not in 0..9", t, g);
    types.t[g] = (int8_t)t;
  }
  const long long ntot = (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  if (bc->nlev > 0) return apply_bcs_levels<T>(bc, NUM_GFS, ntot, types, gfs);
  const int B = 128;
  for (int g = 0; g < bc->NGHOSTS; g++) {
    for (int d = 0; d < 3; d++) {
      const int a = bc->ob_dir_start[g][d], b = bc->ob_dir_start[g][d + 1];
      const int n = b - a;
      if (n <= 0) continue;
      dim3 grid((n + B - 1) / B, NUM_GFS);
      bc_outer_kernel<T><<<grid, B, 0, stream()>>>(bc->outer_dest + a, bc->outer_step + a, n, NUM_GFS, ntot, gfs);
      NRGPU_LAUNCH_CHECK();
    }
    const int n = bc->num_ib_gz_pts[g];
    if (n > 0) {
      const int a = bc->ib_start[g];
      dim3 grid((n + B - 1) / B, NUM_GFS);
      bc_inner_kernel<T><<<grid, B, 0, stream()>>>(bc->inner_dest + a, bc->inner_src + a,
                                                   bc->inner_parity + a, n, NUM_GFS, ntot, types, gfs);
      NRGPU_LAUNCH_CHECK();
    }
  }
  return NRGPU_OK;
}

int apply_bcs_pair_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity,
                        float2 *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(bc != nullptr && gfs != nullptr, "NULL argument");
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64, "NUM_GFS %d out of range", NUM_GFS);
  NRGPU_REQUIRE(bc->NGHOSTS == p->NGHOSTS, "bcstruct built for NGHOSTS=%d, params say %d", bc->NGHOSTS,
                p->NGHOSTS);
  ParityTypes types;
  memset(&types, 0, sizeof(types));
  for (int g = 0; g < NUM_GFS; g++) {
    const int t = gfs_parity ? gfs_parity[g] : 0;
    NRGPU_REQUIRE(t >= 0 && t <= 9, "parity type %d of gf %d not in 0..9", t, g);
    types.t[g] = (int8_t)t;
  }
  const long long ntot = (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  if (bc->nlev > 0) return apply_bcs_levels<float2>(bc, NUM_GFS, ntot, types, gfs);
  const int B = 128;
  for (int g = 0; g < bc->NGHOSTS; g++) {
    for (int d = 0; d < 3; d++) {
      const int a = bc->ob_dir_start[g][d], b = bc->ob_dir_start[g][d + 1];
      const int n = b - a;
      if (n <= 0) continue;
      dim3 grid((n + B - 1) / B, NUM_GFS);
      bc_outer_pair_kernel<<<grid, B, 0, stream()>>>(bc->outer_dest + a, bc->outer_step + a, n, NUM_GFS, ntot, gfs);
      NRGPU_LAUNCH_CHECK();
    }
    const int n = bc->num_ib_gz_pts[g];
    if (n > 0) {
      const int a = bc->ib_start[g];
      dim3 grid((n + B - 1) / B, NUM_GFS);
      bc_inner_pair_kernel<<<grid, B, 0, stream()>>>(bc->inner_dest + a, bc->inner_src + a, bc->inner_parity + a,
                                                     n, NUM_GFS, ntot, types, gfs);
      NRGPU_LAUNCH_CHECK();
    }
  }
  return NRGPU_OK;
}

// ------------------------------------------------------------- adjoint
// Transpose of apply_bcs_curvilinear (FP64): the phases in reverse order;
// each ghost point hands its adjoint to the points it was computed from and
// is zeroed.  Sources are updated with atomicAdd (several ghost points of a
// parity phase can share a source; the outer faces of one phase never do,
// so Cartesian grids give the same bits every run).
__global__ void bc_outer_adjoint_kernel(const int *__restrict__ dest, const int *__restrict__ step, int npts,
                                        int ngfs, long long ntot, double *gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  double *f = gfs + (long long)gf * ntot;
  const long long d = dest[p], s = step[p];
  const double v = f[d];
  f[d] = 0.0;
  atomicAdd(f + d + s, 3.0 * v);
  atomicAdd(f + d + 2 * s, -3.0 * v);
  atomicAdd(f + d + 3 * s, v);
}

__global__ void bc_inner_adjoint_kernel(const int *__restrict__ dest, const int *__restrict__ src,
                                        const int *__restrict__ parity, int npts, int ngfs, long long ntot,
                                        ParityTypes types, double *gfs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  double *f = gfs + (long long)gf * ntot;
  const bool neg = (parity[p] >> types.t[gf]) & 1;
  const double v = f[dest[p]];
  f[dest[p]] = 0.0;
  atomicAdd(f + src[p], neg ? -v : v);
}

int apply_bcs_adjoint_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity,
                           double *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(bc != nullptr && gfs != nullptr, "NULL argument");
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64, "NUM_GFS %d out of range", NUM_GFS);
  NRGPU_REQUIRE(bc->NGHOSTS == p->NGHOSTS, "bcstruct built for NGHOSTS=%d, params say %d", bc->NGHOSTS,
                p->NGHOSTS);
  ParityTypes types;
  memset(&types, 0, sizeof(types));
  for (int g = 0; g < NUM_GFS; g++) {
    const int t = gfs_parity ? gfs_parity[g] : 0;
    NRGPU_REQUIRE(t >= 0 && t <= 9, "parity type %d of gf %d not in 0..9", t, g);
    types.t[g] = (int8_t)t;
  }
  const long long ntot = (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  const int B = 128;
  for (int g = bc->NGHOSTS - 1; g >= 0; g--) {
    const int n = bc->num_ib_gz_pts[g];
    if (n > 0) {
      const int a = bc->ib_start[g];
      dim3 grid((n + B - 1) / B, NUM_GFS);
      bc_inner_adjoint_kernel<<<grid, B, 0, stream()>>>(bc->inner_dest + a, bc->inner_src + a,
                                                        bc->inner_parity + a, n, NUM_GFS, ntot, types, gfs);
      NRGPU_LAUNCH_CHECK();
    }
    for (int d = 2; d >= 0; d--) {
      const int a = bc->ob_dir_start[g][d], b = bc->ob_dir_start[g][d + 1];
      const int m = b - a;
      if (m <= 0) continue;
      dim3 grid((m + B - 1) / B, NUM_GFS);
      bc_outer_adjoint_kernel<<<grid, B, 0, stream()>>>(bc->outer_dest + a, bc->outer_step + a, m, NUM_GFS, ntot,
                                                        gfs);
      NRGPU_LAUNCH_CHECK();
    }
  }
  return NRGPU_OK;
}

template int apply_bcs_impl<double>(const paramstruct *, const bc_struct *, int, const int8_t *, double *);
template int apply_bcs_impl<float>(const paramstruct *, const bc_struct *, int, const int8_t *, float *);

// ----------------------------------------------------------- Sommerfeld
// CurviBoundaryConditions.py:259-658 (apply_bcs_sommerfeld): on the RHS at
// every outer ghost point, rhs = -c (d_r f + (f - f_inf)/r), plus for a radial
// falloff power n > 0 the correction (rhs(o) + c (d_r f(o) + (f(o) -
// f_inf)/r(o))) (r(o)/r)^n from the point o one step inward along the face
// normal.  d_r f = sum_i d_i f dx^i/dr with d_i f one-sided (shifted into the
// grid along the face normal, or away from the array edge) or centred, at the
// FD order of the Sommerfeld parameters (2, 4 or 6).  Inner ghost points copy
// the RHS with parity.  FP64.
struct SommerfeldParams {
  int fd_order;
  double speed[64], f_inf[64], falloff[64];
};
static SommerfeldParams g_somm = [] {
  SommerfeldParams s{};
  s.fd_order = 2;
  for (int g = 0; g < 64; g++) {
    s.speed[g] = 1.0;
    s.f_inf[g] = 0.0;
    s.falloff[g] = 3.0;
  }
  return s;
}();

struct SommerfeldGeom {
  int cs, n[3], ng;
  double xxmin[3], dxx[3], invdx[3], AMPL, SINHW, const_dr;
  CoordParams c;
  const double *xx[3];  // caller's coordinates, or NULL: cell-centred from xxmin/dxx
};

__device__ __forceinline__ double somm_xx(const SommerfeldGeom &G, int d, int i) {
  return G.xx[d] ? G.xx[d][i] : xx_of(G.xxmin[d], G.dxx[d], i, G.ng);
}

template <int FD>
__device__ __forceinline__ void somm_contraction(const SommerfeldGeom &G, const double *f, long long ntot_unused,
                                                 const int idx3[3], const int face[3], double &r, double &pif) {
  double J[3];
  const double x0 = somm_xx(G, 0, idx3[0]);
  if (G.cs == NRGPU_COORD_CARTESIAN) {
    const double x1 = somm_xx(G, 1, idx3[1]), x2 = somm_xx(G, 2, idx3[2]);
    r = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
    J[0] = x0 / r;
    J[1] = x1 / r;
    J[2] = x2 / r;
  } else if (G.cs == NRGPU_COORD_SPHERICAL) {
    r = x0;
    J[0] = 1.0;
    J[1] = J[2] = 0.0;
  } else if (symtp_family(G.cs)) {
    // dxx^i/dr along the radial direction x/r: (J^-1 x / r)^i
    double X[3], Jm[3][3], Ji[3][3];
    cart_jacobian(G.c, x0, somm_xx(G, 1, idx3[1]), somm_xx(G, 2, idx3[2]), X, Jm);
    inverse3(Jm, Ji);
    r = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    for (int i = 0; i < 3; i++) J[i] = (Ji[i][0] * X[0] + Ji[i][1] * X[1] + Ji[i][2] * X[2]) / r;
  } else if (cylindrical_family(G.cs)) {
    // r = sqrt(rho^2 + z^2); dxx0/dr = (rho/r) / (drho/dxx0), dxx2/dr = (z/r) / (dz/dxx2)
    double rho[4], z[4];
    cylinder_maps(G.c, x0, somm_xx(G, 2, idx3[2]), rho, z);
    r = sqrt(rho[0] * rho[0] + z[0] * z[0]);
    J[0] = rho[0] / r / rho[1];
    J[1] = 0.0;
    J[2] = z[0] / r / z[1];
  } else {
    // SinhSpherical; SinhSphericalv2 adds AMPL const_dr xx0 to r
    const double sw = sinh(1.0 / G.SINHW);
    const double lin = G.cs == NRGPU_COORD_SINHSPHERICALV2 ? G.AMPL * G.const_dr : 0.0;
    r = G.AMPL * sinh(x0 / G.SINHW) / sw + lin * x0;
    J[0] = 1.0 / (G.AMPL * cosh(x0 / G.SINHW) / (G.SINHW * sw) + lin);
    J[1] = J[2] = 0.0;
  }
  constexpr int NU = FD + 1;
  const double up2[3] = {-1.5, 2.0, -0.5}, cen2[1] = {0.5};
  const double up4[5] = {-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -1.0 / 4.0}, cen4[2] = {2.0 / 3.0, -1.0 / 12.0};
  const double up6[7] = {-49.0 / 20.0, 6.0, -15.0 / 2.0, 20.0 / 3.0, -15.0 / 4.0, 6.0 / 5.0, -1.0 / 6.0},
               cen6[3] = {3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0};
  const double *up = FD == 2 ? up2 : (FD == 4 ? up4 : up6);
  const double *cen = FD == 2 ? cen2 : (FD == 4 ? cen4 : cen6);
  const long long st[3] = {1, G.n[0], (long long)G.n[0] * G.n[1]};
  const long long c = idx3[0] + st[1] * idx3[1] + st[2] * idx3[2];
  pif = 0.0;
  for (int d = 0; d < 3; d++) {
    if (J[d] == 0.0) continue;
    const int i = idx3[d];
    double fd;
    if (face[d] != 0 || i + G.ng >= G.n[d] || i - G.ng <= 0) {
      int shift = face[d];
      if (i + G.ng >= G.n[d]) shift = -1;
      if (i - G.ng <= 0) shift = 1;
      double s = 0.0;
      for (int k = 0; k < NU; k++) s += up[k] * f[c + (long long)k * shift * st[d]];
      fd = shift * s * G.invdx[d];
    } else {
      double s = 0.0;
      for (int k = 1; k <= FD / 2; k++) s += cen[k - 1] * (f[c + k * st[d]] - f[c - k * st[d]]);
      fd = s * G.invdx[d];
    }
    pif += fd * J[d];
  }
}

template <int FD>
__global__ void sommerfeld_outer_kernel(SommerfeldGeom G, SommerfeldParams P, const int *__restrict__ dest,
                                        const int *__restrict__ step, int npts, int dir, int ngfs, long long ntot,
                                        const double *__restrict__ gfs, double *rhs) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int gf = blockIdx.y;
  if (p >= npts || gf >= ngfs) return;
  const double *f = gfs + (long long)gf * ntot;
  double *R = rhs + (long long)gf * ntot;
  const long long d = dest[p];
  const int idx3[3] = {(int)(d % G.n[0]), (int)((d / G.n[0]) % G.n[1]), (int)(d / ((long long)G.n[0] * G.n[1]))};
  int face[3] = {0, 0, 0};
  face[dir] = step[p] > 0 ? 1 : -1;
  const double c = P.speed[gf], finf = P.f_inf[gf], n = P.falloff[gf];
  double r, pif;
  somm_contraction<FD>(G, f, ntot, idx3, face, r, pif);
  double val = -c * (pif + (f[d] - finf) / r);
  if (n > 0) {
    int o3[3] = {idx3[0], idx3[1], idx3[2]};
    o3[dir] += face[dir];
    const long long o = d + step[p];
    double ro, pifo;
    somm_contraction<FD>(G, f, ntot, o3, face, ro, pifo);
    const double extrap = c * (pifo + (f[o] - finf) / ro);
    val += (R[o] + extrap) * pow(ro / r, n);
  }
  R[d] = val;
}

int apply_sommerfeld_impl(const paramstruct *p, double *const xx[3], const bc_struct *bc, int NUM_GFS,
                          const int8_t *gfs_parity, const double *gfs, double *rhs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(bc != nullptr && gfs != nullptr && rhs != nullptr, "NULL argument");
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64, "NUM_GFS %d out of range", NUM_GFS);
  NRGPU_REQUIRE(bc->NGHOSTS == p->NGHOSTS, "bcstruct built for NGHOSTS=%d, params say %d", bc->NGHOSTS,
                p->NGHOSTS);
  const int FD = g_somm.fd_order;
  // centred stencils stay inside the array when NGHOSTS >= FD/2, one-sided
  // ones when every extent is at least NGHOSTS + FD + 1
  NRGPU_REQUIRE(p->NGHOSTS >= FD / 2, "Sommerfeld FD%d needs NGHOSTS >= %d", FD, FD / 2);
  NRGPU_REQUIRE(p->Nxx_plus_2NGHOSTS0 >= p->NGHOSTS + FD + 1 && p->Nxx_plus_2NGHOSTS1 >= p->NGHOSTS + FD + 1 &&
                    p->Nxx_plus_2NGHOSTS2 >= p->NGHOSTS + FD + 1,
                "grid too small for the Sommerfeld FD%d stencils", FD);
  ParityTypes types;
  memset(&types, 0, sizeof(types));
  for (int g = 0; g < NUM_GFS; g++) {
    const int t = gfs_parity ? gfs_parity[g] : 0;
    NRGPU_REQUIRE(t >= 0 && t <= 9, "parity type %d of gf %d not in 0..9", t, g);
    types.t[g] = (int8_t)t;
  }
  SommerfeldGeom G;
  G.cs = p->CoordSystem;
  G.n[0] = p->Nxx_plus_2NGHOSTS0;
  G.n[1] = p->Nxx_plus_2NGHOSTS1;
  G.n[2] = p->Nxx_plus_2NGHOSTS2;
  G.ng = p->NGHOSTS;
  G.xxmin[0] = p->xxmin0; G.xxmin[1] = p->xxmin1; G.xxmin[2] = p->xxmin2;
  G.dxx[0] = p->dxx0; G.dxx[1] = p->dxx1; G.dxx[2] = p->dxx2;
  G.invdx[0] = p->invdx0; G.invdx[1] = p->invdx1; G.invdx[2] = p->invdx2;
  G.AMPL = p->AMPL;
  G.SINHW = p->SINHW;
  G.const_dr = p->const_dr;
  G.c = coord_params(*p);
  for (int d = 0; d < 3; d++) G.xx[d] = xx ? xx[d] : nullptr;
  const long long ntot = (long long)G.n[0] * G.n[1] * G.n[2];
  const int B = 128;
  for (int g = 0; g < bc->NGHOSTS; g++) {
    for (int d = 0; d < 3; d++) {
      const int a = bc->ob_dir_start[g][d], b = bc->ob_dir_start[g][d + 1];
      const int n = b - a;
      if (n <= 0) continue;
      dim3 grid((n + B - 1) / B, NUM_GFS);
#define SOMM(F) sommerfeld_outer_kernel<F><<<grid, B, 0, stream()>>>(G, g_somm, bc->outer_dest + a, \
                                                                    bc->outer_step + a, n, d, NUM_GFS, ntot, gfs, rhs)
      if (FD == 2) SOMM(2);
      else if (FD == 4) SOMM(4);
      else SOMM(6);
#undef SOMM
      NRGPU_LAUNCH_CHECK();
    }
    const int n = bc->num_ib_gz_pts[g];
    if (n > 0) {
      const int a = bc->ib_start[g];
      dim3 grid((n + B - 1) / B, NUM_GFS);
      bc_inner_kernel<double><<<grid, B, 0, stream()>>>(bc->inner_dest + a, bc->inner_src + a,
                                                        bc->inner_parity + a, n, NUM_GFS, ntot, types, rhs);
      NRGPU_LAUNCH_CHECK();
    }
  }
  return NRGPU_OK;
}

}  // namespace nrgpu

using namespace nrgpu;

extern "C" {

int driver_bcstruct(const paramstruct *p, bc_struct *bc) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(bc != nullptr, "bcstruct is NULL");
  memset(bc, 0, sizeof(*bc));
  std::vector<GzMap> map;
  st = build_gz_map(p, map);
  if (st) return st;
  const int ng = p->NGHOSTS;
  const int n0 = p->Nxx_plus_2NGHOSTS0, n1 = p->Nxx_plus_2NGHOSTS1, n2 = p->Nxx_plus_2NGHOSTS2;
  auto IDX3 = [&](int i0, int i1, int i2) { return i0 + n0 * (i1 + n1 * i2); };
  const int stride[3] = {1, n0, n0 * n1};
  std::vector<int> od, os, id_, is_, ip;
  int imin[3] = {ng, ng, ng};
  int imax[3] = {n0 - ng, n1 - ng, n2 - ng};
  bc->NGHOSTS = ng;
  for (int g = 0; g < ng; g++) {
    // The six faces of this layer, each with the box widened afterwards
    // (set_bcstruct.h:94-100 and :111-116 use the same sequence).
    int lo[3] = {imin[0], imin[1], imin[2]}, hi[3] = {imax[0], imax[1], imax[2]};
    struct Face { int d, side; int r[3][2]; };
    Face faces[6];
    int nf = 0;
    for (int d = 0; d < 3; d++)
      for (int side = 0; side < 2; side++) {
        Face f;
        f.d = d;
        f.side = side;
        for (int e = 0; e < 3; e++) { f.r[e][0] = lo[e]; f.r[e][1] = hi[e]; }
        if (side == 0) { f.r[d][0] = lo[d] - 1; f.r[d][1] = lo[d]; lo[d]--; }
        else           { f.r[d][0] = hi[d];     f.r[d][1] = hi[d] + 1; hi[d]++; }
        faces[nf++] = f;
      }
    bc->ob_dir_start[g][0] = (int)od.size();
    for (int fi = 0; fi < 6; fi++) {
      const Face &f = faces[fi];
      const int face_sign = (f.side == 0) ? +1 : -1;  // MINFACE = +1, MAXFACE = -1
      for (int i2 = f.r[2][0]; i2 < f.r[2][1]; i2++)
        for (int i1 = f.r[1][0]; i1 < f.r[1][1]; i1++)
          for (int i0 = f.r[0][0]; i0 < f.r[0][1]; i0++) {
            const int idx = IDX3(i0, i1, i2);
            if (map[idx].i0 == -1) {
              od.push_back(idx);
              os.push_back(face_sign * stride[f.d]);
            }
          }
      if (fi % 2 == 1) bc->ob_dir_start[g][fi / 2 + 1] = (int)od.size();
    }
    bc->num_ob_gz_pts[g] = (int)od.size() - bc->ob_dir_start[g][0];
    bc->ib_start[g] = (int)id_.size();
    for (int fi = 0; fi < 6; fi++) {
      const Face &f = faces[fi];
      for (int i2 = f.r[2][0]; i2 < f.r[2][1]; i2++)
        for (int i1 = f.r[1][0]; i1 < f.r[1][1]; i1++)
          for (int i0 = f.r[0][0]; i0 < f.r[0][1]; i0++) {
            const int idx = IDX3(i0, i1, i2);
            const GzMap &m = map[idx];
            if (m.i0 != -1) {
              id_.push_back(idx);
              is_.push_back(IDX3(m.i0, m.i1, m.i2));
              ip.push_back(m.parity_bits);
            }
          }
    }
    bc->num_ib_gz_pts[g] = (int)id_.size() - bc->ib_start[g];
    for (int d = 0; d < 3; d++) { imin[d]--; imax[d]++; }
  }
  // Every point reached through an outer stencil must be a grid point.
  const long long ntot = (long long)n0 * n1 * n2;
  for (size_t k = 0; k < od.size(); k++)
    if ((long long)od[k] + 3LL * os[k] < 0 || (long long)od[k] + 3LL * os[k] >= ntot) {
      set_error("outer boundary stencil leaves the grid (grid too small for NGHOSTS)");
      return NRGPU_ERR_BCMAP;
    }
  bc->total_outer = (int)od.size();
  bc->total_inner = (int)id_.size();
  auto upload = [&](int **dst, const std::vector<int> &v) -> int {
    *dst = nullptr;
    if (v.empty()) return NRGPU_OK;
    NRGPU_CUDA_CHECK(cudaMalloc(dst, v.size() * sizeof(int)));
    NRGPU_CUDA_CHECK(cudaMemcpy(*dst, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
    return NRGPU_OK;
  };
  if ((st = upload(&bc->outer_dest, od))) return st;
  if ((st = upload(&bc->outer_step, os))) return st;
  if ((st = upload(&bc->inner_dest, id_))) return st;
  if ((st = upload(&bc->inner_src, is_))) return st;
  if ((st = upload(&bc->inner_parity, ip))) return st;
  // Level schedule.  The sequential order: per layer the outer points (by
  // face direction), then the inner points.
  struct Ent {
    int d, a, par;
    bool inner;
  };
  std::vector<Ent> seq;
  seq.reserve(od.size() + id_.size());
  for (int g = 0; g < ng; g++) {
    for (int k = bc->ob_dir_start[g][0]; k < bc->ob_dir_start[g][3]; k++) seq.push_back({od[k], os[k], 0, false});
    for (int k = bc->ib_start[g]; k < bc->ib_start[g] + bc->num_ib_gz_pts[g]; k++)
      seq.push_back({id_[k], is_[k], ip[k], true});
  }
  std::vector<int> worder(ntot, -1), lvl(ntot, 0);
  bool ok = true;
  for (int k = 0; k < (int)seq.size() && ok; k++) {
    if (worder[seq[k].d] >= 0) ok = false;  // a point written twice
    worder[seq[k].d] = k;
  }
  int L = 0;
  for (int k = 0; k < (int)seq.size() && ok; k++) {
    const Ent &e = seq[k];
    int lv = 0;
    for (int j = 0; j < (e.inner ? 1 : 3); j++) {
      const long long x = e.inner ? e.a : (long long)e.d + (long long)(j + 1) * e.a;
      if (worder[x] > k) ok = false;  // read before the sequence writes it: keep the phases
      else if (worder[x] >= 0) lv = std::max(lv, lvl[x]);
    }
    lvl[e.d] = lv + 1;
    L = std::max(L, lv + 1);
  }
  if (ok && L >= 1 && L <= NRGPU_MAX_BC_LEVELS) {
    std::vector<int> ld, la, lp;
    std::vector<int> count(L + 1, 0);
    for (int l = 1; l <= L; l++) {
      bc->lev_start[l - 1] = (int)ld.size();
      for (int inner = 0; inner < 2; inner++) {
        if (inner) bc->lev_inner[l - 1] = (int)ld.size();
        for (const Ent &e : seq)
          if (lvl[e.d] == l && (int)e.inner == inner) {
            ld.push_back(e.d);
            la.push_back(e.a);
            lp.push_back(e.par);
          }
      }
      count[l] = (int)ld.size() - bc->lev_start[l - 1];
    }
    bc->lev_start[L] = (int)ld.size();
    // the trailing levels of at most kBcTailMax points go to the per-gridfunction tail kernel
    int tail = L;
    while (tail > 0 && count[tail] <= 2048) tail--;
    bc->lev_tail = tail;  // levels [tail, L) (0-based) form the tail
    if ((st = upload(&bc->lev_dest, ld))) return st;
    if ((st = upload(&bc->lev_arg, la))) return st;
    if ((st = upload(&bc->lev_parity, lp))) return st;
    bc->nlev = L;
  }
  return NRGPU_OK;
}

int bcstruct_freemem(bc_struct *bc) {
  if (!bc) return NRGPU_OK;
  int **ptrs[8] = {&bc->outer_dest, &bc->outer_step, &bc->inner_dest, &bc->inner_src, &bc->inner_parity,
                   &bc->lev_dest, &bc->lev_arg, &bc->lev_parity};
  bc->nlev = 0;
  for (int k = 0; k < 8; k++)
    if (*ptrs[k]) {
      cudaFree(*ptrs[k]);
      *ptrs[k] = nullptr;
    }
  return NRGPU_OK;
}

int bcstruct_download(const bc_struct *bc, int *outer_dest, int *outer_step, int *inner_dest,
                      int *inner_src, int *inner_parity) {
  NRGPU_REQUIRE(bc != nullptr, "bcstruct is NULL");
  auto dl = [&](int *dst, const int *src, int n) -> int {
    if (n > 0 && dst && src) NRGPU_CUDA_CHECK(cudaMemcpy(dst, src, n * sizeof(int), cudaMemcpyDeviceToHost));
    return NRGPU_OK;
  };
  int st;
  if ((st = dl(outer_dest, bc->outer_dest, bc->total_outer))) return st;
  if ((st = dl(outer_step, bc->outer_step, bc->total_outer))) return st;
  if ((st = dl(inner_dest, bc->inner_dest, bc->total_inner))) return st;
  if ((st = dl(inner_src, bc->inner_src, bc->total_inner))) return st;
  if ((st = dl(inner_parity, bc->inner_parity, bc->total_inner))) return st;
  return NRGPU_OK;
}

int apply_bcs_curvilinear(const paramstruct *p, const bc_struct *bc, int NUM_GFS,
                          const int8_t *gfs_parity, double *gfs) {
  return apply_bcs_impl<double>(p, bc, NUM_GFS, gfs_parity, gfs);
}
int apply_bcs_curvilinear_f32(const paramstruct *p, const bc_struct *bc, int NUM_GFS,
                              const int8_t *gfs_parity, float *gfs) {
  return apply_bcs_impl<float>(p, bc, NUM_GFS, gfs_parity, gfs);
}

// ------------------------------------------------ slab (one rank's share)
// The boundary conditions of a grid split into slabs along i2, applied by
// each rank to the ghost points it owns; indices are the slab's own idx3.
int nrgpu_bc_outer_points(const paramstruct *p, int NUM_GFS, const int *dest, const int *step, int n,
                          double *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64 && n >= 0, "bad arguments");
  if (n == 0) return NRGPU_OK;
  NRGPU_REQUIRE(dest && step && gfs, "NULL argument");
  const long long ntot = (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  dim3 grid((n + 127) / 128, NUM_GFS);
  bc_outer_kernel<double><<<grid, 128, 0, stream()>>>(dest, step, n, NUM_GFS, ntot, gfs);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_bc_gather_points(const paramstruct *p, int NUM_GFS, const int *src, int n, const double *gfs,
                           double *buf) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64 && n >= 0, "bad arguments");
  if (n == 0) return NRGPU_OK;
  NRGPU_REQUIRE(src && gfs && buf, "NULL argument");
  const long long ntot = (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  dim3 grid((n + 127) / 128, NUM_GFS);
  bc_gather_kernel<<<grid, 128, 0, stream()>>>(src, n, NUM_GFS, ntot, gfs, buf);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_bc_scatter_parity(const paramstruct *p, int NUM_GFS, const int8_t *gfs_parity, const int *dest,
                            const int *parity_bits, int n, const double *buf, double *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(NUM_GFS >= 1 && NUM_GFS <= 64 && n >= 0, "bad arguments");
  if (n == 0) return NRGPU_OK;
  NRGPU_REQUIRE(dest && parity_bits && buf && gfs, "NULL argument");
  ParityTypes types;
  memset(&types, 0, sizeof(types));
  for (int g = 0; g < NUM_GFS; g++) {
    const int t = gfs_parity ? gfs_parity[g] : 0;
    NRGPU_REQUIRE(t >= 0 && t <= 9, "parity type %d of gf %d not in 0..9", t, g);
    types.t[g] = (int8_t)t;
  }
  const long long ntot = (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  dim3 grid((n + 127) / 128, NUM_GFS);
  bc_scatter_parity_kernel<<<grid, 128, 0, stream()>>>(dest, parity_bits, n, NUM_GFS, ntot, types, buf, gfs);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

}  // extern "C"

extern "C" int nrgpu_sommerfeld_params(int fd_order, int NUM_GFS, const double *speed, const double *f_inf,
                                       const double *radial_falloff_power) {
  NRGPU_REQUIRE(fd_order == 2 || fd_order == 4 || fd_order == 6, "Sommerfeld fd_order must be 2, 4 or 6");
  NRGPU_REQUIRE(NUM_GFS >= 0 && NUM_GFS <= 64, "NUM_GFS %d out of range", NUM_GFS);
  g_somm.fd_order = fd_order;
  for (int g = 0; g < NUM_GFS; g++) {
    if (speed) g_somm.speed[g] = speed[g];
    if (f_inf) g_somm.f_inf[g] = f_inf[g];
    if (radial_falloff_power) g_somm.falloff[g] = radial_falloff_power[g];
  }
  return NRGPU_OK;
}

extern "C" int apply_bcs_sommerfeld(const paramstruct *p, double *xx[3], const bc_struct *bc, int NUM_GFS,
                                    const int8_t *gfs_parity, const double *gfs, double *rhs_gfs) {
  return apply_sommerfeld_impl(p, xx, bc, NUM_GFS, gfs_parity, gfs, rhs_gfs);
}
