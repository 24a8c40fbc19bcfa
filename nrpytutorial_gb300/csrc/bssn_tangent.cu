// bssn_tangent.cu -- the tangent-linear BSSN evolution: RK4 steps of a state
// and N tangent states, Brill-Lindquist data with its parameter
// derivatives, and a radial-shell observable with its derivatives (the
// C ABI of the forward-mode gradient).
//
// One step is the reference's RK4 (MoLtimestepping/C_Code_Generation.py:
// 266-329) in the unfused order of MoL_step_forward_in_time_unfused: per
// substep Ricci_eval and rhs_eval at interior points (value and tangents,
// bssn_tangent.cuh), the RK update at every point, apply_bcs_curvilinear on
// the value and on each tangent (the boundary conditions are linear), then
// the det(gammabar) rescale of the value and its linearisation on the
// tangents.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "bssn_tangent.cuh"

namespace nrgpu {
template <typename T>
int apply_bcs_impl(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity, T *gfs);

namespace bssn {
namespace tangent {

NRGPU_TANGENT_DECLARE(NRGPU_COORD_CARTESIAN, 4, 0)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_CARTESIAN, 4, 1)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_CARTESIAN, 4, 2)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_CARTESIAN, 4, 4)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_SINHSPHERICAL, 4, 0)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_SINHSPHERICAL, 4, 1)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_SINHSPHERICAL, 4, 2)
NRGPU_TANGENT_DECLARE(NRGPU_COORD_SINHSPHERICAL, 4, 4)

static int check_tangent(const rfm_struct *rfm, const paramstruct *p, int ntan) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(ntan == 0 || ntan == 1 || ntan == 2 || ntan == 4, "ntan %d not in {0, 1, 2, 4}", ntan);
  const int cs = dispatch_cs(p->CoordSystem);
  NRGPU_REQUIRE(p->FD_order == 4 && (cs == NRGPU_COORD_CARTESIAN || cs == NRGPU_COORD_SINHSPHERICAL),
                "the tangent BSSN evolution is built for FD_order 4 on Cartesian and SinhSpherical(v2) grids");
  NRGPU_REQUIRE(cs == NRGPU_COORD_CARTESIAN || rfm_matches(rfm, p),
                "curvilinear grids need an rfm_struct defined for this grid");
  NRGPU_REQUIRE(!p->enable_stress_energy_source_terms && p->diss_strength == 0.0,
                "the tangent BSSN evolution has no source terms and no dissipation");
  return NRGPU_OK;
}

static int rhs_dispatch(const rfm_struct *rfm, const paramstruct *p, int ntan, const double *in, double *aux,
                        double *out) {
  const Grid g = make_grid(p);
  const long long ts = (long long)NUM_EVOL_GFS * g.ntot, ats = (long long)NUM_AUXEVOL_GFS * g.ntot;
  const bool cart = dispatch_cs(p->CoordSystem) == NRGPU_COORD_CARTESIAN;
#define TAN_CASE(NT)                                                                                           \
  if (ntan == NT)                                                                                            \
    return cart ? rhs_launch<NRGPU_COORD_CARTESIAN, 4, NT>(rfm, g, in, ts, aux, ats, p->eta, out)            \
                : rhs_launch<NRGPU_COORD_SINHSPHERICAL, 4, NT>(rfm, g, in, ts, aux, ats, p->eta, out);
  TAN_CASE(0) TAN_CASE(1) TAN_CASE(2) TAN_CASE(4)
#undef TAN_CASE
  set_error("ntan %d not built", ntan);
  return NRGPU_ERR_UNSUPPORTED;
}

// RK4 update of substep s over n values (value and tangents alike), in the
// expressions of the reference's RK_MoL.h: k is the substep's RHS on input
// and the next substep's input on output (s < 3).
__global__ void rk_update_kernel(long long n, int s, double dt, double *__restrict__ y, double *__restrict__ rt,
                                 double *__restrict__ k) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double ki = k[i];
    if (s == 0) {
      rt[i] = ki * dt * (1.0 / 6.0);
      k[i] = y[i] + ki * dt * (1.0 / 2.0);
    } else if (s == 1) {
      rt[i] = rt[i] + ki * dt * (1.0 / 3.0);
      k[i] = y[i] + ki * dt * (1.0 / 2.0);
    } else if (s == 2) {
      rt[i] = rt[i] + ki * dt * (1.0 / 3.0);
      k[i] = y[i] + ki * dt;
    } else {
      y[i] = y[i] + rt[i] + ki * dt * (1.0 / 6.0);
    }
  }
}

// Linearisation of the det(gammabar) rescale on the tangents, from the
// value before the rescale: h' = f (delta + h) - delta with f = s^{-1/3},
// s = det(gammabar)/|det(ghat)|, so dh' = df (delta + h) + f dh with
// df = -(f / 3s) ds and ds the derivative of det(gammabar) along dh.
template <int CS>
__global__ void enforce_tangent_kernel(Grid g, const double *__restrict__ tab, int ntan, double *__restrict__ Y,
                                       long long ts) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  if (i0 >= g.n0) return;
  const long long idx = (long long)i0 + (long long)g.n0 * ((long long)i1 + (long long)g.n1 * i2);
  const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
  double h[3][3], gb[3][3], sc[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      h[i][j] = h[j][i] = Y[(long long)(HDD00 + S6(i, j)) * g.ntot + idx];
      sc[i][j] = sc[j][i] = RfmMask<CS>::trivial ? 1.0 : rf.ReDD(i, j);
      double v = h[i][j] * sc[i][j];
      if (i == j) v += rf.ghatDD(i);
      gb[i][j] = gb[j][i] = v;
    }
  // cofactors: d det = sum_ij C_ij d gb_ij
  double C[3][3];
  C[0][0] = gb[1][1] * gb[2][2] - gb[1][2] * gb[1][2];
  C[1][1] = gb[0][0] * gb[2][2] - gb[0][2] * gb[0][2];
  C[2][2] = gb[0][0] * gb[1][1] - gb[0][1] * gb[0][1];
  C[0][1] = C[1][0] = gb[0][2] * gb[1][2] - gb[0][1] * gb[2][2];
  C[0][2] = C[2][0] = gb[0][1] * gb[1][2] - gb[0][2] * gb[1][1];
  C[1][2] = C[2][1] = gb[0][1] * gb[0][2] - gb[0][0] * gb[1][2];
  const double det = gb[0][0] * C[0][0] + gb[0][1] * C[0][1] + gb[0][2] * C[0][2];
  const double adg = fabs(rf.detg());
  const double s = det / adg;
  // f = s^{-1/3} as the value's rescale computes it (enforce_kernel: Newton
  // on w^{-3} = s from the FP32 reciprocal cube root), so that the tangent is
  // the derivative of that map at every point, ghost points included.
  double f = (double)rcbrtf((float)s);
#pragma unroll
  for (int it = 0; it < 2; it++) f = f * (4.0 - s * f * f * f) * (1.0 / 3.0);
  for (int k = 1; k <= ntan; k++) {
    double *t = Y + k * ts;
    double dh[3][3], ddet = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++) dh[i][j] = dh[j][i] = t[(long long)(HDD00 + S6(i, j)) * g.ntot + idx];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) ddet += C[i][j] * dh[i][j] * sc[i][j];
    const double df = -(f / (3.0 * s)) * (ddet / adg);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = i; j < 3; j++) {
        const double d = (i == j) ? 1.0 : 0.0;
        t[(long long)(HDD00 + S6(i, j)) * g.ntot + idx] = df * (d + h[i][j]) + f * dh[i][j];
      }
  }
}

// Brill-Lindquist parameter derivatives.  The library's data
// (BSSN_initial_data_BrillLindquist) depend on the parameters only through
// psi = 1 + m1/(2 r1) + m2/(2 r2): W = alpha = psi^-2, hDD and lambdaU are
// psi-independent (gammabar = ghat).  Parameters: 0 m1, 1 m2, 2..4 x1, 5..7 x2.
struct BLTangent {
  double m1, x1[3], m2, x2[3];
  int ntan, param[4];
};
__global__ void bl_tangent_kernel(paramstruct p, BLTangent b, double *__restrict__ Y, long long ts) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  const int n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1, n2 = p.Nxx_plus_2NGHOSTS2;
  if (i0 >= n0) return;
  const long long ntot = (long long)n0 * n1 * n2;
  const long long idx = (long long)i0 + (long long)n0 * ((long long)i1 + (long long)n1 * i2);
  double x[3], J[3][3];
  cart_jacobian(coord_params(p), xx_of(p.xxmin0, p.dxx0, i0, p.NGHOSTS), xx_of(p.xxmin1, p.dxx1, i1, p.NGHOSTS),
                xx_of(p.xxmin2, p.dxx2, i2, p.NGHOSTS), x, J);
  double d1[3], d2[3];
  for (int a = 0; a < 3; a++) d1[a] = x[a] - b.x1[a], d2[a] = x[a] - b.x2[a];
  const double r1 = sqrt(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
  const double r2 = sqrt(d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2]);
  const double psi = 1.0 + b.m1 / (2.0 * r1) + b.m2 / (2.0 * r2);
  const double dW = -2.0 / (psi * psi * psi);  // d(psi^-2)/d psi
  for (int k = 0; k < b.ntan; k++) {
    const int q = b.param[k];
    double dpsi;
    if (q == 0) dpsi = 1.0 / (2.0 * r1);
    else if (q == 1) dpsi = 1.0 / (2.0 * r2);
    else if (q <= 4) dpsi = b.m1 * d1[q - 2] / (2.0 * r1 * r1 * r1);
    else dpsi = b.m2 * d2[q - 5] / (2.0 * r2 * r2 * r2);
    double *t = Y + (long long)(k + 1) * ts;
    for (int gf = 0; gf < NUM_EVOL_GFS; gf++) t[(long long)gf * ntot + idx] = 0.0;
    t[(long long)CF * ntot + idx] = dW * dpsi;
    t[(long long)ALPHA * ntot + idx] = dW * dpsi;
  }
}

// J^2 accumulation on the shell i0: accum[0] += scale sum_q w_q (f_q - off)^2,
// accum[k] += 2 scale sum_q w_q (f_q - off) t_k,q (k = 1..ntan).
__global__ void shell_tangent_kernel(Grid g, const double *__restrict__ Y, long long ts, int ntan, int gf, int i0,
                                     const double *__restrict__ wts, double scale, double off,
                                     double *__restrict__ accum) {
  const int m1 = g.n1 - 2 * g.ng, nq = m1 * (g.n2 - 2 * g.ng);
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double loc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (q < nq) {
    const long long idx =
        (long long)gf * g.ntot + i0 + (long long)g.n0 * ((g.ng + q % m1) + (long long)g.n1 * (g.ng + q / m1));
    const double f = Y[idx] - off, w = scale * wts[q];
    loc[0] = w * f * f;
    for (int k = 1; k <= ntan; k++) loc[k] = 2.0 * w * f * Y[(long long)k * ts + idx];
  }
  __shared__ double sh[5][32];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    double v = loc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5 && threadIdx.x <= ntan) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sh[threadIdx.x][w];
    atomicAdd(accum + threadIdx.x, v);
  }
}

}  // namespace tangent
}  // namespace bssn
}  // namespace nrgpu

using namespace nrgpu;
using namespace nrgpu::bssn;
using namespace nrgpu::bssn::tangent;

extern "C" {

int BSSN_tangent_rhs_eval(const rfm_struct *rfm, const paramstruct *p, int ntan, const double *in, double *aux,
                          double *rhs) {
  NRGPU_REQUIRE(p && in && aux && rhs, "NULL argument");
  int st = check_tangent(rfm, p, ntan);
  if (st) return st;
  return rhs_dispatch(rfm, p, ntan, in, aux, rhs);
}

int BSSN_tangent_step(const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc, int ntan, double *Y,
                      double *scratch, double dt) {
  NRGPU_REQUIRE(p && bc && Y && scratch, "NULL argument");
  int st = check_tangent(rfm, p, ntan);
  if (st) return st;
  const Grid g = make_grid(p);
  const long long ts = (long long)NUM_EVOL_GFS * g.ntot, n = (long long)(ntan + 1) * ts;
  double *rt = scratch, *kbuf[2] = {scratch + n, scratch + 2 * n}, *aux = scratch + 3 * n;
  const int8_t *par = system_parity(NRGPU_SYS_BSSN);
  const int threads = 256;
  const int blocks = (int)std::min<long long>((n + threads - 1) / threads, 152LL * 16);
  const double *tab = rfm ? rfm->table64 : nullptr;
  const bool cart = dispatch_cs(p->CoordSystem) == NRGPU_COORD_CARTESIAN;
  dim3 eblock(64), egrid((g.n0 + 63) / 64, g.n1, g.n2);
  for (int s = 0; s < 4; s++) {
    const double *in = (s == 0) ? Y : kbuf[(s + 1) % 2];
    double *k = kbuf[s % 2];
    if ((st = rhs_dispatch(rfm, p, ntan, in, aux, k))) return st;
    rk_update_kernel<<<blocks, threads, 0, stream()>>>(n, s, dt, Y, rt, k);
    NRGPU_LAUNCH_CHECK();
    double *post = (s == 3) ? Y : k;
    for (int c = 0; c <= ntan; c++)
      if ((st = apply_bcs_impl<double>(p, bc, NUM_EVOL_GFS, par, post + c * ts))) return st;
    if (ntan > 0) {
      if (cart) enforce_tangent_kernel<NRGPU_COORD_CARTESIAN><<<egrid, eblock, 0, stream()>>>(g, tab, ntan, post, ts);
      else enforce_tangent_kernel<NRGPU_COORD_SINHSPHERICAL><<<egrid, eblock, 0, stream()>>>(g, tab, ntan, post, ts);
      NRGPU_LAUNCH_CHECK();
    }
    if ((st = bssn_enforce_launch(rfm, p, post, true))) return st;
  }
  return NRGPU_OK;
}

int BSSN_tangent_initial_data_BrillLindquist(const paramstruct *p, double m1, const double x1[3], double m2,
                                             const double x2[3], int ntan, const int *param_index, double *Y) {
  NRGPU_REQUIRE(p && x1 && x2 && Y && (ntan == 0 || param_index), "NULL argument");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(ntan >= 0 && ntan <= 4, "ntan %d not in 0..4", ntan);
  BLTangent b{};
  b.m1 = m1, b.m2 = m2, b.ntan = ntan;
  for (int a = 0; a < 3; a++) b.x1[a] = x1[a], b.x2[a] = x2[a];
  for (int k = 0; k < ntan; k++) {
    NRGPU_REQUIRE(param_index[k] >= 0 && param_index[k] <= 7, "parameter index %d not in 0..7", param_index[k]);
    b.param[k] = param_index[k];
  }
  if ((st = BSSN_initial_data_BrillLindquist(p, m1, x1, m2, x2, Y))) return st;
  if (ntan == 0) return NRGPU_OK;
  const long long ts = (long long)NUM_EVOL_GFS * p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 *
                       p->Nxx_plus_2NGHOSTS2;
  dim3 block(64), grid((p->Nxx_plus_2NGHOSTS0 + 63) / 64, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2);
  bl_tangent_kernel<<<grid, block, 0, stream()>>>(*p, b, Y, ts);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int BSSN_tangent_shell_accumulate(const paramstruct *p, int ntan, const double *Y, int gf, int i0,
                                  const double *wts, double scale, double offset, double *accum) {
  NRGPU_REQUIRE(p && Y && wts && accum, "NULL argument");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(ntan >= 0 && ntan <= 4, "ntan %d not in 0..4", ntan);
  NRGPU_REQUIRE(gf >= 0 && gf < NUM_EVOL_GFS, "gridfunction %d out of range", gf);
  NRGPU_REQUIRE(i0 >= p->NGHOSTS && i0 < p->Nxx_plus_2NGHOSTS0 - p->NGHOSTS, "shell i0 %d not interior", i0);
  const Grid g = make_grid(p);
  const int nq = p->Nxx1 * p->Nxx2;
  shell_tangent_kernel<<<(nq + 127) / 128, 128, 0, stream()>>>(g, Y, (long long)NUM_EVOL_GFS * g.ntot, ntan, gf, i0,
                                                               wts, scale, offset, accum);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

}  // extern "C"
