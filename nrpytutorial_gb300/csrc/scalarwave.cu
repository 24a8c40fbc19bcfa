// scalarwave.cu -- scalar wave equation RHS, Cartesian and curvilinear.
//
// Cartesian (ScalarWave/ScalarWave_RHSs.py:46-71):
//   uu_rhs = vv,   vv_rhs = c^2 sum_i d_i d_i uu
// Curvilinear (ScalarWave/ScalarWaveCurvilinear_RHSs.py:43-98):
//   vv_rhs = c^2 ( ghat^{ij} d_i d_j uu - ghat^{ij} Gammahat^k_{ij} d_k uu )
// (ghat is diagonal for the supported coordinate systems, so only the
// unmixed second derivatives enter).  Gridfunctions: uu = 0, vv = 1.
#include "epilogue.cuh"
#include "fd.cuh"
#include "rfm.cuh"
#include "systems.cuh"

namespace nrgpu {

template <typename R, typename Tin, int CS, int ORDER, typename TStage>
__global__ void __launch_bounds__(256)
    scalarwave_kernel(Grid g, typename InRef<Tin>::type in, const R *__restrict__ rfmtab, R c2,
                      RKEpilogue<TStage> epi) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  const auto uu = in + idx;
  const R vv = val<R>(in + g.ntot + idx);
  const long long st[3] = {1, g.n0, (long long)g.n0 * g.n1};
  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  R lap = (R)0;
  if constexpr (RfmMask<CS>::trivial) {
#pragma unroll
    for (int d = 0; d < 3; d++) lap += fd_d2<ORDER, R>(uu, st[d]) * (inv[d] * inv[d]);
  } else {
    using M = RfmMask<CS>;
    const Rfm<CS, R> rf = rfm_at<CS, R>(rfmtab, g, i0, i1, i2);
    R contracted[3] = {(R)0, (R)0, (R)0};
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        if (M::Gammahat(k, i, i)) contracted[k] += rf.ghatUU(i) * rf.G(k, i, i);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      lap += rf.ghatUU(d) * (fd_d2<ORDER, R>(uu, st[d]) * (inv[d] * inv[d]));
      bool any = false;
#pragma unroll
      for (int i = 0; i < 3; i++) any = any || M::Gammahat(d, i, i);
      if (any) lap -= contracted[d] * (fd_d1<ORDER, R>(uu, st[d]) * inv[d]);
    }
  }
  epi(0, idx, vv);
  epi(1, idx, c2 * lap);
}

template <typename R, typename Tin, typename TStage, int CS, int ORDER>
static int launch_one(const Grid &g, typename InRef<Tin>::type in, const rfm_struct *rfm, double c2,
                      const RKEpilogue<TStage> &epi) {
  const R *tab = nullptr;
  if constexpr (CS != NRGPU_COORD_CARTESIAN) {
    if (!rfm) {
      set_error("curvilinear ScalarWave needs an rfm_struct");
      return NRGPU_ERR_ARG;
    }
    if constexpr (sizeof(R) == 8) tab = (const R *)rfm->table64;
    else tab = (const R *)rfm->table32;
  }
  InteriorLaunch L = interior_launch(g, 64, 4);
  scalarwave_kernel<R, Tin, CS, ORDER, TStage>
      <<<L.grid, L.block, 0, stream()>>>(g, in, tab, (R)c2, epi);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <typename R, typename Tin, typename TStage>
static int dispatch(const paramstruct *p, const Grid &g, typename InRef<Tin>::type in, const rfm_struct *rfm,
                    const RKEpilogue<TStage> &epi) {
  const double c2 = p->wavespeed * p->wavespeed;
#define SW_CASE(CSV, ORD) \
  if (dispatch_cs(p->CoordSystem) == CSV && p->FD_order == ORD)                                             \
    return launch_one<R, Tin, TStage, CSV, ORD>(g, in, rfm, c2, epi);
  SW_CASE(NRGPU_COORD_CARTESIAN, 2) SW_CASE(NRGPU_COORD_CARTESIAN, 4)
  SW_CASE(NRGPU_COORD_CARTESIAN, 6) SW_CASE(NRGPU_COORD_CARTESIAN, 8)
  SW_CASE(NRGPU_COORD_SPHERICAL, 2) SW_CASE(NRGPU_COORD_SPHERICAL, 4)
  SW_CASE(NRGPU_COORD_SPHERICAL, 6) SW_CASE(NRGPU_COORD_SPHERICAL, 8)
  SW_CASE(NRGPU_COORD_SINHSPHERICAL, 2) SW_CASE(NRGPU_COORD_SINHSPHERICAL, 4)
  SW_CASE(NRGPU_COORD_SINHSPHERICAL, 6) SW_CASE(NRGPU_COORD_SINHSPHERICAL, 8)
  SW_CASE(NRGPU_COORD_SINHCYLINDRICAL, 2) SW_CASE(NRGPU_COORD_SINHCYLINDRICAL, 4)
  SW_CASE(NRGPU_COORD_SINHCYLINDRICAL, 6) SW_CASE(NRGPU_COORD_SINHCYLINDRICAL, 8)
  SW_CASE(NRGPU_COORD_SINHSYMTP, 2) SW_CASE(NRGPU_COORD_SINHSYMTP, 4)
  SW_CASE(NRGPU_COORD_SINHSYMTP, 6) SW_CASE(NRGPU_COORD_SINHSYMTP, 8)
#undef SW_CASE
  set_error("ScalarWave: CoordSystem %d with FD_order %d not built", p->CoordSystem, p->FD_order);
  return NRGPU_ERR_UNSUPPORTED;
}

int scalarwave_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  int st = check_params(p);
  if (st) return st;
  Grid g = make_grid(p);
  if (a.prec == NRGPU_PREC_FP64) {
    RKEpilogue<double> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (double *)a.out};
    return dispatch<double, double, double>(p, g, stage_input<double>(a), rfm, epi);
  }
  if (pair_precision(a.prec)) {
    RKEpilogue<float2> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float2 *)a.out, stage_consts(a.dt),
                           a.prec == NRGPU_PREC_COMPENSATED_FP64RK};
    return dispatch<float, Pair32, float2>(p, g, stage_input<Pair32>(a), rfm, epi);
  }
  RKEpilogue<float> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float *)a.out, stage_consts(a.dt)};
  if (a.in_is_f64) return dispatch<float, double, float>(p, g, stage_input<double>(a), rfm, epi);
  return dispatch<float, float, float>(p, g, stage_input<float>(a), rfm, epi);
}

// Initial data of ScalarWave/InitialData.py:27-88 at every point, at
// Cartesian positions xx_to_Cart(xx) of the grid's CoordSystem:
//   PlaneWave          uu = sin(khat.x - c t) + 2, vv = -c cos(khat.x - c t)
//   SphericalGaussian  uu = (r-ct)/r e^{-(r-ct)^2/(2s^2)} + (r+ct)/r e^{-(r+ct)^2/(2s^2)} + 1,
//                      vv = c/r [e_a ((r-ct)^2/s^2 - 1) + e_b (1 - (r+ct)^2/s^2)]
__global__ void sw_initial_data_kernel(paramstruct p, int kind, double t, double k0, double k1, double k2,
                                       double sigma, double *__restrict__ gfs) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  const int n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1;
  if (i0 >= n0) return;
  const long long ntot = (long long)n0 * n1 * p.Nxx_plus_2NGHOSTS2;
  const long long idx = i0 + (long long)n0 * (i1 + (long long)n1 * i2);
  const double x0 = xx_of(p.xxmin0, p.dxx0, i0, p.NGHOSTS), x1 = xx_of(p.xxmin1, p.dxx1, i1, p.NGHOSTS),
               x2 = xx_of(p.xxmin2, p.dxx2, i2, p.NGHOSTS);
  double X[3], J[3][3];
  cart_jacobian(coord_params(p), x0, x1, x2, X, J);  // xx_to_Cart
  const double x = X[0], y = X[1], z = X[2];
  const double c = p.wavespeed;
  double uu, vv;
  if (kind == 0) {
    const double ph = (k0 * x + k1 * y + k2 * z) / sqrt(k0 * k0 + k1 * k1 + k2 * k2) - c * t;
    uu = sin(ph) + 2.0;
    vv = -c * cos(ph);
  } else {
    const double r = sqrt(x * x + y * y + z * z);
    const double a = r - c * t, b = r + c * t, s2 = sigma * sigma;
    const double ea = exp(-a * a / (2.0 * s2)), eb = exp(-b * b / (2.0 * s2));
    uu = a / r * ea + b / r * eb + 1.0;
    vv = c / r * (ea * (a * a / s2 - 1.0) + eb * (1.0 - b * b / s2));
  }
  gfs[idx] = uu;
  gfs[ntot + idx] = vv;
}

}  // namespace nrgpu

using namespace nrgpu;

static int sw_plain(const rfm_struct *rfm, const paramstruct *p, const void *in, void *rhs, int prec,
                    bool want_curvi) {
  NRGPU_REQUIRE(p && in && rhs, "NULL argument");
  NRGPU_REQUIRE(want_curvi == (p->CoordSystem != NRGPU_COORD_CARTESIAN),
                want_curvi ? "ScalarWaveCurvilinear_rhs_eval needs a curvilinear CoordSystem"
                           : "ScalarWave_rhs_eval needs CoordSystem Cartesian");
  StageArgs a{};
  a.stage = -1;
  a.prec = prec;
  a.in = in;
  a.in_is_f64 = (prec == NRGPU_PREC_FP64);
  a.out = rhs;
  return scalarwave_launch(rfm, p, a);
}

extern "C" {
int ScalarWave_rhs_eval(const paramstruct *p, const double *in, double *rhs) {
  return sw_plain(nullptr, p, in, rhs, NRGPU_PREC_FP64, false);
}
int ScalarWave_rhs_eval_f32(const paramstruct *p, const float *in, float *rhs) {
  return sw_plain(nullptr, p, in, rhs, NRGPU_PREC_MIXED, false);
}
int ScalarWaveCurvilinear_rhs_eval(const rfm_struct *rfm, const paramstruct *p, const double *in,
                                   double *rhs) {
  return sw_plain(rfm, p, in, rhs, NRGPU_PREC_FP64, true);
}
int ScalarWaveCurvilinear_rhs_eval_f32(const rfm_struct *rfm, const paramstruct *p, const float *in,
                                       float *rhs) {
  return sw_plain(rfm, p, in, rhs, NRGPU_PREC_MIXED, true);
}
int ScalarWave_initial_data(const paramstruct *p, int kind, double time, const double kk[3], double sigma,
                            double *in_gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(in_gfs, "NULL argument");
  NRGPU_REQUIRE(kind == 0 || kind == 1, "kind must be 0 (PlaneWave) or 1 (SphericalGaussian)");
  NRGPU_REQUIRE(kind == 1 || (kk && (kk[0] != 0.0 || kk[1] != 0.0 || kk[2] != 0.0)), "PlaneWave needs k != 0");
  NRGPU_REQUIRE(kind == 0 || sigma > 0.0, "SphericalGaussian needs sigma > 0");
  dim3 block(64), grid((p->Nxx_plus_2NGHOSTS0 + 63) / 64, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2);
  sw_initial_data_kernel<<<grid, block, 0, stream()>>>(*p, kind, time, kk ? kk[0] : 0.0, kk ? kk[1] : 0.0,
                                                       kk ? kk[2] : 0.0, sigma, in_gfs);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
}
