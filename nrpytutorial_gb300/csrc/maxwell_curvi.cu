// maxwell_curvi.cu -- vacuum Maxwell equations, System II, in rescaled
// curvilinear form (Maxwell/VacuumMaxwell_Flat_Evol_Curvilinear_rescaled.py:22-190):
//   A^i = a^i ReU^i, E^i = e^i ReU^i, auxiliary Gamma = d_i A^i + ...
//   d_t a^i   = -e^i - ghat^ij psi_,j / ReU^i
//   d_t e^i   = [ ghat^ij Gamma_,j - ghat^jk ( A^i_,kj + d_j Gammahat^i_mk A^m
//               + Gammahat^i_mk A^m_,j + Gammahat^i_mj A^m_,k - Gammahat^m_kj A^i_,m
//               + (Gammahat^i_dj Gammahat^d_mk - Gammahat^d_kj Gammahat^i_md) A^m ) ] / ReU^i
//   d_t psi   = -Gamma
//   d_t Gamma = -ghat^ij psi_,ij + ghat^ij Gammahat^k_ji psi_,k
// Constraints: C = E^i_,i + Gammahat^i_ji E^j, G = Gamma - A^i_,i + Gammahat^i_ji A^j.
// ghat is diagonal for the supported coordinate systems, so only j == k
// terms enter (no mixed second derivatives).  Gridfunctions, alphabetical
// (uppercase first): Gamma, aU0, aU1, aU2, eU0, eU1, eU2, psi.
#include "epilogue.cuh"
#include "fd.cuh"
#include "rfm.cuh"
#include "systems.cuh"

namespace nrgpu {
namespace mcurvi {

enum { GAMMA = 0, AU0 = 1, EU0 = 4, PSI = 7, NGF = 8 };

template <typename R, typename Tin, int CS, int ORDER, typename TStage>
__global__ void __launch_bounds__(128)
    maxwell_curvi_kernel(Grid g, typename InRef<Tin>::type in, const R *__restrict__ tab, RKEpilogue<TStage> epi) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  using M = RfmMask<CS>;
  const long long st[3] = {1, g.n0, (long long)g.n0 * g.n1};
  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g, i0, i1, i2);
  auto gf = [&](int k) { return in + (long long)k * g.ntot + idx; };
  // A^i, A^i_,j and the unmixed A^i_,jj
  R A[3], Ad[3][3], Add[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const R a = val<R>(gf(AU0 + i));
    const R reu = rf.ReU(i);
    A[i] = M::trivial ? a : a * reu;
    R ad[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      ad[j] = fd_d1<ORDER, R>(gf(AU0 + i), st[j]) * inv[j];
      R v = M::trivial ? ad[j] : ad[j] * reu;
      if (M::ReUdD(i, j)) v += a * rf.ReUdD(i, j);
      Ad[i][j] = v;
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const R a2 = fd_d2<ORDER, R>(gf(AU0 + i), st[j]) * (inv[j] * inv[j]);
      R v = M::trivial ? a2 : a2 * reu;
      if (M::ReUdD(i, j)) v += (R)2 * ad[j] * rf.ReUdD(i, j);
      if (M::ReUdDD(i, j, j)) v += a * rf.ReUdDD(i, j, j);
      Add[i][j] = v;
    }
  }
  // a^i RHS
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const R e = val<R>(gf(EU0 + i));
    const R dpsi = fd_d1<ORDER, R>(gf(PSI), st[i]) * inv[i];
    R t = rf.ghatUU(i) * dpsi;
    if constexpr (!M::trivial) t /= rf.ReU(i);
    epi(AU0 + i, idx, -e - t);
  }
  // e^i RHS
  R dGam[3];
#pragma unroll
  for (int j = 0; j < 3; j++) dGam[j] = fd_d1<ORDER, R>(gf(GAMMA), st[j]) * inv[j];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R E = rf.ghatUU(i) * dGam[i];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R t = Add[i][j];
      if constexpr (!M::trivial) {
#pragma unroll
        for (int m = 0; m < 3; m++) {
          if (M::GammahatdD(i, m, j, j)) t += rf.GdD(i, m, j, j) * A[m];
          if (M::Gammahat(i, m, j)) t += (R)2 * rf.G(i, m, j) * Ad[m][j];
          if (M::Gammahat(m, j, j)) t -= rf.G(m, j, j) * Ad[i][m];
#pragma unroll
          for (int d = 0; d < 3; d++) {
            if (M::Gammahat(i, d, j) && M::Gammahat(d, m, j)) t += rf.G(i, d, j) * rf.G(d, m, j) * A[m];
            if (M::Gammahat(d, j, j) && M::Gammahat(i, m, d)) t -= rf.G(d, j, j) * rf.G(i, m, d) * A[m];
          }
        }
      }
      E -= rf.ghatUU(j) * t;
    }
    if constexpr (!M::trivial) E /= rf.ReU(i);
    epi(EU0 + i, idx, E);
  }
  // psi, Gamma RHS
  const R Gam = val<R>(gf(GAMMA));
  epi(PSI, idx, -Gam);
  R Grhs = (R)0;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Grhs -= rf.ghatUU(i) * (fd_d2<ORDER, R>(gf(PSI), st[i]) * (inv[i] * inv[i]));
    if constexpr (!M::trivial) {
#pragma unroll
      for (int k = 0; k < 3; k++)
        if (M::Gammahat(k, i, i)) Grhs += rf.ghatUU(i) * rf.G(k, i, i) * (fd_d1<ORDER, R>(gf(PSI), st[k]) * inv[k]);
    }
  }
  epi(GAMMA, idx, Grhs);
}

template <int CS, int ORDER>
__global__ void maxwell_curvi_constraint_kernel(Grid g, const double *__restrict__ in, const double *__restrict__ tab,
                                                double *__restrict__ aux) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  using M = RfmMask<CS>;
  const long long st[3] = {1, g.n0, (long long)g.n0 * g.n1};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
  double C = 0.0, G = __ldg(in + (long long)GAMMA * g.ntot + idx);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double *pa = in + (long long)(AU0 + i) * g.ntot + idx, *pe = in + (long long)(EU0 + i) * g.ntot + idx;
    const double a = __ldg(pa), e = __ldg(pe);
    double dA = fd_d1<ORDER, double>(pa, st[i]) * inv[i], dE = fd_d1<ORDER, double>(pe, st[i]) * inv[i];
    if constexpr (!M::trivial) {
      dA *= rf.ReU(i);
      dE *= rf.ReU(i);
      if (M::ReUdD(i, i)) {
        dA += a * rf.ReUdD(i, i);
        dE += e * rf.ReUdD(i, i);
      }
    }
    C += dE;
    G -= dA;
  }
  if constexpr (!M::trivial) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        if (M::Gammahat(i, j, i)) {
          const double Aj = __ldg(in + (long long)(AU0 + j) * g.ntot + idx) * rf.ReU(j);
          const double Ej = __ldg(in + (long long)(EU0 + j) * g.ntot + idx) * rf.ReU(j);
          C += rf.G(i, j, i) * Ej;
          G += rf.G(i, j, i) * Aj;
        }
  }
  aux[idx] = C;
  aux[g.ntot + idx] = G;
}

// Toroidal dipole (Maxwell/InitialData.py:26-117, System II: psi = Gamma = 0)
// in the grid's basis: A_Cart = F (-y, x, 0), E_Cart = -d_t A_Cart carried to
// xx by the inverse Jacobian of xx_to_Cart and divided by ReU (the
// Curvilinear driver's AidU/ReU, EidU/ReU).  Every point.
template <int CS>
__global__ void maxwell_curvi_id_kernel(paramstruct p, double amp, double lam, double t, double *__restrict__ gfs) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  const int n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1, n2 = p.Nxx_plus_2NGHOSTS2;
  if (i0 >= n0) return;
  const long long ntot = (long long)n0 * n1 * n2, idx = i0 + (long long)n0 * (i1 + (long long)n1 * i2);
  const double xx0 = xx_of(p.xxmin0, p.dxx0, i0, p.NGHOSTS), xx1 = xx_of(p.xxmin1, p.dxx1, i1, p.NGHOSTS),
               xx2 = xx_of(p.xxmin2, p.dxx2, i2, p.NGHOSTS);
  double x[3], J[3][3], Ji[3][3];
  cart_jacobian(coord_params(p), xx0, xx1, xx2, x, J);
  inverse3(J, Ji);
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  const double u = t + r, v = t - r;
  const double eu = exp(-lam * u * u), ev = exp(-lam * v * v);
  const double deu = -2.0 * lam * u * eu, dev = -2.0 * lam * v * ev;
  const double F = amp / r * ((ev - eu) / (r * r) - 2.0 * lam * (v * ev + u * eu) / r);
  const double dF = amp / r * ((dev - deu) / (r * r) - 2.0 * lam * (ev + v * dev + eu + u * deu) / r);
  const double Ac[3] = {-x[1] * F, x[0] * F, 0.0}, Ec[3] = {x[1] * dF, -x[0] * dF, 0.0};
  double s[3] = {1.0, 1.0, 1.0};
  if constexpr (CS != NRGPU_COORD_CARTESIAN) {
    ScaleFactors S;
    scale_factors(coord_params(p), xx0, xx1, xx2, &S);
    for (int i = 0; i < 3; i++) s[i] = S.s[i];  // 1/ReU^i
  }
  for (int i = 0; i < 3; i++) {
    double a = 0.0, e = 0.0;
    for (int j = 0; j < 3; j++) {
      a += Ji[i][j] * Ac[j];
      e += Ji[i][j] * Ec[j];
    }
    gfs[(long long)(AU0 + i) * ntot + idx] = a * s[i];
    gfs[(long long)(EU0 + i) * ntot + idx] = e * s[i];
  }
  gfs[(long long)GAMMA * ntot + idx] = 0.0;
  gfs[(long long)PSI * ntot + idx] = 0.0;
}

template <typename R, typename Tin, typename TStage, int CS, int ORDER>
static int launch_one(const Grid &g, typename InRef<Tin>::type in, const rfm_struct *rfm,
                      const RKEpilogue<TStage> &epi) {
  const R *tab = nullptr;
  if constexpr (CS != NRGPU_COORD_CARTESIAN) {
    if (!rfm) {
      set_error("curvilinear Maxwell needs an rfm_struct");
      return NRGPU_ERR_ARG;
    }
    if constexpr (sizeof(R) == 8) tab = (const R *)rfm->table64;
    else tab = (const R *)rfm->table32;
  }
  InteriorLaunch L = interior_launch(g, 32, 4);
  maxwell_curvi_kernel<R, Tin, CS, ORDER, TStage><<<L.grid, L.block, 0, stream()>>>(g, in, tab, epi);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <typename R, typename Tin, typename TStage>
static int dispatch(const paramstruct *p, const Grid &g, typename InRef<Tin>::type in, const rfm_struct *rfm,
                    const RKEpilogue<TStage> &epi) {
#define MC_CASE(CSV, ORD) \
  if (dispatch_cs(p->CoordSystem) == CSV && p->FD_order == ORD)                                     \
    return launch_one<R, Tin, TStage, CSV, ORD>(g, in, rfm, epi);
  MC_CASE(NRGPU_COORD_CARTESIAN, 2) MC_CASE(NRGPU_COORD_CARTESIAN, 4)
  MC_CASE(NRGPU_COORD_SPHERICAL, 2) MC_CASE(NRGPU_COORD_SPHERICAL, 4)
  MC_CASE(NRGPU_COORD_SINHSPHERICAL, 2) MC_CASE(NRGPU_COORD_SINHSPHERICAL, 4)
  MC_CASE(NRGPU_COORD_SINHCYLINDRICAL, 2) MC_CASE(NRGPU_COORD_SINHCYLINDRICAL, 4)
  MC_CASE(NRGPU_COORD_SINHSYMTP, 2) MC_CASE(NRGPU_COORD_SINHSYMTP, 4)
#undef MC_CASE
  set_error("curvilinear Maxwell: CoordSystem %d with FD_order %d not built", p->CoordSystem, p->FD_order);
  return NRGPU_ERR_UNSUPPORTED;
}

}  // namespace mcurvi

int maxwell_curvi_launch(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a) {
  using namespace mcurvi;
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

}  // namespace nrgpu

using namespace nrgpu;
using namespace nrgpu::mcurvi;

extern "C" {
int MaxwellCurvilinear_rhs_eval(const rfm_struct *rfm, const paramstruct *p, const double *in, double *rhs) {
  NRGPU_REQUIRE(p && in && rhs, "NULL argument");
  StageArgs a{};
  a.stage = -1;
  a.prec = NRGPU_PREC_FP64;
  a.in = in;
  a.in_is_f64 = true;
  a.out = rhs;
  return maxwell_curvi_launch(rfm, p, a);
}
int MaxwellCurvilinear_rhs_eval_f32(const rfm_struct *rfm, const paramstruct *p, const float *in, float *rhs) {
  NRGPU_REQUIRE(p && in && rhs, "NULL argument");
  StageArgs a{};
  a.stage = -1;
  a.prec = NRGPU_PREC_MIXED;
  a.in = in;
  a.in_is_f64 = false;
  a.out = rhs;
  return maxwell_curvi_launch(rfm, p, a);
}
int MaxwellCurvilinear_constraints(const rfm_struct *rfm, const paramstruct *p, const double *in, double *aux) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(in && aux, "NULL argument");
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN || (rfm && rfm->table64), "curvilinear grid needs rfm");
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, 64, 4);
  const double *tab = rfm ? rfm->table64 : nullptr;
#define MCC(CSV, ORD) maxwell_curvi_constraint_kernel<CSV, ORD><<<L.grid, L.block, 0, stream()>>>(g, in, tab, aux)
  switch (dispatch_cs(p->CoordSystem) * 16 + p->FD_order) {
    case NRGPU_COORD_CARTESIAN * 16 + 2: MCC(NRGPU_COORD_CARTESIAN, 2); break;
    case NRGPU_COORD_CARTESIAN * 16 + 4: MCC(NRGPU_COORD_CARTESIAN, 4); break;
    case NRGPU_COORD_SPHERICAL * 16 + 2: MCC(NRGPU_COORD_SPHERICAL, 2); break;
    case NRGPU_COORD_SPHERICAL * 16 + 4: MCC(NRGPU_COORD_SPHERICAL, 4); break;
    case NRGPU_COORD_SINHSPHERICAL * 16 + 2: MCC(NRGPU_COORD_SINHSPHERICAL, 2); break;
    case NRGPU_COORD_SINHSPHERICAL * 16 + 4: MCC(NRGPU_COORD_SINHSPHERICAL, 4); break;
    case NRGPU_COORD_SINHCYLINDRICAL * 16 + 2: MCC(NRGPU_COORD_SINHCYLINDRICAL, 2); break;
    case NRGPU_COORD_SINHCYLINDRICAL * 16 + 4: MCC(NRGPU_COORD_SINHCYLINDRICAL, 4); break;
    case NRGPU_COORD_SINHSYMTP * 16 + 2: MCC(NRGPU_COORD_SINHSYMTP, 2); break;
    case NRGPU_COORD_SINHSYMTP * 16 + 4: MCC(NRGPU_COORD_SINHSYMTP, 4); break;
    default: set_error("curvilinear Maxwell constraints: FD_order %d not built", p->FD_order); return NRGPU_ERR_UNSUPPORTED;
  }
#undef MCC
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
int MaxwellCurvilinear_initial_data_toroidal_dipole(const paramstruct *p, double amp, double lam, double time,
                                                    double *gfs) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(gfs != nullptr, "NULL argument");
  NRGPU_REQUIRE(lam > 0.0, "lam must be positive");
  dim3 block(64), grid((p->Nxx_plus_2NGHOSTS0 + 63) / 64, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2);
  switch (p->CoordSystem) {
    case NRGPU_COORD_CARTESIAN:
      maxwell_curvi_id_kernel<NRGPU_COORD_CARTESIAN><<<grid, block, 0, stream()>>>(*p, amp, lam, time, gfs);
      break;
    case NRGPU_COORD_SPHERICAL:
      maxwell_curvi_id_kernel<NRGPU_COORD_SPHERICAL><<<grid, block, 0, stream()>>>(*p, amp, lam, time, gfs);
      break;
    default:
      maxwell_curvi_id_kernel<NRGPU_COORD_SINHSPHERICAL><<<grid, block, 0, stream()>>>(*p, amp, lam, time, gfs);
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
}
