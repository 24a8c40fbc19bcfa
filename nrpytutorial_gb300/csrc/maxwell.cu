// maxwell.cu -- vacuum Maxwell equations, System I, Cartesian
// (Maxwell/VacuumMaxwell_Flat_Evol_Cartesian.py:54-74):
//   d_t A^i = -E^i - d_i psi
//   d_t E^i = sum_j ( -d_j d_j A^i + d_j d_i A^j )
//   d_t psi = -d_i A^i
// The j == i terms of the E equation cancel identically (the reference's
// symbolic sum drops them), so only j != i is evaluated.  Gridfunctions
// in alphabetical order: AU0 AU1 AU2 EU0 EU1 EU2 psi.
// Constraint (:49-52): C = d_i E^i.
#include "epilogue.cuh"
#include "fd.cuh"
#include "systems.cuh"

namespace nrgpu {

template <typename R, typename Tin, int ORDER, typename TStage>
__global__ void __launch_bounds__(256)
    maxwell_kernel(Grid g, typename InRef<Tin>::type in, RKEpilogue<TStage> epi) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  const long long st[3] = {1, g.n0, (long long)g.n0 * g.n1};
  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  decltype(in + idx) A[3], E[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    A[i] = in + (long long)i * g.ntot + idx;
    E[i] = in + (long long)(3 + i) * g.ntot + idx;
  }
  const auto psi = in + 6LL * g.ntot + idx;
  R divA = (R)0;
#pragma unroll
  for (int i = 0; i < 3; i++) divA += fd_d1<ORDER, R>(A[i], st[i]) * inv[i];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const R Ei = val<R>(E[i]);
    const R dpsi = fd_d1<ORDER, R>(psi, st[i]) * inv[i];
    epi(i, idx, -Ei - dpsi);
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R rhs = (R)0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (j == i) continue;
      rhs += -(fd_d2<ORDER, R>(A[i], st[j]) * (inv[j] * inv[j]));
      rhs += fd_d11<ORDER, R>(A[j], st[j], st[i]) * (inv[j] * inv[i]);
    }
    epi(3 + i, idx, rhs);
  }
  epi(6, idx, -divA);
}

template <int ORDER>
__global__ void maxwell_constraint_kernel(Grid g, const double *__restrict__ in, double *__restrict__ aux) {
  int i0, i1, i2;
  long long idx;
  if (!interior_point(g, i0, i1, i2, idx)) return;
  const long long st[3] = {1, g.n0, (long long)g.n0 * g.n1};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  double c = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) c += fd_d1<ORDER, double>(in + (long long)(3 + i) * g.ntot + idx, st[i]) * inv[i];
  aux[idx] = c;
}

template <typename R, typename Tin, typename TStage>
static int dispatch(const paramstruct *p, const Grid &g, typename InRef<Tin>::type in,
                    const RKEpilogue<TStage> &epi) {
  InteriorLaunch L = interior_launch(g, 64, 4);
  switch (p->FD_order) {
    case 2: maxwell_kernel<R, Tin, 2, TStage><<<L.grid, L.block, 0, stream()>>>(g, in, epi); break;
    case 4: maxwell_kernel<R, Tin, 4, TStage><<<L.grid, L.block, 0, stream()>>>(g, in, epi); break;
    case 6: maxwell_kernel<R, Tin, 6, TStage><<<L.grid, L.block, 0, stream()>>>(g, in, epi); break;
    case 8: maxwell_kernel<R, Tin, 8, TStage><<<L.grid, L.block, 0, stream()>>>(g, in, epi); break;
    default: set_error("Maxwell: FD_order %d not built", p->FD_order); return NRGPU_ERR_UNSUPPORTED;
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int maxwell_launch(const paramstruct *p, const StageArgs &a) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN, "Maxwell System I is Cartesian only");
  Grid g = make_grid(p);
  if (a.prec == NRGPU_PREC_FP64) {
    RKEpilogue<double> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (double *)a.out};
    return dispatch<double, double, double>(p, g, stage_input<double>(a), epi);
  }
  if (pair_precision(a.prec)) {
    RKEpilogue<float2> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float2 *)a.out, stage_consts(a.dt),
                           a.prec == NRGPU_PREC_COMPENSATED_FP64RK};
    return dispatch<float, Pair32, float2>(p, g, stage_input<Pair32>(a), epi);
  }
  RKEpilogue<float> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float *)a.out, stage_consts(a.dt)};
  if (a.in_is_f64) return dispatch<float, double, float>(p, g, stage_input<double>(a), epi);
  return dispatch<float, float, float>(p, g, stage_input<float>(a), epi);
}

}  // namespace nrgpu

using namespace nrgpu;

extern "C" {
int Maxwell_rhs_eval(const paramstruct *p, const double *in, double *rhs) {
  NRGPU_REQUIRE(p && in && rhs, "NULL argument");
  StageArgs a{};
  a.stage = -1;
  a.prec = NRGPU_PREC_FP64;
  a.in = in;
  a.in_is_f64 = true;
  a.out = rhs;
  return maxwell_launch(p, a);
}
int Maxwell_rhs_eval_f32(const paramstruct *p, const float *in, float *rhs) {
  NRGPU_REQUIRE(p && in && rhs, "NULL argument");
  StageArgs a{};
  a.stage = -1;
  a.prec = NRGPU_PREC_MIXED;
  a.in = in;
  a.in_is_f64 = false;
  a.out = rhs;
  return maxwell_launch(p, a);
}
int Maxwell_Constraints(const paramstruct *p, const double *in, double *aux) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(in && aux, "NULL argument");
  Grid g = make_grid(p);
  InteriorLaunch L = interior_launch(g, 64, 4);
  switch (p->FD_order) {
    case 2: maxwell_constraint_kernel<2><<<L.grid, L.block, 0, stream()>>>(g, in, aux); break;
    case 4: maxwell_constraint_kernel<4><<<L.grid, L.block, 0, stream()>>>(g, in, aux); break;
    case 6: maxwell_constraint_kernel<6><<<L.grid, L.block, 0, stream()>>>(g, in, aux); break;
    case 8: maxwell_constraint_kernel<8><<<L.grid, L.block, 0, stream()>>>(g, in, aux); break;
    default: set_error("FD_order %d not built", p->FD_order); return NRGPU_ERR_UNSUPPORTED;
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
}
