// epilogue.cuh -- what an RHS kernel does with the RHS value it computed at
// an interior point: store it (plain rhs_eval) or apply the RK4 update of
// that substep in place (fused MoL step).
//
// The RK4 update is the "diagonal" low-storage form that
// MoLtimestepping/C_Code_Generation.py:266-329 emits for RK_method "RK4"
// (Butcher table RK_Butcher_Table_Dictionary.py:86-91), with k the RHS:
//   substep 0: rt  = k*dt*(1/6);        out = y_n + k*dt*(1/2)
//   substep 1: rt  = rt + k*dt*(1/3);   out = y_n + k*dt*(1/2)
//   substep 2: rt  = rt + k*dt*(1/3);   out = y_n + k*dt
//   substep 3: y_n = y_n + rt + k*dt*(1/6)
// evaluated left to right in FP64 without FMA contraction, exactly as the
// generated C writes it, so the fused update rounds like the reference's.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "fd.cuh"

namespace nrgpu {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// RK4 substep update of one value; stage < 0 stores k itself into `out`.
template <typename TStage> struct RKEpilogue {
  int stage;          // -1: plain store; 0..3: RK4 substep
  double dt;
  long long ntot;     // gridfunction stride
  double *y_n;        // FP64 state
  double *rt;         // FP64 running total
  TStage *out;        // stage buffer (or rhs buffer for stage -1); float2:
                      // FP32 (hi, lo) pairs of the FP64 stage value

  // Stage value (computed in FP64) into the stage buffer.
  __device__ __forceinline__ void put(long long i, double v) const {
    if constexpr (std::is_same<TStage, float2>::value) out[i] = split_pair(v);
    else out[i] = (TStage)v;
  }

  template <typename R> __device__ __forceinline__ void operator()(int gf, long long idx, R value) const {
    const long long i = (long long)gf * ntot + idx;
    if (stage < 0) {
      if constexpr (std::is_same<TStage, float2>::value) out[i] = make_float2((float)value, 0.f);
      else out[i] = (TStage)value;
      return;
    }
    const double kdt = dmul((double)value, dt);
    switch (stage) {
      case 0:
        rt[i] = dmul(kdt, 1.0 / 6.0);
        put(i, dadd(y_n[i], dmul(kdt, 1.0 / 2.0)));
        break;
      case 1:
        rt[i] = dadd(rt[i], dmul(kdt, 1.0 / 3.0));
        put(i, dadd(y_n[i], dmul(kdt, 1.0 / 2.0)));
        break;
      case 2:
        rt[i] = dadd(rt[i], dmul(kdt, 1.0 / 3.0));
        put(i, dadd(y_n[i], kdt));
        break;
      default:
        y_n[i] = dadd(dadd(y_n[i], rt[i]), dmul(kdt, 1.0 / 6.0));
        break;
    }
  }
};

// Interior point indices of the standard interior launch; false if outside.
__device__ __forceinline__ bool interior_point(const Grid &g, int &i0, int &i1, int &i2, long long &idx) {
  i0 = g.ng + blockIdx.x * blockDim.x + threadIdx.x;
  i1 = g.ng + blockIdx.y * blockDim.y + threadIdx.y;
  i2 = g.ng + blockIdx.z;
  if (i0 >= g.n0 - g.ng || i1 >= g.n1 - g.ng) return false;
  idx = (long long)i0 + (long long)g.n0 * ((long long)i1 + (long long)g.n1 * i2);
  return true;
}

}  // namespace nrgpu
