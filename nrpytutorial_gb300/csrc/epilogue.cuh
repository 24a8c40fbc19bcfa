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
// With FP32 stage buffers (mixed and compensated precision) GB300's FP64
// pipe, which issues at 1/64 of the FP32 rate, would bound the update, so
// the RK accumulation runs in float-float arithmetic on the FP32 pipe: at
// the start of the step y_n is split in place into (hi, lo) pairs (the
// y_n buffer holds pairs until substep 3), the running total is kept as
// pairs in the rt buffer, dt*c are pair constants formed on the host, and
// substep 3 writes y_n back as the FP64 sum hi + lo.  Accumulation then
// carries ~48 significant bits (2^-48 ~ 3.6e-15 relative per update)
// instead of FP64's 53, far below the FP32 RHS arithmetic's error, with
// about 3 FP64-pipe instructions per value per step instead of ~26.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "fd.cuh"

namespace nrgpu {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// dt/6, dt/3, dt/2 and dt as FP32 (hi, lo) pairs (host).
struct StageConsts {
  float2 c6, c3, c2, c1;
};
inline float2 pair_const(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}
inline StageConsts stage_consts(double dt) {
  return StageConsts{pair_const(dt * (1.0 / 6.0)), pair_const(dt * (1.0 / 3.0)), pair_const(dt * 0.5),
                     pair_const(dt)};
}

// Float-float RK4 substep on loaded values (FP32 stage modes): y the y_n
// pair, r the running-total pair (not read by substep 0; updated in place by
// substeps 0..2); returns the stage value (substeps 0..2) or the new y_n
// pair (substep 3).  Every FP32-stage update goes through this function, so
// all of them round alike.
__device__ __forceinline__ float2 ff_rk4_pairs(int stage, float k, const StageConsts &kc, float2 y, float2 &r) {
  switch (stage) {
    case 0:
      r = ff_mul(k, kc.c6);
      return ff_add(y, ff_mul(k, kc.c2));
    case 1:
      r = ff_add(r, ff_mul(k, kc.c3));
      return ff_add(y, ff_mul(k, kc.c2));
    case 2:
      r = ff_add(r, ff_mul(k, kc.c3));
      return ff_add(y, ff_mul(k, kc.c1));
    default:
      return ff_add(ff_add(y, r), ff_mul(k, kc.c6));
  }
}

// The same update of value i in memory: y_n and rt hold (hi, lo) pairs;
// returns the stage value (substeps 0..2) or writes y_n[i] as FP64
// (substep 3).  Used by the unfused update kernel.
__device__ __forceinline__ float2 ff_rk4_update(int stage, float k, const StageConsts &kc, double *y_n, double *rt,
                                                long long i) {
  float2 *y2 = (float2 *)y_n, *r2 = (float2 *)rt;
  float2 r = (stage > 0) ? r2[i] : make_float2(0.f, 0.f);
  const float2 s = ff_rk4_pairs(stage, k, kc, y2[i], r);
  if (stage < 3) r2[i] = r;
  else y_n[i] = f2d_bits(s.x) + f2d_bits(s.y);
  return s;
}

// RK4 substep update of one value; stage < 0 stores k itself into `out`.
template <typename TStage> struct RKEpilogue {
  int stage;          // -1: plain store; 0..3: RK4 substep
  double dt;
  long long ntot;     // gridfunction stride
  double *y_n;        // FP64 state
  double *rt;         // FP64 running total
  TStage *out;        // stage buffer (or rhs buffer for stage -1); float2:
                      // FP32 (hi, lo) pairs of the FP64 stage value
  StageConsts kc;     // FP32 stage buffers: dt*c pairs (stage_consts(dt))
  bool f64_update;    // FP32 stage buffers: RK update in FP64 arithmetic on the
                      // FP64 y_n and running total (NRGPU_PREC_COMPENSATED_FP64RK)
                      // instead of float-float on their pair form

  // Stage value (computed in FP64) into the stage buffer.
  __device__ __forceinline__ void put(long long i, double v) const {
    if constexpr (std::is_same<TStage, float2>::value) out[i] = split_pair(v);
    else out[i] = (TStage)v;
  }
  // Stage value (a normalised pair) into an FP32 stage buffer: the pair, or
  // its leading part (the FP32 rounding of the sum) for plain FP32 stages.
  __device__ __forceinline__ void put_pair(long long i, float2 v) const {
    if constexpr (std::is_same<TStage, float2>::value) out[i] = v;
    else out[i] = (TStage)v.x;
  }

  // The y_n and running-total words the update of value (gf, idx) reads
  // (FP64 values, or (hi, lo) pairs as raw 8-byte words), so that a kernel
  // can issue these loads early, with its stencil loads; apply() then does
  // the update on them.
  struct Operands {
    double y, r;
  };
  __device__ __forceinline__ Operands fetch(int gf, long long idx) const {
    Operands o{0.0, 0.0};
    if (stage < 0) return o;
    const long long i = (long long)gf * ntot + idx;
    o.y = y_n[i];
    if (stage > 0) o.r = rt[i];
    return o;
  }
  __device__ __forceinline__ static float2 as_pair(double w) {
    const long long b = __double_as_longlong(w);
    return make_float2(__int_as_float((int)(b & 0xffffffffLL)), __int_as_float((int)(b >> 32)));
  }

  template <typename R>
  __device__ __forceinline__ void apply(int gf, long long idx, R value, const Operands &o) const {
    const long long i = (long long)gf * ntot + idx;
    if (stage < 0) {
      if constexpr (std::is_same<TStage, float2>::value) out[i] = make_float2((float)value, 0.f);
      else out[i] = (TStage)value;
      return;
    }
    if constexpr (!std::is_same<TStage, double>::value) {
      if (!f64_update) {
        float2 r = as_pair(o.r);
        const float2 v = ff_rk4_pairs(stage, (float)value, kc, as_pair(o.y), r);
        if (stage < 3) {
          ((float2 *)rt)[i] = r;
          put_pair(i, v);
        } else {
          y_n[i] = f2d_bits(v.x) + f2d_bits(v.y);
        }
        return;
      }
    }
    const double kdt = dmul((double)value, dt);
    switch (stage) {
      case 0:
        rt[i] = dmul(kdt, 1.0 / 6.0);
        put(i, dadd(o.y, dmul(kdt, 1.0 / 2.0)));
        break;
      case 1:
        rt[i] = dadd(o.r, dmul(kdt, 1.0 / 3.0));
        put(i, dadd(o.y, dmul(kdt, 1.0 / 2.0)));
        break;
      case 2:
        rt[i] = dadd(o.r, dmul(kdt, 1.0 / 3.0));
        put(i, dadd(o.y, kdt));
        break;
      default:
        y_n[i] = dadd(dadd(o.y, o.r), dmul(kdt, 1.0 / 6.0));
        break;
    }
  }

  template <typename R> __device__ __forceinline__ void operator()(int gf, long long idx, R value) const {
    apply(gf, idx, value, fetch(gf, idx));
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

// Start of an FP32-stage step (single grid or batch): the n doubles of y_n
// split in place into (hi, lo) pairs (the float-float accumulation state of
// the epilogue, and the compensated substep-0 input); for plain FP32 stages
// also y_n rounded to FP32 into f (substep 0's input).
// In place, so each thread loads 4 values before it stores their pairs.
template <bool ROUND>
__global__ void split_state_kernel(long long n, double *__restrict__ y, float *__restrict__ f) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
    double v[4];
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (i0 + j * stride < n) v[j] = y[i0 + j * stride];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const long long i = i0 + j * stride;
      if (i < n) {
        const float2 p = split_pair_fast(v[j]);
        if (ROUND) f[i] = p.x;
        ((float2 *)y)[i] = p;
      }
    }
  }
}

}  // namespace nrgpu
