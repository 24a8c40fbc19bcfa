// fd.cuh -- finite-difference stencils on IDX4S gridfunctions.
//
// Coefficients are those of finite_difference.py:252-369 (Vandermonde
// inverse, exact rationals), written out for orders 2..8:
//   centred 1st derivative  f' = invdx * sum_{k=1..R} C1[k] (f[+k] - f[-k])
//   centred 2nd derivative  f''= invdx^2 (C2[0] f[0] + sum_k C2[k](f[+k]+f[-k]))
//   mixed 2nd derivative    product of two centred 1st-derivative stencils
//   upwind 1st derivative   ("dupD", stencil shifted +1) and its mirror
//                           ("ddnD", shifted -1, weights negated and reversed)
// Control-vector upwinding (finite_difference_helpers.py:790-820) picks dupD
// where the control component is > 0 and ddnD otherwise; here one stencil is
// evaluated with a signed stride instead of blending both.
#pragma once
#include "common.cuh"

namespace nrgpu {

template <int ORDER> struct FDCoef;

// Coefficients as constexpr functions of the (unrolled, hence constant)
// offset, usable from both host and device code.  ko(k), k = 0..R+1, are the
// Kreiss-Oliger weights of the symmetric (ORDER+3)-point stencil: the
// (ORDER+2)-th derivative times (-1)^((ORDER+4)/2) / 2^(ORDER+2)
// (finite_difference.py:252-258, 310-313, 331-334).
#define NRGPU_FD_TABLE(NAME, ...)                                              \
  __host__ __device__ static constexpr double NAME(int k) {                    \
    constexpr double t[] = {__VA_ARGS__};                                      \
    return t[k];                                                               \
  }

template <> struct FDCoef<2> {
  static constexpr int R = 1;
  static constexpr int UPLO = 0;  // dupD offsets 0..2
  NRGPU_FD_TABLE(c1, 0.0, 1.0 / 2.0)
  NRGPU_FD_TABLE(c2, -2.0, 1.0)
  NRGPU_FD_TABLE(up, -3.0 / 2.0, 2.0, -1.0 / 2.0)
  NRGPU_FD_TABLE(ko, -3.0 / 8.0, 1.0 / 4.0, -1.0 / 16.0)
};
template <> struct FDCoef<4> {
  static constexpr int R = 2;
  static constexpr int UPLO = -1;  // dupD offsets -1..3
  NRGPU_FD_TABLE(c1, 0.0, 2.0 / 3.0, -1.0 / 12.0)
  NRGPU_FD_TABLE(c2, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0)
  NRGPU_FD_TABLE(up, -1.0 / 4.0, -5.0 / 6.0, 3.0 / 2.0, -1.0 / 2.0, 1.0 / 12.0)
  NRGPU_FD_TABLE(ko, -5.0 / 16.0, 15.0 / 64.0, -3.0 / 32.0, 1.0 / 64.0)
};
template <> struct FDCoef<6> {
  static constexpr int R = 3;
  static constexpr int UPLO = -2;  // dupD offsets -2..4
  NRGPU_FD_TABLE(c1, 0.0, 3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0)
  NRGPU_FD_TABLE(c2, -49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0)
  NRGPU_FD_TABLE(up, 1.0 / 30.0, -2.0 / 5.0, -7.0 / 12.0, 4.0 / 3.0, -1.0 / 2.0, 2.0 / 15.0, -1.0 / 60.0)
  NRGPU_FD_TABLE(ko, -35.0 / 128.0, 7.0 / 32.0, -7.0 / 64.0, 1.0 / 32.0, -1.0 / 256.0)
};
template <> struct FDCoef<8> {
  static constexpr int R = 4;
  static constexpr int UPLO = -3;  // dupD offsets -3..5
  NRGPU_FD_TABLE(c1, 0.0, 4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0)
  NRGPU_FD_TABLE(c2, -205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0)
  NRGPU_FD_TABLE(up, -1.0 / 168.0, 1.0 / 14.0, -1.0 / 2.0, -9.0 / 20.0, 5.0 / 4.0, -1.0 / 2.0, 1.0 / 6.0,
                 -1.0 / 28.0, 1.0 / 280.0)
  NRGPU_FD_TABLE(ko, -63.0 / 256.0, 105.0 / 512.0, -15.0 / 128.0, 45.0 / 1024.0, -5.0 / 512.0, 1.0 / 1024.0)
};
#undef NRGPU_FD_TABLE

// Loads go through the read-only path; p points at the stencil centre.
template <typename T, typename R>
__device__ __forceinline__ R ld(const T *p, long long off) {
  return (R)__ldg(p + off);
}

// Centred first derivative along stride s (unscaled by invdx).
template <int ORDER, typename R, typename T>
__device__ __forceinline__ R fd_d1(const T *__restrict__ p, long long s) {
  using C = FDCoef<ORDER>;
  R acc = (R)C::c1(1) * (ld<T, R>(p, s) - ld<T, R>(p, -s));
#pragma unroll
  for (int k = 2; k <= C::R; k++) acc += (R)C::c1(k) * (ld<T, R>(p, k * s) - ld<T, R>(p, -k * s));
  return acc;
}

// Centred second derivative along stride s (unscaled by invdx^2).
template <int ORDER, typename R, typename T>
__device__ __forceinline__ R fd_d2(const T *__restrict__ p, long long s) {
  using C = FDCoef<ORDER>;
  R acc = (R)C::c2(0) * ld<T, R>(p, 0);
#pragma unroll
  for (int k = 1; k <= C::R; k++) acc += (R)C::c2(k) * (ld<T, R>(p, k * s) + ld<T, R>(p, -k * s));
  return acc;
}

// Mixed second derivative along strides s and t (unscaled).
template <int ORDER, typename R, typename T>
__device__ __forceinline__ R fd_d11(const T *__restrict__ p, long long s, long long t) {
  using C = FDCoef<ORDER>;
  R acc = (R)0;
#pragma unroll
  for (int a = 1; a <= C::R; a++) {
    R inner = (R)0;
#pragma unroll
    for (int b = 1; b <= C::R; b++) {
      const long long ps = a * s, qt = b * t;
      inner += (R)C::c1(b) * ((ld<T, R>(p, ps + qt) - ld<T, R>(p, ps - qt)) -
                              (ld<T, R>(p, -ps + qt) - ld<T, R>(p, -ps - qt)));
    }
    acc += (R)C::c1(a) * inner;
  }
  return acc;
}

// Kreiss-Oliger derivative along stride s (unscaled by invdx).
template <int ORDER, typename R, typename T>
__device__ __forceinline__ R fd_ko(const T *__restrict__ p, long long s) {
  using C = FDCoef<ORDER>;
  R acc = (R)C::ko(0) * ld<T, R>(p, 0);
#pragma unroll
  for (int k = 1; k <= C::R + 1; k++) acc += (R)C::ko(k) * (ld<T, R>(p, k * s) + ld<T, R>(p, -k * s));
  return acc;
}

// ------------------------------------------------ FP32 pair gridfunctions
// A gridfunction stored as interleaved FP32 pairs (hi, lo) whose sum is the
// FP64 value v: hi = FP32(v), lo = FP32(v - hi).  Stencils treat the two
// parts separately: differences of neighbouring hi values are exact in
// FP32 whenever the values are within a factor 2 of each other (Sterbenz)
// and otherwise round relative to the difference, so a derivative loses
// nothing to the FP32 storage of a large smooth field; lo is small and goes
// through the plain stencil.  One 8-byte load fetches both parts.
struct Pair32 {};  // stage-input tag: the input array is `const float2 *`

// Input pointer type of a kernel whose stage input is `Tin`.
template <typename Tin> struct InRef {
  using type = const Tin *__restrict__;
};
template <> struct InRef<Pair32> {
  using type = const float2 *__restrict__;
};

// Value at the stencil centre.
template <typename R, typename T> __device__ __forceinline__ R val(const T *p) { return (R)__ldg(p); }
template <typename R> __device__ __forceinline__ R val(const float2 *p) {
  const float2 v = __ldg(p);
  return (R)v.x + (R)v.y;
}

template <int ORDER, typename R> __device__ __forceinline__ R fd_d1(const float2 *__restrict__ p, long long s) {
  using C = FDCoef<ORDER>;
  R hi = (R)0, lo = (R)0;
#pragma unroll
  for (int k = 1; k <= C::R; k++) {
    const float2 a = __ldg(p + k * s), b = __ldg(p - k * s);
    hi += (R)C::c1(k) * ((R)a.x - (R)b.x);
    lo += (R)C::c1(k) * ((R)a.y - (R)b.y);
  }
  return hi + lo;
}
// Second derivative over v[k] - v[0] (the weights sum to zero).
template <int ORDER, typename R> __device__ __forceinline__ R fd_d2(const float2 *__restrict__ p, long long s) {
  using C = FDCoef<ORDER>;
  const float2 c = __ldg(p);
  R hi = (R)0, lo = (R)C::c2(0) * (R)c.y;
#pragma unroll
  for (int k = 1; k <= C::R; k++) {
    const float2 a = __ldg(p + k * s), b = __ldg(p - k * s);
    hi += (R)C::c2(k) * (((R)a.x - (R)c.x) + ((R)b.x - (R)c.x));
    lo += (R)C::c2(k) * ((R)a.y + (R)b.y);
  }
  return hi + lo;
}
// Kreiss-Oliger derivative over v[k] - v[0] (the weights sum to zero).
template <int ORDER, typename R> __device__ __forceinline__ R fd_ko(const float2 *__restrict__ p, long long s) {
  using C = FDCoef<ORDER>;
  const float2 c = __ldg(p);
  R hi = (R)0, lo = (R)C::ko(0) * (R)c.y;
#pragma unroll
  for (int k = 1; k <= C::R + 1; k++) {
    const float2 a = __ldg(p + k * s), b = __ldg(p - k * s);
    hi += (R)C::ko(k) * (((R)a.x - (R)c.x) + ((R)b.x - (R)c.x));
    lo += (R)C::ko(k) * ((R)a.y + (R)b.y);
  }
  return hi + lo;
}
template <int ORDER, typename R>
__device__ __forceinline__ R fd_d11(const float2 *__restrict__ p, long long s, long long t) {
  using C = FDCoef<ORDER>;
  R hi = (R)0, lo = (R)0;
#pragma unroll
  for (int a = 1; a <= C::R; a++) {
    R ih = (R)0, il = (R)0;
#pragma unroll
    for (int b = 1; b <= C::R; b++) {
      const long long ps = a * s, qt = b * t;
      const float2 pp = __ldg(p + ps + qt), pm = __ldg(p + ps - qt);
      const float2 mp = __ldg(p - ps + qt), mm = __ldg(p - ps - qt);
      ih += (R)C::c1(b) * (((R)pp.x - (R)pm.x) - ((R)mp.x - (R)mm.x));
      il += (R)C::c1(b) * (((R)pp.y - (R)pm.y) - ((R)mp.y - (R)mm.y));
    }
    hi += (R)C::c1(a) * ih;
    lo += (R)C::c1(a) * il;
  }
  return hi + lo;
}
// Upwinded derivative over v[k] - v[0] (the weights sum to zero).
template <int ORDER, typename R>
__device__ __forceinline__ R fd_dupwind(const float2 *__restrict__ p, long long s, bool positive) {
  using C = FDCoef<ORDER>;
  const long long ss = positive ? s : -s;
  const float2 c = __ldg(p);
  R hi = (R)0, lo = (R)0;
#pragma unroll
  for (int j = 0; j <= ORDER; j++) {
    const int k = j + C::UPLO;
    if (C::up(j) == 0.0) continue;
    if (k == 0) {
      lo += (R)C::up(j) * (R)c.y;
    } else {
      const float2 v = __ldg(p + k * ss);
      hi += (R)C::up(j) * ((R)v.x - (R)c.x);
      lo += (R)C::up(j) * (R)v.y;
    }
  }
  const R acc = hi + lo;
  return positive ? acc : -acc;
}

// ------------------------------------------- float-float (FP32 pair) arithmetic
// Error-free transformations on the FP32 pipe (Dekker 1971; Knuth, TAOCP
// vol. 2, 4.2.2; the FMA form of the product): a value is the unevaluated
// sum hi + lo with |lo| <= ulp(hi)/2, about 48 significant bits.  Written
// with round-to-nearest intrinsics so no contraction changes them.
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
// a + b, both pairs; normalised result.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  float2 s = ff_two_sum(a.x, b.x);
  const float2 t = ff_two_sum(a.y, b.y);
  s = ff_fast_two_sum(s.x, __fadd_rn(s.y, t.x));
  return ff_fast_two_sum(s.x, __fadd_rn(s.y, t.y));
}
// k * C, k an FP32 value, C a pair constant; normalised result.
__device__ __forceinline__ float2 ff_mul(float k, float2 C) {
  const float p = __fmul_rn(k, C.x);
  const float e = __fmaf_rn(k, C.x, -p);
  return ff_fast_two_sum(p, __fmaf_rn(k, C.y, e));
}

// a * b, both pairs (Dekker's product with the FMA error term).
__device__ __forceinline__ float2 ff_mul_ff(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }

// FP64 value -> (hi, lo) pair.
__device__ __forceinline__ float2 split_pair(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(__dsub_rn(v, (double)h)));
}
__device__ __forceinline__ double pair_value(float2 p) { return (double)p.x + (double)p.y; }

// The same conversions without the FP64 pipe (GB300 issues FP64 at 1/64 of
// the FP32 rate).  float -> double is exact bit manipulation for zero and
// normal floats; double -> pair truncates the significand after 24 bits for
// hi (integer ops), converts the remaining 29 bits with one int->float
// conversion scaled by an exact power of two, and normalises with an FP32
// fast two-sum, so hi = RN(v) up to double rounding and hi + lo = v to
// 2^-48 relative.  Zero is exact; values outside [2^-74, 2^128) (and inf,
// NaN) take the FP64-pipe path.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if ((u << 1) == 0) return __longlong_as_double((long long)sign);  // +-0
  const unsigned ex = (u >> 23) & 0xFFu;
  if (ex == 0 || ex == 0xFFu) return (double)f;                   // subnormal, inf, NaN
  return __longlong_as_double((long long)(sign | ((unsigned long long)(ex + 896u) << 52) |
                                          ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}
__device__ __forceinline__ float2 split_pair_fast(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  if ((b << 1) == 0) return make_float2(__uint_as_float(sign), 0.f);  // +-0
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < -74 || e > 127) return split_pair(v);
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
  const float mag = __fmul_rn(__uint2float_rn((unsigned)(b & 0x1FFFFFFFu)), __uint_as_float((unsigned)(e + 75) << 23));
  return ff_fast_two_sum(hi, sign ? -mag : mag);
}

// Upwinded first derivative (unscaled): dupD if positive, else ddnD.
// ddnD weights are the negated mirror image of dupD's, so one loop with a
// signed stride evaluates whichever one the control vector selects.
template <int ORDER, typename R, typename T>
__device__ __forceinline__ R fd_dupwind(const T *__restrict__ p, long long s, bool positive) {
  using C = FDCoef<ORDER>;
  const long long ss = positive ? s : -s;
  R acc = (R)0;
#pragma unroll
  for (int j = 0; j <= ORDER; j++) {
    const int k = j + C::UPLO;
    if (C::up(j) != 0.0) acc += (R)C::up(j) * ld<T, R>(p, k * ss);
  }
  return positive ? acc : -acc;
}

}  // namespace nrgpu
