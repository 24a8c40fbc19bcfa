// dualn.cuh -- forward-mode dual numbers with N tangent components.
//
// DualN<N> carries a value v and its derivatives d[0..N-1] with respect to N
// parameters; + - * / propagate them by the chain rule, comparisons look at
// the value only (so a branch such as the upwind switch beta^k > 0 follows
// the value, and the tangent is that branch's derivative).  The BSSN algebra
// of bssn.cuh is generic in its arithmetic type and uses only + - * / on it,
// so instantiating it with DualN gives the tangent-linear RHS: the value
// and N directional derivatives in one pass.
#pragma once

namespace nrgpu {

template <int N> struct DualN {
  double v;
  double d[N];
  __host__ __device__ DualN() {}
  __host__ __device__ DualN(double c) : v(c) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.0;
  }
  __host__ __device__ DualN &operator+=(const DualN &b) {
    v += b.v;
#pragma unroll
    for (int k = 0; k < N; k++) d[k] += b.d[k];
    return *this;
  }
  __host__ __device__ DualN &operator-=(const DualN &b) {
    v -= b.v;
#pragma unroll
    for (int k = 0; k < N; k++) d[k] -= b.d[k];
    return *this;
  }
  __host__ __device__ DualN &operator*=(const DualN &b) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = d[k] * b.v + v * b.d[k];
    v *= b.v;
    return *this;
  }
};

template <int N> __host__ __device__ __forceinline__ DualN<N> operator+(DualN<N> a, const DualN<N> &b) {
  a += b;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator-(DualN<N> a, const DualN<N> &b) {
  a -= b;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator-(const DualN<N> &a) {
  DualN<N> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -a.d[k];
  return r;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator*(DualN<N> a, const DualN<N> &b) {
  a *= b;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator/(const DualN<N> &a, const DualN<N> &b) {
  DualN<N> r;
  r.v = a.v / b.v;  // the value exactly as plain FP64 arithmetic computes it
  const double inv = 1.0 / b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
  return r;
}
// mixed with plain doubles
template <int N> __host__ __device__ __forceinline__ DualN<N> operator*(double c, DualN<N> a) {
  a.v *= c;
#pragma unroll
  for (int k = 0; k < N; k++) a.d[k] *= c;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator*(DualN<N> a, double c) { return c * a; }
template <int N> __host__ __device__ __forceinline__ DualN<N> operator+(DualN<N> a, double c) {
  a.v += c;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator+(double c, DualN<N> a) { return a + c; }
template <int N> __host__ __device__ __forceinline__ DualN<N> operator-(DualN<N> a, double c) {
  a.v -= c;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator-(double c, const DualN<N> &a) {
  return DualN<N>(c) - a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator/(DualN<N> a, double c) {
  a.v /= c;
#pragma unroll
  for (int k = 0; k < N; k++) a.d[k] /= c;
  return a;
}
template <int N> __host__ __device__ __forceinline__ DualN<N> operator/(double c, const DualN<N> &b) {
  return DualN<N>(c) / b;
}
template <int N> __host__ __device__ __forceinline__ bool operator>(const DualN<N> &a, const DualN<N> &b) {
  return a.v > b.v;
}
template <int N> __host__ __device__ __forceinline__ bool operator<(const DualN<N> &a, const DualN<N> &b) {
  return a.v < b.v;
}
template <int N> __host__ __device__ __forceinline__ bool operator!=(const DualN<N> &a, const DualN<N> &b) {
  return a.v != b.v;
}

}  // namespace nrgpu
