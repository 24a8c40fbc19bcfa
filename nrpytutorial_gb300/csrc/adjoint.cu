// adjoint.cu -- discrete adjoints of the Maxwell (System I, Cartesian) and
// ScalarWave (Cartesian and curvilinear) method-of-lines evolutions, their
// initial data with parameter derivatives (toroidal dipole; Gaussian pulse),
// and the extraction observables (a sphere for Cartesian grids, a radial
// shell for curvilinear ones).
//
// The evolution being differentiated is this library's RK4 step
// (MoLtimestepping/C_Code_Generation.py:266-329): per substep an RHS at
// interior points, the RK update there, then apply_bcs_curvilinear on every
// ghost point.  With L the RHS operator (interior rows only), B the boundary
// conditions (ghost values from interior values) and P the restriction to
// interior points, one step is
//   y1 = B P(y + dt/2 L y), y2 = B P(y + dt/2 L y1), y3 = B P(y + dt L y2),
//   y' = B P(y + dt/6 (L y + 2 L y1 + 2 L y2 + L y3)),
// which is linear in y for Maxwell; its transpose is applied by
// MoL_adjoint_step_backward below.  Maxwell's RHS
// (Maxwell/VacuumMaxwell_Flat_Evol_Cartesian.py:54-74)
//   A_i' = -E_i - D_i psi,  E_i' = sum_{j!=i} (-D_jj A_i + D_ji A_j),
//   psi' = -sum_i D_i A_i
// has the transpose (D_i antisymmetric, D_jj and D_ij symmetric stencils,
// applied to the adjoint restricted to interior points, at every point)
//   adjA_i = sum_{j!=i} (-D_jj a_Ei + D_ij a_Ej) + D_i a_psi,
//   adjE_i = -a_Ai,   adjpsi = sum_i D_i a_Ai.
#include <math.h>

#include <algorithm>

#include "fd.cuh"
#include "rfm.cuh"
#include "systems.cuh"

namespace nrgpu {

// The adjoint operand a (zero at ghost points), read with zero padding
// outside the array.
struct AdjIn {
  const double *a;
  Grid g;
  __device__ __forceinline__ double at(int gf, int i0, int i1, int i2) const {
    if (i0 < 0 || i0 >= g.n0 || i1 < 0 || i1 >= g.n1 || i2 < 0 || i2 >= g.n2) return 0.0;
    return __ldg(a + (long long)gf * g.ntot + i0 + (long long)g.n0 * (i1 + (long long)g.n1 * i2));
  }
};

// Masked stencils of the adjoint operand at point (i0,i1,i2), unscaled.
template <int ORDER>
__device__ __forceinline__ double adj_d1(const AdjIn &a, int gf, const int c[3], int d) {
  using C = FDCoef<ORDER>;
  double acc = 0.0;
#pragma unroll
  for (int k = 1; k <= C::R; k++) {
    int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
    p[d] += k;
    m[d] -= k;
    acc += C::c1(k) * (a.at(gf, p[0], p[1], p[2]) - a.at(gf, m[0], m[1], m[2]));
  }
  return acc;
}
template <int ORDER>
__device__ __forceinline__ double adj_d2(const AdjIn &a, int gf, const int c[3], int d) {
  using C = FDCoef<ORDER>;
  double acc = C::c2(0) * a.at(gf, c[0], c[1], c[2]);
#pragma unroll
  for (int k = 1; k <= C::R; k++) {
    int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
    p[d] += k;
    m[d] -= k;
    acc += C::c2(k) * (a.at(gf, p[0], p[1], p[2]) + a.at(gf, m[0], m[1], m[2]));
  }
  return acc;
}
template <int ORDER>
__device__ __forceinline__ double adj_d11(const AdjIn &a, int gf, const int c[3], int d, int e) {
  using C = FDCoef<ORDER>;
  double acc = 0.0;
#pragma unroll
  for (int u = 1; u <= C::R; u++) {
    double inner = 0.0;
#pragma unroll
    for (int v = 1; v <= C::R; v++) {
      int pp[3] = {c[0], c[1], c[2]}, pm[3] = {c[0], c[1], c[2]}, mp[3] = {c[0], c[1], c[2]},
          mm[3] = {c[0], c[1], c[2]};
      pp[d] += u; pp[e] += v;
      pm[d] += u; pm[e] -= v;
      mp[d] -= u; mp[e] += v;
      mm[d] -= u; mm[e] -= v;
      inner += C::c1(v) * ((a.at(gf, pp[0], pp[1], pp[2]) - a.at(gf, pm[0], pm[1], pm[2])) -
                           (a.at(gf, mp[0], mp[1], mp[2]) - a.at(gf, mm[0], mm[1], mm[2])));
    }
    acc += C::c1(u) * inner;
  }
  return acc;
}

// a = c1*mu + c2*mus at interior points, 0 at ghost points; and the running
// sum of the substeps' direct terms: acc_mode 1: acc = mu + mus;
// 2: acc += mus; 3: acc += mus, read back by the last transpose.
__global__ void adjoint_combine_kernel(Grid g, int ngf, const double *__restrict__ mu, const double *__restrict__ mus,
                                       double c1, double c2, double *__restrict__ a, double *__restrict__ acc,
                                       int acc_mode) {
  const long long n = (long long)ngf * g.ntot;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long p = k % g.ntot;
    const int i0 = (int)(p % g.n0), i1 = (int)((p / g.n0) % g.n1), i2 = (int)(p / ((long long)g.n0 * g.n1));
    const bool interior =
        i0 >= g.ng && i0 < g.n0 - g.ng && i1 >= g.ng && i1 < g.n1 - g.ng && i2 >= g.ng && i2 < g.n2 - g.ng;
    double v = 0.0, m = 0.0, ms = 0.0;
    if (interior) {
      m = mu[k];
      ms = mus ? mus[k] : 0.0;
      v = c1 * m + c2 * ms;
    }
    a[k] = v;
    if (acc_mode == 1) acc[k] = m + ms;
    else if (acc_mode >= 2) acc[k] += ms;
  }
}

// out = L^T a at every point (+ acc at interior points if add_acc).
template <int ORDER>
__global__ void maxwell_adjoint_kernel(AdjIn a, double *__restrict__ out, const double *__restrict__ acc) {
  const Grid &g = a.g;
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  if (i0 >= g.n0) return;
  const long long idx = i0 + (long long)g.n0 * (i1 + (long long)g.n1 * i2);
  const int c[3] = {i0, i1, i2};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  const bool interior =
      i0 >= g.ng && i0 < g.n0 - g.ng && i1 >= g.ng && i1 < g.n1 - g.ng && i2 >= g.ng && i2 < g.n2 - g.ng;
  double res[7];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double v = adj_d1<ORDER>(a, 6, c, i) * inv[i];  // from psi' = -D_i A_i
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (j == i) continue;
      v -= adj_d2<ORDER>(a, 3 + i, c, j) * (inv[j] * inv[j]);
      const int lo = i < j ? i : j, hi = i < j ? j : i;
      v += adj_d11<ORDER>(a, 3 + j, c, lo, hi) * (inv[lo] * inv[hi]);
    }
    res[i] = v;
    res[3 + i] = -a.at(i, i0, i1, i2);
  }
  double dpsi = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) dpsi += adj_d1<ORDER>(a, i, c, i) * inv[i];
  res[6] = dpsi;
#pragma unroll
  for (int gf = 0; gf < 7; gf++) {
    const long long k = (long long)gf * g.ntot + idx;
    out[k] = (acc && interior) ? res[gf] + acc[k] : res[gf];
  }
}

// ScalarWave (ScalarWave/ScalarWave_RHSs.py:46-71, ScalarWaveCurvilinear_RHSs.py:
// 43-98): at interior points p, (L y)_u = v and (L y)_v = c^2 sum_d [g_d(p)
// D2_d u - G_d(p) D1_d u] with g_d = ghat^dd and G_d = ghat^ii Gammahat^d_ii
// (1 and 0 on Cartesian grids).  D2 is symmetric and D1 antisymmetric, so at
// every point q
//   (L^T a)_u(q) = c^2 sum_d [D2_d(g_d a_v)(q) + D1_d(G_d a_v)(q)],
//   (L^T a)_v(q) = a_u(q),
// with the coefficients taken at the stencil's centre p and a zero outside
// interior points.
template <int CS>
__device__ __forceinline__ void sw_coeffs(const double *tab, const Grid &g, int i0, int i1, int i2, double gd[3],
                                          double Gd[3]) {
  using M = RfmMask<CS>;
  if constexpr (M::trivial) {
#pragma unroll
    for (int d = 0; d < 3; d++) gd[d] = 1.0, Gd[d] = 0.0;
  } else {
    const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      gd[d] = rf.ghatUU(d);
      double c = 0.0;
#pragma unroll
      for (int i = 0; i < 3; i++)
        if (M::Gammahat(d, i, i)) c += rf.ghatUU(i) * rf.G(d, i, i);
      Gd[d] = c;
    }
  }
}

template <int CS, int ORDER>
__global__ void scalarwave_adjoint_kernel(AdjIn a, const double *__restrict__ tab, double c2, double *__restrict__ out,
                                          const double *__restrict__ acc) {
  using C = FDCoef<ORDER>;
  const Grid &g = a.g;
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  if (i0 >= g.n0) return;
  const long long idx = i0 + (long long)g.n0 * (i1 + (long long)g.n1 * i2);
  const int c[3] = {i0, i1, i2};
  const int n[3] = {g.n0, g.n1, g.n2};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  const bool interior =
      i0 >= g.ng && i0 < g.n0 - g.ng && i1 >= g.ng && i1 < g.n1 - g.ng && i2 >= g.ng && i2 < g.n2 - g.ng;
  double res_u = 0.0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double s2 = 0.0, s1 = 0.0;
#pragma unroll
    for (int k = -C::R; k <= C::R; k++) {
      int q[3] = {c[0], c[1], c[2]};
      q[d] += k;  // a stencil centre p = c + k e_d reads c with offset -k
      if (q[d] < g.ng || q[d] >= n[d] - g.ng) continue;
      const double av = a.at(1, q[0], q[1], q[2]);
      if (av == 0.0) continue;
      double gd[3], Gd[3];
      sw_coeffs<CS>(tab, g, q[0], q[1], q[2], gd, Gd);
      const int ak = k < 0 ? -k : k;
      s2 += (ak == 0 ? C::c2(0) : C::c2(ak)) * gd[d] * av;
      if (k != 0) s1 += (k > 0 ? -C::c1(ak) : C::c1(ak)) * Gd[d] * av;  // weight of offset -k in D1
    }
    res_u += s2 * (inv[d] * inv[d]) - s1 * inv[d];
  }
  res_u *= c2;
  const double res_v = a.at(0, i0, i1, i2);
  const long long k0 = idx, k1 = g.ntot + idx;
  out[k0] = (acc && interior) ? res_u + acc[k0] : res_u;
  out[k1] = (acc && interior) ? res_v + acc[k1] : res_v;
}

static int check_adjoint_system(int system, const rfm_struct *rfm, const paramstruct *p) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(system == NRGPU_SYS_MAXWELL || system == NRGPU_SYS_SCALARWAVE,
                "adjoints are built for the linear systems ScalarWave and Maxwell System I");
  NRGPU_REQUIRE(system != NRGPU_SYS_MAXWELL || p->CoordSystem == NRGPU_COORD_CARTESIAN,
                "Maxwell System I is Cartesian only");
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN || rfm_matches(rfm, p),
                "curvilinear grids need an rfm_struct defined for this grid");
  return NRGPU_OK;
}

// out = L^T (c1*mu + c2*mus); tmp receives the combined operand.
static int system_adjoint_launch(int system, const rfm_struct *rfm, const paramstruct *p, const Grid &g,
                                 const double *mu, const double *mus, double c1, double c2, double *tmp,
                                 double *out, double *acc, int acc_mode) {
  const int ngf = system_num_gfs(system);
  const long long n = ngf * g.ntot;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  adjoint_combine_kernel<<<blocks, 256, 0, stream()>>>(g, ngf, mu, mus, c1, c2, tmp, acc, acc_mode);
  NRGPU_LAUNCH_CHECK();
  AdjIn a{tmp, g};
  const double *add = acc_mode == 3 ? acc : nullptr;
  dim3 block(64), grid((g.n0 + 63) / 64, g.n1, g.n2);
  if (system == NRGPU_SYS_MAXWELL) {
    switch (p->FD_order) {
      case 2: maxwell_adjoint_kernel<2><<<grid, block, 0, stream()>>>(a, out, add); break;
      case 4: maxwell_adjoint_kernel<4><<<grid, block, 0, stream()>>>(a, out, add); break;
      case 6: maxwell_adjoint_kernel<6><<<grid, block, 0, stream()>>>(a, out, add); break;
      case 8: maxwell_adjoint_kernel<8><<<grid, block, 0, stream()>>>(a, out, add); break;
      default: set_error("Maxwell adjoint: FD_order %d not built", p->FD_order); return NRGPU_ERR_UNSUPPORTED;
    }
  } else {
    const double *tab = rfm ? rfm->table64 : nullptr;
    const double cc = p->wavespeed * p->wavespeed;
    const int cs = dispatch_cs(p->CoordSystem);
#define SWA(CSV, ORD)                                                                            \
  if (cs == CSV && p->FD_order == ORD) {                                                         \
    scalarwave_adjoint_kernel<CSV, ORD><<<grid, block, 0, stream()>>>(a, tab, cc, out, add);     \
    NRGPU_LAUNCH_CHECK();                                                                        \
    return NRGPU_OK;                                                                             \
  }
#define SWA_ORDERS(CSV) SWA(CSV, 2) SWA(CSV, 4) SWA(CSV, 6) SWA(CSV, 8)
    SWA_ORDERS(NRGPU_COORD_CARTESIAN)
    SWA_ORDERS(NRGPU_COORD_SPHERICAL)
    SWA_ORDERS(NRGPU_COORD_SINHSPHERICAL)
    SWA_ORDERS(NRGPU_COORD_SINHCYLINDRICAL)
    SWA_ORDERS(NRGPU_COORD_SINHSYMTP)
#undef SWA_ORDERS
#undef SWA
    set_error("ScalarWave adjoint: CoordSystem %d with FD_order %d not built", p->CoordSystem, p->FD_order);
    return NRGPU_ERR_UNSUPPORTED;
  }
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

static int check_maxwell(const paramstruct *p) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN, "Maxwell System I is Cartesian only");
  return NRGPU_OK;
}

// ------------------------------------------------ toroidal dipole + derivs
// Value and derivative with respect to lam (forward-mode dual number).
struct DualL {
  double v, d;
};
__device__ __forceinline__ DualL operator+(DualL a, DualL b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ DualL operator-(DualL a, DualL b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ DualL operator*(DualL a, DualL b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ DualL operator*(double s, DualL a) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ DualL operator/(DualL a, double s) { return {a.v / s, a.d / s}; }
__device__ __forceinline__ DualL dexp(DualL a) {
  const double e = exp(a.v);
  return {e, e * a.d};
}

// Maxwell/InitialData.py:41-104: A = F(r,t) (-y, x, 0), E = -dA/dt, psi = 0,
// F = amp/r [ (e^{-lam v^2} - e^{-lam u^2})/r^2 - 2 lam (v e^{-lam v^2} + u e^{-lam u^2})/r ],
// u = t + r, v = t - r (the z/r factors of A_phi and of dx/dphi cancel).
__global__ void toroidal_dipole_kernel(Grid g, double xmin0, double xmin1, double xmin2, double dx0, double dx1,
                                       double dx2, double amp, double lam, double t, double *__restrict__ y,
                                       double *__restrict__ d_amp, double *__restrict__ d_lam) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  if (i0 >= g.n0) return;
  const long long idx = i0 + (long long)g.n0 * (i1 + (long long)g.n1 * i2);
  const double x = xx_of(xmin0, dx0, i0, g.ng), yy = xx_of(xmin1, dx1, i1, g.ng), z = xx_of(xmin2, dx2, i2, g.ng);
  const double r = sqrt(x * x + yy * yy + z * z);
  const DualL L{lam, 1.0};
  const double u = t + r, v = t - r;
  const DualL eu = dexp((-u * u) * L), ev = dexp((-v * v) * L);
  const DualL deu = (-2.0 * u) * (L * eu), dev = (-2.0 * v) * (L * ev);  // d/dt of eu, ev
  const DualL F = ((ev - eu) / (r * r) - (2.0 / r) * (L * (v * ev + u * eu))) / r;  // F / amp
  const DualL dF = ((dev - deu) / (r * r) - (2.0 / r) * (L * (ev + v * dev + eu + u * deu))) / r;
  const double vals[7][2] = {{-yy * F.v, -yy * F.d}, {x * F.v, x * F.d},   {0.0, 0.0},
                             {yy * dF.v, yy * dF.d}, {-x * dF.v, -x * dF.d}, {0.0, 0.0},
                             {0.0, 0.0}};
#pragma unroll
  for (int gf = 0; gf < 7; gf++) {
    const long long k = (long long)gf * g.ntot + idx;
    if (y) y[k] = amp * vals[gf][0];
    if (d_amp) d_amp[k] = vals[gf][0];
    if (d_lam) d_lam[k] = amp * vals[gf][1];
  }
}

// -------------------------------------------- Gaussian pulse + derivatives
// u = A exp(-(r - r0)^2 / w^2), v = 0 at every point (r the Cartesian radius
// of the point), and du/dA, du/dr0, du/dw.
__global__ void gaussian_pulse_kernel(paramstruct p, double A, double r0, double w, double *__restrict__ y,
                                      double *__restrict__ dA, double *__restrict__ dr0, double *__restrict__ dw) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, i1 = blockIdx.y, i2 = blockIdx.z;
  const int n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1, n2 = p.Nxx_plus_2NGHOSTS2;
  if (i0 >= n0) return;
  const long long ntot = (long long)n0 * n1 * n2;
  const long long idx = i0 + (long long)n0 * (i1 + (long long)n1 * i2);
  double x[3], J[3][3];
  cart_jacobian(coord_params(p), xx_of(p.xxmin0, p.dxx0, i0, p.NGHOSTS), xx_of(p.xxmin1, p.dxx1, i1, p.NGHOSTS),
                xx_of(p.xxmin2, p.dxx2, i2, p.NGHOSTS), x, J);
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  const double s = (r - r0) / w, e = exp(-s * s);
  if (y) {
    y[idx] = A * e;
    y[ntot + idx] = 0.0;
  }
  if (dA) dA[idx] = e, dA[ntot + idx] = 0.0;
  if (dr0) dr0[idx] = A * e * 2.0 * s / w, dr0[ntot + idx] = 0.0;
  if (dw) dw[idx] = A * e * 2.0 * s * s / w, dw[ntot + idx] = 0.0;
}

// ------------------------------------------------------ radial shell
// Samples of gridfunction gf on the interior (i1, i2) points of the shell
// i0: samples[q] = f(i0, ng + q % Nxx1, ng + q / Nxx1), and
// accum[0] += scale * sum_q wts[q] samples[q]^2 (one atomic per block).
__global__ void shell_sample_kernel(Grid g, const double *__restrict__ f, int i0, const double *__restrict__ wts,
                                   double scale, double *__restrict__ samples, double *__restrict__ accum) {
  const int m1 = g.n1 - 2 * g.ng, nq = m1 * (g.n2 - 2 * g.ng);
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double local = 0.0;
  if (q < nq) {
    const long long idx = i0 + (long long)g.n0 * ((g.ng + q % m1) + (long long)g.n1 * (g.ng + q / m1));
    const double v = f[idx];
    samples[q] = v;
    local = scale * wts[q] * v * v;
  }
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sh[k];
    atomicAdd(accum, t);
  }
}

// Transpose of J = sqrt(accum) for one sample set: adj_f += (scale/J) w_q samples_q
// at the shell points.
__global__ void shell_adjoint_kernel(Grid g, const double *__restrict__ samples, int i0, const double *__restrict__ wts,
                                     double scale, const double *__restrict__ accum, double *adj_f) {
  const int m1 = g.n1 - 2 * g.ng, nq = m1 * (g.n2 - 2 * g.ng);
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const double J = sqrt(accum[0]);
  if (!(J > 0.0)) return;
  const long long idx = i0 + (long long)g.n0 * ((g.ng + q % m1) + (long long)g.n1 * (g.ng + q / m1));
  adj_f[idx] += scale * wts[q] * samples[q] / J;
}

// ------------------------------------------------------ extraction sphere
// Tricubic Lagrange interpolation from the 4x4x4 nodes around a point.
struct Tricubic {
  int base[3];
  double w[3][4];
};

__device__ __forceinline__ bool tricubic(const paramstruct &p, const double *xyz, Tricubic &T) {
  const double xmin[3] = {p.xxmin0, p.xxmin1, p.xxmin2}, dx[3] = {p.dxx0, p.dxx1, p.dxx2};
  const int n[3] = {p.Nxx_plus_2NGHOSTS0, p.Nxx_plus_2NGHOSTS1, p.Nxx_plus_2NGHOSTS2};
  for (int d = 0; d < 3; d++) {
    // grid index coordinate: x = xmin + (j - NGHOSTS + 1/2) dx
    const double j = (xyz[d] - xmin[d]) / dx[d] + p.NGHOSTS - 0.5;
    const double f = floor(j);
    const int b = (int)f - 1;
    if (b < 0 || b + 3 >= n[d]) return false;
    const double s = j - f;
    T.base[d] = b;
    T.w[d][0] = -s * (s - 1.0) * (s - 2.0) / 6.0;
    T.w[d][1] = (s + 1.0) * (s - 1.0) * (s - 2.0) / 2.0;
    T.w[d][2] = -(s + 1.0) * s * (s - 2.0) / 2.0;
    T.w[d][3] = (s + 1.0) * s * (s - 1.0) / 6.0;
  }
  return true;
}

// samples[p*ngf + i] = f_{gf0+i}(x_p); accum[0] += scale * sum_p w_p |f(x_p)|^2.
__global__ void sphere_sample_kernel(paramstruct p, const double *__restrict__ gfs, int gf0, int ngf,
                                     const double *__restrict__ pts, const double *__restrict__ wts, int npts,
                                     double scale, double *__restrict__ samples, double *__restrict__ accum,
                                     int *__restrict__ err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double local = 0.0;
  if (q < npts) {
    Tricubic T;
    if (!tricubic(p, pts + 3 * q, T)) {
      atomicExch(err, 1);
    } else {
      const long long n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1;
      const long long ntot = n0 * n1 * p.Nxx_plus_2NGHOSTS2;
      for (int i = 0; i < ngf; i++) {
        const double *f = gfs + (long long)(gf0 + i) * ntot;
        double v = 0.0;
        for (int c = 0; c < 4; c++)
          for (int b = 0; b < 4; b++) {
            const double wbc = T.w[1][b] * T.w[2][c];
            const double *row = f + T.base[0] + n0 * ((T.base[1] + b) + n1 * (T.base[2] + c));
            v += wbc * (T.w[0][0] * row[0] + T.w[0][1] * row[1] + T.w[0][2] * row[2] + T.w[0][3] * row[3]);
          }
        samples[(long long)q * ngf + i] = v;
        local += v * v;
      }
      local *= wts[q] * scale;
    }
  }
  // block sum, one atomic per block
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
    atomicAdd(accum, s);
  }
}

// Adjoint of the observable J = sqrt(accum) for one sample set:
// adj_gfs += (scale / J) * sum_p w_p f(x_p) (x) interpolation weights.
__global__ void sphere_adjoint_kernel(paramstruct p, const double *__restrict__ samples, int gf0, int ngf,
                                      const double *__restrict__ pts, const double *__restrict__ wts, int npts,
                                      double scale, const double *__restrict__ accum, double *adj_gfs,
                                      int *__restrict__ err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npts) return;
  Tricubic T;
  if (!tricubic(p, pts + 3 * q, T)) {
    atomicExch(err, 1);
    return;
  }
  const double J = sqrt(accum[0]);
  const double coef = J > 0.0 ? scale * wts[q] / J : 0.0;
  const long long n0 = p.Nxx_plus_2NGHOSTS0, n1 = p.Nxx_plus_2NGHOSTS1;
  const long long ntot = n0 * n1 * p.Nxx_plus_2NGHOSTS2;
  for (int i = 0; i < ngf; i++) {
    const double gq = coef * samples[(long long)q * ngf + i];
    double *f = adj_gfs + (long long)(gf0 + i) * ntot;
    for (int c = 0; c < 4; c++)
      for (int b = 0; b < 4; b++)
        for (int a = 0; a < 4; a++)
          atomicAdd(f + (T.base[0] + a) + n0 * ((T.base[1] + b) + n1 * (T.base[2] + c)),
                    gq * T.w[0][a] * T.w[1][b] * T.w[2][c]);
  }
}

// ------------------------------------------------------------------ dot
__global__ void dot_partial_kernel(const double *__restrict__ a, const double *__restrict__ b, long long n,
                                   double *__restrict__ partial) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
    partial[blockIdx.x] = s;
  }
}
__global__ void dot_final_kernel(const double *__restrict__ partial, int nparts, double *__restrict__ result) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nparts; i++) s += partial[i];  // fixed order: reproducible
    result[0] = s;
  }
}

static int error_flag(int **flag) {
  static int *d = nullptr;  // one flag per process, reset before each use
  if (!d) NRGPU_CUDA_CHECK(cudaMalloc(&d, sizeof(int)));
  *flag = d;
  return NRGPU_OK;
}

}  // namespace nrgpu

using namespace nrgpu;

extern "C" {

int Maxwell_rhs_eval_adjoint(const paramstruct *p, const double *adj_rhs, double *adj_in) {
  NRGPU_REQUIRE(p && adj_rhs && adj_in, "NULL argument");
  int st = check_maxwell(p);
  if (st) return st;
  NRGPU_REQUIRE(adj_rhs != adj_in, "adj_rhs and adj_in must not alias");
  const Grid g = make_grid(p);
  double *tmp = nullptr;
  NRGPU_CUDA_CHECK(cudaMallocAsync((void **)&tmp, 7 * g.ntot * sizeof(double), stream()));
  st = system_adjoint_launch(NRGPU_SYS_MAXWELL, nullptr, p, g, adj_rhs, nullptr, 1.0, 0.0, tmp, adj_in, nullptr, 0);
  cudaFreeAsync(tmp, stream());
  return st;
}

int ScalarWave_rhs_eval_adjoint(const rfm_struct *rfm, const paramstruct *p, const double *adj_rhs, double *adj_in) {
  NRGPU_REQUIRE(p && adj_rhs && adj_in, "NULL argument");
  int st = check_adjoint_system(NRGPU_SYS_SCALARWAVE, rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(adj_rhs != adj_in, "adj_rhs and adj_in must not alias");
  const Grid g = make_grid(p);
  double *tmp = nullptr;
  NRGPU_CUDA_CHECK(cudaMallocAsync((void **)&tmp, 2 * g.ntot * sizeof(double), stream()));
  st = system_adjoint_launch(NRGPU_SYS_SCALARWAVE, rfm, p, g, adj_rhs, nullptr, 1.0, 0.0, tmp, adj_in, nullptr, 0);
  cudaFreeAsync(tmp, stream());
  return st;
}

int apply_bcs_curvilinear_adjoint(const paramstruct *p, const bc_struct *bc, int NUM_GFS, const int8_t *gfs_parity,
                                  double *adj_gfs) {
  return apply_bcs_adjoint_impl(p, bc, NUM_GFS, gfs_parity, adj_gfs);
}

int MoL_adjoint_step_backward(int system, const rfm_struct *rfm, const paramstruct *p, const bc_struct *bc,
                              double *lam_in, double *lam_out, double *scratch, double dt) {
  NRGPU_REQUIRE(p && bc && lam_in && lam_out && scratch, "NULL argument");
  int st = check_adjoint_system(system, rfm, p);
  if (st) return st;
  NRGPU_REQUIRE(lam_in != lam_out, "lam_in and lam_out must differ");
  const Grid g = make_grid(p);
  const int ngf = system_num_gfs(system);
  const long long len = ngf * g.ntot;
  double *S0 = scratch, *S1 = scratch + len, *acc = scratch + 2 * len, *tmp = scratch + 3 * len;
  const int8_t *par = system_parity(system);
  // mu = P B^T lam_{n+1}
  if ((st = apply_bcs_adjoint_impl(p, bc, ngf, par, lam_in))) return st;
  const double *mu = lam_in;
  // substep 4: k4 = L y3 enters y' with dt/6
  if ((st = system_adjoint_launch(system, rfm, p, g, mu, nullptr, dt / 6.0, 0.0, tmp, S0, nullptr, 0))) return st;
  if ((st = apply_bcs_adjoint_impl(p, bc, ngf, par, S0))) return st;  // mu3
  // substep 3: y3 = B P(y + dt k3); k3 enters y' with dt/3
  if ((st = system_adjoint_launch(system, rfm, p, g, mu, S0, dt / 3.0, dt, tmp, S1, acc, 1))) return st;
  if ((st = apply_bcs_adjoint_impl(p, bc, ngf, par, S1))) return st;  // mu2
  // substep 2: y2 = B P(y + dt/2 k2)
  if ((st = system_adjoint_launch(system, rfm, p, g, mu, S1, dt / 3.0, dt / 2.0, tmp, S0, acc, 2))) return st;
  if ((st = apply_bcs_adjoint_impl(p, bc, ngf, par, S0))) return st;  // mu1
  // substep 1: y1 = B P(y + dt/2 k1), k1 = L y; plus every direct y term
  return system_adjoint_launch(system, rfm, p, g, mu, S0, dt / 6.0, dt / 2.0, tmp, lam_out, acc, 3);
}

int Maxwell_initial_data_toroidal_dipole(const paramstruct *p, double amp, double lam, double time,
                                         double *in_gfs, double *d_amp, double *d_lam) {
  NRGPU_REQUIRE(p && (in_gfs || d_amp || d_lam), "NULL argument");
  int st = check_maxwell(p);
  if (st) return st;
  NRGPU_REQUIRE(lam > 0.0, "lam must be positive");
  const Grid g = make_grid(p);
  dim3 block(64), grid((g.n0 + 63) / 64, g.n1, g.n2);
  toroidal_dipole_kernel<<<grid, block, 0, stream()>>>(g, p->xxmin0, p->xxmin1, p->xxmin2, p->dxx0, p->dxx1,
                                                       p->dxx2, amp, lam, time, in_gfs, d_amp, d_lam);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int ScalarWave_initial_data_gaussian(const paramstruct *p, double A, double r0, double w, double *in_gfs,
                                     double *d_A, double *d_r0, double *d_w) {
  NRGPU_REQUIRE(p && (in_gfs || d_A || d_r0 || d_w), "NULL argument");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(w > 0.0, "w must be positive");
  dim3 block(64), grid((p->Nxx_plus_2NGHOSTS0 + 63) / 64, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2);
  gaussian_pulse_kernel<<<grid, block, 0, stream()>>>(*p, A, r0, w, in_gfs, d_A, d_r0, d_w);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_shell_sample(const paramstruct *p, const double *gfs, int gf, int i0, const double *wts, double scale,
                       double *samples, double *accum) {
  NRGPU_REQUIRE(p && gfs && wts && samples && accum && gf >= 0, "bad arguments");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(i0 >= p->NGHOSTS && i0 < p->Nxx_plus_2NGHOSTS0 - p->NGHOSTS, "shell i0 %d not interior", i0);
  const Grid g = make_grid(p);
  const int nq = p->Nxx1 * p->Nxx2;
  shell_sample_kernel<<<(nq + 127) / 128, 128, 0, stream()>>>(g, gfs + (long long)gf * g.ntot, i0, wts, scale,
                                                               samples, accum);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_shell_sample_adjoint(const paramstruct *p, const double *samples, int gf, int i0, const double *wts,
                               double scale, const double *accum, double *adj_gfs) {
  NRGPU_REQUIRE(p && samples && wts && accum && adj_gfs && gf >= 0, "bad arguments");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(i0 >= p->NGHOSTS && i0 < p->Nxx_plus_2NGHOSTS0 - p->NGHOSTS, "shell i0 %d not interior", i0);
  const Grid g = make_grid(p);
  const int nq = p->Nxx1 * p->Nxx2;
  shell_adjoint_kernel<<<(nq + 127) / 128, 128, 0, stream()>>>(g, samples, i0, wts, scale, accum,
                                                                adj_gfs + (long long)gf * g.ntot);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_sphere_sample(const paramstruct *p, const double *gfs, int gf0, int ngf, const double *pts,
                        const double *wts, int npts, double scale, double *samples, double *accum) {
  NRGPU_REQUIRE(p && gfs && pts && wts && samples && accum && npts >= 1 && ngf >= 1, "bad arguments");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN, "sphere sampling needs a Cartesian grid");
  int *err;
  if ((st = error_flag(&err))) return st;
  NRGPU_CUDA_CHECK(cudaMemsetAsync(err, 0, sizeof(int), stream()));
  sphere_sample_kernel<<<(npts + 127) / 128, 128, 0, stream()>>>(*p, gfs, gf0, ngf, pts, wts, npts, scale, samples,
                                                                 accum, err);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_sphere_sample_adjoint(const paramstruct *p, const double *samples, int gf0, int ngf, const double *pts,
                                const double *wts, int npts, double scale, const double *accum, double *adj_gfs) {
  NRGPU_REQUIRE(p && samples && pts && wts && accum && adj_gfs && npts >= 1 && ngf >= 1, "bad arguments");
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN, "sphere sampling needs a Cartesian grid");
  int *err;
  if ((st = error_flag(&err))) return st;
  NRGPU_CUDA_CHECK(cudaMemsetAsync(err, 0, sizeof(int), stream()));
  sphere_adjoint_kernel<<<(npts + 127) / 128, 128, 0, stream()>>>(*p, samples, gf0, ngf, pts, wts, npts, scale,
                                                                  accum, adj_gfs, err);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int nrgpu_sphere_check(const paramstruct *p, int *outside) {
  NRGPU_REQUIRE(p && outside, "NULL argument");
  int *err;
  int st = error_flag(&err);
  if (st) return st;
  NRGPU_CUDA_CHECK(cudaMemcpyAsync(outside, err, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  NRGPU_CUDA_CHECK(cudaStreamSynchronize(stream()));
  return NRGPU_OK;
}

int nrgpu_dot(const double *a, const double *b, long long n, double *scratch, int scratch_len, double *result) {
  NRGPU_REQUIRE(a && b && scratch && result && n >= 1 && scratch_len >= 1, "bad arguments");
  const int threads = 256;
  const int blocks = (int)std::min<long long>((n + threads - 1) / threads, (long long)scratch_len);
  dot_partial_kernel<<<blocks, threads, 0, stream()>>>(a, b, n, scratch);
  NRGPU_LAUNCH_CHECK();
  dot_final_kernel<<<1, 32, 0, stream()>>>(scratch, blocks, result);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

}  // extern "C"
