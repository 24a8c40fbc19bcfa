// psi4.cu -- the Weyl scalar psi_4 from the BSSN variables, in the
// quasi-Kinnersley tetrad, and its spin-weight -2 spherical-harmonic modes on
// an extraction shell of a spherical-like grid.
//
// psi_4 per point (FP64; a diagnostic):
//   BSSN/ADM_in_terms_of_BSSN.py:20-170  gamma_ij = e^{4phi} gammabar_ij
//       (e^{4phi} = 1/W^2), its first and second derivatives, Christoffels,
//       K_ij = e^{4phi} Abar_ij + gamma_ij K/3 and d_k K_ij;
//   BSSN/Psi4.py:50-193  the 3+1 Riemann tensor of gamma and the three terms of
//       Baker, Campanelli & Lousto (2002) eq. 5.1, contracted with n and m;
//   BSSN/Psi4_tetrads.py:50-193  the tetrad: Gram-Schmidt, in gamma, of
//       phi-hat (-y, x, 0), r-hat (x, y, z) and their gamma-cross product,
//       carried to the xx basis by the inverse Jacobian of xx_to_Cart;
//       u = (1, 0, 0, 0) (UseCorrectUnitNormal = False), so m has no time
//       component and only the n^0 terms of the tetrad products survive.
// Modes: lowlevel_decompose_psi4_into_swm2_modes of
//   Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide-Psi4.ipynb:
//   psi4_lm = sum over the shell's interior (theta, phi) cells of
//   psi4 conj(sY_lm) sin(theta) dxx1 dxx2, with sY_lm (s = -2) from Goldberg's
//   formula (SpinWeight_minus2_SphHarmonics.py:31-43), evaluated as
//   sin^{2l-k}(theta/2) cos^k(theta/2) products (no division at the poles).
#include <math.h>

#include "bssn.cuh"

namespace nrgpu {
namespace psi4 {
using namespace bssn;

constexpr double kIsqrt2 = 0.707106781186547524400844362104849039;

__device__ __forceinline__ double omega(const double u[3], const double w[3], const double g[3][3]) {
  double s = 0.0;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) s += u[a] * w[b] * g[a][b];
  return s;
}

template <int ORDER, int CS>
__device__ void psi4_point(const Point<double> &P, const Rfm<CS, double> &rf, const double inv[3], double xx0,
                           double xx1, double xx2, const paramstruct &prm, double &re, double &im) {
  using M = RfmMask<CS>;
  // ---- BSSN variables and their centred derivatives; gammabar, Abar
  double g[3][3], gd[6][3], gdd[6][6], Ab[3][3], Abd[6][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const int s = S6(i, j);
      const double h = __ldg(P.gf(HDD00 + s)), a = __ldg(P.gf(ADD00 + s));
      const double red = M::trivial ? 1.0 : rf.ReDD(i, j);
      double hd[3];
#pragma unroll
      for (int k = 0; k < 3; k++) hd[k] = D1<ORDER, double>(P, HDD00 + s, k, inv);
      g[i][j] = g[j][i] = h * red + (i == j ? rf.ghatDD(i) : 0.0);
      Ab[i][j] = Ab[j][i] = a * red;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        double v = hd[k] * red;
        if (M::ReDDdD(i, j, k)) v += h * rf.ReDDdD(i, j, k);
        if (M::ghatDDdD(i, j, k)) v += rf.ghatDDdD(i, j, k);
        gd[s][k] = v;
        double w = D1<ORDER, double>(P, ADD00 + s, k, inv) * red;
        if (M::ReDDdD(i, j, k)) w += a * rf.ReDDdD(i, j, k);
        Abd[s][k] = w;
      }
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = k; l < 3; l++) {
          double v = D2<ORDER, double>(P, HDD00 + s, k, l, inv) * red;
          if (M::ReDDdD(i, j, l)) v += hd[k] * rf.ReDDdD(i, j, l);
          if (M::ReDDdD(i, j, k)) v += hd[l] * rf.ReDDdD(i, j, k);
          if (M::ReDDdDD(i, j, k, l)) v += h * rf.ReDDdDD(i, j, k, l);
          if (M::ghatDDdDD(i, j, k, l)) v += rf.ghatDDdDD(i, j, k, l);
          gdd[s][S6(k, l)] = v;
        }
    }
  // ---- conformal factor W: e^{4phi} = 1/W^2 and its derivatives
  const double cf = __ldg(P.gf(CF)), trK = __ldg(P.gf(TRK));
  const double e4 = 1.0 / (cf * cf), e2 = 1.0 / cf;
  double phid[3], e4d[3], e4dd[6], trKd[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    phid[k] = -0.5 * e2 * D1<ORDER, double>(P, CF, k, inv);
    trKd[k] = D1<ORDER, double>(P, TRK, k, inv);
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    e4d[k] = 4.0 * e4 * phid[k];
#pragma unroll
    for (int l = k; l < 3; l++) {
      const double cfk = -2.0 * cf * phid[k], cfl = -2.0 * cf * phid[l];  // d_k W
      const double phidd = 0.5 * (e4 * cfk * cfl - e2 * D2<ORDER, double>(P, CF, k, l, inv));
      e4dd[S6(k, l)] = 16.0 * e4 * phid[k] * phid[l] + 4.0 * e4 * phidd;
    }
  }
  // ---- physical metric, derivatives (in place), K_ij and d_k K_ij
  double K[3][3], Kd[6][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const int s = S6(i, j);
      const double gb = g[i][j];
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = k; l < 3; l++)
          gdd[s][S6(k, l)] = e4dd[S6(k, l)] * gb + e4d[k] * gd[s][l] + e4d[l] * gd[s][k] + e4 * gdd[s][S6(k, l)];
      double gdn[3];
#pragma unroll
      for (int k = 0; k < 3; k++) gdn[k] = e4d[k] * gb + e4 * gd[s][k];
      const double gij = e4 * gb;
      g[i][j] = g[j][i] = gij;
      const double kij = e4 * Ab[i][j] + gij * trK * (1.0 / 3.0);
      K[i][j] = K[j][i] = kij;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        Kd[s][k] = e4d[k] * Ab[i][j] + e4 * Abd[s][k] + (gdn[k] * trK + gij * trKd[k]) * (1.0 / 3.0);
        gd[s][k] = gdn[k];
      }
    }
  double gUU[3][3], detg;
  sym_inverse(g, gUU, detg);
  // lowered Christoffels GL_{p,jk} and Gamma^i_jk
  double GL[3][6], G[3][6];
#pragma unroll
  for (int p = 0; p < 3; p++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = j; k < 3; k++)
        GL[p][S6(j, k)] = 0.5 * (gd[S6(p, j)][k] + gd[S6(p, k)][j] - gd[S6(j, k)][p]);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int s = 0; s < 6; s++) G[i][s] = gUU[i][0] * GL[0][s] + gUU[i][1] * GL[1][s] + gUU[i][2] * GL[2][s];

  // ---- tetrad (xx basis)
  double x[3], J[3][3], Ji[3][3];
  cart_jacobian(coord_params(prm), xx0, xx1, xx2, x, J);
  inverse3(J, Ji);
  const double v1C[3] = {-x[1], x[0], 0.0};
  double v1[3], v2[3], v3[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    v1[i] = Ji[i][0] * v1C[0] + Ji[i][1] * v1C[1] + Ji[i][2] * v1C[2];
    v2[i] = Ji[i][0] * x[0] + Ji[i][1] * x[1] + Ji[i][2] * x[2];
  }
  const double cr[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
  const double sq = sqrt(detg);
#pragma unroll
  for (int a = 0; a < 3; a++) v3[a] = sq * (gUU[a][0] * cr[0] + gUU[a][1] * cr[1] + gUU[a][2] * cr[2]);
  double e1[3], e2v[3], e3[3];
  {
    const double n1 = 1.0 / sqrt(omega(v1, v1, g));
#pragma unroll
    for (int a = 0; a < 3; a++) e1[a] = v1[a] * n1;
    const double w01 = omega(e1, v2, g);
#pragma unroll
    for (int a = 0; a < 3; a++) e2v[a] = v2[a] - w01 * e1[a];
    const double n2 = 1.0 / sqrt(omega(e2v, e2v, g));
#pragma unroll
    for (int a = 0; a < 3; a++) e2v[a] *= n2;
    const double w02 = omega(e1, v3, g), w12 = omega(e2v, v3, g);
#pragma unroll
    for (int a = 0; a < 3; a++) e3[a] = v3[a] - w02 * e1[a] - w12 * e2v[a];
    const double n3 = 1.0 / sqrt(omega(e3, e3, g));
#pragma unroll
    for (int a = 0; a < 3; a++) e3[a] *= n3;
  }
  // n = (u - r)/sqrt2, Re m = theta/sqrt2, Im m = phi/sqrt2 (spatial parts)
  double n[3], A[3][3], B[3][3];
  const double n0 = kIsqrt2;
#pragma unroll
  for (int a = 0; a < 3; a++) n[a] = -kIsqrt2 * e2v[a];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) {
      const double mra = kIsqrt2 * e3[a], mrb = kIsqrt2 * e3[b];
      const double mia = kIsqrt2 * e1[a], mib = kIsqrt2 * e1[b];
      A[a][b] = mra * mrb - mia * mib;   // real part of m_a m_b
      B[a][b] = mra * mib + mia * mrb;   // imaginary part
    }

  // ---- Riemann R_iklm of gamma (Psi4.py:50-72) and its contractions
  // term 1: sum_ijkl (R_ijkl + K_ik K_lj - K_il K_kj) n^i n^k m^j m^l
  // term 3 needs R_jl = gamma^im R_ijml.
  double p0r = 0.0, p0i = 0.0, Rjl[3][3];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int l = 0; l < 3; l++) Rjl[j][l] = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int l = 0; l < 3; l++)
#pragma unroll
        for (int m = 0; m < 3; m++) {
          // R[i][k][l][m]
          double r = 0.5 * (gdd[S6(i, m)][S6(k, l)] + gdd[S6(k, l)][S6(i, m)] - gdd[S6(i, l)][S6(k, m)] -
                            gdd[S6(k, m)][S6(i, l)]);
#pragma unroll
          for (int p = 0; p < 3; p++) r += GL[p][S6(k, l)] * G[p][S6(i, m)] - GL[p][S6(k, m)] * G[p][S6(i, l)];
          // as R_{i j k' l'} with (j, k', l') = (k, l, m): term 1 index roles
          const double t1 = r + K[i][l] * K[m][k] - K[i][m] * K[l][k];
          const double w = n[i] * n[l];
          p0r += t1 * w * A[k][m];
          p0i -= t1 * w * B[k][m];
          // R_jl = gamma^im R_ijml: here (i, k, l, m) -> contributes to R_{k m} with gamma^{i l}
          Rjl[k][m] += gUU[i][l] * r;
        }
  // term 2: t2_jkl = -8 (K_j[k,l] + Gamma^p_j[k K_l]p), contracted with n^0 n^k m^j m^l / 2
  double p1r = 0.0, p1i = 0.0;
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int l = 0; l < 3; l++) {
        double a = 0.5 * (Kd[S6(j, k)][l] - Kd[S6(j, l)][k]);
#pragma unroll
        for (int p = 0; p < 3; p++) a += 0.5 * (G[p][S6(j, k)] * K[l][p] - G[p][S6(j, l)] * K[k][p]);
        const double t2 = -8.0 * a;
        const double w = 0.5 * n0 * n[k];
        p1r += t2 * w * A[j][l];
        p1i -= t2 * w * B[j][l];
      }
  // term 3: t3_jl = 4 (R_jl + K K_jl - K_jp K^p_l), contracted with n^0 n^0 m^j m^l / 4
  double KUD[3][3], trKp = 0.0;
#pragma unroll
  for (int p = 0; p < 3; p++)
#pragma unroll
    for (int l = 0; l < 3; l++) KUD[p][l] = gUU[p][0] * K[0][l] + gUU[p][1] * K[1][l] + gUU[p][2] * K[2][l];
#pragma unroll
  for (int i = 0; i < 3; i++) trKp += KUD[i][i];
  double p2r = 0.0, p2i = 0.0;
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int l = 0; l < 3; l++) {
      double a = Rjl[j][l] + trKp * K[j][l];
#pragma unroll
      for (int p = 0; p < 3; p++) a -= K[j][p] * KUD[p][l];
      const double t3 = 4.0 * a;
      const double w = 0.25 * n0 * n0;
      p2r += t3 * w * A[j][l];
      p2i -= t3 * w * B[j][l];
    }
  re = p0r + p1r + p2r;
  im = p0i + p1i + p2i;
}

// One thread per point of the i0 range x interior (i1, i2), i0 fastest: a
// single extraction shell fills whole warps too.
constexpr int kPsi4Threads = 32;
template <int CS, int ORDER>
__global__ void __launch_bounds__(kPsi4Threads) psi4_kernel(Grid g, const double *__restrict__ in,
                                                            const double *__restrict__ tab, paramstruct p, int i0lo,
                                                            int i0hi, double *__restrict__ out_re,
                                                            double *__restrict__ out_im) {
  const long long t = (long long)blockIdx.x * kPsi4Threads + threadIdx.x;
  const int nr = i0hi - i0lo, n1i = g.n1 - 2 * g.ng, n2i = g.n2 - 2 * g.ng;
  if (t >= (long long)nr * n1i * n2i) return;
  const int i0 = i0lo + (int)(t % nr);
  const int i1 = g.ng + (int)((t / nr) % n1i);
  const int i2 = g.ng + (int)(t / ((long long)nr * n1i));
  const long long idx = i0 + (long long)g.n0 * (i1 + (long long)g.n1 * i2);
  Point<double> P{in + idx, g.ntot, {1, (long long)g.n0, (long long)g.n0 * g.n1}};
  const double inv[3] = {g.invdx0, g.invdx1, g.invdx2};
  const Rfm<CS, double> rf = rfm_at<CS, double>(tab, g, i0, i1, i2);
  const double xx0 = xx_of(p.xxmin0, p.dxx0, i0, g.ng);
  const double xx1 = xx_of(p.xxmin1, p.dxx1, i1, g.ng);
  const double xx2 = xx_of(p.xxmin2, p.dxx2, i2, g.ng);
  double re, im;
  psi4_point<ORDER, CS>(P, rf, inv, xx0, xx1, xx2, p, re, im);
  out_re[idx] = re;
  out_im[idx] = im;
}

// ------------------------------------------------ spin-weight -2 modes
constexpr int kModeThreads = 256;
constexpr int kMaxL = 12;

// One block per (l, m), l = 2..l_max, m = -l..l in that order.  Thread 0
// tabulates Goldberg's coefficients for the mode; the block then tabulates
// sY_lm's theta factor times sin(theta) for every interior i1 and
// cos(m phi), sin(m phi) for every interior i2 in shared memory, and every
// thread accumulates a strided share of the shell's points; a fixed-order
// tree reduction makes the result independent of scheduling.
__global__ void __launch_bounds__(kModeThreads) swm2_modes_kernel(Grid g, paramstruct p, int i0,
                                                                  const double *__restrict__ re_gf,
                                                                  const double *__restrict__ im_gf,
                                                                  double *__restrict__ out) {
  extern __shared__ double tabs[];  // [n1i] theta factors, then [n2i] cos(m phi), [n2i] sin(m phi)
  __shared__ double coef[kMaxL + 3];
  __shared__ int kexp[kMaxL + 3];
  __shared__ int nterm;
  __shared__ double sre[kModeThreads], sim[kModeThreads];
  int mode = blockIdx.x, l = 2;
  while (mode >= 2 * l + 1) {
    mode -= 2 * l + 1;
    l++;
  }
  const int m = mode - l;
  if (threadIdx.x == 0) {
    // sY_lm = (-1)^m sqrt((l+m)!(l-m)!(2l+1) / (4 pi (l+s)!(l-s)!)) sin^{2l}(th/2)
    //         sum_r C(l-s, r) C(l+s, r+s-m) (-1)^{l-r-s} e^{i m ph} cot^{2r+s-m}(th/2),  s = -2
    double fact[2 * kMaxL + 3];
    fact[0] = 1.0;
    for (int k = 1; k < 2 * kMaxL + 3; k++) fact[k] = fact[k - 1] * k;
    const int s = -2;
    const double norm = ((m & 1) ? -1.0 : 1.0) *
                        sqrt(fact[l + m] * fact[l - m] * (2 * l + 1) / (4.0 * M_PI * fact[l + s] * fact[l - s]));
    int nt = 0;
    for (int r = 0; r <= l - s; r++) {
      const int b2 = r + s - m;
      if (b2 < 0 || b2 > l + s) continue;
      const double c1 = fact[l - s] / (fact[r] * fact[l - s - r]);
      const double c2 = fact[l + s] / (fact[b2] * fact[l + s - b2]);
      coef[nt] = norm * c1 * c2 * (((l - r - s) & 1) ? -1.0 : 1.0);
      kexp[nt] = 2 * r + s - m;
      nt++;
    }
    nterm = nt;
  }
  __syncthreads();
  const int n1i = g.n1 - 2 * g.ng, n2i = g.n2 - 2 * g.ng;
  double *thf = tabs, *cph = tabs + n1i, *sph = tabs + n1i + n2i;
  for (int j = threadIdx.x; j < n1i; j += kModeThreads) {
    const double th = xx_of(p.xxmin1, p.dxx1, g.ng + j, g.ng);
    const double sh = sin(0.5 * th), ch = cos(0.5 * th);
    double y = 0.0;
    for (int t = 0; t < nterm; t++) {
      const int k = kexp[t];
      double pw = 1.0;
      for (int e = 0; e < 2 * l - k; e++) pw *= sh;
      for (int e = 0; e < k; e++) pw *= ch;
      y += coef[t] * pw;
    }
    thf[j] = y * sin(th);
  }
  for (int j = threadIdx.x; j < n2i; j += kModeThreads) {
    const double ph = xx_of(p.xxmin2, p.dxx2, g.ng + j, g.ng);
    cph[j] = cos(m * ph);
    sph[j] = sin(m * ph);
  }
  __syncthreads();
  double ar = 0.0, ai = 0.0;
  for (int q = threadIdx.x; q < n1i * n2i; q += kModeThreads) {
    const int j1 = q / n2i, j2 = q % n2i;
    const double c = thf[j1] * cph[j2], d = thf[j1] * sph[j2];
    const long long idx = i0 + (long long)g.n0 * ((g.ng + j1) + (long long)g.n1 * (g.ng + j2));
    const double a = re_gf[idx], b = im_gf[idx];
    ar += a * c + b * d;
    ai += b * c - a * d;
  }
  sre[threadIdx.x] = ar;
  sim[threadIdx.x] = ai;
  __syncthreads();
  for (int h = kModeThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      sre[threadIdx.x] += sre[threadIdx.x + h];
      sim[threadIdx.x] += sim[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = sre[0] * p.dxx1 * p.dxx2;
    out[2 * blockIdx.x + 1] = sim[0] * p.dxx1 * p.dxx2;
  }
}

}  // namespace psi4
}  // namespace nrgpu

using namespace nrgpu;
using namespace nrgpu::psi4;

int BSSN_psi4(const rfm_struct *rfm, const paramstruct *p, const double *in_gfs, double *psi4_gfs, int i0_min,
              int i0_max) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(in_gfs && psi4_gfs, "NULL gridfunctions");
  NRGPU_REQUIRE(p->NGHOSTS >= p->FD_order / 2, "psi4 needs NGHOSTS >= FD_order/2");
  NRGPU_REQUIRE(p->CoordSystem == NRGPU_COORD_CARTESIAN || rfm_matches(rfm, p),
                "curvilinear psi4 needs an rfm_struct defined for this grid");
  const int ng = p->NGHOSTS;
  if (i0_min < 0 && i0_max < 0) {
    i0_min = ng;
    i0_max = p->Nxx_plus_2NGHOSTS0 - ng;
  }
  NRGPU_REQUIRE(i0_min >= ng && i0_max <= p->Nxx_plus_2NGHOSTS0 - ng && i0_min < i0_max,
                "i0 range [%d, %d) outside the interior [%d, %d)", i0_min, i0_max, ng, p->Nxx_plus_2NGHOSTS0 - ng);
  Grid g = make_grid(p);
  const long long npts = (long long)(i0_max - i0_min) * p->Nxx1 * p->Nxx2;
  dim3 block(kPsi4Threads), grid((unsigned)((npts + kPsi4Threads - 1) / kPsi4Threads));
  const double *tab = rfm ? rfm->table64 : nullptr;
  double *re = psi4_gfs, *im = psi4_gfs + g.ntot;
#define P4(CS, ORD) psi4_kernel<CS, ORD><<<grid, block, 0, stream()>>>(g, in_gfs, tab, *p, i0_min, i0_max, re, im)
  switch (dispatch_cs(p->CoordSystem) * 16 + p->FD_order) {
    case NRGPU_COORD_CARTESIAN * 16 + 2: P4(NRGPU_COORD_CARTESIAN, 2); break;
    case NRGPU_COORD_CARTESIAN * 16 + 4: P4(NRGPU_COORD_CARTESIAN, 4); break;
    case NRGPU_COORD_CARTESIAN * 16 + 6: P4(NRGPU_COORD_CARTESIAN, 6); break;
    case NRGPU_COORD_CARTESIAN * 16 + 8: P4(NRGPU_COORD_CARTESIAN, 8); break;
    case NRGPU_COORD_SINHSPHERICAL * 16 + 4: P4(NRGPU_COORD_SINHSPHERICAL, 4); break;
    case NRGPU_COORD_SINHCYLINDRICAL * 16 + 4: P4(NRGPU_COORD_SINHCYLINDRICAL, 4); break;
    case NRGPU_COORD_SINHSYMTP * 16 + 4: P4(NRGPU_COORD_SINHSYMTP, 4); break;
    case NRGPU_COORD_SPHERICAL * 16 + 4: P4(NRGPU_COORD_SPHERICAL, 4); break;
    default:
      set_error("psi4: CoordSystem %d FD_order %d not built", p->CoordSystem, p->FD_order);
      return NRGPU_ERR_UNSUPPORTED;
  }
#undef P4
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int BSSN_psi4_spinweightm2_decomposition(const paramstruct *p, const double *psi4_gfs, int i0, int l_max,
                                         double *modes) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(psi4_gfs && modes, "NULL argument");
  NRGPU_REQUIRE(spherical_family(p->CoordSystem), "the mode decomposition needs a spherical-like grid");
  NRGPU_REQUIRE(l_max >= 2 && l_max <= kMaxL, "l_max %d outside [2, %d]", l_max, kMaxL);
  NRGPU_REQUIRE(i0 >= p->NGHOSTS && i0 < p->Nxx_plus_2NGHOSTS0 - p->NGHOSTS, "i0 %d is not an interior shell", i0);
  Grid g = make_grid(p);
  const int n_modes = (l_max + 1) * (l_max + 1) - 4;
  const size_t smem = sizeof(double) * (size_t)(p->Nxx1 + 2 * p->Nxx2);
  NRGPU_REQUIRE(smem <= 40 * 1024, "shell of %d x %d points too large for the mode tables", p->Nxx1, p->Nxx2);
  swm2_modes_kernel<<<n_modes, kModeThreads, smem, stream()>>>(g, *p, i0, psi4_gfs, psi4_gfs + g.ntot, modes);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}
