// bssn.cuh -- BSSN in reference-metric (rescaled) form: conformal Ricci
// tensor, evolution RHSs with the 1+log lapse and the covariant second-order
// Gamma-driver shift, Hamiltonian constraint.  Tensor expressions are
// written as index loops that the compiler unrolls; hatted quantities come
// from rfm.cuh with compile-time sparsity.
//
// Formulas (file:line in zachetienne/nrpytutorial):
//   basic tensors, Christoffels, Ricci  BSSN/BSSN_quantities.py:84-425
//   beta derivatives                    BSSN/BSSN_quantities.py:431-456
//   phi (W = e^{-2 phi}) derivatives    BSSN/BSSN_quantities.py:462-534
//   gammabar/Abar/cf/trK/Lambdabar RHS  BSSN/BSSN_RHSs.py:50-328
//   lapse/shift RHS                     BSSN/BSSN_gauge_RHSs.py:33-293
//   Hamiltonian constraint              BSSN/BSSN_constraints.py:19-74
// Derivatives of the rescaled gridfunctions are finite differences; every
// advection term beta^k d_k(...) uses the control-vector-upwinded
// derivative, as the reference's dupD symbols do.
#pragma once
#include "fd.cuh"
#include "rfm.cuh"

namespace nrgpu {
namespace bssn {

// Alphabetical gridfunction indices (grid.py:226-243).
enum GF {
  ADD00 = 0, ADD01, ADD02, ADD11, ADD12, ADD22, ALPHA, BETU0, BETU1, BETU2, CF,
  HDD00, HDD01, HDD02, HDD11, HDD12, HDD22, LAMBDAU0, LAMBDAU1, LAMBDAU2, TRK,
  VETU0, VETU1, VETU2, NUM_EVOL_GFS
};
// auxevol: RbarDD00 RbarDD01 RbarDD02 RbarDD11 RbarDD12 RbarDD22
constexpr int NUM_AUXEVOL_GFS = 6;

__host__ __device__ constexpr int S6(int i, int j) {
  return (i <= j) ? (i == 0 ? j : (i == 1 ? 2 + j : 5)) : (j == 0 ? i : (j == 1 ? 2 + i : 5));
}

// Stencil access to all gridfunctions at one point.
template <typename Tin> struct Point {
  typename InRef<Tin>::type c;  // in_gfs + idx (or hi + idx, lo + idx)
  long long ntot;
  long long st[3];
  __device__ __forceinline__ auto gf(int g) const { return c + (long long)g * ntot; }
};

template <int ORDER, typename R, typename Tin>
__device__ __forceinline__ R D1(const Point<Tin> &P, int g, int d, const R *inv) {
  return fd_d1<ORDER, R>(P.gf(g), P.st[d]) * inv[d];
}
template <int ORDER, typename R, typename Tin>
__device__ __forceinline__ R D2(const Point<Tin> &P, int g, int d, int e, const R *inv) {
  if (d == e) return fd_d2<ORDER, R>(P.gf(g), P.st[d]) * (inv[d] * inv[d]);
  // One canonical index order, so d_kl and d_lk are the same expression.
  const int a = d < e ? d : e, b = d < e ? e : d;
  return fd_d11<ORDER, R>(P.gf(g), P.st[a], P.st[b]) * (inv[a] * inv[b]);
}
template <int ORDER, typename R, typename Tin>
__device__ __forceinline__ R DUP(const Point<Tin> &P, int g, int d, const R *inv, const bool *pos) {
  return fd_dupwind<ORDER, R>(P.gf(g), P.st[d], pos[d]) * inv[d];
}
// Value of gridfunction g at the point.
template <typename R, typename Tin> __device__ __forceinline__ R pval(const Point<Tin> &P, int g) {
  return val<R>(P.gf(g));
}
// Advection of gridfunction g along the shift, beta^k d_k g with every d_k
// upwinded by the sign of beta^k.  The reference's RHSs use the upwinded
// derivatives (dupD symbols) only in these contractions with beta^k
// (BSSN_RHSs.py:69-318, BSSN_gauge_RHSs.py:61-67, 191-255), so each
// gridfunction contributes this one scalar.
template <int ORDER, typename R, typename Tin>
__device__ __forceinline__ R ADV(const Point<Tin> &P, int g, const R *betaU, const bool *pos, const R *inv) {
  R s = (R)0;
#pragma unroll
  for (int k = 0; k < 3; k++) s += betaU[k] * DUP<ORDER, R>(P, g, k, inv, pos);
  return s;
}

// Symmetric 3x3 inverse via the adjugate (indexedexp.py:331, symm_matrix_inverter3x3).
template <typename R>
__device__ __forceinline__ void sym_inverse(const R g[3][3], R gUU[3][3], R &det) {
  det = -g[0][2] * g[0][2] * g[1][1] + (R)2 * g[0][1] * g[0][2] * g[1][2] - g[0][0] * g[1][2] * g[1][2] -
        g[0][1] * g[0][1] * g[2][2] + g[0][0] * g[1][1] * g[2][2];
  const R inv = (R)1 / det;
  gUU[0][0] = (g[1][1] * g[2][2] - g[1][2] * g[1][2]) * inv;
  gUU[0][1] = (g[0][2] * g[1][2] - g[0][1] * g[2][2]) * inv;
  gUU[0][2] = (g[0][1] * g[1][2] - g[0][2] * g[1][1]) * inv;
  gUU[1][1] = (g[0][0] * g[2][2] - g[0][2] * g[0][2]) * inv;
  gUU[1][2] = (g[0][2] * g[0][1] - g[0][0] * g[1][2]) * inv;
  gUU[2][2] = (g[0][0] * g[1][1] - g[0][1] * g[0][1]) * inv;
  gUU[1][0] = gUU[0][1];
  gUU[2][0] = gUU[0][2];
  gUU[2][1] = gUU[1][2];
}

// ------------------------------------------------------------------ metric
// gammabar_ij, its inverse, and the barred Christoffels from hDD and its
// centred first derivatives (BSSN_quantities.py:84-158).
template <int CS, typename R> struct Metric {
  R h[3][3], eps[3][3], gbar[3][3], gUU[3][3], detgbar;
  R epsd[3][3][3];   // d_k eps_ij = d_k (h_ij ReDD_ij)
  R gbard[3][3][3];  // d_k gammabar_ij
  R Gbar[3][3][3];   // Gammabar^i_kl
};

template <int ORDER, int CS, typename R, typename PT, int LOC>
__device__ __forceinline__ void metric_point(const PT &P, const Rfm<CS, R, LOC> &rf, const R *inv,
                                             Metric<CS, R> &m) {
  using M = RfmMask<CS>;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const int g = HDD00 + S6(i, j);
      const R hij = pval<R>(P, g);
      m.h[i][j] = m.h[j][i] = hij;
      const R e = M::trivial ? hij : hij * rf.ReDD(i, j);
      m.eps[i][j] = m.eps[j][i] = e;
      R gb = e;
      if (i == j) gb += rf.ghatDD(i);
      m.gbar[i][j] = m.gbar[j][i] = gb;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const R hd = D1<ORDER, R>(P, g, k, inv);
        R ed = M::trivial ? hd : hd * rf.ReDD(i, j);
        if (M::ReDDdD(i, j, k)) ed += hij * rf.ReDDdD(i, j, k);
        m.epsd[i][j][k] = m.epsd[j][i][k] = ed;
        R gd = ed;
        if (M::ghatDDdD(i, j, k)) gd += rf.ghatDDdD(i, j, k);
        m.gbard[i][j][k] = m.gbard[j][i][k] = gd;
      }
    }
  sym_inverse(m.gbar, m.gUU, m.detgbar);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int l = k; l < 3; l++) {
        R s = (R)0;
#pragma unroll
        for (int mm = 0; mm < 3; mm++)
          s += m.gUU[i][mm] * (m.gbard[mm][k][l] + m.gbard[mm][l][k] - m.gbard[k][l][mm]);
        m.Gbar[i][k][l] = m.Gbar[i][l][k] = (R)0.5 * s;
      }
}

// Delta^i_jk = Gammabar - Gammahat, and Delta^i = gammabar^jk Delta^i_jk.
template <int CS, typename R, int LOC>
__device__ __forceinline__ void delta_gamma(const Metric<CS, R> &m, const Rfm<CS, R, LOC> &rf, R DG[3][3][3],
                                            R DGU[3]) {
  using M = RfmMask<CS>;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        R v = m.Gbar[i][j][k];
        if (M::Gammahat(i, j, k)) v -= rf.G(i, j, k);
        DG[i][j][k] = v;
      }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R s = (R)0;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) s += m.gUU[j][k] * DG[i][j][k];
    DGU[i] = s;
  }
}

// ------------------------------------------------------------------ Ricci
// Rbar_ij (BSSN_quantities.py:260-425), needs second derivatives of hDD and
// first derivatives of lambdaU.
template <int ORDER, int CS, typename R, typename PT, int LOC>
__device__ __forceinline__ void ricci_point(const PT &P, const Rfm<CS, R, LOC> &rf, const R *inv,
                                            const Metric<CS, R> &m, R Rbar[6]) {
  using M = RfmMask<CS>;
  R DG[3][3][3], DGU[3];
  delta_gamma<CS, R>(m, rf, DG, DGU);
  // Delta_ijk = gammabar_im Delta^m_jk
  R DGD[3][3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        R s = (R)0;
#pragma unroll
        for (int mm = 0; mm < 3; mm++) s += m.gbar[i][mm] * DG[mm][j][k];
        DGD[i][j][k] = s;
      }
  // \hat{D}_l gammabar_ij (gammabarDD_dHatD)
  R dH[3][3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int l = 0; l < 3; l++) {
        R v = m.epsd[i][j][l];
        if constexpr (!M::trivial) {
#pragma unroll
          for (int mm = 0; mm < 3; mm++) {
            if (M::Gammahat(mm, i, l)) v -= rf.G(mm, i, l) * m.eps[mm][j];
            if (M::Gammahat(mm, j, l)) v -= rf.G(mm, j, l) * m.eps[i][mm];
          }
        }
        dH[i][j][l] = v;
      }
  // lambda: \hat{D}_j Lambdabar^k (LambarU_dHatD)
  R lam[3], LdH[3][3];
#pragma unroll
  for (int k = 0; k < 3; k++) lam[k] = pval<R>(P, LAMBDAU0 + k);
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const R ld = D1<ORDER, R>(P, LAMBDAU0 + k, j, inv);
      R v = M::trivial ? ld : ld * rf.ReU(k);
      if (M::ReUdD(k, j)) v += lam[k] * rf.ReUdD(k, j);
      if constexpr (!M::trivial) {
#pragma unroll
        for (int mm = 0; mm < 3; mm++)
          if (M::Gammahat(k, mm, j)) v += rf.G(k, mm, j) * lam[mm] * rf.ReU(mm);
      }
      LdH[k][j] = v;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const int gij = HDD00 + S6(i, j);
      // the six distinct second derivatives of hDD_ij, each evaluated once
      R hdd[6];
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = k; l < 3; l++) hdd[S6(k, l)] = D2<ORDER, R>(P, gij, k, l, inv);
      // Term 1: -1/2 gammabar^kl \hat{D}_k \hat{D}_l gammabar_ij (dHatDD[i][j][l][k])
      R t1 = (R)0;
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = 0; l < 3; l++) {
          // eps_ij,lk
          R edd = hdd[S6(l, k)];
          if constexpr (!M::trivial) {
            edd *= rf.ReDD(i, j);
            if (M::ReDDdD(i, j, k)) edd += D1<ORDER, R>(P, gij, l, inv) * rf.ReDDdD(i, j, k);
            if (M::ReDDdD(i, j, l)) edd += D1<ORDER, R>(P, gij, k, inv) * rf.ReDDdD(i, j, l);
            if (M::ReDDdDD(i, j, l, k)) edd += m.h[i][j] * rf.ReDDdDD(i, j, l, k);
          }
          R v = edd;  // gammabarDD_dHatD_dD[i][j][l][k]
          if constexpr (!M::trivial) {
#pragma unroll
            for (int mm = 0; mm < 3; mm++) {
              if (M::GammahatdD(mm, i, l, k)) v -= rf.GdD(mm, i, l, k) * m.eps[mm][j];
              if (M::Gammahat(mm, i, l)) v -= rf.G(mm, i, l) * m.epsd[mm][j][k];
              if (M::GammahatdD(mm, j, l, k)) v -= rf.GdD(mm, j, l, k) * m.eps[i][mm];
              if (M::Gammahat(mm, j, l)) v -= rf.G(mm, j, l) * m.epsd[i][mm][k];
            }
#pragma unroll
            for (int mm = 0; mm < 3; mm++) {
              if (M::Gammahat(mm, l, k)) v -= rf.G(mm, l, k) * dH[i][j][mm];
              if (M::Gammahat(mm, i, k)) v -= rf.G(mm, i, k) * dH[mm][j][l];
              if (M::Gammahat(mm, j, k)) v -= rf.G(mm, j, k) * dH[i][mm][l];
            }
          }
          t1 += m.gUU[k][l] * v;
        }
      R r = (R)-0.5 * t1;
      // Term 2: 1/2 (gammabar_ki LdH^k_j + gammabar_kj LdH^k_i)
      R t2 = (R)0;
#pragma unroll
      for (int k = 0; k < 3; k++) t2 += m.gbar[k][i] * LdH[k][j] + m.gbar[k][j] * LdH[k][i];
      r += (R)0.5 * t2;
      // Term 3: 1/2 Delta^k (Delta_ijk + Delta_jik)
      R t3 = (R)0;
#pragma unroll
      for (int k = 0; k < 3; k++) t3 += DGU[k] * (DGD[i][j][k] + DGD[j][i][k]);
      r += (R)0.5 * t3;
      // Term 4
      R t4 = (R)0;
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = 0; l < 3; l++) {
          R s = (R)0;
#pragma unroll
          for (int mm = 0; mm < 3; mm++)
            s += DG[mm][k][i] * DGD[j][mm][l] + DG[mm][k][j] * DGD[i][mm][l] + DG[mm][i][k] * DGD[mm][j][l];
          t4 += m.gUU[k][l] * s;
        }
      Rbar[S6(i, j)] = r + t4;
    }
}

// --------------------------------------------------- momentum constraint
// M^i = e^{-4 phi}/ReU^i [gammabar^ik gammabar^jl Dbar_j Abar_kl
//       + 6 Abar^ij d_j phi - 2/3 gammabar^ij d_j K]  (BSSN_constraints.py:76-126;
// AbarDD_dD from BSSN_quantities.py:247-255; W = e^{-2 phi}).
template <int ORDER, int CS, typename R, typename Tin, int LOC>
__device__ __forceinline__ void momentum_point(const Point<Tin> &P, const Rfm<CS, R, LOC> &rf, const R *inv, R MU[3]) {
  using M = RfmMask<CS>;
  Metric<CS, R> m;
  metric_point<ORDER, CS, R>(P, rf, inv, m);
  const R cf = pval<R>(P, CF);
  R a[3][3], Abar[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      a[i][j] = a[j][i] = pval<R>(P, ADD00 + S6(i, j));
      Abar[i][j] = Abar[j][i] = M::trivial ? a[i][j] : a[i][j] * rf.ReDD(i, j);
    }
  R AUD[3][3], AUU[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R s = (R)0;
#pragma unroll
      for (int k = 0; k < 3; k++) s += m.gUU[i][k] * Abar[k][j];
      AUD[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R s = (R)0;
#pragma unroll
      for (int l = 0; l < 3; l++) s += AUD[i][l] * m.gUU[j][l];
      AUU[i][j] = s;
    }
  R phid[3], trKd[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    phid[j] = -D1<ORDER, R>(P, CF, j, inv) / ((R)2 * cf);
    trKd[j] = D1<ORDER, R>(P, TRK, j, inv);
  }
  // Dbar_k Abar_ij (symmetric in ij)
  R AdBar[3][3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const R ad = D1<ORDER, R>(P, ADD00 + S6(i, j), k, inv);
        R v = M::trivial ? ad : ad * rf.ReDD(i, j);
        if (M::ReDDdD(i, j, k)) v += rf.ReDDdD(i, j, k) * a[i][j];
#pragma unroll
        for (int l = 0; l < 3; l++) v -= m.Gbar[l][k][i] * Abar[l][j] + m.Gbar[l][k][j] * Abar[i][l];
        AdBar[i][j][k] = AdBar[j][i][k] = v;
      }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R r = (R)0;
#pragma unroll
    for (int j = 0; j < 3; j++) r += (R)6 * AUU[i][j] * phid[j] - (R)(2.0 / 3.0) * m.gUU[i][j] * trKd[j];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int l = 0; l < 3; l++)
#pragma unroll
        for (int j = 0; j < 3; j++) r += m.gUU[i][k] * m.gUU[j][l] * AdBar[k][l][j];
    r *= cf * cf;
    MU[i] = M::trivial ? r : r / rf.ReU(i);
  }
}

// -------------------------------------------------------------------- RHS
// All 24 right-hand sides at one interior point, in gridfunction order.
template <int ORDER, int CS, typename R, typename PT, int LOC>
__device__ __forceinline__ void rhs_point(const PT &P, const Rfm<CS, R, LOC> &rf, const R *inv,
                                          const R Rbar[6], R eta, R out[NUM_EVOL_GFS]) {
  using M = RfmMask<CS>;
  Metric<CS, R> m;
  metric_point<ORDER, CS, R>(P, rf, inv, m);

  const R alpha = pval<R>(P, ALPHA);
  const R cf = pval<R>(P, CF);
  const R trK = pval<R>(P, TRK);
  R vet[3], bet[3], lam[3], betaU[3], BU[3], LambdabarU[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    vet[i] = pval<R>(P, VETU0 + i);
    bet[i] = pval<R>(P, BETU0 + i);
    lam[i] = pval<R>(P, LAMBDAU0 + i);
    betaU[i] = M::trivial ? vet[i] : vet[i] * rf.ReU(i);
    BU[i] = M::trivial ? bet[i] : bet[i] * rf.ReU(i);
    LambdabarU[i] = M::trivial ? lam[i] : lam[i] * rf.ReU(i);
  }
  // UPWIND_ALG(UpwindControlVectorU) = (betaU > 0)
  bool pos[3];
#pragma unroll
  for (int d = 0; d < 3; d++) pos[d] = betaU[d] > (R)0;

  // beta^j d_j (f^i ReU^i) for a rescaled vector f (upwinded): ReU^i times
  // the advection of f^i, plus f^i beta^j d_j ReU^i.
  auto vec_adv = [&](int g0, int i, R fi) -> R {
    R u = ADV<ORDER, R>(P, g0 + i, betaU, pos, inv);
    if constexpr (!M::trivial) u *= rf.ReU(i);
#pragma unroll
    for (int j = 0; j < 3; j++)
      if (M::ReUdD(i, j)) u += betaU[j] * fi * rf.ReUdD(i, j);
    return u;
  };

  // beta^i_{,j}, beta^i_{,jk} (BSSN_quantities.py:431-456)
  R vetd[3][3], betad[3][3], betadd[3][3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      vetd[i][j] = D1<ORDER, R>(P, VETU0 + i, j, inv);
      R v = M::trivial ? vetd[i][j] : vetd[i][j] * rf.ReU(i);
      if (M::ReUdD(i, j)) v += vet[i] * rf.ReUdD(i, j);
      betad[i][j] = v;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = j; k < 3; k++) {
        R v = D2<ORDER, R>(P, VETU0 + i, j, k, inv);
        if constexpr (!M::trivial) v *= rf.ReU(i);
        if (M::ReUdD(i, k)) v += vetd[i][j] * rf.ReUdD(i, k);
        if (M::ReUdD(i, j)) v += vetd[i][k] * rf.ReUdD(i, j);
        if (M::ReUdDD(i, j, k)) v += vet[i] * rf.ReUdDD(i, j, k);
        betadd[i][j][k] = betadd[i][k][j] = v;
      }

  // Abar_ij, Abar^ij, Abar^i_j, trace (BSSN_quantities.py:189-240)
  R Abar[3][3], a[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      a[i][j] = a[j][i] = pval<R>(P, ADD00 + S6(i, j));
      Abar[i][j] = Abar[j][i] = M::trivial ? a[i][j] : a[i][j] * rf.ReDD(i, j);
    }
  R AUD[3][3], AUU[3][3], trAbar = (R)0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R s = (R)0;
#pragma unroll
      for (int k = 0; k < 3; k++) s += m.gUU[i][k] * Abar[k][j];
      AUD[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      R s = (R)0;
#pragma unroll
      for (int l = 0; l < 3; l++) s += AUD[i][l] * m.gUU[j][l];
      AUU[i][j] = AUU[j][i] = s;
    }
#pragma unroll
  for (int k = 0; k < 3; k++) trAbar += AUD[k][k];

  // det(gammabar) = det(gammahat) (detgbarOverdetghat_equals_one) and
  // Dbar_k beta^k = beta^k_{,k} + beta^k d_k detg / (2 detg)
  const R detg = rf.detg();
  R Dbarbeta = (R)0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    Dbarbeta += betad[k][k];
    if (M::detgdD(k)) Dbarbeta += betaU[k] * rf.detgdD(k) / ((R)2 * detg);
  }

  // phi derivatives for W = e^{-2 phi} (BSSN_quantities.py:496-508)
  R cfd[3], phid[3], phidd[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    cfd[i] = D1<ORDER, R>(P, CF, i, inv);
    phid[i] = -cfd[i] / ((R)2 * cf);
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++)
      phidd[i][j] = phidd[j][i] = (-D2<ORDER, R>(P, CF, i, j, inv) + cfd[i] * cfd[j] / cf) / ((R)2 * cf);
  const R exp_m4phi = cf * cf;

  R alphad[3], alphadBarDD[3][3], phidBarDD[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) alphad[i] = D1<ORDER, R>(P, ALPHA, i, inv);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      R va = D2<ORDER, R>(P, ALPHA, i, j, inv), vp = phidd[i][j];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        va -= m.Gbar[k][i][j] * alphad[k];
        vp -= m.Gbar[k][i][j] * phid[k];
      }
      alphadBarDD[i][j] = alphadBarDD[j][i] = va;
      phidBarDD[i][j] = phidBarDD[j][i] = vp;
    }

  // ---- gammabar_ij RHS (BSSN_RHSs.py:69-96), rescaled to h_rhsDD
  // ---- Abar_ij RHS (BSSN_RHSs.py:98-165), rescaled to a_rhsDD
  R curly[3][3], curly_tr = (R)0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const R c = (R)-2 * alpha * phidBarDD[i][j] + (R)4 * alpha * phid[i] * phid[j] +
                  (R)2 * alphad[i] * phid[j] + (R)2 * alphad[j] * phid[i] - alphadBarDD[i][j] +
                  alpha * Rbar[S6(i, j)];
      curly[i][j] = curly[j][i] = c;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) curly_tr += m.gUU[i][j] * curly[i][j];

#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      const int gij = S6(i, j);
      // upwinded beta^k d_k gammabar_ij and beta^k d_k Abar_ij
      R grhs = ADV<ORDER, R>(P, HDD00 + gij, betaU, pos, inv);
      R arhs = ADV<ORDER, R>(P, ADD00 + gij, betaU, pos, inv);
      if constexpr (!M::trivial) {
        grhs *= rf.ReDD(i, j);
        arhs *= rf.ReDD(i, j);
      }
#pragma unroll
      for (int k = 0; k < 3; k++) {
        if (M::ReDDdD(i, j, k)) {
          grhs += betaU[k] * (m.h[i][j] * rf.ReDDdD(i, j, k));
          arhs += betaU[k] * (rf.ReDDdD(i, j, k) * a[i][j]);
        }
        if (M::ghatDDdD(i, j, k)) grhs += betaU[k] * rf.ghatDDdD(i, j, k);
        grhs += betad[k][i] * m.gbar[k][j] + betad[k][j] * m.gbar[i][k];
        arhs += betad[k][i] * Abar[k][j] + betad[k][j] * Abar[i][k];
      }
      grhs += (R)(2.0 / 3.0) * m.gbar[i][j] * (alpha * trAbar - Dbarbeta);
      grhs += (R)-2 * alpha * Abar[i][j];
      arhs += (R)(-2.0 / 3.0) * Abar[i][j] * Dbarbeta + alpha * Abar[i][j] * trK;
#pragma unroll
      for (int k = 0; k < 3; k++) arhs += (R)-2 * alpha * Abar[i][k] * AUD[k][j];
      arhs += exp_m4phi * (curly[i][j] - (R)(1.0 / 3.0) * m.gbar[i][j] * curly_tr);
      if constexpr (M::trivial) {
        out[HDD00 + gij] = grhs;
        out[ADD00 + gij] = arhs;
      } else {
        const R re = rf.ReDD(i, j);
        out[HDD00 + gij] = grhs / re;
        out[ADD00 + gij] = arhs / re;
      }
    }

  // ---- cf RHS for W (BSSN_RHSs.py:167-194)
  {
    // beta^k d_k phi upwinded: -beta^k d_k cf / (2 cf)
    R phirhs = (R)(1.0 / 6.0) * (Dbarbeta - alpha * trK);
    phirhs += -ADV<ORDER, R>(P, CF, betaU, pos, inv) / ((R)2 * cf);
    out[CF] = phirhs * ((R)-2 * cf);
  }

  // ---- trK RHS (BSSN_RHSs.py:196-223)
  {
    R r = (R)(1.0 / 3.0) * alpha * trK * trK;
#pragma unroll
    r += ADV<ORDER, R>(P, TRK, betaU, pos, inv);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        r += -exp_m4phi * m.gUU[i][j] * (alphadBarDD[i][j] + (R)2 * alphad[j] * phid[i]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) r += alpha * Abar[i][j] * AUU[i][j];
    out[TRK] = r;
  }

  // ---- Lambdabar^i RHS (BSSN_RHSs.py:225-318)
  R DG[3][3][3], DGU[3];
  delta_gamma<CS, R>(m, rf, DG, DGU);
  // beta^k LambdabarU_dupD[i][k], upwinded
  R LAdv[3];
#pragma unroll
  for (int i = 0; i < 3; i++) LAdv[i] = vec_adv(LAMBDAU0, i, lam[i]);
  R trKd[3];
#pragma unroll
  for (int j = 0; j < 3; j++) trKd[j] = D1<ORDER, R>(P, TRK, j, inv);
  // Dbar^i Dbar_j beta^j pieces: Dbarbetacontraction_dBarD[m]
  R DbbdBar[3];
#pragma unroll
  for (int mm = 0; mm < 3; mm++) {
    R s = (R)0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      s += betadd[k][k][mm];
      if constexpr (!M::trivial) {
        R num = (R)0;
        bool any = false;
        if (M::detgdD(k)) { num += betad[k][mm] * rf.detgdD(k); any = true; }
        if (M::detgdDD(k, mm)) { num += betaU[k] * rf.detgdDD(k, mm); any = true; }
        if (any) s += num / ((R)2 * detg);
        if (M::detgdD(k) && M::detgdD(mm))
          s -= betaU[k] * rf.detgdD(k) * rf.detgdD(mm) / ((R)2 * detg * detg);
      }
    }
    DbbdBar[mm] = s;
  }
  R Lrhs[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R r = (R)0;
    // Term 1
#pragma unroll
    for (int k = 0; k < 3; k++) r += -betad[i][k] * LambdabarU[k];
    r += LAdv[i];
    // Term 2: gammabar^jk (beta^i_{,kj} + hatted pieces)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        R t = betadd[i][k][j];
        if constexpr (!M::trivial) {
#pragma unroll
          for (int mm = 0; mm < 3; mm++) {
            if (M::GammahatdD(i, mm, k, j)) t += rf.GdD(i, mm, k, j) * betaU[mm];
            if (M::Gammahat(i, mm, k)) t += rf.G(i, mm, k) * betad[mm][j];
            if (M::Gammahat(i, mm, j)) t += rf.G(i, mm, j) * betad[mm][k];
            if (M::Gammahat(mm, k, j)) t -= rf.G(mm, k, j) * betad[i][mm];
          }
#pragma unroll
          for (int mm = 0; mm < 3; mm++) {
            R c = (R)0;
            bool any = false;
#pragma unroll
            for (int d = 0; d < 3; d++) {
              if (M::Gammahat(i, d, j) && M::Gammahat(d, mm, k)) { c += rf.G(i, d, j) * rf.G(d, mm, k); any = true; }
              if (M::Gammahat(d, k, j) && M::Gammahat(i, mm, d)) { c -= rf.G(d, k, j) * rf.G(i, mm, d); any = true; }
            }
            if (any) t += c * betaU[mm];
          }
        }
        r += m.gUU[j][k] * t;
      }
    // Term 3
    r += (R)(2.0 / 3.0) * DGU[i] * Dbarbeta;
    // Term 4
#pragma unroll
    for (int mm = 0; mm < 3; mm++) r += (R)(1.0 / 3.0) * m.gUU[i][mm] * DbbdBar[mm];
    // Term 5
#pragma unroll
    for (int j = 0; j < 3; j++) r += (R)-2 * AUU[i][j] * (alphad[j] - (R)6 * alpha * phid[j]);
    // Term 6
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) r += (R)2 * alpha * AUU[j][k] * DG[i][j][k];
    // Term 7
#pragma unroll
    for (int j = 0; j < 3; j++) r += (R)(-4.0 / 3.0) * alpha * m.gUU[i][j] * trKd[j];
    Lrhs[i] = r;
    out[LAMBDAU0 + i] = M::trivial ? r : r / rf.ReU(i);
  }

  // ---- gauge: 1+log lapse, covariant 2nd-order Gamma-driver
  // (BSSN_gauge_RHSs.py:61-67, :191-255)
  {
    R r = (R)-2 * alpha * trK;
    r += ADV<ORDER, R>(P, ALPHA, betaU, pos, inv);
    out[ALPHA] = r;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    // upwinded beta^j d_j beta^i and beta^j d_j B^i
    R brhs = vec_adv(VETU0, i, vet[i]), Brhs = vec_adv(BETU0, i, bet[i]);
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) brhs += betaU[j] * m.Gbar[i][mm][j] * betaU[mm];
    brhs += BU[i];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) Brhs += betaU[j] * m.Gbar[i][mm][j] * BU[mm];
    Brhs += (R)(3.0 / 4.0) * Lrhs[i];
    Brhs += (R)(-3.0 / 4.0) * LAdv[i];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) Brhs += (R)(-3.0 / 4.0) * betaU[j] * m.Gbar[i][mm][j] * LambdabarU[mm];
    Brhs += -eta * BU[i];
    if constexpr (M::trivial) {
      out[VETU0 + i] = brhs;
      out[BETU0 + i] = Brhs;
    } else {
      out[VETU0 + i] = brhs / rf.ReU(i);
      out[BETU0 + i] = Brhs / rf.ReU(i);
    }
  }
}

}  // namespace bssn
}  // namespace nrgpu
