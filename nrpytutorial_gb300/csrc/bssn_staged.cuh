// bssn_staged.cuh -- BSSN Ricci / RHS kernels with shared-memory staging.
//
// The point kernels (bssn_kernels.cuh) read every stencil tap of every
// gridfunction from global memory inside the RHS algebra: ~900 dependent
// loads per point at the occupancy the algebra's live state allows.  Here a
// block owns a brick of TX x TY x TZ interior points and works in two phases:
//
//  A. For each gridfunction in turn, one thread issues a TMA bulk tensor
//     load (cp.async.bulk.tensor, completion on an mbarrier) of the brick
//     plus an H = FD_order/2 + 1 halo on every side into a ring of shared
//     buffers (the next boxes are in flight while one is used; every later
//     box is prefetched into L2 when the block starts, so the ring's loads
//     see L2 rather than DRAM latency).  Every thread then evaluates, from shared memory, what the
//     algebra needs of that gridfunction at its point -- the value, centred
//     first and second derivatives, and the upwinded advection
//     beta^k d_k f -- and stores them in its own column of a per-block
//     slot array in shared memory ([slot][thread], conflict-free).
//  B. The unchanged algebra of bssn.cuh (metric_point, ricci_point,
//     rhs_point) runs on a StagedPoint accessor that reads those slots, and
//     the fused RK4 epilogue writes the stage.
//
// Variants: RHS (reads RbarDD from auxevol, like rhs_eval), RICCI (writes
// RbarDD, like Ricci_eval), FUSED (Ricci computed in the block from staged
// second derivatives of hDD, then the RHSs: one launch per substep and no
// auxevol round trip).  Finite differences use the weights of fd.cuh
// (finite_difference.py:252-369) and the same hi/lo split for FP32 pairs.
#pragma once
#include <type_traits>

#include "bssn.cuh"
#include "epilogue.cuh"
#include "systems.cuh"
#include "bssn_kernels.cuh"
#include "tma.cuh"

// Unroll factor of the RK4 epilogue loop over the 24 gridfunctions.
// Boxes in flight per block of the RHS and Ricci variants.
#ifndef NRGPU_STAGED_NBUF
#define NRGPU_STAGED_NBUF 3
#endif
#ifndef NRGPU_STAGED_EPILOGUE_UNROLL
#define NRGPU_STAGED_EPILOGUE_UNROLL 4
#endif

namespace nrgpu {
namespace bssn {
namespace stage {

constexpr int kEpilogueUnroll = NRGPU_STAGED_EPILOGUE_UNROLL;

enum Variant { RHS = 0, RICCI = 1, FUSED = 2 };

__host__ __device__ constexpr bool is_hdd(int g) { return g >= HDD00 && g <= HDD22; }
__host__ __device__ constexpr bool is_lam(int g) { return g >= LAMBDAU0 && g <= LAMBDAU2; }
__host__ __device__ constexpr bool is_vet(int g) { return g >= VETU0 && g <= VETU2; }

// What a variant keeps of gridfunction g (all in slots, already scaled by
// the inverse grid spacings).
__host__ __device__ constexpr bool staged(int V, int g) { return V != RICCI || is_hdd(g) || is_lam(g); }
__host__ __device__ constexpr bool has_d1(int V, int g) {
  return V == RICCI ? (is_hdd(g) || is_lam(g))
                    : (g == ALPHA || g == CF || is_hdd(g) || g == TRK || is_vet(g) || (V == FUSED && is_lam(g)));
}
__host__ __device__ constexpr bool has_d2(int V, int g) {
  return V == RICCI ? is_hdd(g) : (g == ALPHA || g == CF || is_vet(g) || (V == FUSED && is_hdd(g)));
}
__host__ __device__ constexpr bool has_adv(int V, int g) { return V != RICCI && staged(V, g); }
__host__ __device__ constexpr int nslots(int V, int g) {
  return staged(V, g) ? 1 + 3 * (int)has_d1(V, g) + 6 * (int)has_d2(V, g) + (int)has_adv(V, g) : 0;
}
__host__ __device__ constexpr int base(int V, int g) {
  int b = 0;
  for (int k = 0; k < g; k++) b += nslots(V, k);
  return b;
}
__host__ __device__ constexpr int total_slots(int V) { return base(V, NUM_EVOL_GFS); }
__host__ __device__ constexpr int num_staged(int V) { return V == RICCI ? 9 : NUM_EVOL_GFS; }
// The it-th gridfunction a variant stages (RICCI: hDD then lambdaU).
__host__ __device__ constexpr int staged_gf(int V, int it) { return V == RICCI ? HDD00 + it : it; }
__host__ __device__ constexpr int slot_d1(int V, int g, int d) { return base(V, g) + 1 + d; }
__host__ __device__ constexpr int slot_d2(int V, int g, int s6) { return base(V, g) + 1 + 3 * (int)has_d1(V, g) + s6; }
__host__ __device__ constexpr int slot_adv(int V, int g) {
  return base(V, g) + 1 + 3 * (int)has_d1(V, g) + 6 * (int)has_d2(V, g);
}

// Brick and box geometry for arithmetic type R and stage element E.  FP32
// arithmetic: 16 x 4 x 2 points (128 threads); FP64: 16 x 4 x 1 (64 threads,
// the FP64 slots being twice as large).
template <typename R, typename E, int ORDER, int V> struct Tile {
  static constexpr int TX = 16, TY = 4, TZ = sizeof(R) == 8 ? 1 : 2;
  static constexpr int NT = TX * TY * TZ;
  static constexpr int H = ORDER / 2 + 1;
  static constexpr int ES = sizeof(E);
  static constexpr int QX = 16 / ES;  // box x extent in multiples of 16 bytes
  static constexpr int BX = (TX + 2 * H + QX - 1) / QX * QX, BY = TY + 2 * H, BZ = TZ + 2 * H;
  static constexpr int BOX_BYTES = BX * BY * BZ * ES;
  static constexpr int BOX_STRIDE = (BOX_BYTES + 127) / 128 * 128;
  // Boxes in flight per block: the most (up to NRGPU_STAGED_NBUF) with which
  // two blocks still fit an SM's shared memory (228 KB, 1 KB reserved per
  // block).  FD4: the fused variant's larger slot array leaves room for two
  // boxes, the others for three; FD6: one box for the fused variant and two
  // for RHS (deeper rings would leave one block, 4 warps, per SM: 128^3
  // Cartesian compensated step 11.85 -> 9.94 ms on the RHS variant).  When
  // not even one box leaves room for two blocks (FD8 fused), two boxes: a
  // single box would expose every copy's latency at one block per SM
  // (15.8 -> 20.9 ms).
  static constexpr int SLOT_BYTES = total_slots(V) * NT * (int)sizeof(R);
  static constexpr int kTwoBlockSmem = 113 * 1024;
  static constexpr bool fits(int nb) { return 128 + nb * BOX_STRIDE + SLOT_BYTES <= kTwoBlockSmem; }
  static constexpr int NBUF = (NRGPU_STAGED_NBUF >= 3 && fits(3)) ? 3 : fits(2) ? 2 : fits(1) ? 1 : 2;
  static constexpr int SLOT_OFFSET = 128 + NBUF * BOX_STRIDE;
  static_assert(TX % QX == 0, "box start must stay 16-byte aligned");
};
template <typename R, typename E, int ORDER, int V> constexpr int smem_bytes() {
  using T = Tile<R, E, ORDER, V>;
  return T::SLOT_OFFSET + total_slots(V) * T::NT * (int)sizeof(R);
}

// ------------------------------------------ stencils on a shared-memory box
// p points at the stencil centre; s is a stride in elements.  Same weights
// and, for FP32 pairs, the same hi/lo treatment as the global versions in
// fd.cuh.
template <typename R, typename E> __device__ __forceinline__ R sval(const E *p) {
  if constexpr (std::is_same<E, float2>::value) return (R)p[0].x + (R)p[0].y;
  else return (R)p[0];
}

template <int ORDER, typename R, typename E> __device__ __forceinline__ R s_d1(const E *p, int s) {
  using C = FDCoef<ORDER>;
  if constexpr (std::is_same<E, float2>::value) {
    R hi = (R)0, lo = (R)0;
#pragma unroll
    for (int k = 1; k <= C::R; k++) {
      const float2 a = p[k * s], b = p[-k * s];
      hi += (R)C::c1(k) * ((R)a.x - (R)b.x);
      lo += (R)C::c1(k) * ((R)a.y - (R)b.y);
    }
    return hi + lo;
  } else {
    R acc = (R)C::c1(1) * ((R)p[s] - (R)p[-s]);
#pragma unroll
    for (int k = 2; k <= C::R; k++) acc += (R)C::c1(k) * ((R)p[k * s] - (R)p[-k * s]);
    return acc;
  }
}

template <int ORDER, typename R, typename E> __device__ __forceinline__ R s_d2(const E *p, int s) {
  using C = FDCoef<ORDER>;
  if constexpr (std::is_same<E, float2>::value) {
    const float2 c = p[0];
    R hi = (R)0, lo = (R)C::c2(0) * (R)c.y;
#pragma unroll
    for (int k = 1; k <= C::R; k++) {
      const float2 a = p[k * s], b = p[-k * s];
      hi += (R)C::c2(k) * (((R)a.x - (R)c.x) + ((R)b.x - (R)c.x));
      lo += (R)C::c2(k) * ((R)a.y + (R)b.y);
    }
    return hi + lo;
  } else {
    R acc = (R)C::c2(0) * (R)p[0];
#pragma unroll
    for (int k = 1; k <= C::R; k++) acc += (R)C::c2(k) * ((R)p[k * s] + (R)p[-k * s]);
    return acc;
  }
}

template <int ORDER, typename R, typename E> __device__ __forceinline__ R s_d11(const E *p, int s, int t) {
  using C = FDCoef<ORDER>;
  if constexpr (std::is_same<E, float2>::value) {
    R hi = (R)0, lo = (R)0;
#pragma unroll
    for (int a = 1; a <= C::R; a++) {
      R ih = (R)0, il = (R)0;
#pragma unroll
      for (int b = 1; b <= C::R; b++) {
        const int ps = a * s, qt = b * t;
        const float2 pp = p[ps + qt], pm = p[ps - qt], mp = p[-ps + qt], mm = p[-ps - qt];
        ih += (R)C::c1(b) * (((R)pp.x - (R)pm.x) - ((R)mp.x - (R)mm.x));
        il += (R)C::c1(b) * (((R)pp.y - (R)pm.y) - ((R)mp.y - (R)mm.y));
      }
      hi += (R)C::c1(a) * ih;
      lo += (R)C::c1(a) * il;
    }
    return hi + lo;
  } else {
    R acc = (R)0;
#pragma unroll
    for (int a = 1; a <= C::R; a++) {
      R inner = (R)0;
#pragma unroll
      for (int b = 1; b <= C::R; b++) {
        const int ps = a * s, qt = b * t;
        inner += (R)C::c1(b) * (((R)p[ps + qt] - (R)p[ps - qt]) - ((R)p[-ps + qt] - (R)p[-ps - qt]));
      }
      acc += (R)C::c1(a) * inner;
    }
    return acc;
  }
}

// Upwinded first derivative: dupD where positive, else ddnD (signed stride).
template <int ORDER, typename R, typename E> __device__ __forceinline__ R s_dup(const E *p, int s, bool positive) {
  using C = FDCoef<ORDER>;
  const int ss = positive ? s : -s;
  if constexpr (std::is_same<E, float2>::value) {
    const float2 c = p[0];
    R hi = (R)0, lo = (R)0;
#pragma unroll
    for (int j = 0; j <= ORDER; j++) {
      const int k = j + C::UPLO;
      if (C::up(j) == 0.0) continue;
      if (k == 0) {
        lo += (R)C::up(j) * (R)c.y;
      } else {
        const float2 v = p[k * ss];
        hi += (R)C::up(j) * ((R)v.x - (R)c.x);
        lo += (R)C::up(j) * (R)v.y;
      }
    }
    const R acc = hi + lo;
    return positive ? acc : -acc;
  } else {
    R acc = (R)0;
#pragma unroll
    for (int j = 0; j <= ORDER; j++) {
      const int k = j + C::UPLO;
      if (C::up(j) != 0.0) acc += (R)C::up(j) * (R)p[k * ss];
    }
    return positive ? acc : -acc;
  }
}

// Phase A for one gridfunction: this thread's slots from the box centred
// at p (strides 1, sy, sz).  out: this thread's slot `b` (stride NT).
template <int ORDER, typename R, typename E, int NT>
__device__ __forceinline__ void stage_one(const E *__restrict__ p, int sy, int sz, const R inv[3], const R betaU[3],
                                          const bool pos[3], bool d1, bool d2, bool adv, R *__restrict__ out) {
  const int st[3] = {1, sy, sz};
  out[0] = sval<R>(p);
  int n = 1;
  if (d1) {
#pragma unroll
    for (int d = 0; d < 3; d++) out[(n + d) * NT] = s_d1<ORDER, R>(p, st[d]) * inv[d];
    n += 3;
  }
  if (d2) {
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = a; b < 3; b++)
        out[(n + S6(a, b)) * NT] = a == b ? s_d2<ORDER, R>(p, st[a]) * (inv[a] * inv[a])
                                          : s_d11<ORDER, R>(p, st[a], st[b]) * (inv[a] * inv[b]);
    n += 6;
  }
  if (adv) {
    R s = (R)0;
#pragma unroll
    for (int k = 0; k < 3; k++) s += betaU[k] * (s_dup<ORDER, R>(p, st[k], pos[k]) * inv[k]);
    out[n * NT] = s;
  }
}

}  // namespace stage

// ------------------------------------------------- phase B point accessor
// This thread's staged values: slot k at s[k * NT].
template <typename RS, int V, int NT> struct StagedPoint {
  const RS *s;
  __device__ __forceinline__ RS at(int k) const { return s[k * NT]; }
};

template <typename R, typename RS, int V, int NT>
__device__ __forceinline__ R pval(const StagedPoint<RS, V, NT> &P, int g) {
  return (R)P.at(stage::base(V, g));
}
template <int ORDER, typename R, typename RS, int V, int NT>
__device__ __forceinline__ R D1(const StagedPoint<RS, V, NT> &P, int g, int d, const R *) {
  return (R)P.at(stage::slot_d1(V, g, d));
}
template <int ORDER, typename R, typename RS, int V, int NT>
__device__ __forceinline__ R D2(const StagedPoint<RS, V, NT> &P, int g, int d, int e, const R *) {
  return (R)P.at(stage::slot_d2(V, g, S6(d, e)));
}
template <int ORDER, typename R, typename RS, int V, int NT>
__device__ __forceinline__ R ADV(const StagedPoint<RS, V, NT> &P, int g, const R *, const bool *, const R *) {
  return (R)P.at(stage::slot_adv(V, g));
}

// Phase B: the algebra on the staged values and the reference metric `rf`,
// then the variant's stores.
template <typename R, int CS, int ORDER, typename TStage, int V, int NT, typename RF>
__device__ __forceinline__ void staged_phase_b(const StagedPoint<R, V, NT> &P, const RF &rf, const R inv[3],
                                               const R *__restrict__ aux_in, R eta, const RKEpilogue<TStage> &epi,
                                               R *__restrict__ aux_out, const Grid &g, long long idx) {
  if constexpr (V == stage::RICCI) {
    Metric<CS, R> m;
    metric_point<ORDER, CS, R>(P, rf, inv, m);
    R Rbar[6];
    ricci_point<ORDER, CS, R>(P, rf, inv, m, Rbar);
#pragma unroll
    for (int k = 0; k < 6; k++) aux_out[(long long)k * g.ntot + idx] = Rbar[k];
  } else {
    R Rbar[6];
    if constexpr (V == stage::FUSED) {
      Metric<CS, R> m;
      metric_point<ORDER, CS, R>(P, rf, inv, m);
      ricci_point<ORDER, CS, R>(P, rf, inv, m, Rbar);
    } else {
#pragma unroll
      for (int k = 0; k < 6; k++) Rbar[k] = (R)__ldg(aux_in + (long long)k * g.ntot + idx);
    }
    R out[NUM_EVOL_GFS];
    rhs_point<ORDER, CS, R>(P, rf, inv, Rbar, eta, out);
#pragma unroll stage::kEpilogueUnroll
    for (int gf = 0; gf < NUM_EVOL_GFS; gf++) epi(gf, idx, out[gf]);
  }
}

// ------------------------------------------------------------------ kernel
// R arithmetic type; Tin stage-input tag (double, float, or Pair32 for FP32
// (hi, lo) pairs); TStage the epilogue's stage type (unused by RICCI).
// in: the stage input (global, for the shift at the point); tmap: the same
// array as a TMA tensor map; aux_in: RbarDD (RHS); aux_out: RbarDD (RICCI);
// status: device status word (set when a bounded wait gives up).
template <typename R, typename Tin, int CS, int ORDER, typename TStage, int V>
__global__ void __launch_bounds__(stage::Tile<R, typename std::conditional<std::is_same<Tin, Pair32>::value, float2,
                                                                           Tin>::type, ORDER, V>::NT, 2)
    staged_kernel(Grid g, const __grid_constant__ CUtensorMap tmap, typename InRef<Tin>::type in,
                  const R *__restrict__ aux_in, const R *__restrict__ tab, R eta, RKEpilogue<TStage> epi,
                  R *__restrict__ aux_out, int *status) {
  using E = typename std::conditional<std::is_same<Tin, Pair32>::value, float2, Tin>::type;
  using T = stage::Tile<R, E, ORDER, V>;
  constexpr int NT = T::NT, H = T::H, NSTG = stage::num_staged(V);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)smem;                // NBUF mbarriers
  int *abort_flag = (int *)(smem + 120);
  unsigned char *bufs = smem + 128;                // NBUF boxes of BOX_STRIDE bytes
  R *slots = (R *)(smem + T::SLOT_OFFSET);
  static_assert(T::NBUF * 8 <= 120, "mbarriers overlap the abort flag");

  const int t = threadIdx.x;
  const int tx = t % T::TX, ty = (t / T::TX) % T::TY, tz = t / (T::TX * T::TY);
  const int x0 = blockIdx.x * T::TX, y0 = blockIdx.y * T::TY, z0 = blockIdx.z * T::TZ;
  const int nx = g.n0 - 2 * g.ng, ny = g.n1 - 2 * g.ng, nz = g.n2 - 2 * g.ng;
  const bool valid = x0 + tx < nx && y0 + ty < ny && z0 + tz < nz;
  // Threads past the interior's edge compute on the last interior point
  // (every address in bounds) and store nothing.
  const int i0 = g.ng + min(x0 + tx, nx - 1), i1 = g.ng + min(y0 + ty, ny - 1), i2 = g.ng + min(z0 + tz, nz - 1);
  const long long idx = (long long)i0 + (long long)g.n0 * ((long long)i1 + (long long)g.n1 * i2);

  if (t == 0) {
#pragma unroll
    for (int b = 0; b < T::NBUF; b++) mbar_init(&bar[b], 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  // Box origin: the brick's first interior point minus the halo.  x is
  // ng - H + 16 * blockIdx.x with ng == H (checked by the launcher), a
  // multiple of 16 bytes for every element size.
  const int bx0 = g.ng + x0 - H, by0 = g.ng + y0 - H, bz0 = g.ng + z0 - H;
  int issued = NSTG < T::NBUF ? NSTG : T::NBUF;  // box loads issued so far (thread 0's count)
  if (t == 0) {
    for (int it = 0; it < issued; it++) {
      mbar_arrive_expect_tx(&bar[it], T::BOX_BYTES);
      tma_load_4d(bufs + it * T::BOX_STRIDE, &tmap, bx0, by0, bz0, stage::staged_gf(V, it), &bar[it]);
    }
    for (int it = issued; it < NSTG; it++) tma_prefetch_l2_4d(&tmap, bx0, by0, bz0, stage::staged_gf(V, it));
  }

  // The epilogue's y_n and running-total values of this point start on their
  // way to L2 now and arrive while phase A runs.
  if constexpr (V != stage::RICCI) {
    if (epi.stage >= 0) {
#pragma unroll 1
      for (int gf = 0; gf < NUM_EVOL_GFS; gf++) {
        const long long i = (long long)gf * g.ntot + idx;
        prefetch_l2(epi.y_n + i);
        if (epi.stage > 0) prefetch_l2(epi.rt + i);
      }
    }
  }

  const R inv[3] = {(R)g.invdx0, (R)g.invdx1, (R)g.invdx2};
  const Rfm<CS, R> rf = rfm_at<CS, R>(tab, g, i0, i1, i2);
  R betaU[3] = {(R)0, (R)0, (R)0};
  bool pos[3] = {false, false, false};
  if constexpr (V != stage::RICCI) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const R vet = val<R>(in + (long long)(VETU0 + k) * g.ntot + idx);
      betaU[k] = RfmMask<CS>::trivial ? vet : vet * rf.ReU(k);
      pos[k] = betaU[k] > (R)0;  // UPWIND_ALG(UpwindControlVectorU)
    }
  }

  // ---- phase A
  const int centre = (tx + H) + T::BX * ((ty + H) + T::BY * (tz + H));
  R *myslots = slots + t;
  int sbase = 0, b = 0;
  uint32_t parity = 0;
#pragma unroll 1
  for (int it = 0; it < NSTG; it++) {
    const int gf = stage::staged_gf(V, it);
    const E *box = (const E *)(bufs + b * T::BOX_STRIDE);
    if (!mbar_wait_bounded(&bar[b], parity)) {
      *abort_flag = 1;
    } else {
      stage::stage_one<ORDER, R, E, NT>(box + centre, T::BX, T::BX * T::BY, inv, betaU, pos, stage::has_d1(V, gf),
                                        stage::has_d2(V, gf), stage::has_adv(V, gf), myslots + (long long)sbase * NT);
    }
    sbase += stage::nslots(V, gf);
    __syncthreads();  // every thread is done with this box
    if (*abort_flag) break;
    if (t == 0 && it + T::NBUF < NSTG) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[b], T::BOX_BYTES);
      tma_load_4d(bufs + b * T::BOX_STRIDE, &tmap, bx0, by0, bz0, stage::staged_gf(V, it + T::NBUF), &bar[b]);
      issued = it + T::NBUF + 1;
    }
    if (++b == T::NBUF) {
      b = 0;
      parity ^= 1u;
    }
  }
  if (*abort_flag) {
    // A copy did not arrive in time: record it, let the copies in flight
    // land (bounded) before the block's shared memory goes away, store
    // nothing.
    if (t == 0) {
      atomicOr(status, 1);
      for (int it = issued - T::NBUF < 0 ? 0 : issued - T::NBUF; it < issued; it++)
        mbar_wait_bounded(&bar[it % T::NBUF], (uint32_t)((it / T::NBUF) & 1));
    }
    return;
  }

  // ---- phase B
  if (!valid) return;
  staged_phase_b<R, CS, ORDER, TStage, V, NT>(StagedPoint<R, V, NT>{slots + t}, rf, inv, aux_in, eta, epi, aux_out,
                                              g, idx);
}

// ---------------------------------------------------------------- launchers
// NRGPU_ERR_UNSUPPORTED (no message) when the grid cannot take the staged
// path: ghost width other than FD_order/2 + 1, a stage array whose strides
// or base are not 16-byte aligned, or an FP32-arithmetic step on FP64 input.
// The caller then runs the point kernels.

template <typename R, typename Tin, int CS, int ORDER, typename TStage, int V>
int staged_launch(const rfm_struct *rfm, const paramstruct *p, const void *in, const R *aux_in, R *aux_out, R eta,
                  const RKEpilogue<TStage> &epi) {
  using E = typename std::conditional<std::is_same<Tin, Pair32>::value, float2, Tin>::type;
  using T = stage::Tile<R, E, ORDER, V>;
  Grid g = make_grid(p);
  if (g.ng != T::H) return NRGPU_ERR_UNSUPPORTED;
  CUtensorMap map;
  if (!tma_map_gridfunctions(&map, in, (int)sizeof(E), g.n0, g.n1, g.n2, NUM_EVOL_GFS, T::BX, T::BY, T::BZ))
    return NRGPU_ERR_UNSUPPORTED;
  int *status = device_status_word();
  NRGPU_REQUIRE(status != nullptr, "staged BSSN kernel: device status word unavailable");
  constexpr int smem = stage::smem_bytes<R, E, ORDER, V>();
  auto kern = staged_kernel<R, Tin, CS, ORDER, TStage, V>;
  static bool attr_done[64];
  int dev = 0;
  NRGPU_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || !attr_done[dev]) {
    NRGPU_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    if (dev >= 0 && dev < 64) attr_done[dev] = true;
  }
  const int nx = g.n0 - 2 * g.ng, ny = g.n1 - 2 * g.ng, nz = g.n2 - 2 * g.ng;
  const dim3 grid((nx + T::TX - 1) / T::TX, (ny + T::TY - 1) / T::TY, (nz + T::TZ - 1) / T::TZ);
  kern<<<grid, T::NT, smem, stream()>>>(g, map, (typename InRef<Tin>::type)in, aux_in, table_of<R>(rfm), eta, epi,
                                        aux_out, status);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

template <int CS, int ORDER>
int staged_ricci_launch_t(const rfm_struct *rfm, const paramstruct *p, const void *in, bool in_is_f64, int prec,
                          void *aux) {
  if (prec == NRGPU_PREC_FP64)
    return staged_launch<double, double, CS, ORDER, double, stage::RICCI>(rfm, p, in, nullptr, (double *)aux, 0.0,
                                                                        RKEpilogue<double>{});
  if (in_is_f64) return NRGPU_ERR_UNSUPPORTED;
  if (pair_precision(prec))
    return staged_launch<float, Pair32, CS, ORDER, float2, stage::RICCI>(rfm, p, in, nullptr, (float *)aux, 0.f,
                                                                        RKEpilogue<float2>{});
  return staged_launch<float, float, CS, ORDER, float, stage::RICCI>(rfm, p, in, nullptr, (float *)aux, 0.f,
                                                                    RKEpilogue<float>{});
}

// fused: Ricci computed in the block (auxevol neither read nor written).
template <int CS, int ORDER>
int staged_rhs_launch_t(const rfm_struct *rfm, const paramstruct *p, const StageArgs &a, bool fused) {
  Grid g = make_grid(p);
  if (a.prec == NRGPU_PREC_FP64) {
    RKEpilogue<double> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (double *)a.out};
    return fused ? staged_launch<double, double, CS, ORDER, double, stage::FUSED>(rfm, p, a.in, nullptr, nullptr,
                                                                                  p->eta, epi)
                 : staged_launch<double, double, CS, ORDER, double, stage::RHS>(
                       rfm, p, a.in, (const double *)a.auxevol, nullptr, p->eta, epi);
  }
  if (a.in_is_f64) return NRGPU_ERR_UNSUPPORTED;
  const float eta32 = (float)p->eta;
  if (pair_precision(a.prec)) {
    RKEpilogue<float2> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float2 *)a.out, stage_consts(a.dt),
                           a.prec == NRGPU_PREC_COMPENSATED_FP64RK};
    return fused ? staged_launch<float, Pair32, CS, ORDER, float2, stage::FUSED>(rfm, p, a.in, nullptr, nullptr,
                                                                                 eta32, epi)
                 : staged_launch<float, Pair32, CS, ORDER, float2, stage::RHS>(
                       rfm, p, a.in, (const float *)a.auxevol, nullptr, eta32, epi);
  }
  RKEpilogue<float> epi{a.stage, a.dt, g.ntot, a.y_n, a.rt, (float *)a.out, stage_consts(a.dt)};
  return fused ? staged_launch<float, float, CS, ORDER, float, stage::FUSED>(rfm, p, a.in, nullptr, nullptr, eta32,
                                                                             epi)
               : staged_launch<float, float, CS, ORDER, float, stage::RHS>(rfm, p, a.in, (const float *)a.auxevol,
                                                                           nullptr, eta32, epi);
}

#define NRGPU_BSSN_STAGED_DECLARE(CS, ORDER)                                                                  \
  extern template int staged_ricci_launch_t<CS, ORDER>(const rfm_struct *, const paramstruct *, const void *, \
                                                       bool, int, void *);                                    \
  extern template int staged_rhs_launch_t<CS, ORDER>(const rfm_struct *, const paramstruct *, const StageArgs &, \
                                                     bool);
#define NRGPU_BSSN_STAGED_INSTANTIATE(CS, ORDER)                                                             \
  template int staged_ricci_launch_t<CS, ORDER>(const rfm_struct *, const paramstruct *, const void *, bool, \
                                                int, void *);                                                \
  template int staged_rhs_launch_t<CS, ORDER>(const rfm_struct *, const paramstruct *, const StageArgs &, bool);

}  // namespace bssn
}  // namespace nrgpu
