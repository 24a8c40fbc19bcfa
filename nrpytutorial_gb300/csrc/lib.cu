// lib.cu -- library state (status messages, stream, launch counter), grid
// set-up, CFL timestep and the reference-metric precompute tables.
#include <cmath>
#include <math.h>
#include <stdarg.h>
#include <string.h>

#include <atomic>
#include <string>

#include "common.cuh"
#include "fd.cuh"
#include "rfm.cuh"

namespace nrgpu {

static thread_local char g_err[1024] = "";
static cudaStream_t g_stream = nullptr;
static std::atomic<long long> g_launches{0};

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
cudaStream_t stream() { return g_stream; }
void count_launch(int n) { g_launches += n; }

int check_params(const paramstruct *p) {
  NRGPU_REQUIRE(p != nullptr, "params is NULL");
  NRGPU_REQUIRE(p->CoordSystem >= 0 && p->CoordSystem <= 8, "unknown CoordSystem %d", p->CoordSystem);
  NRGPU_REQUIRE(p->FD_order == 2 || p->FD_order == 4 || p->FD_order == 6 || p->FD_order == 8,
                "FD_order %d not in {2,4,6,8}", p->FD_order);
  NRGPU_REQUIRE(p->NGHOSTS >= p->FD_order / 2 && p->NGHOSTS <= NRGPU_MAX_GHOSTS,
                "NGHOSTS %d invalid for FD_order %d", p->NGHOSTS, p->FD_order);
  NRGPU_REQUIRE(p->Nxx0 >= 1 && p->Nxx1 >= 1 && p->Nxx2 >= 1, "Nxx must be positive");
  NRGPU_REQUIRE(p->Nxx_plus_2NGHOSTS0 == p->Nxx0 + 2 * p->NGHOSTS &&
                    p->Nxx_plus_2NGHOSTS1 == p->Nxx1 + 2 * p->NGHOSTS &&
                    p->Nxx_plus_2NGHOSTS2 == p->Nxx2 + 2 * p->NGHOSTS,
                "Nxx_plus_2NGHOSTS inconsistent with Nxx and NGHOSTS");
  const long long ntot =
      (long long)p->Nxx_plus_2NGHOSTS0 * p->Nxx_plus_2NGHOSTS1 * p->Nxx_plus_2NGHOSTS2;
  NRGPU_REQUIRE(ntot < (1LL << 31) / 32, "grid of %lld points too large for 32-bit gf indexing", ntot);
  NRGPU_REQUIRE(std::isfinite(p->diss_strength), "diss_strength is not finite");
  return NRGPU_OK;
}

// ----------------------------------------------------------------- rfm define
// One thread per (i0, iB) column: iB = i1 for the Spherical family, i2 for
// the Cylindrical family (the coordinate the reference metric depends on).
__global__ void rfm_define_kernel(paramstruct p, double *tab64, float *tab32) {
  const bool cyl = cylindrical_family(p.CoordSystem);
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int iB = blockIdx.y;
  const int n0 = p.Nxx_plus_2NGHOSTS0, nB = cyl ? p.Nxx_plus_2NGHOSTS2 : p.Nxx_plus_2NGHOSTS1;
  if (i0 >= n0 || iB >= nB) return;
  const double xx0 = xx_of(p.xxmin0, p.dxx0, i0, p.NGHOSTS);
  const double xxB = cyl ? xx_of(p.xxmin2, p.dxx2, iB, p.NGHOSTS) : xx_of(p.xxmin1, p.dxx1, iB, p.NGHOSTS);
  ScaleFactors S;
  scale_factors(coord_params(p), xx0, xxB, xxB, &S);
  double out[rq::NQ];
  hatted_quantities(S, out);
  const long long plane = (long long)n0 * nB, col = (long long)iB * n0 + i0;
  for (int q = 0; q < rq::NQ; q++) {
    tab64[q * plane + col] = out[q];
    tab32[q * plane + col] = (float)out[q];
  }
}

}  // namespace nrgpu

using namespace nrgpu;

extern "C" {

int nrgpu_version(void) { return 1; }

int nrgpu_set_stream(void *s) {
  g_stream = (cudaStream_t)s;
  return NRGPU_OK;
}
void *nrgpu_get_stream(void) { return (void *)g_stream; }
const char *nrgpu_last_error(void) { return g_err; }
long long nrgpu_kernel_launch_count(void) { return g_launches.load(); }

int nrgpu_fd_coeffs(int order, int kind, double *out) {
  NRGPU_REQUIRE(out != nullptr, "out is NULL");
  NRGPU_REQUIRE(kind >= 0 && kind <= 3, "kind must be 0, 1, 2 or 3");
  auto fill = [&](auto C) {
    using CC = decltype(C);
    const int R = CC::R;
    if (kind == 3) {
      for (int j = 0; j <= 2 * R + 2; j++) out[j] = CC::ko(j >= R + 1 ? j - R - 1 : R + 1 - j);
      return;
    }
    for (int j = 0; j <= 2 * R; j++) {
      const int k = j - R;
      if (kind == 0) out[j] = (k == 0) ? 0.0 : (k > 0 ? CC::c1(k) : -CC::c1(-k));
      if (kind == 1) out[j] = CC::c2(k >= 0 ? k : -k);
      if (kind == 2) out[j] = CC::up(j);
    }
  };
  switch (order) {
    case 2: fill(FDCoef<2>{}); break;
    case 4: fill(FDCoef<4>{}); break;
    case 6: fill(FDCoef<6>{}); break;
    case 8: fill(FDCoef<8>{}); break;
    default: set_error("order %d unsupported", order); return NRGPU_ERR_ARG;
  }
  return NRGPU_OK;
}

int set_Nxx_dxx_invdx_params__and__xx(int EigenCoord, const int Nxx[3], paramstruct *p,
                                      double *xx[3]) {
  NRGPU_REQUIRE(p != nullptr && Nxx != nullptr, "NULL argument");
  NRGPU_REQUIRE(p->NGHOSTS >= 1 && p->NGHOSTS <= NRGPU_MAX_GHOSTS, "NGHOSTS %d out of range", p->NGHOSTS);
  p->Nxx0 = Nxx[0];
  p->Nxx1 = Nxx[1];
  p->Nxx2 = Nxx[2];
  p->Nxx_plus_2NGHOSTS0 = Nxx[0] + 2 * p->NGHOSTS;
  p->Nxx_plus_2NGHOSTS1 = Nxx[1] + 2 * p->NGHOSTS;
  p->Nxx_plus_2NGHOSTS2 = Nxx[2] + 2 * p->NGHOSTS;
  double xmin[3], xmax[3];
  int cs = p->CoordSystem;
  // EigenCoord of the Spherical family is Spherical, of the Cylindrical
  // family Cylindrical (reference_metric.py:946-952).
  if (EigenCoord && spherical_family(cs)) cs = NRGPU_COORD_SPHERICAL;
  if (EigenCoord && cylindrical_family(cs)) cs = NRGPU_COORD_CYLINDRICAL;
  if (EigenCoord && symtp_family(cs)) cs = NRGPU_COORD_SYMTP;
  if (cs == NRGPU_COORD_CARTESIAN) {
    xmin[0] = p->xmin; xmax[0] = p->xmax;
    xmin[1] = p->ymin; xmax[1] = p->ymax;
    xmin[2] = p->zmin; xmax[2] = p->zmax;
  } else if (symtp_family(cs)) {  // reference_metric.py:317-322
    xmin[0] = 0.0;   xmax[0] = cs == NRGPU_COORD_SYMTP ? p->AMAX : 1.0;
    xmin[1] = 0.0;   xmax[1] = M_PI;
    xmin[2] = -M_PI; xmax[2] = M_PI;
  } else if (cylindrical_family(cs)) {
    // Cylindrical :233-234; SinhCylindrical :246-247
    const bool plain = cs == NRGPU_COORD_CYLINDRICAL;
    xmin[0] = 0.0;                     xmax[0] = plain ? p->RHOMAX : 1.0;
    xmin[1] = -M_PI;                   xmax[1] = M_PI;
    xmin[2] = plain ? p->ZMIN : -1.0;  xmax[2] = plain ? p->ZMAX : 1.0;
  } else {
    xmin[0] = 0.0;
    xmax[0] = (cs == NRGPU_COORD_SPHERICAL) ? p->RMAX : 1.0;
    xmin[1] = 0.0; xmax[1] = M_PI;
    xmin[2] = -M_PI; xmax[2] = M_PI;
  }
  p->xxmin0 = xmin[0]; p->xxmin1 = xmin[1]; p->xxmin2 = xmin[2];
  p->xxmax0 = xmax[0]; p->xxmax1 = xmax[1]; p->xxmax2 = xmax[2];
  p->dxx0 = (xmax[0] - xmin[0]) / ((double)Nxx[0]);
  p->dxx1 = (xmax[1] - xmin[1]) / ((double)Nxx[1]);
  p->dxx2 = (xmax[2] - xmin[2]) / ((double)Nxx[2]);
  p->invdx0 = 1.0 / p->dxx0;
  p->invdx1 = 1.0 / p->dxx1;
  p->invdx2 = 1.0 / p->dxx2;
  const double dxx[3] = {p->dxx0, p->dxx1, p->dxx2};
  const int np[3] = {p->Nxx_plus_2NGHOSTS0, p->Nxx_plus_2NGHOSTS1, p->Nxx_plus_2NGHOSTS2};
  if (xx)
    for (int d = 0; d < 3; d++)
      if (xx[d])
        for (int j = 0; j < np[d]; j++) xx[d][j] = xx_of(xmin[d], dxx[d], j, p->NGHOSTS);
  return NRGPU_OK;
}

int xx_to_Cart(const paramstruct *p, double *xx[3], int i0, int i1, int i2, double xCart[3]) {
  NRGPU_REQUIRE(p && xCart, "NULL argument");
  NRGPU_REQUIRE(i0 >= 0 && i0 < p->Nxx_plus_2NGHOSTS0 && i1 >= 0 && i1 < p->Nxx_plus_2NGHOSTS1 && i2 >= 0 &&
                    i2 < p->Nxx_plus_2NGHOSTS2,
                "point (%d, %d, %d) outside the grid", i0, i1, i2);
  const double x0 = (xx && xx[0]) ? xx[0][i0] : xx_of(p->xxmin0, p->dxx0, i0, p->NGHOSTS);
  const double x1 = (xx && xx[1]) ? xx[1][i1] : xx_of(p->xxmin1, p->dxx1, i1, p->NGHOSTS);
  const double x2 = (xx && xx[2]) ? xx[2][i2] : xx_of(p->xxmin2, p->dxx2, i2, p->NGHOSTS);
  double J[3][3];
  cart_jacobian(coord_params(*p), x0, x1, x2, xCart, J);
  return NRGPU_OK;
}

double find_timestep(const paramstruct *p, double CFL_FACTOR) {
  if (check_params(p) != NRGPU_OK) return -1.0;
  // min over interior points of dxx_i s_i; the scale factors depend on
  // (xx0, xx1) (Spherical family) or (xx0, xx2) (Cylindrical family) only
  const bool cyl = cylindrical_family(p->CoordSystem);
  const int ng = p->NGHOSTS, nB = cyl ? p->Nxx_plus_2NGHOSTS2 : p->Nxx_plus_2NGHOSTS1;
  double dsmin = 1e38;
  for (int iB = ng; iB < nB - ng; iB++)
    for (int i0 = ng; i0 < p->Nxx_plus_2NGHOSTS0 - ng; i0++) {
      const double xx0 = xx_of(p->xxmin0, p->dxx0, i0, ng);
      const double xxB = cyl ? xx_of(p->xxmin2, p->dxx2, iB, ng) : xx_of(p->xxmin1, p->dxx1, iB, ng);
      ScaleFactors S;
      scale_factors(coord_params(*p), xx0, xxB, xxB, &S);
      const double ds0 = p->dxx0 * S.s[0], ds1 = p->dxx1 * S.s[1], ds2 = p->dxx2 * S.s[2];
      dsmin = fmin(dsmin, fmin(ds0, fmin(ds1, ds2)));
    }
  return dsmin * CFL_FACTOR / p->wavespeed;
}

int rfm_struct__malloc(const paramstruct *p, rfm_struct *rfm) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(rfm != nullptr, "rfm is NULL");
  memset(rfm, 0, sizeof(*rfm));
  rfm->CoordSystem = p->CoordSystem;
  rfm->N0 = p->Nxx_plus_2NGHOSTS0;
  rfm->N1 = rfm_second_extent(p);
  rfm->nquant = rq::NQ;
  const size_t n = (size_t)rq::NQ * rfm->N0 * rfm->N1;
  NRGPU_CUDA_CHECK(cudaMalloc(&rfm->table64, n * sizeof(double)));
  NRGPU_CUDA_CHECK(cudaMalloc(&rfm->table32, n * sizeof(float)));
  return NRGPU_OK;
}

int rfm_struct__define(const paramstruct *p, rfm_struct *rfm) {
  int st = check_params(p);
  if (st) return st;
  NRGPU_REQUIRE(rfm && rfm->table64 && rfm->table32, "rfm tables not allocated");
  NRGPU_REQUIRE(rfm_matches(rfm, p), "rfm tables sized for another grid");
  dim3 block(64), grid((rfm->N0 + 63) / 64, rfm->N1);
  rfm_define_kernel<<<grid, block, 0, stream()>>>(*p, rfm->table64, rfm->table32);
  NRGPU_LAUNCH_CHECK();
  return NRGPU_OK;
}

int rfm_struct__freemem(rfm_struct *rfm) {
  if (!rfm) return NRGPU_OK;
  if (rfm->table64) cudaFree(rfm->table64);
  if (rfm->table32) cudaFree(rfm->table32);
  rfm->table64 = nullptr;
  rfm->table32 = nullptr;
  return NRGPU_OK;
}

int rfm_struct__download(const rfm_struct *rfm, double *host) {
  NRGPU_REQUIRE(rfm && rfm->table64 && host, "NULL argument");
  const size_t n = (size_t)rfm->nquant * rfm->N0 * rfm->N1;
  NRGPU_CUDA_CHECK(cudaMemcpyAsync(host, rfm->table64, n * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  NRGPU_CUDA_CHECK(cudaStreamSynchronize(stream()));
  return NRGPU_OK;
}

}  // extern "C"
