// common.cuh -- shared device/host plumbing for libnrgpu: status handling,
// the library stream, launch accounting, grid indexing.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include "../../include/nrgpu.h"

namespace nrgpu {

// ---------------------------------------------------------------- status
void set_error(const char *fmt, ...);
cudaStream_t stream();
void count_launch(int n = 1);
// Device address of the library's status word on the current device (set by
// a kernel whose bounded wait gave up), or NULL.
int *device_status_word();

#define NRGPU_CUDA_CHECK(call)                                                   \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      ::nrgpu::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,              \
                         cudaGetErrorString(e_));                                \
      return NRGPU_ERR_CUDA;                                                     \
    }                                                                            \
  } while (0)

// Check a launch that was just issued (configuration errors only; no sync).
#define NRGPU_LAUNCH_CHECK()                                                     \
  do {                                                                           \
    cudaError_t e_ = cudaGetLastError();                                         \
    if (e_ != cudaSuccess) {                                                     \
      ::nrgpu::set_error("%s:%d launch: %s", __FILE__, __LINE__,                 \
                         cudaGetErrorString(e_));                                \
      return NRGPU_ERR_CUDA;                                                     \
    }                                                                            \
    ::nrgpu::count_launch();                                                     \
  } while (0)

#define NRGPU_REQUIRE(cond, ...)                                                 \
  do {                                                                           \
    if (!(cond)) {                                                               \
      ::nrgpu::set_error(__VA_ARGS__);                                           \
      return NRGPU_ERR_ARG;                                                      \
    }                                                                            \
  } while (0)

// Stage buffers of FP32 (hi, lo) pairs: both compensated precisions.
__host__ __device__ inline bool pair_precision(int prec) {
  return prec == NRGPU_PREC_COMPENSATED || prec == NRGPU_PREC_COMPENSATED_FP64RK;
}

// Validates the parts of a paramstruct every kernel depends on.
int check_params(const paramstruct *p);

// ---------------------------------------------------------------- grid view
// Extents and strides of one IDX4S-laid-out grid, passed by value to kernels.
struct Grid {
  int n0, n1, n2;      // Nxx_plus_2NGHOSTS0..2
  int ng;              // NGHOSTS
  long long ntot;      // n0*n1*n2 (gridfunction stride)
  double invdx0, invdx1, invdx2;
};

// The kernel instantiation a coordinate system runs on.  Kernels specialise
// on the structure of the reference metric (which scale factor depends on
// which coordinate, RfmMask) and read its values from the rfm tables;
// SinhSphericalv2 has SinhSpherical's structure and differs only in r(xx0),
// Cylindrical has SinhCylindrical's with the identity maps, SymTP
// SinhSymTP's; the tables and the runtime CoordSystem carry the values.
inline int dispatch_cs(int cs) {
  return cs == NRGPU_COORD_SINHSPHERICALV2 ? NRGPU_COORD_SINHSPHERICAL
         : (cs == NRGPU_COORD_CYLINDRICAL || cs == NRGPU_COORD_SINHCYLINDRICALV2) ? NRGPU_COORD_SINHCYLINDRICAL
         : cs == NRGPU_COORD_SYMTP ? NRGPU_COORD_SINHSYMTP
                                   : cs;
}

inline Grid make_grid(const paramstruct *p) {
  Grid g;
  g.n0 = p->Nxx_plus_2NGHOSTS0;
  g.n1 = p->Nxx_plus_2NGHOSTS1;
  g.n2 = p->Nxx_plus_2NGHOSTS2;
  g.ng = p->NGHOSTS;
  g.ntot = (long long)g.n0 * g.n1 * g.n2;
  g.invdx0 = p->invdx0;
  g.invdx1 = p->invdx1;
  g.invdx2 = p->invdx2;
  return g;
}

// Standard launch shape for interior-point kernels: x covers i0 (coalesced
// along the fastest axis), y covers i1, z covers i2.
struct InteriorLaunch {
  dim3 grid, block;
};
inline InteriorLaunch interior_launch(const Grid &g, int bx, int by) {
  InteriorLaunch L;
  const int nx = g.n0 - 2 * g.ng, ny = g.n1 - 2 * g.ng, nz = g.n2 - 2 * g.ng;
  L.block = dim3(bx, by, 1);
  L.grid = dim3((nx + bx - 1) / bx, (ny + by - 1) / by, nz);
  return L;
}

template <typename T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

}  // namespace nrgpu
