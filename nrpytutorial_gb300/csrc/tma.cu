// tma.cu -- host side of the TMA plumbing: the tiled tensor map of an IDX4S
// gridfunction array, and the device status word that the staged kernels set
// when a bounded wait gives up.
#include <mutex>

#include "common.cuh"
#include "tma.cuh"

namespace nrgpu {

// cuTensorMapEncodeTiled is a driver entry point; the runtime hands it out
// without linking libcuda directly.
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    else
      cudaGetLastError();
  });
  return fn;
}

bool tma_map_gridfunctions(CUtensorMap *map, const void *base, int esize, int n0, int n1, int n2, int ngf, int bx,
                           int by, int bz) {
  if (!map || !base || (esize != 4 && esize != 8)) return false;
  if (((uintptr_t)base & 15) != 0) return false;
  const unsigned long long row = (unsigned long long)n0 * esize;
  const unsigned long long plane = row * n1, vol = plane * n2;
  if (row % 16 || plane % 16 || vol % 16) return false;
  if ((unsigned long long)bx * esize % 16) return false;
  if (bx < 1 || by < 1 || bz < 1 || bx > 256 || by > 256 || bz > 256) return false;
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)n0, (cuuint64_t)n1, (cuuint64_t)n2, (cuuint64_t)ngf};
  const cuuint64_t strides[3] = {row, plane, vol};
  const cuuint32_t box[4] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUtensorMap m;
  const CUresult r =
      fn(&m, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
         const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  *map = m;
  return true;
}

// ------------------------------------------------------ device status word
// Set (never cleared by a kernel) when a staged kernel's bounded wait for a
// TMA copy gives up; the host reads and clears it with nrgpu_device_status.
static __device__ int g_device_status;
static int *g_status_ptr[64];
static std::mutex g_status_mu;

int *device_status_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_status_mu);
  if (!g_status_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_status) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    g_status_ptr[dev] = (int *)p;
  }
  return g_status_ptr[dev];
}

}  // namespace nrgpu

using namespace nrgpu;

extern "C" int nrgpu_device_status(int clear) {
  int *p = device_status_word();
  if (!p) {
    set_error("device status word unavailable");
    return -NRGPU_ERR_CUDA;
  }
  int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, p, sizeof(int), cudaMemcpyDeviceToHost, stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
  if (e == cudaSuccess && clear && v) {
    const int zero = 0;
    e = cudaMemcpyAsync(p, &zero, sizeof(int), cudaMemcpyHostToDevice, stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream());
  }
  if (e != cudaSuccess) {
    set_error("nrgpu_device_status: %s", cudaGetErrorString(e));
    return -NRGPU_ERR_CUDA;
  }
  return v;
}
