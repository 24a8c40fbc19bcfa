// bssn_inst_sinh4.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_SINHSPHERICAL, FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_SINHSPHERICAL, 4)
}  // namespace bssn
}  // namespace nrgpu
