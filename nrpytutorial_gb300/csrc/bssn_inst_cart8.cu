// bssn_inst_cart8.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_CARTESIAN, FD order 8.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_CARTESIAN, 8)
}  // namespace bssn
}  // namespace nrgpu
