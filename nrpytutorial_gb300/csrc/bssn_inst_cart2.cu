// bssn_inst_cart2.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_CARTESIAN, FD order 2.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_CARTESIAN, 2)
}  // namespace bssn
}  // namespace nrgpu
