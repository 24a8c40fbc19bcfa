// bssn_inst_cart6.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_CARTESIAN, FD order 6.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_CARTESIAN, 6)
}  // namespace bssn
}  // namespace nrgpu
