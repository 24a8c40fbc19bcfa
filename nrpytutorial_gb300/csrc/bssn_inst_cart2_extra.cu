// bssn_inst_cart2_extra.cu -- BSSN RHS kernels with Kreiss-Oliger dissipation and T^{mu nu} source terms for CoordSystem NRGPU_COORD_CARTESIAN, FD order 2.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE_EXTRA(NRGPU_COORD_CARTESIAN, 2)
}  // namespace bssn
}  // namespace nrgpu
