// bssn_inst_cart8_extra.cu -- BSSN RHS kernels with Kreiss-Oliger dissipation and T^{mu nu} source terms for CoordSystem NRGPU_COORD_CARTESIAN, FD order 8.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE_EXTRA(NRGPU_COORD_CARTESIAN, 8)
}  // namespace bssn
}  // namespace nrgpu
