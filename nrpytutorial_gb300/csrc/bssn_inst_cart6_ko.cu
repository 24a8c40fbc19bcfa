// bssn_inst_cart6_ko.cu -- BSSN RHS kernels with Kreiss-Oliger dissipation for CoordSystem NRGPU_COORD_CARTESIAN, FD order 6.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE_KO(NRGPU_COORD_CARTESIAN, 6)
}  // namespace bssn
}  // namespace nrgpu
