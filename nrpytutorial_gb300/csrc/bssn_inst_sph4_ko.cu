// bssn_inst_sph4_ko.cu -- BSSN RHS kernels with Kreiss-Oliger dissipation for CoordSystem NRGPU_COORD_SPHERICAL, FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE_KO(NRGPU_COORD_SPHERICAL, 4)
}  // namespace bssn
}  // namespace nrgpu
