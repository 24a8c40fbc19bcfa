// bssn_inst_sph4.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_SPHERICAL, FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_SPHERICAL, 4)
}  // namespace bssn
}  // namespace nrgpu
