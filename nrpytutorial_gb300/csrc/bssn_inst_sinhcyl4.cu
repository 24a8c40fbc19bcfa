// bssn_inst_sinhcyl4.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_SINHCYLINDRICAL (and Cylindrical), FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_SINHCYLINDRICAL, 4)
}  // namespace bssn
}  // namespace nrgpu
