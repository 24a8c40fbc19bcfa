// bssn_inst_sinhsymtp4.cu -- BSSN Ricci/RHS kernels for CoordSystem NRGPU_COORD_SINHSYMTP (and SymTP), FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE(NRGPU_COORD_SINHSYMTP, 4)
}  // namespace bssn
}  // namespace nrgpu
