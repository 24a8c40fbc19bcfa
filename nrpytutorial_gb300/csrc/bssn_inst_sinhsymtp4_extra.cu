// bssn_inst_sinhsymtp4_extra.cu -- BSSN RHS kernels with Kreiss-Oliger dissipation and T^{mu nu} source terms for CoordSystem NRGPU_COORD_SINHSYMTP (and SymTP), FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE_EXTRA(NRGPU_COORD_SINHSYMTP, 4)
}  // namespace bssn
}  // namespace nrgpu
