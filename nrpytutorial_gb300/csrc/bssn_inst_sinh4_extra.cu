// bssn_inst_sinh4_extra.cu -- BSSN RHS kernels with Kreiss-Oliger dissipation and T^{mu nu} source terms for CoordSystem NRGPU_COORD_SINHSPHERICAL, FD order 4.
#include "bssn_kernels.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_INSTANTIATE_EXTRA(NRGPU_COORD_SINHSPHERICAL, 4)
}  // namespace bssn
}  // namespace nrgpu
