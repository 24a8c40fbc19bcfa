// Staged BSSN kernels (bssn_staged.cuh), SymTP-family grids at FD order 4.
#include "bssn_staged.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_STAGED_INSTANTIATE(NRGPU_COORD_SINHSYMTP, 4)
}  // namespace bssn
}  // namespace nrgpu
