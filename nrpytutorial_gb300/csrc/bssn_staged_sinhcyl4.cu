// Staged BSSN kernels (bssn_staged.cuh), Cylindrical-family grids at FD order 4.
#include "bssn_staged.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_STAGED_INSTANTIATE(NRGPU_COORD_SINHCYLINDRICAL, 4)
}  // namespace bssn
}  // namespace nrgpu
