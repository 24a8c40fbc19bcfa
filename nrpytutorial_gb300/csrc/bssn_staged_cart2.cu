// Staged BSSN kernels (bssn_staged.cuh), Cartesian grids at FD order 2.
#include "bssn_staged.cuh"
namespace nrgpu {
namespace bssn {
NRGPU_BSSN_STAGED_INSTANTIATE(NRGPU_COORD_CARTESIAN, 2)
}  // namespace bssn
}  // namespace nrgpu
