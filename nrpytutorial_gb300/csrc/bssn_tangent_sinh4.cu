// Tangent-linear BSSN RHS kernels (bssn_tangent.cuh), SinhSpherical family grids at FD
// order 4, with 0 (plain FP64), 1, 2 and 4 tangents.
#include "bssn_tangent.cuh"
namespace nrgpu {
namespace bssn {
namespace tangent {
NRGPU_TANGENT_INSTANTIATE(NRGPU_COORD_SINHSPHERICAL, 4, 0)
NRGPU_TANGENT_INSTANTIATE(NRGPU_COORD_SINHSPHERICAL, 4, 1)
NRGPU_TANGENT_INSTANTIATE(NRGPU_COORD_SINHSPHERICAL, 4, 2)
NRGPU_TANGENT_INSTANTIATE(NRGPU_COORD_SINHSPHERICAL, 4, 4)
}  // namespace tangent
}  // namespace bssn
}  // namespace nrgpu
