// Step kernels instantiated for 3D grids (Grid3D / Solid3D).
#include "mpm_launch.cuh"

namespace jmpm {
template struct Launchers<3>;
}  // namespace jmpm
