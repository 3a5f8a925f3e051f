// Step kernels instantiated for 2D grids (Grid2D / Solid2D).
#include "mpm_launch.cuh"

namespace jmpm {
template struct Launchers<2>;
}  // namespace jmpm
