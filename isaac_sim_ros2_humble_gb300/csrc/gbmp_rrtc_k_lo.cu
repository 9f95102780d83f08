// gbmp_rrtc_k_lo.cu -- single-problem planning kernels for 1 to 4 spheres per lane (one of the
// four translation units that instantiate the planner's kernels, so that they compile in
// parallel).
#include "gbmp_rrtc_device.cuh"

namespace gbmp {
GBMP_RRTC_DEFINE_LAUNCHER(rrtc_launch_lo, 1)
}  // namespace gbmp
