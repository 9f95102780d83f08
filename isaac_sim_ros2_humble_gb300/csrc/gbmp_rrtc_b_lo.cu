// gbmp_rrtc_b_lo.cu -- batched planning kernels for 1 to 4 spheres per lane (one of the
// four translation units that instantiate the planner's kernels, so that they compile in
// parallel).
#include "gbmp_rrtc_device.cuh"

namespace gbmp {
GBMP_RRTC_DEFINE_BATCH_LAUNCHER(rrtc_batch_launch_lo, 1)
}  // namespace gbmp
