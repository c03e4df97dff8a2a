// Level kernels of the lane engine for 256-thread CTAs (one of the three CTA
// shapes the autotuner chooses from).
#include "lane_kernels.cuh"

namespace gbc {

void level_kernels_256(LevelKernels& k) { fill_level_kernels<256>(k); }

}  // namespace gbc
