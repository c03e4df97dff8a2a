// Level kernels of the lane engine for 512-thread CTAs (one of the three CTA
// shapes the autotuner chooses from).
#include "lane_kernels.cuh"

namespace gbc {

void level_kernels_512(LevelKernels& k) { fill_level_kernels<512>(k); }

}  // namespace gbc
