// Level kernels of the lane engine for 128-thread CTAs (one of the three CTA
// shapes the autotuner chooses from).
#include "lane_kernels.cuh"

namespace gbc {

void level_kernels_128(LevelKernels& k) { fill_level_kernels<128>(k); }

}  // namespace gbc
