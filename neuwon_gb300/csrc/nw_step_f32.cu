// FP32 instances of the batched step kernel (one translation unit per
// precision, so the two compile in parallel).
#include "nw_step_batched.cuh"

namespace nw {
template int config_batched<float>(nw_ctx*, BatchedCfg<float>&);
}  // namespace nw
