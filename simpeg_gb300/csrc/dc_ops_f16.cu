// Instantiation of the node kernels for the fp32 inner solve with fp16 multigrid vectors (half the V-cycle's bytes).
#include "dc_kernels.cuh"

namespace dc {

DC_OPS_INSTANTIATE(float, __half)

}  // namespace dc
