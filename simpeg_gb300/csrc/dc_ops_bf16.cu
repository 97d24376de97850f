// Instantiation of the node kernels for the fp32 inner solve with bf16
// multigrid vectors (fp32 range, 8-bit mantissa; conversions are bit shifts).
#include <cuda_bf16.h>

#include "dc_kernels.cuh"

namespace dc {

DC_OPS_INSTANTIATE(float, __nv_bfloat16)

}  // namespace dc
