// Instantiation of the node kernels for the fp32 inner solve with fp32 multigrid vectors.
#include "dc_kernels.cuh"

namespace dc {

DC_OPS_INSTANTIATE(float, float)

}  // namespace dc
