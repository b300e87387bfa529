// Dense passes over FP32 M in launch configuration 0 (dense_pass.cuh).
#include "dense_pass.cuh"

namespace regot {
template void launch_pass_cfg<float, 0>(int, const PassParams&, cudaStream_t, int);
template int occupancy_cfg<float, 0>(int);
}  // namespace regot
