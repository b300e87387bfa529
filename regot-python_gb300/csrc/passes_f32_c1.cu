// Dense passes over FP32 M in launch configuration 1 (dense_pass.cuh).
#include "dense_pass.cuh"

namespace regot {
template void launch_pass_cfg<float, 1>(int, const PassParams&, cudaStream_t, int);
template int occupancy_cfg<float, 1>(int);
}  // namespace regot
