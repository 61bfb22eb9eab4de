// Fused kernel instantiations for A = 3 surfaces.
#include "pbr_fused_launch.cuh"

namespace pbr {
template int launch_fused<3>(int, int, int, const FusedArgs&, cudaStream_t);
}  // namespace pbr
