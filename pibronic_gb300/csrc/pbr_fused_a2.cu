// Fused kernel instantiations for A = 2 surfaces.
#include "pbr_fused_launch.cuh"

namespace pbr {
template int launch_fused<2>(int, int, int, const FusedArgs&, cudaStream_t);
}  // namespace pbr
