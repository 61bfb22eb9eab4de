// Fused kernel instantiations for A = 4 surfaces.
#include "pbr_fused_launch.cuh"

namespace pbr {
template int launch_fused<4>(int, int, int, const FusedArgs&, cudaStream_t);
}  // namespace pbr
