// Row-team kernel instantiations for A = 5 surfaces.
#include "pbr_team_launch.cuh"

namespace pbr {
template int launch_team<5>(int, int, int, const TeamArgs&, cudaStream_t);
}  // namespace pbr
