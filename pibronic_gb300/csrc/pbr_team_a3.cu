// Row-team kernel instantiations for A = 3 surfaces.
#include "pbr_team_launch.cuh"

namespace pbr {
template int launch_team<3>(int, int, int, const TeamArgs&, cudaStream_t);
}  // namespace pbr
