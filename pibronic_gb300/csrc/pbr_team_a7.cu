// Row-team kernel instantiations for A = 7 surfaces.
#include "pbr_team_launch.cuh"

namespace pbr {
template int launch_team<7>(int, int, int, const TeamArgs&, cudaStream_t);
template int launch_team_batch<7>(int, const TeamBatchItem*, int, int64_t, int, int, int, cudaStream_t);
}  // namespace pbr
