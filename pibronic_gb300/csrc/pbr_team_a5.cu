// Row-team kernel instantiations for A = 5 surfaces.
#include "pbr_team_launch.cuh"

namespace pbr {
template int launch_team<5>(int, int, int, const TeamArgs&, cudaStream_t);
template int launch_team_batch<5>(int, const TeamBatchItem*, int, int64_t, int, int, int, cudaStream_t);
}  // namespace pbr
