// Row-team kernel instantiations for A = 8 surfaces.
#include "pbr_team_launch.cuh"

namespace pbr {
template int launch_team<8>(int, int, int, const TeamArgs&, cudaStream_t);
template int launch_team_batch<8>(int, const TeamBatchItem*, int, int64_t, int, int, int, cudaStream_t);
}  // namespace pbr
