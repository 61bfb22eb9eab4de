// pbr_wide_a12.cu -- instantiation of the wide block evaluation for surfaces padded to 12.
#include "pbr_wide.cuh"

namespace pbr {
template int launch_wide<12>(int, const WideArgs&, cudaStream_t);
template int wide_resident<12>(int, const WideArgs&);
}
