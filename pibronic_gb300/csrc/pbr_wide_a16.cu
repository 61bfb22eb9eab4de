// pbr_wide_a16.cu -- instantiation of the wide block evaluation for surfaces padded to 16.
#include "pbr_wide.cuh"

namespace pbr {
template int launch_wide<16>(int, const WideArgs&, cudaStream_t);
template int wide_resident<16>(int, const WideArgs&);
}
