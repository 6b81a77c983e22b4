// kernels_force_smooth.cu — pair-force kernels for smooth_r4 truncation.
#include "force.cuh"

namespace hmd {

template void launch_force_kind<FK_SMOOTH>(const Dev& d, bool aux, cudaStream_t st);

} // namespace hmd
