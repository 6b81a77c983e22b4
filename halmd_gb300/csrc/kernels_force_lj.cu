// kernels_force_lj.cu — pair-force kernels for one species, sharp or shifted truncation.
#include "force.cuh"

namespace hmd {

template void launch_force_kind<FK_LJ1>(const Dev& d, bool aux, cudaStream_t st);

} // namespace hmd
