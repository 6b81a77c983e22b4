// kernels_force_other.cu — pair-force kernels for systems of several species
// with a sharp or shifted truncation, and for the force_shifted truncation.
#include "force.cuh"

namespace hmd {

template void launch_force_kind<FK_SHIFTED>(const Dev& d, bool aux, cudaStream_t st);
template void launch_force_kind<FK_FSHIFT>(const Dev& d, bool aux, cudaStream_t st);

} // namespace hmd
