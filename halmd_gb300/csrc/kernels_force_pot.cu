// kernels_force_pot.cu — pair-force kernels for the mie, morse and power_law
// potentials with any truncation.
#include "force.cuh"

namespace hmd {

template void launch_force_kind<FK_POT>(const Dev& d, bool aux, cudaStream_t st);

} // namespace hmd
