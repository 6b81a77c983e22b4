// kernels_force_mixed.cu — the pair-force kernel that handles every kind of
// pair interaction, for engines whose systems change after commit (capacity
// mode), where the kinds present are not known when the step is captured.
#include "force.cuh"

namespace hmd {

template void launch_force_kind<FK_GENERIC>(const Dev& d, bool aux, cudaStream_t st);

} // namespace hmd
