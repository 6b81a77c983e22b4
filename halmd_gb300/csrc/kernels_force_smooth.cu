// kernels_force_smooth.cu — pair-force kernels for smooth_r4 truncation.
//
// This kind aims for 6 resident blocks of 128 threads per SM (80 registers)
// instead of 7: its smoothing factors need more registers, and at KA-64k
// (four lanes per particle, two entries per load) it measured 34.5 us
// against 35.2 us per launch with 7 (two runs each).
#ifndef HMD_FORCE_MINB
#define HMD_FORCE_MINB 6
#endif
#include "force.cuh"

namespace hmd {

template void launch_force_kind<FK_SMOOTH>(const Dev& d, bool aux, cudaStream_t st);

} // namespace hmd
