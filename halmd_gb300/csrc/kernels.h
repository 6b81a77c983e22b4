// kernels.h — host-side launchers of the MD kernels (one engine = struct Dev).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hmd {

struct Dev;

// kinds of pair interaction, one pair-force kernel each (force.cuh):
// FK_LJ1 one species with a sharp or shifted truncation, FK_SHIFTED several
// species with a sharp or shifted truncation, FK_SMOOTH smooth_r4, FK_FSHIFT
// force_shifted, FK_POT the other pair potentials (mie, morse, power_law) with
// any truncation; FK_GENERIC handles every list kind in one kernel; FK_FULL
// untruncated potentials over all pairs (no list, launch_force_full)
enum ForceKind : int { FK_GENERIC = 0, FK_LJ1 = 1, FK_SHIFTED = 2, FK_SMOOTH = 3, FK_FSHIFT = 4, FK_POT = 5, FK_FULL = 6 };
template <int KIND> void launch_force_kind(const Dev& d, bool aux, cudaStream_t st);
void launch_force_full(const Dev& d, bool aux, cudaStream_t st);

// step (kernels_step.cu)
void launch_integrate(const Dev& d, bool ds, cudaGraphConditionalHandle h, bool use_handle, cudaStream_t st);
void launch_mark(const Dev& d, bool rebuild_all, cudaStream_t st);
// the force kernels of the kinds in Dev::force_kinds (all kinds in one when 0)
void launch_force(const Dev& d, bool aux, cudaStream_t st);
void launch_finalize(const Dev& d, bool ds, cudaStream_t st);
// finalize of step k fused with the integrate of step k + 1 (captured chunks)
void launch_finalize_integrate(const Dev& d, bool ds, cudaGraphConditionalHandle h, cudaStream_t st);
void launch_thermo(const Dev& d, cudaStream_t st);
// the FP64 variant of the step (kernels_fp64.cu)
void launch_force64(const Dev& d, bool aux, cudaStream_t st);
void launch_integrate64(const Dev& d, bool fin, cudaGraphConditionalHandle h, bool use_handle, cudaStream_t st);
void launch_finalize64(const Dev& d, cudaStream_t st);
// the force kernel's gather records of every real slot (dsfloat engines)
void launch_pack_fpos(const Dev& d, cudaStream_t st);
// largest |min_image(r - r0)|^2 of system s as float bits into *out
void launch_max_displacement(const Dev& d, uint32_t s, uint32_t slots, uint32_t* out, cudaStream_t st);
// engines with a Nose-Hoover system: the chain's half step before integrate
void launch_integrate_prepare(const Dev& d, cudaStream_t st);
// kernels of one captured step that is not fused and rebuilds nothing
int step_kernel_count(const Dev& d);

// rebuild (kernels_rebuild.cu)
int radix_passes(uint32_t key_bits);
constexpr uint32_t SORT_TILE = 2048;   // keys per tile of the segmented radix sort
void launch_rebuild_list(const Dev& d, cudaStream_t st);
void launch_sort(const Dev& d, int passes, cudaStream_t st);
int sort_kernel_count(int passes);
void launch_rearrange(const Dev& d, bool ds, const uint32_t* perm, cudaStream_t st);
void launch_binning(const Dev& d, cudaStream_t st);
void launch_neighbour(const Dev& d, cudaStream_t st);
void launch_hilbert_keys(const Dev& d, uint32_t* keys, cudaStream_t st);

// observables (kernels_obs.cu)
void launch_sample_position(const Dev& d, uint32_t first, uint32_t count, double* out, cudaStream_t st);
void launch_msd(const double* r1, const double* r2, const uint32_t* range, uint32_t nrange, const uint32_t* blk_range,
                const uint32_t* blk_begin, uint32_t nblk, double* partial, double* out, cudaStream_t st);
// kind 0 MSD, 2 MQD, 3 VACF (r1, r2: velocity samples) over particle ranges
void launch_tcf(int kind, const double* r1, const double* r2, const uint32_t* range, uint32_t nrange,
                const uint32_t* blk_range, const uint32_t* blk_begin, uint32_t nblk, double* partial, double* out,
                cudaStream_t st);
void launch_sample_velocity(const Dev& d, uint32_t first, uint32_t count, double* out, cudaStream_t st);
void launch_density_modes(const Dev& d, const uint32_t* range, uint32_t nrange, const uint32_t* blk_range,
                          const uint32_t* blk_begin, uint32_t nblk, const float4* q, uint32_t nq, double* partial,
                          double* out, cudaStream_t st);

// phase-space transfer in tag order (kernels_io.cu): set what = 0 position,
// 1 velocity; get what = 0 position, 1 unwrapped position, 2 velocity,
// 3 force, 4 image (arrays of 3 n doubles on the device)
void launch_set_vector(const Dev& d, uint32_t s, uint32_t n, int what, bool ds, const double* in, cudaStream_t st);
void launch_get_vector(const Dev& d, uint32_t s, uint32_t n, int what, double* out, cudaStream_t st);
// *flag = 1 if any of in[0, n) is not finite (a staged set array)
void launch_check_finite(const double* in, size_t n, uint32_t* flag, cudaStream_t st);
// set-up (kernels_io.cu): fcc lattice positions and Maxwell-Boltzmann
// velocities of tags < n into out[3 n] on the device
void launch_lattice(double* out, uint32_t n, const uint32_t cells[3], double a, const double offset[3], uint32_t skip,
                    cudaStream_t st);
void launch_boltzmann(const Dev& d, uint32_t s, uint32_t n, double T, uint64_t seed, double* out, double* scratch,
                      cudaStream_t st);

// MSD of one sample pair with fixed scratch and no allocation (msd_noalloc.cu)
void msd_pair_noalloc(const double* origin, const double* position, uint32_t count, double* out, cudaStream_t st);

} // namespace hmd
