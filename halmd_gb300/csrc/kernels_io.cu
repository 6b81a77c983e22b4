// kernels_io.cu — phase-space transfer between the caller's tag-ordered
// double arrays (one device staging copy) and the Hilbert-ordered float /
// double-single arrays: the conversion of particle.cpp's set/get
// (mdsim/gpu/particle.cpp:221-330, particle_kernel.cu) done on the device,
// so a set or get is one host copy and one kernel instead of a read-back,
// a host loop and a write per array.  Double arithmetic uses the _rn
// intrinsics: no contraction, the same rounding as the host formulas.
#include "hmd_device.cuh"
#include <algorithm>
#include "kernels.h"

namespace hmd {

// position: reduce into the box (image += rint(x / L)), split into hi + lo
template <bool DS>
__global__ void __launch_bounds__(256) k_set_position(Dev d, uint32_t s, const double* in)
{
    const SysParam& P = d.sys[s];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.n) return;
    const uint32_t k = d.rid[P.off + t];
    float4 h = pos_hi(d.pos, k), g = d.img[k];
    float4 l = make_float4(0, 0, 0, 0);
    float* hp = &h.x;
    float* lp = &l.x;
    float* gp = &g.x;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double x = in[3 * (size_t)t + q];
        const double L = (double)P.L[q];
        const double w = rint(__ddiv_rn(x, L));
        const double xr = __dsub_rn(x, __dmul_rn(w, L));
        hp[q] = __double2float_rn(xr);
        lp[q] = DS ? __double2float_rn(__dsub_rn(xr, (double)hp[q])) : 0.0f;
        gp[q] = __double2float_rn(__dadd_rn((double)gp[q], w));
    }
    pos_hi(d.pos, k) = h;               // w (species) unchanged
    if (DS) pos_lo(d.pos, k) = l;
    d.img[k] = g;
}

template <bool DS>
__global__ void __launch_bounds__(256) k_set_velocity(Dev d, uint32_t s, const double* in)
{
    const SysParam& P = d.sys[s];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.n) return;
    const uint32_t k = d.rid[P.off + t];
    float4 h = d.vel[k];
    float4 l = make_float4(0, 0, 0, 0);
    float* hp = &h.x;
    float* lp = &l.x;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double v = in[3 * (size_t)t + q];
        hp[q] = __double2float_rn(v);
        lp[q] = DS ? __double2float_rn(__dsub_rn(v, (double)hp[q])) : 0.0f;
    }
    d.vel[k] = h;                       // w (mass) unchanged
    if (DS) d.vel[d.S + k] = l;
}

// out[3 t + q] for tags t < n: what = 0 position, 1 unwrapped position,
// 2 velocity, 3 force, 4 image
__global__ void __launch_bounds__(256) k_get_vector(Dev d, uint32_t s, int what, double* out)
{
    const SysParam& P = d.sys[s];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.n) return;
    const uint32_t k = d.rid[P.off + t];
    float4 a, b = make_float4(0, 0, 0, 0), g = make_float4(0, 0, 0, 0);
    if (what <= 1) { a = pos_hi(d.pos, k); b = pos_lo(d.pos, k); if (what == 1) g = d.img[k]; }
    else if (what == 2) { a = d.vel[k]; b = d.vel[d.S + k]; }
    else if (what == 3) a = d.force[k];
    else a = d.img[k];
    const float* ap = &a.x;
    const float* bp = &b.x;
    const float* gp = &g.x;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        double v = (double)ap[q];
        if (what <= 2) v = __dadd_rn(v, (double)bp[q]);
        if (what <= 1) v = __dadd_rn(v, what == 1 ? __dmul_rn((double)gp[q], (double)P.L[q]) : 0.0);
        out[3 * (size_t)t + q] = v;
    }
}

// ---------------------------------------------------------------------------
// set-up modules: positions on an fcc lattice (mdsim/host/positions/lattice.cpp:63-175,
// gpu/positions/lattice_kernel.cu) and Maxwell-Boltzmann velocities
// (mdsim/gpu/velocities/boltzmann_kernel.cu:47-140), written in tag order
// into a staging array that the set conversions above then store
// ---------------------------------------------------------------------------

// site of particle tag t: sites with index i = skip - 1 (mod skip) stay empty
// (particle t takes site t + floor(t / (skip - 1))); the four sites of a
// cell (mdsim/positions/lattice_primitive.hpp, close_packed_lattice) in
// cells numbered with x fastest, scaled by a and shifted by offset
__global__ void __launch_bounds__(256) k_lattice(double* out, uint32_t n, uint32_t cx, uint32_t cy, double a,
                                                 double ox, double oy, double oz, uint32_t skip)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint64_t i = skip > 1 ? (uint64_t)t + t / (skip - 1u) : t;
    const uint64_t c = i >> 2;
    const uint32_t b = (uint32_t)(i & 3u);
    const double x = (double)(c % cx) + (double)((((b ^ (b >> 1)) & 1u) * 2u + 1u)) / 4.0;
    const double y = (double)((c / cx) % cy) + (double)(((b & 1u) * 2u + 1u)) / 4.0;
    const double z = (double)(c / ((uint64_t)cx * cy)) + (double)(((b & 2u) + 1u)) / 4.0;
    out[3 * (size_t)t + 0] = __dadd_rn(__dmul_rn(x, a), ox);
    out[3 * (size_t)t + 1] = __dadd_rn(__dmul_rn(y, a), oy);
    out[3 * (size_t)t + 2] = __dadd_rn(__dmul_rn(z, a), oz);
}

// velocity of tag t: each component N(0, sqrt(T)) / sqrt(m), Box-Muller in
// FP64 on Philox4x32-10 words keyed by (seed, tag); per-block sums of m v and
// m into partial[4 b + 0..3]
__global__ void __launch_bounds__(256) k_boltzmann(Dev d, uint32_t s, double T, uint32_t seed_lo, uint32_t seed_hi,
                                                   double* out, double* partial)
{
    const SysParam& P = d.sys[s];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    if (t < P.n) {
        const double m = (double)d.vel[d.rid[P.off + t]].w;
        const uint4 w = philox4x32_10(make_uint4(t, 0u, 0u, 0x424F4C54u), seed_lo, seed_hi);
        const double inv = 1.0 / 4294967296.0;
        const double u0 = ((double)w.x + 0.5) * inv, u1 = ((double)w.y + 0.5) * inv;
        const double u2 = ((double)w.z + 0.5) * inv, u3 = ((double)w.w + 0.5) * inv;
        const double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
        double s0, c0, s1, c1;
        sincospi(2.0 * u1, &s0, &c0);
        sincospi(2.0 * u3, &s1, &c1);
        const double f = sqrt(T / m);
        const double v[3] = {f * r0 * c0, f * r0 * s0, f * r1 * c1};
        for (int q = 0; q < 3; ++q) {
            out[3 * (size_t)t + q] = v[q];
            acc[q] = m * v[q];
        }
        acc[3] = m;
    }
    __shared__ double s_acc[8][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double x = warp_sum(acc[k]);
        if ((threadIdx.x & 31) == 0) s_acc[threadIdx.x >> 5][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double x = 0.0;
        for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) x += s_acc[w2][threadIdx.x];
        partial[4 * (size_t)blockIdx.x + threadIdx.x] = x;
    }
}

// one block: the centre-of-mass velocity (fixed-order sum of the block sums)
// into vcm[0..2]
__global__ void __launch_bounds__(256) k_boltzmann_vcm(const double* partial, uint32_t nblocks, double* vcm)
{
    __shared__ double s_red[256];
    __shared__ double s_sum[4];
    for (int k = 0; k < 4; ++k) {
        double x = 0.0;
        for (uint32_t b = threadIdx.x; b < nblocks; b += blockDim.x) x += partial[4 * (size_t)b + k];
        s_red[threadIdx.x] = x;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) s_red[threadIdx.x] += s_red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) s_sum[k] = s_red[0];
        __syncthreads();
    }
    if (threadIdx.x < 3) vcm[threadIdx.x] = s_sum[threadIdx.x] / s_sum[3];
}

__global__ void __launch_bounds__(256) k_shift(double* out, uint32_t n, const double* vcm)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    for (int q = 0; q < 3; ++q) out[3 * (size_t)t + q] = __dsub_rn(out[3 * (size_t)t + q], vcm[q]);
}

void launch_lattice(double* out, uint32_t n, const uint32_t cells[3], double a, const double offset[3], uint32_t skip,
                    cudaStream_t st)
{
    const unsigned grid = (n + 255) / 256;
    if (grid > 0) k_lattice<<<grid, 256, 0, st>>>(out, n, cells[0], cells[1], a, offset[0], offset[1], offset[2], skip);
}

// velocities into out[3 n]; scratch: 4 ceil(n / 256) + 3 doubles
void launch_boltzmann(const Dev& d, uint32_t s, uint32_t n, double T, uint64_t seed, double* out, double* scratch,
                      cudaStream_t st)
{
    const unsigned grid = (n + 255) / 256;
    if (grid == 0) return;
    double* vcm = scratch + 4 * (size_t)grid;
    k_boltzmann<<<grid, 256, 0, st>>>(d, s, T, (uint32_t)seed, (uint32_t)(seed >> 32), out, scratch);
    k_boltzmann_vcm<<<1, 256, 0, st>>>(scratch, grid, vcm);
    k_shift<<<grid, 256, 0, st>>>(out, n, vcm);
}

// flag[0] = 1 if any of the n values is not finite
__global__ void __launch_bounds__(256) k_check_finite(const double* in, size_t n, uint32_t* flag)
{
    bool bad = false;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        bad |= !isfinite(in[k]);
    if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

void launch_check_finite(const double* in, size_t n, uint32_t* flag, cudaStream_t st)
{
    cudaMemsetAsync(flag, 0, sizeof(uint32_t), st);
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 1024);
    if (grid > 0) k_check_finite<<<grid, 256, 0, st>>>(in, n, flag);
}

void launch_set_vector(const Dev& d, uint32_t s, uint32_t n, int what, bool ds, const double* in, cudaStream_t st)
{
    const unsigned grid = (n + 255) / 256;
    if (grid == 0) return;
    if (what == 0) {
        if (ds) k_set_position<true><<<grid, 256, 0, st>>>(d, s, in);
        else k_set_position<false><<<grid, 256, 0, st>>>(d, s, in);
    } else {
        if (ds) k_set_velocity<true><<<grid, 256, 0, st>>>(d, s, in);
        else k_set_velocity<false><<<grid, 256, 0, st>>>(d, s, in);
    }
}

void launch_get_vector(const Dev& d, uint32_t s, uint32_t n, int what, double* out, cudaStream_t st)
{
    const unsigned grid = (n + 255) / 256;
    if (grid > 0) k_get_vector<<<grid, 256, 0, st>>>(d, s, what, out);
}

} // namespace hmd
