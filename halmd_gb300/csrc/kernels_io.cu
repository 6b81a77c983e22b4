// kernels_io.cu — phase-space transfer between the caller's tag-ordered
// double arrays (one device staging copy) and the Hilbert-ordered float /
// double-single arrays: the conversion of particle.cpp's set/get
// (mdsim/gpu/particle.cpp:221-330, particle_kernel.cu) done on the device,
// so a set or get is one host copy and one kernel instead of a read-back,
// a host loop and a write per array.  Double arithmetic uses the _rn
// intrinsics: no contraction, the same rounding as the host formulas.
#include "hmd_device.cuh"
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
    float4 h = d.pos[k], g = d.img[k];
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
    d.pos[k] = h;                       // w (species) unchanged
    if (DS) d.pos[d.S + k] = l;
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
    if (what <= 1) { a = d.pos[k]; b = d.pos[d.S + k]; if (what == 1) g = d.img[k]; }
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
