// kernels_obs.cu — observables on the device: unwrapped positions and
// velocities in tag order (observables/gpu/phase_space_kernel.cu:39-64),
// mean-square / mean-quartic displacement and velocity autocorrelation of
// two samples with an FP64 Welford accumulator per particle range
// (observables/gpu/dynamics/mean_square_displacement.cpp:55-68,
// numeric/accumulator.hpp:83-119), and density modes rho(q) = Σ exp(i q·r)
// (observables/gpu/density_mode_kernel.cu:46-108) summed in FP64.
#include "hmd_device.cuh"
#include "kernels.h"

namespace hmd {

// out[tag * 3 + c] = hi + lo + image * L for the slots [first, first + count)
// of one system (double; L is the float box length the integrator wraps with)
__global__ void __launch_bounds__(256) k_sample_position(Dev d, uint32_t first, double* out)
{
    const uint32_t i = first + blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    const float4 r = pos_hi(d.pos, i);
    if (!P.active || species_bits(r.w) == PLACEHOLDER) return;
    const float4 rl = pos_lo(d.pos, i);
    const float4 im = d.img[i];
    const uint32_t tag = d.id[i];
    double* o = out + (size_t)tag * 3;
    o[0] = ((double)r.x + (double)rl.x) + (double)im.x * (double)P.L[0];
    o[1] = ((double)r.y + (double)rl.y) + (double)im.y * (double)P.L[1];
    o[2] = ((double)r.z + (double)rl.z) + (double)im.z * (double)P.L[2];
}

// Chan et al. pairwise merge of (count, mean, M2)
__device__ __forceinline__ void acc_merge(double& n, double& m, double& v, double n2, double m2, double v2)
{
    if (n2 > 0) {
        const double c = n + n2;
        const double diff = m - m2;
        v = v + v2 + diff * diff * n * n2 / c;
        m = (n * m + n2 * m2) / c;
        n = c;
    }
}

constexpr uint32_t MSD_CHUNK = 8192;

// velocities in tag order: out[tag * 3 + c] = hi + lo
__global__ void __launch_bounds__(256) k_sample_velocity(Dev d, uint32_t first, double* out)
{
    const uint32_t i = first + blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    if (!P.active || species_bits(pos_hi(d.pos, i).w) == PLACEHOLDER) return;
    const float4 v = d.vel[i];
    const float4 vl = d.vel[d.S + i];
    double* o = out + (size_t)d.id[i] * 3;
    o[0] = (double)v.x + (double)vl.x;
    o[1] = (double)v.y + (double)vl.y;
    o[2] = (double)v.z + (double)vl.z;
}

// per-particle value of a correlation of two samples: KIND 0 |r2 - r1|^2
// (MSD), 2 |r2 - r1|^4 (MQD, mean_quartic_displacement.hpp:34-41),
// 3 r1 . r2 (VACF on velocity samples, velocity_autocorrelation.hpp:34-38)
template <int KIND>
__device__ __forceinline__ double tcf_value(const double* r1, const double* r2, size_t k)
{
    if (KIND == 3) return r1[3 * k] * r2[3 * k] + r1[3 * k + 1] * r2[3 * k + 1] + r1[3 * k + 2] * r2[3 * k + 2];
    const double dx = r2[3 * k] - r1[3 * k];
    const double dy = r2[3 * k + 1] - r1[3 * k + 1];
    const double dz = r2[3 * k + 2] - r1[3 * k + 2];
    const double x = dx * dx + dy * dy + dz * dz;
    return KIND == 2 ? x * x : x;
}

template <int KIND>
__global__ void __launch_bounds__(256) k_msd_partial(const double* r1, const double* r2, const uint32_t* range,
                                                     const uint32_t* blk_range, const uint32_t* blk_begin,
                                                     double* partial)
{
    const uint32_t b = blockIdx.x;
    const uint32_t rg = blk_range[b];
    const uint32_t beg = blk_begin[b];
    const uint32_t end = min(beg + MSD_CHUNK, range[2 * rg + 1]);
    double n = 0, m = 0, v = 0;
    for (uint32_t k = beg + threadIdx.x; k < end; k += blockDim.x) {
        const double x = tcf_value<KIND>(r1, r2, k);
        const double t = x - m;
        n += 1;
        m += t / n;
        v += t * (x - m);
    }
    __shared__ double sn[256], sm[256], sv[256];
    sn[threadIdx.x] = n; sm[threadIdx.x] = m; sv[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            double a = sn[threadIdx.x], am = sm[threadIdx.x], av = sv[threadIdx.x];
            acc_merge(a, am, av, sn[threadIdx.x + o], sm[threadIdx.x + o], sv[threadIdx.x + o]);
            sn[threadIdx.x] = a; sm[threadIdx.x] = am; sv[threadIdx.x] = av;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[3 * b] = sn[0]; partial[3 * b + 1] = sm[0]; partial[3 * b + 2] = sv[0];
    }
}

__global__ void k_msd_reduce(const uint32_t* blk_range, uint32_t nblk, const double* partial, uint32_t nrange,
                             double* out)
{
    const uint32_t rg = blockIdx.x * blockDim.x + threadIdx.x;
    if (rg >= nrange) return;
    double n = 0, m = 0, v = 0;
    for (uint32_t b = 0; b < nblk; ++b)
        if (blk_range[b] == rg) acc_merge(n, m, v, partial[3 * b], partial[3 * b + 1], partial[3 * b + 2]);
    out[3 * rg] = n;
    out[3 * rg + 1] = m;
    out[3 * rg + 2] = n > 0 ? v / n : 0.0;
}

constexpr uint32_t DM_CHUNK = 2048;

// ranges index the reverse-id table (off + tag); positions are the wrapped
// hi words; q·r = (qx x + qy y) + qz z in float, cos/sin in float, sums in FP64
__global__ void __launch_bounds__(256) k_density_partial(Dev d, const uint32_t* range, const uint32_t* blk_range,
                                                         const uint32_t* blk_begin, const float4* q, uint32_t nq,
                                                         double* partial)
{
    __shared__ float4 s_r[DM_CHUNK];
    __shared__ double s_re[8], s_im[8];
    const uint32_t b = blockIdx.x;
    const uint32_t rg = blk_range[b];
    const uint32_t beg = blk_begin[b];
    const uint32_t end = min(beg + DM_CHUNK, range[2 * rg + 1]);
    const uint32_t cnt = end - beg;
    for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) s_r[k] = pos_hi(d.pos, d.rid[beg + k]);
    __syncthreads();
    for (uint32_t w = 0; w < nq; ++w) {
        const float4 qq = q[w];
        double re = 0, im = 0;
        for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
            const float4 r = s_r[k];
            const float qr = __fadd_rn(__fadd_rn(__fmul_rn(qq.x, r.x), __fmul_rn(qq.y, r.y)), __fmul_rn(qq.z, r.z));
            float sn, cs;
            sincosf(qr, &sn, &cs);
            re += cs;
            im += sn;
        }
        re = warp_sum(re);
        im = warp_sum(im);
        if ((threadIdx.x & 31) == 0) { s_re[threadIdx.x >> 5] = re; s_im[threadIdx.x >> 5] = im; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0, c = 0;
            for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += s_re[k]; c += s_im[k]; }
            partial[((size_t)b * nq + w) * 2] = a;
            partial[((size_t)b * nq + w) * 2 + 1] = c;
        }
        __syncthreads();
    }
}

__global__ void k_density_reduce(const uint32_t* blk_range, uint32_t nblk, uint32_t nq, const double* partial,
                                 uint32_t nrange, double* out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrange * nq) return;
    const uint32_t rg = t / nq, w = t % nq;
    double re = 0, im = 0;
    for (uint32_t b = 0; b < nblk; ++b)
        if (blk_range[b] == rg) { re += partial[((size_t)b * nq + w) * 2]; im += partial[((size_t)b * nq + w) * 2 + 1]; }
    out[2 * t] = re;
    out[2 * t + 1] = -im;   // density_mode.cpp:128
}

void launch_sample_position(const Dev& d, uint32_t first, uint32_t count, double* out, cudaStream_t st)
{
    k_sample_position<<<count / 256, 256, 0, st>>>(d, first, out);
}

void launch_sample_velocity(const Dev& d, uint32_t first, uint32_t count, double* out, cudaStream_t st)
{
    k_sample_velocity<<<count / 256, 256, 0, st>>>(d, first, out);
}

void launch_tcf(int kind, const double* r1, const double* r2, const uint32_t* range, uint32_t nrange,
                const uint32_t* blk_range, const uint32_t* blk_begin, uint32_t nblk, double* partial, double* out,
                cudaStream_t st)
{
    if (nblk > 0) {
        if (kind == 2) k_msd_partial<2><<<nblk, 256, 0, st>>>(r1, r2, range, blk_range, blk_begin, partial);
        else if (kind == 3) k_msd_partial<3><<<nblk, 256, 0, st>>>(r1, r2, range, blk_range, blk_begin, partial);
        else k_msd_partial<0><<<nblk, 256, 0, st>>>(r1, r2, range, blk_range, blk_begin, partial);
    }
    k_msd_reduce<<<(nrange + 127) / 128, 128, 0, st>>>(blk_range, nblk, partial, nrange, out);
}

void launch_msd(const double* r1, const double* r2, const uint32_t* range, uint32_t nrange, const uint32_t* blk_range,
                const uint32_t* blk_begin, uint32_t nblk, double* partial, double* out, cudaStream_t st)
{
    launch_tcf(0, r1, r2, range, nrange, blk_range, blk_begin, nblk, partial, out, st);
}

void launch_density_modes(const Dev& d, const uint32_t* range, uint32_t nrange, const uint32_t* blk_range,
                          const uint32_t* blk_begin, uint32_t nblk, const float4* q, uint32_t nq, double* partial,
                          double* out, cudaStream_t st)
{
    if (nblk > 0 && nq > 0) k_density_partial<<<nblk, 256, 0, st>>>(d, range, blk_range, blk_begin, q, nq, partial);
    const uint32_t tot = nrange * nq;
    if (tot > 0) k_density_reduce<<<(tot + 127) / 128, 128, 0, st>>>(blk_range, nblk, nq, partial, nrange, out);
}

} // namespace hmd
