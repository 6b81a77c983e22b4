// kernels_fp64.cu — the FP64 variant of the MD step (HMD_PRECISION_DOUBLE):
// pair forces, integrate and finalize in double precision, the reference
// run from the same start against which the float and dsfloat engines'
// energy drift and force error are measured.  Positions and velocities keep
// the double-single storage (hi + lo words, 48 significant bits; every
// kernel reads hi + lo as a double and splits the result again), so the
// neighbour list, binning, Hilbert sort and rebuild decision are the
// dsfloat engine's.  Forces are kept in double (Dev::force64).  Lennard-
// Jones with every truncation and velocity Verlet only; the pair set is
// r^2 < r_c^2 in double, as in the host backend
// (mdsim/host/forces/pair_trunc.hpp:219-344).
#include "hmd_device.cuh"
#include "kernels.h"
#include "step_device.cuh"

namespace hmd {

__device__ __forceinline__ double pos_d(float hi, float lo) { return (double)hi + (double)lo; }

// one component: double -> (hi, lo) words
__device__ __forceinline__ void split_d(double x, float& hi, float& lo)
{
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

// LJ + truncation in double (lennard_jones.hpp:56-66 and the truncations'
// host formulas, the same as pair_eval in force.cuh)
__device__ __forceinline__ void lj64(const PairParam64& p, uint32_t trunc, double rri_smooth, double rr,
                                     double& fval, double& en)
{
    const double rri = p.sigma2 / rr;
    const double ri6 = rri * rri * rri;
    fval = p.c48 * rri * ri6 * (ri6 - 0.5);
    en = p.eps4 * ri6 * (ri6 - 1.0) - p.en_cut;
    if (trunc == TRUNC_SMOOTH_R4) {
        const double r = sqrt(rr);
        const double dr = r - p.r_cut;
        const double x2 = dr * dr * rri_smooth;
        const double x4 = x2 * x2;
        const double x4i = 1.0 / (1.0 + x4);
        const double h0 = x4 * x4i;
        const double h1 = 4.0 * dr * rri_smooth * x2 * x4i * x4i;
        fval = h0 * fval - h1 * (en / r);
        en = h0 * en;
    } else if (trunc == TRUNC_FORCE_SHIFTED) {
        const double r = sqrt(rr);
        fval = fval - p.f_cut / r;
        en = en + (r - p.r_cut) * p.f_cut;
    }
}

// F_i = Σ_j fval r_ij over the list entries with r_ij^2 < r_c^2 (double);
// one thread a particle, near entries from the front of the blocked list,
// far entries from its back (hmd_device.cuh Dev::nbr)
template <bool AUX>
__global__ void __launch_bounds__(128) k_force64(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const SysParam& P = d.sys[d.chunk_sys[i / CHUNK]];
    const uint32_t s = d.chunk_sys[i / CHUNK];
    if (!P.active || !d.st[s].live || *d.status != 0u) return;
    float4 hi, lo;
    ldg_pos2(d.pos, i, hi, lo);
    const uint32_t a = species_bits(hi.w);
    if (a == PLACEHOLDER) return;
    const double ri[3] = {pos_d(hi.x, lo.x), pos_d(hi.y, lo.y), pos_d(hi.z, lo.z)};
    const double L[3] = {(double)P.L[0], (double)P.L[1], (double)P.L[2]};
    const uint32_t packed = d.nbr_count[i];
    const uint32_t nn = packed & 0xFFFFu, nf = packed >> 16;
    const uint32_t lw = d.lb_log2, lmask = (1u << lw) - 1u;
    const PairParam64* row = d.pair64 + P.pair_off + a * P.ns;
    const double rri_smooth = (double)P.rri_smooth64;
    double f[3] = {0, 0, 0}, en = 0, st[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t k = 0; k < nn + nf; ++k) {
        const uint32_t e = k < nn ? k : d.nbr_cap - 1u - (k - nn);
        const uint32_t j = d.nbr[(((size_t)(e >> lw) * d.S + i) << lw) + (e & lmask)];
        float4 hj, lj;
        ldg_pos2(d.pos, j, hj, lj);
        const uint32_t b = species_bits(hj.w);
        if (b >= P.ns) continue;
        double dr[3] = {ri[0] - pos_d(hj.x, lj.x), ri[1] - pos_d(hj.y, lj.y), ri[2] - pos_d(hj.z, lj.z)};
        for (int q = 0; q < 3; ++q) dr[q] -= L[q] * rint(dr[q] / L[q]);
        const double rr = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
        const PairParam64& p = row[b];
        if (d.float_cutoff) {
            // the float cut-off test of the other engines (force.cuh): the
            // squared minimum-image distance of the hi words below float r_c^2
            const float sx = min_image(__fsub_rn(hi.x, hj.x), P.L[0], P.Linv[0]);
            const float sy = min_image(__fsub_rn(hi.y, hj.y), P.L[1], P.Linv[1]);
            const float sz = min_image(__fsub_rn(hi.z, hj.z), P.L[2], P.Linv[2]);
            if (!(rr_exact(sx, sy, sz) < (float)p.rr_cut)) continue;
        } else if (!(rr < p.rr_cut)) {
            continue;
        }
        double fval, e_pair;
        lj64(p, P.trunc, rri_smooth, rr, fval, e_pair);
        for (int q = 0; q < 3; ++q) f[q] += fval * dr[q];
        if (AUX) {
            en += e_pair;
            st[0] += fval * dr[0] * dr[0]; st[1] += fval * dr[1] * dr[1]; st[2] += fval * dr[2] * dr[2];
            st[3] += fval * dr[0] * dr[1]; st[4] += fval * dr[0] * dr[2]; st[5] += fval * dr[1] * dr[2];
        }
    }
    d.force64[i] = Force64{f[0], f[1], f[2], 0.0};
    d.force[i] = make_float4((float)f[0], (float)f[1], (float)f[2], 0.0f);
    if (AUX) {
        // full list: half of each pair's energy and stress per particle (pair_trunc.hpp:291-294)
        d.en_pot[i] = (float)(0.5 * en);
        for (int c = 0; c < 6; ++c) d.stress[(size_t)c * d.S + i] = (float)(0.5 * st[c]);
    }
}

// half-kick v += F dt / (2 m) of slot i in double, velocities split back
__device__ __forceinline__ void kick64(const Dev& d, uint32_t i, double hdt, double v[3], float4& vh, float4& vl)
{
    const Force64 f = d.force64[i];
    const double m = (double)vh.w;
    v[0] += f.x * hdt / m;
    v[1] += f.y * hdt / m;
    v[2] += f.z * hdt / m;
}

// integrate (and with FIN the finalize of the previous step) in double:
// verlet_kernel.cu:38-98 with the arithmetic of host/integrators/verlet.cpp
template <bool FIN>
__global__ void __launch_bounds__(256) k_integrate64(Dev d, cudaGraphConditionalHandle h, int use_handle)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    SysState& st = d.st[s];
    const bool clean = *d.status == 0u;
    const bool live = P.active && st.steps_left != 0u && clean;
    const bool fin = FIN && P.active && st.live && clean;
    float rr = 0.0f;
    float4 r = pos_hi(d.pos, i);
    const bool real = species_bits(r.w) != PLACEHOLDER;
    if (real && (fin || live)) {
        float4 rl = pos_lo(d.pos, i);
        float4 vh = d.vel[i], vl = d.vel[d.S + i];
        double v[3] = {pos_d(vh.x, vl.x), pos_d(vh.y, vl.y), pos_d(vh.z, vl.z)};
        const double hdt = 0.5 * P.dt64;
        if (fin) kick64(d, i, hdt, v, vh, vl);
        if (live) {
            kick64(d, i, hdt, v, vh, vl);
            double x[3] = {pos_d(r.x, rl.x), pos_d(r.y, rl.y), pos_d(r.z, rl.z)};
            float4 im = d.img[i];
            float* imp = &im.x;
            float* rh = &r.x;
            float* rlo = &rl.x;
            bool wrapped = false;
            for (int q = 0; q < 3; ++q) {
                x[q] += v[q] * P.dt64;
                const double L = (double)P.L[q];
                const double k = rint(x[q] / L);
                x[q] -= k * L;
                if (k != 0.0) { imp[q] = __fadd_rn(imp[q], (float)k); wrapped = true; }
                split_d(x[q], rh[q], rlo[q]);
            }
            pos_hi(d.pos, i) = r;
            pos_lo(d.pos, i) = rl;
            if (wrapped) d.img[i] = im;
            const float4 q0 = d.r0[i];
            const float dx = min_image(__fsub_rn(r.x, q0.x), P.L[0], P.Linv[0]);
            const float dy = min_image(__fsub_rn(r.y, q0.y), P.L[1], P.Linv[1]);
            const float dz = min_image(__fsub_rn(r.z, q0.z), P.L[2], P.Linv[2]);
            rr = rr_exact(dx, dy, dz);
        }
        split_d(v[0], vh.x, vl.x);
        split_d(v[1], vh.y, vl.y);
        split_d(v[2], vh.z, vl.z);
        d.vel[i] = vh;
        d.vel[d.S + i] = vl;
    }
    step_decision(d, st, rr, h, use_handle);
}

__global__ void __launch_bounds__(256) k_finalize64(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    const SysState& st = d.st[s];
    if (!(P.active && st.live && *d.status == 0u)) return;
    if (species_bits(pos_hi(d.pos, i).w) == PLACEHOLDER) return;
    float4 vh = d.vel[i], vl = d.vel[d.S + i];
    double v[3] = {pos_d(vh.x, vl.x), pos_d(vh.y, vl.y), pos_d(vh.z, vl.z)};
    kick64(d, i, 0.5 * P.dt64, v, vh, vl);
    split_d(v[0], vh.x, vl.x);
    split_d(v[1], vh.y, vl.y);
    split_d(v[2], vh.z, vl.z);
    d.vel[i] = vh;
    d.vel[d.S + i] = vl;
}

void launch_force64(const Dev& d, bool aux, cudaStream_t st)
{
    const unsigned grid = d.S_grid / 128;
    if (aux) k_force64<true><<<grid, 128, 0, st>>>(d);
    else k_force64<false><<<grid, 128, 0, st>>>(d);
}

void launch_integrate64(const Dev& d, bool fin, cudaGraphConditionalHandle h, bool use_handle, cudaStream_t st)
{
    const unsigned grid = d.S_grid / 256;
    if (fin) k_integrate64<true><<<grid, 256, 0, st>>>(d, h, 1);
    else k_integrate64<false><<<grid, 256, 0, st>>>(d, h, use_handle ? 1 : 0);
}

void launch_finalize64(const Dev& d, cudaStream_t st)
{
    k_finalize64<<<d.S_grid / 256, 256, 0, st>>>(d);
}

} // namespace hmd
