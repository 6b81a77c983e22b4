// kernels_step.cu — per-step kernels: velocity-Verlet integrate (fused with the
// maximum-displacement reduction and the rebuild decision), Verlet / Andersen
// finalize, FP64 reductions, and the dispatch of the pair-force kernels
// (force.cuh, compiled per interaction kind in kernels_force_*.cu).
//
// Every kernel runs over all slots of all systems of an engine; a block never
// straddles two systems (blocks of <= 256 threads, systems padded to 256
// slots), so per-system parameters are block-uniform.
#include "hmd_device.cuh"
#include <algorithm>
#include "kernels.h"
#include "step_device.cuh"

namespace hmd {

// per-block sums of m v^2, m v (3) and m of the velocities (FP64, fixed
// order) into Dev::partial[block][0..4], for the thermostats of
// verlet_nvt_hoover (m v^2) and verlet_nvt_boltzmann (m v, m)
constexpr int NMOM = 5;

__device__ __forceinline__ void moment_terms(float4 v, float4 vl, double* acc)
{
    const double m = v.w;
    const double vx = (double)v.x + (double)vl.x, vy = (double)v.y + (double)vl.y, vz = (double)v.z + (double)vl.z;
    acc[0] = m * (vx * vx + vy * vy + vz * vz);
    acc[1] = m * vx;
    acc[2] = m * vy;
    acc[3] = m * vz;
    acc[4] = m;
}

__device__ __forceinline__ void block_moments(const Dev& d, double* acc)
{
    __shared__ double s_acc[8][NMOM];
#pragma unroll
    for (int k = 0; k < NMOM; ++k) {
        const double v = warp_sum(acc[k]);
        if ((threadIdx.x & 31) == 0) s_acc[threadIdx.x >> 5][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < NMOM) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += s_acc[w][threadIdx.x];
        d.partial[(size_t)blockIdx.x * NTHERMO + threadIdx.x] = v;
    }
}

// Second half-kick (gpu/integrators/verlet_kernel.cu:78-98) or Andersen
// collisions (verlet_nvt_andersen_kernel.cu:97-171, with the per-particle
// host convention of host/integrators/verlet_nvt_andersen.cpp:111-137).
// MOM: also the per-block moments of the new velocities (engines with a
// Nose-Hoover or Maxwell-Boltzmann thermostat)
template <bool DS, bool MOM>
__global__ void __launch_bounds__(256) k_finalize(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // the slot's words first: they do not depend on the system's parameters
    const float w = pos_hi(d.pos, i).w;
    float4 v = d.vel[i];
    float4 vl = DS ? d.vel[d.S + i] : make_float4(0, 0, 0, 0);
    const float4 f = d.force[i];
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    const SysState& st = d.st[s];
    double acc[NMOM] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const bool run = P.active && st.live && *d.status == 0u && P.integrator != INTEG_DESCENT;   // block-uniform
    if (run && species_bits(w) != PLACEHOLDER) {
        finalize_slot<DS>(d, P, st, i, v, vl, f);
        d.vel[i] = v;
        if (DS) d.vel[d.S + i] = vl;
        if (MOM) moment_terms(v, vl, acc);
    }
    if (MOM) block_moments(d, acc);
}

// the moments of the current velocities (before a Nose-Hoover integrate)
__global__ void __launch_bounds__(256) k_moments(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[NMOM] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const float4 r = pos_hi(d.pos, i);
    if (species_bits(r.w) != PLACEHOLDER) moment_terms(d.vel[i], d.vel[d.S + i], acc);
    block_moments(d, acc);
}

// Nose-Hoover chain of two, one half step (verlet_nvt_hoover.cpp:141-185
// propagate_chain), in FP64; en_kin_2 = sum m v^2.  Returns the velocity
// scale of this half step.
__device__ double propagate_chain(const SysParam& P, SysState& st, double en_kin_2)
{
    const double dt = P.nhc_dt, dt2 = dt / 2, dt4 = dt / 4, dt8 = dt / 8;
    const double M0 = P.nhc_mass[0], M1 = P.nhc_mass[1], T = P.nhc_T, target = P.nhc_target2;
    st.v_xi[1] += (M0 * st.v_xi[0] * st.v_xi[0] - T) / M1 * dt4;
    const double t = exp(-st.v_xi[1] * dt8);
    st.v_xi[0] *= t;
    st.v_xi[0] += (en_kin_2 - target) / M0 * dt4;
    st.v_xi[0] *= t;
    st.xi[0] += st.v_xi[0] * dt2;
    st.xi[1] += st.v_xi[1] * dt2;
    const double sc = exp(-st.v_xi[0] * dt2);
    en_kin_2 *= sc * sc;
    st.v_xi[0] *= t;
    st.v_xi[0] += (en_kin_2 - target) / M0 * dt4;
    st.v_xi[0] *= t;
    st.v_xi[1] += (M0 * st.v_xi[0] * st.v_xi[0] - T) / M1 * dt4;
    return sc;
}

// One block per system: the system's moments (fixed-order sum of its block
// partials) drive its thermostat.  post = 0: before integrate (Nose-Hoover
// chain -> scale); post = 1: after finalize (Nose-Hoover chain -> scale, or
// the centre-of-mass velocity of a Maxwell-Boltzmann draw).
__global__ void __launch_bounds__(256) k_thermostat(Dev d, int post)
{
    const uint32_t s = blockIdx.x;
    const SysParam& P = d.sys[s];
    SysState& st = d.st[s];
    const bool clean = *d.status == 0u;
    const bool advancing = post ? (P.active && st.live && clean) : (P.active && st.steps_left != 0u && clean);
    const bool hoover = P.integrator == INTEG_HOOVER;
    const bool draw = post && boltzmann_due(P, st);
    if (!advancing || !(hoover || draw)) return;   // block-uniform
    const uint32_t b0 = P.off / 256, nb = P.A / 256;
    __shared__ double s_red[256];
    __shared__ double s_sum[NMOM];
    for (int k = hoover ? 0 : 1; k < (hoover ? 1 : NMOM); ++k) {
        double v = 0.0;
        for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) v += d.partial[(size_t)(b0 + b) * NTHERMO + k];
        s_red[threadIdx.x] = v;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) s_red[threadIdx.x] += s_red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) s_sum[k] = s_red[0];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    if (hoover) {
        st.scale = (float)propagate_chain(P, st, s_sum[0]);
    } else {
        // velocities/boltzmann_kernel.cu:103-140 (shift): vcm = sum m v / sum m
        st.vcm[0] = s_sum[1] / s_sum[4];
        st.vcm[1] = s_sum[2] / s_sum[4];
        st.vcm[2] = s_sum[3] / s_sum[4];
    }
}

// after k_thermostat(post = 1): Nose-Hoover rescale (verlet_nvt_hoover_kernel.cu
// rescale) or the removal of the drawn centre-of-mass velocity
template <bool DS>
__global__ void __launch_bounds__(256) k_thermostat_apply(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    const SysState& st = d.st[s];
    const bool hoover = P.integrator == INTEG_HOOVER;
    if (!P.active || !st.live || *d.status != 0u || !(hoover || boltzmann_due(P, st))) return;
    if (species_bits(pos_hi(d.pos, i).w) == PLACEHOLDER) return;
    float4 v = d.vel[i];
    float4 vl = make_float4(0, 0, 0, 0);
    if (DS) vl = d.vel[d.S + i];
    if (hoover) {
        const float sc = st.scale;
        if (DS) {
            ds_mul(v.x, vl.x, v.x, vl.x, sc, 0.0f);
            ds_mul(v.y, vl.y, v.y, vl.y, sc, 0.0f);
            ds_mul(v.z, vl.z, v.z, vl.z, sc, 0.0f);
        } else {
            v.x = __fmul_rn(v.x, sc); v.y = __fmul_rn(v.y, sc); v.z = __fmul_rn(v.z, sc);
        }
    } else {
        float c[3], cl[3];
        for (int q = 0; q < 3; ++q) {
            c[q] = (float)st.vcm[q];
            cl[q] = (float)(st.vcm[q] - (double)c[q]);
        }
        if (DS) {
            ds_sub(v.x, vl.x, v.x, vl.x, c[0], cl[0]);
            ds_sub(v.y, vl.y, v.y, vl.y, c[1], cl[1]);
            ds_sub(v.z, vl.z, v.z, vl.z, c[2], cl[2]);
        } else {
            v.x = __fsub_rn(v.x, c[0]); v.y = __fsub_rn(v.y, c[1]); v.z = __fsub_rn(v.z, c[2]);
        }
    }
    d.vel[i] = v;
    if (DS) d.vel[d.S + i] = vl;
}

// First half-kick, drift and wrap (gpu/integrators/verlet_kernel.cu:38-72)
// with the displacement maximum (max_displacement_kernel.cu:37-68) and the
// skin/2 rebuild decision (neighbours/from_binning.cpp:130).
// FIN: the finalize of the previous step (its force is in d.force) runs
// first, on the same registers: one pass over the phase space per step
// inside a captured chunk.  The per-system flags it reads (live,
// steps_left) are read before any block arrives at the decision that
// updates them, so both halves see the state of their own step.
template <bool DS, bool FIN>
__global__ void __launch_bounds__(256) k_integrate(Dev d, cudaGraphConditionalHandle h, int use_handle)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const SlotIn<DS> in = load_slot<DS>(d, i);
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    SysState& st = d.st[s];
    const bool clean = *d.status == 0u;
    const bool live = P.active && st.steps_left != 0u && clean;
    const bool fin = FIN && P.active && st.live && clean && P.integrator != INTEG_DESCENT;
    const float rr = step_slot<DS, FIN>(d, P, st, i, in, fin, live);
    step_decision(d, st, rr, h, use_handle);
}

// Mark systems live for a force evaluation outside a step (set-up, or a
// force requested through the module interface, as particle.cpp:221-253
// evaluates forces on demand); `rebuild_all` also flags every active
// system for a list rebuild.
__global__ void k_mark(Dev d, int rebuild_all)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < d.nsys; q += gridDim.x * blockDim.x) {
        SysState& t = d.st[q];
        const bool lv = d.sys[q].active != 0u;
        t.live = lv;
        // an untruncated system (pair_full) has no list and never rebuilds
        t.rebuild = (lv && d.sys[q].trunc != TRUNC_NONE && (rebuild_all || t.rebuild_request)) ? 1u : 0u;
        if (t.rebuild) { t.rebuild_request = 0u; t.rebuilds += 1ull; }
    }
}

// ---------------------------------------------------------------------------
// FP64 reductions (observables/gpu/thermodynamics_kernel.cu:35-106 and
// algorithm/gpu/reduce_kernel.cuh:126): per-block partial sums, then a
// fixed-order per-system reduction (deterministic, no double atomics).
//   0: Σ m v²   1-3: Σ m v   4: Σ m   5: Σ E_pot   6: Σ tr(stress)
//   7-12: Σ stress (xx yy zz xy xz yz)   13: particle count
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_thermo_partial(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[NTHERMO];
#pragma unroll
    for (int k = 0; k < NTHERMO; ++k) acc[k] = 0.0;
    const float4 r = pos_hi(d.pos, i);
    if (species_bits(r.w) != PLACEHOLDER && d.sys[d.chunk_sys[i / CHUNK]].active) {
        const float4 vh = d.vel[i];
        const float4 vl = d.vel[d.S + i];
        const double m = vh.w;
        const double vx = (double)vh.x + (double)vl.x;
        const double vy = (double)vh.y + (double)vl.y;
        const double vz = (double)vh.z + (double)vl.z;
        acc[0] = m * (vx * vx + vy * vy + vz * vz);
        acc[1] = m * vx; acc[2] = m * vy; acc[3] = m * vz;
        acc[4] = m;
        acc[5] = d.en_pot[i];
        const size_t S = d.S;
        double sxx = d.stress[i], syy = d.stress[S + i], szz = d.stress[2 * S + i];
        acc[6] = sxx + syy + szz;
        acc[7] = sxx; acc[8] = syy; acc[9] = szz;
        acc[10] = d.stress[3 * S + i]; acc[11] = d.stress[4 * S + i]; acc[12] = d.stress[5 * S + i];
        acc[13] = 1.0;
    }
    __shared__ double s_acc[8][NTHERMO];
#pragma unroll
    for (int k = 0; k < NTHERMO; ++k) {
        double v = warp_sum(acc[k]);
        if ((threadIdx.x & 31) == 0) s_acc[threadIdx.x >> 5][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < NTHERMO) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += s_acc[w][threadIdx.x];
        d.partial[(size_t)blockIdx.x * NTHERMO + threadIdx.x] = v;
    }
}

// one block per system; `velocity_lo` is ignored for FP32 engines by the
// caller zeroing the lo half once
__global__ void __launch_bounds__(256) k_thermo_reduce(Dev d)
{
    const uint32_t s = blockIdx.x;
    const SysParam& P = d.sys[s];
    const uint32_t b0 = P.off / 256, nb = P.A / 256;
    __shared__ double s_red[256];
    for (int k = 0; k < NTHERMO; ++k) {
        double v = 0.0;
        for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) v += d.partial[(size_t)(b0 + b) * NTHERMO + k];
        s_red[threadIdx.x] = v;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) s_red[threadIdx.x] += s_red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) d.thermo[(size_t)s * NTHERMO + k] = s_red[0];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

// threads per block of the integrate kernels (at most 256: step_decision's
// per-warp maxima; at least 64 so blocks stay inside one system).  128
// measured the same as 256 (KA-64k 1.023e9 against 1.022e9, LJ-1M 3.59e9
// against 3.57e9 particle-steps/s, one run each)
#ifndef HMD_STEP_THREADS
#define HMD_STEP_THREADS 256
#endif
static_assert(HMD_STEP_THREADS >= 64 && HMD_STEP_THREADS <= 256 && HMD_STEP_THREADS % 64 == 0, "step block size");

void launch_integrate(const Dev& d, bool ds, cudaGraphConditionalHandle h, bool use_handle, cudaStream_t st)
{
    if (d.fp64) return launch_integrate64(d, false, h, use_handle, st);
    constexpr unsigned T = HMD_STEP_THREADS;
    const unsigned grid = d.S_grid / T;
    if (ds) k_integrate<true, false><<<grid, T, 0, st>>>(d, h, use_handle ? 1 : 0);
    else k_integrate<false, false><<<grid, T, 0, st>>>(d, h, use_handle ? 1 : 0);
}

void launch_finalize_integrate(const Dev& d, bool ds, cudaGraphConditionalHandle h, cudaStream_t st)
{
    if (d.fp64) return launch_integrate64(d, true, h, true, st);
    constexpr unsigned T = HMD_STEP_THREADS;
    const unsigned grid = d.S_grid / T;
    if (ds) k_integrate<true, true><<<grid, T, 0, st>>>(d, h, 1);
    else k_integrate<false, true><<<grid, T, 0, st>>>(d, h, 1);
}

void launch_mark(const Dev& d, bool rebuild_all, cudaStream_t st)
{
    k_mark<<<(d.nsys + 255) / 256, 256, 0, st>>>(d, rebuild_all ? 1 : 0);
}

// one launch per kind of pair interaction present in the engine (each
// kernel skips the blocks of the other kinds); kinds 0: every kind in one
// kernel (engines whose systems change after commit)
void launch_force(const Dev& d, bool aux, cudaStream_t st)
{
    if (d.fp64) return launch_force64(d, aux, st);
    if (d.force_kinds == 0u) {
        launch_force_kind<FK_GENERIC>(d, aux, st);
        return;
    }
    if (d.force_kinds & (1u << FK_LJ1)) launch_force_kind<FK_LJ1>(d, aux, st);
    if (d.force_kinds & (1u << FK_SHIFTED)) launch_force_kind<FK_SHIFTED>(d, aux, st);
    if (d.force_kinds & (1u << FK_SMOOTH)) launch_force_kind<FK_SMOOTH>(d, aux, st);
    if (d.force_kinds & (1u << FK_FSHIFT)) launch_force_kind<FK_FSHIFT>(d, aux, st);
    if (d.force_kinds & (1u << FK_POT)) launch_force_kind<FK_POT>(d, aux, st);
    if (d.force_kinds & (1u << FK_FULL)) launch_force_full(d, aux, st);
}

// engines with a Nose-Hoover or Maxwell-Boltzmann system: the finalize
// writes the moments of the new velocities, one block per system runs the
// thermostat, and the velocities are rescaled or shifted
void launch_finalize(const Dev& d, bool ds, cudaStream_t st)
{
    if (d.fp64) return launch_finalize64(d, st);
    const unsigned grid = d.S_grid / 256;
    const bool thermo = (d.integ_kinds & ((1u << INTEG_HOOVER) | (1u << INTEG_BOLTZMANN))) != 0u;
    if (!thermo) {
        if (ds) k_finalize<true, false><<<grid, 256, 0, st>>>(d);
        else k_finalize<false, false><<<grid, 256, 0, st>>>(d);
        return;
    }
    if (ds) k_finalize<true, true><<<grid, 256, 0, st>>>(d);
    else k_finalize<false, true><<<grid, 256, 0, st>>>(d);
    k_thermostat<<<d.nsys, 256, 0, st>>>(d, 1);
    if (ds) k_thermostat_apply<true><<<grid, 256, 0, st>>>(d);
    else k_thermostat_apply<false><<<grid, 256, 0, st>>>(d);
}

// engines with a Nose-Hoover system: the chain's first half step, from the
// moments of the current velocities, before integrate
void launch_integrate_prepare(const Dev& d, cudaStream_t st)
{
    if (!(d.integ_kinds & (1u << INTEG_HOOVER))) return;
    k_moments<<<d.S_grid / 256, 256, 0, st>>>(d);
    k_thermostat<<<d.nsys, 256, 0, st>>>(d, 0);
}

int step_kernel_count(const Dev& d)
{
    int n = 2 + (d.force_kinds ? __builtin_popcount(d.force_kinds) : 1);   // integrate, force kinds, finalize
    if (d.integ_kinds & ((1u << INTEG_HOOVER) | (1u << INTEG_BOLTZMANN))) n += 2;   // thermostat, apply
    if (d.integ_kinds & (1u << INTEG_HOOVER)) n += 2;                            // moments, thermostat
    return n;
}

void launch_thermo(const Dev& d, cudaStream_t st)
{
    k_thermo_partial<<<d.S_grid / 256, 256, 0, st>>>(d);
    k_thermo_reduce<<<d.nsys, 256, 0, st>>>(d);
}

// max_displacement::compute (mdsim/gpu/max_displacement.cpp:77-106, kernel
// max_displacement_kernel.cu:37-68): the largest squared minimum-image
// displacement since the last list build over the real particles of system
// s, with the arithmetic of the integrate kernel's fused test (step_slot),
// as float bits (non-negative floats order as their bit patterns)
__global__ void __launch_bounds__(256) k_max_displacement(Dev d, uint32_t s, uint32_t* out)
{
    const SysParam& P = d.sys[s];
    float rr = 0.0f;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < P.A; k += gridDim.x * blockDim.x) {
        const uint32_t i = P.off + k;
        const float4 r = pos_hi(d.pos, i);
        if (species_bits(r.w) == PLACEHOLDER) continue;
        const float4 q = d.r0[i];
        const float dx = min_image(__fsub_rn(r.x, q.x), P.L[0], P.Linv[0]);
        const float dy = min_image(__fsub_rn(r.y, q.y), P.L[1], P.Linv[1]);
        const float dz = min_image(__fsub_rn(r.z, q.z), P.L[2], P.Linv[2]);
        rr = fmaxf(rr, rr_exact(dx, dy, dz));
    }
    rr = warp_max(rr);
    if ((threadIdx.x & 31) == 0 && rr > 0.0f) atomicMax(out, __float_as_uint(rr));
}

void launch_max_displacement(const Dev& d, uint32_t s, uint32_t slots, uint32_t* out, cudaStream_t st)
{
    cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
    const unsigned grid = std::max(1u, std::min((slots + 255u) / 256u, 8u * std::max(d.sm_count, 1u)));
    k_max_displacement<<<grid, 256, 0, st>>>(d, s, out);
}

// the force kernel's gather records (fpos_encode) of every real slot of a
// dsfloat engine; the integrate kernel and the list build write them as they
// go, this pass serves force evaluations outside a step
__global__ void __launch_bounds__(256) k_pack_fpos(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const float4 r = pos_hi(d.pos, i);
    if (species_bits(r.w) == PLACEHOLDER) return;
    const SysParam& P = d.sys[d.chunk_sys[i / CHUNK]];
    d.fpos[i] = fpos_encode(r, pos_lo(d.pos, i), P.lo_inv_scale);
}

void launch_pack_fpos(const Dev& d, cudaStream_t st)
{
    if (!d.ds || d.S_grid == 0) return;
    k_pack_fpos<<<d.S_grid / 256, 256, 0, st>>>(d);
}

} // namespace hmd
