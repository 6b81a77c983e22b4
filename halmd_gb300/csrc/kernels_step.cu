// kernels_step.cu — per-step kernels: velocity-Verlet integrate (fused with the
// maximum-displacement reduction and the rebuild decision), Verlet / Andersen
// finalize, FP64 reductions, and the dispatch of the pair-force kernels
// (force.cuh, compiled per interaction kind in kernels_force_*.cu).
//
// Every kernel runs over all slots of all systems of an engine; a block never
// straddles two systems (blocks of <= 256 threads, systems padded to 256
// slots), so per-system parameters are block-uniform.
#include "hmd_device.cuh"
#include "kernels.h"

namespace hmd {

// ---------------------------------------------------------------------------
// integrate: first half of velocity Verlet (mdsim/gpu/integrators/verlet_kernel.cu:38-72)
//   v += F dt/(2m); r += v dt; image += rint(r/L); r -= image L
// fused with |r - r0|^2 (mdsim/gpu/max_displacement_kernel.cu:37-68) and,
// in the last block to finish, the per-system rebuild decision
// (from_binning.cpp:130: displacement > skin/2), which also drives the
// conditional rebuild node of a captured step graph.
// ---------------------------------------------------------------------------

// kick = false: Euler (mdsim/gpu/integrators/euler_kernel.cu:38-60), r += v dt only
template <bool DS>
__device__ __forceinline__ void integrate_component(float& rh, float& rl, float& vh, float& vl, float& im,
                                                    float f, float m, float dt, float dt_half, float L, float Linv,
                                                    bool kick = true)
{
    float a = __fmul_rn(f, dt_half);
    if (m != 1.0f) a = __fdiv_rn(a, m);   // x / 1 == x exactly: skip the division for unit masses
    float k;
    if (DS) {
        float v0 = vh, v1 = vl, d0, d1, r0, r1;
        if (kick) ds_add(v0, v1, vh, vl, a, 0.0f);
        ds_mul(d0, d1, v0, v1, dt, 0.0f);
        ds_add(r0, r1, rh, rl, d0, d1);
        k = rintf(__fmul_rn(r0, Linv));
        ds_sub(r0, r1, r0, r1, __fmul_rn(k, L), 0.0f);
        vh = v0; vl = v1; rh = r0; rl = r1;
    } else {
        float v = kick ? __fadd_rn(vh, a) : vh;
        float r = __fadd_rn(rh, __fmul_rn(v, dt));
        k = rintf(__fmul_rn(r, Linv));
        r = __fsub_rn(r, __fmul_rn(k, L));
        vh = v; rh = r;
    }
    im = __fadd_rn(im, k);
}

// Steepest descent (energy minimisation of a start configuration; no
// counterpart in the reference): each particle moves by descent_step * F,
// shortened to descent_max.  A non-finite force (two particles almost on
// top of each other) moves the particle by descent_max along its infinite
// components, or not at all when a component is NaN.
__device__ __forceinline__ float3 descent_move(float4 f, float step, float dmax)
{
    float3 g = make_float3(__fmul_rn(f.x, step), __fmul_rn(f.y, step), __fmul_rn(f.z, step));
    if (isnan(g.x) || isnan(g.y) || isnan(g.z)) return make_float3(0.0f, 0.0f, 0.0f);
    const bool inf = isinf(g.x) || isinf(g.y) || isinf(g.z);
    if (inf) {
        g.x = isinf(g.x) ? copysignf(1.0f, g.x) : 0.0f;
        g.y = isinf(g.y) ? copysignf(1.0f, g.y) : 0.0f;
        g.z = isinf(g.z) ? copysignf(1.0f, g.z) : 0.0f;
    }
    const float m = fmaxf(fabsf(g.x), fmaxf(fabsf(g.y), fabsf(g.z)));
    if (m == 0.0f) return g;
    const float ux = g.x / m, uy = g.y / m, uz = g.z / m;   // scaled: no overflow in the norm
    const float len = m * sqrtf(ux * ux + uy * uy + uz * uz);
    if (inf || len > dmax) {
        const float c = dmax / len;
        g.x *= c; g.y *= c; g.z *= c;
    }
    return g;
}

template <bool DS>
__device__ __forceinline__ void descend_component(float& rh, float& rl, float& im, float g, float L, float Linv)
{
    float k;
    if (DS) {
        float r0, r1;
        ds_add(r0, r1, rh, rl, g, 0.0f);
        k = rintf(__fmul_rn(r0, Linv));
        ds_sub(r0, r1, r0, r1, __fmul_rn(k, L), 0.0f);
        rh = r0; rl = r1;
    } else {
        float r = __fadd_rn(rh, g);
        k = rintf(__fmul_rn(r, Linv));
        rh = __fsub_rn(r, __fmul_rn(k, L));
    }
    im = __fadd_rn(im, k);
}

// ---------------------------------------------------------------------------
// finalize: second half-kick (verlet_kernel.cu:78-98) or Andersen
// (per-particle collisions with the heat bath, host convention
// mdsim/host/integrators/verlet_nvt_andersen.cpp:111-137; Philox4x32-10
// streams keyed by (seed, particle tag, step) so results do not depend on
// particle order or on which other systems share the launch)
// ---------------------------------------------------------------------------

template <bool DS>
__device__ __forceinline__ void half_kick(float& vh, float& vl, float f, float m, float dt_half)
{
    float a = __fmul_rn(f, dt_half);
    if (m != 1.0f) a = __fdiv_rn(a, m);
    if (DS) {
        float v0, v1;
        ds_add(v0, v1, vh, vl, a, 0.0f);
        vh = v0; vl = v1;
    } else {
        vh = __fadd_rn(vh, a);
    }
}

// verlet_nvt_boltzmann draws new velocities at the finalize of every step
// that is a multiple of the coupling interval (verlet_nvt_boltzmann.lua.in)
__device__ __forceinline__ bool boltzmann_due(const SysParam& P, const SysState& st)
{
    return P.integrator == INTEG_BOLTZMANN && st.step % P.interval == 0ull;
}

// Maxwell-Boltzmann velocity of one particle for the draw of step `step`
// (velocities/boltzmann_kernel.cu:47-100: each component N(0, sqrt(T)), then
// divided by sqrt(m)); Philox4x32-10 keyed by (seed, tag, step) with a
// stream word of its own, Box-Muller as the Andersen collisions
__device__ __forceinline__ float3 boltzmann_draw(const SysParam& P, uint32_t tag, unsigned long long step, float m)
{
    const uint4 w = philox4x32_10(make_uint4(tag, (uint32_t)step, (uint32_t)(step >> 32), 0x424F4C5Au),
                                  P.seed_lo, P.seed_hi);
    const float rad0 = sqrtf(-2.0f * logf(u01(w.x)));
    const float rad1 = sqrtf(-2.0f * logf(u01(w.z)));
    float sn0, cs0, sn1, cs1;
    sincospif(2.0f * u01(w.y), &sn0, &cs0);
    sincospif(2.0f * u01(w.w), &sn1, &cs1);
    float3 v = make_float3(P.sqrt_T * rad0 * cs0, P.sqrt_T * rad0 * sn0, P.sqrt_T * rad1 * cs1);
    if (m != 1.0f) {
        const float q = sqrtf(m);
        v = make_float3(__fdiv_rn(v.x, q), __fdiv_rn(v.y, q), __fdiv_rn(v.z, q));
    }
    return v;
}

// the second half of step st.step of slot i, on velocities held in registers
template <bool DS>
__device__ __forceinline__ void finalize_slot(const Dev& d, const SysParam& P, const SysState& st, uint32_t i,
                                              float4& v, float4& vl, float4 f)
{
    if (P.integrator == INTEG_EULER) return;
    if (boltzmann_due(P, st)) {
        const float3 u = boltzmann_draw(P, d.id[i], st.step, v.w);
        v.x = u.x; v.y = u.y; v.z = u.z;
        vl = make_float4(0, 0, 0, vl.w);
        return;
    }
    if (P.integrator == INTEG_ANDERSEN) {
        const unsigned long long step = st.step - 1ull;
        const uint4 ctr = make_uint4(d.id[i], (uint32_t)step, (uint32_t)(step >> 32), 0x414E4452u);
        const uint4 u = philox4x32_10(ctr, P.seed_lo, P.seed_hi);
        if (u.x < P.coll_threshold) {
            const uint4 w = philox4x32_10(make_uint4(ctr.x, ctr.y, ctr.z, 0x414E4453u), P.seed_lo, P.seed_hi);
            const float rad0 = sqrtf(-2.0f * logf(u01(w.x)));
            const float rad1 = sqrtf(-2.0f * logf(u01(w.z)));
            float sn0, cs0, sn1, cs1;
            sincospif(2.0f * u01(w.y), &sn0, &cs0);
            sincospif(2.0f * u01(w.w), &sn1, &cs1);
            v.x = P.sqrt_T * rad0 * cs0;
            v.y = P.sqrt_T * rad0 * sn0;
            v.z = P.sqrt_T * rad1 * cs1;
            vl = make_float4(0, 0, 0, vl.w);
            return;
        }
    }
    half_kick<DS>(v.x, vl.x, f.x, v.w, P.dt_half);
    half_kick<DS>(v.y, vl.y, f.y, v.w, P.dt_half);
    half_kick<DS>(v.z, vl.z, f.z, v.w, P.dt_half);
}

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

// MOM: also the per-block moments of the new velocities (engines with a
// Nose-Hoover or Maxwell-Boltzmann thermostat)
template <bool DS, bool MOM>
__global__ void __launch_bounds__(256) k_finalize(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    const SysState& st = d.st[s];
    double acc[NMOM] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const bool run = P.active && st.live && *d.status == 0u && P.integrator != INTEG_DESCENT;   // block-uniform
    if (run && species_bits(d.pos[i].w) != PLACEHOLDER) {
        float4 v = d.vel[i];
        float4 vl = make_float4(0, 0, 0, 0);
        if (DS) vl = d.vel[d.S + i];
        finalize_slot<DS>(d, P, st, i, v, vl, d.force[i]);
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
    const float4 r = d.pos[i];
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
    if (species_bits(d.pos[i].w) == PLACEHOLDER) return;
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

// FIN: the finalize of the previous step (its force is in d.force) runs
// first, on the same registers: one pass over the phase space per step
// inside a captured chunk.  The per-system flags it reads (live,
// steps_left) are read before any block arrives at the decision that
// updates them, so both halves see the state of their own step.
template <bool DS, bool FIN>
__global__ void __launch_bounds__(256) k_integrate(Dev d, cudaGraphConditionalHandle h, int use_handle)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    SysState& st = d.st[s];
    const bool clean = *d.status == 0u;
    const bool live = P.active && st.steps_left != 0u && clean;
    const bool fin = FIN && P.active && st.live && clean && P.integrator != INTEG_DESCENT;
    float rr = 0.0f;
    if (fin && !live) {
        // the system finished with the previous step: its last half-kick only
        if (species_bits(d.pos[i].w) != PLACEHOLDER) {
            float4 v = d.vel[i];
            float4 vl = make_float4(0, 0, 0, 0);
            if (DS) vl = d.vel[d.S + i];
            finalize_slot<DS>(d, P, st, i, v, vl, d.force[i]);
            d.vel[i] = v;
            if (DS) d.vel[d.S + i] = vl;
        }
    }
    if (live) {
        float4 r = d.pos[i];
        if (species_bits(r.w) != PLACEHOLDER) {
            float4 v = d.vel[i];
            const float4 f = d.force[i];
            float4 k = make_float4(0, 0, 0, 0);   // box images crossed in this step
            float4 rl = make_float4(0, 0, 0, 0), vl = make_float4(0, 0, 0, 0);
            if (DS) { rl = d.pos[d.S + i]; vl = d.vel[d.S + i]; }
            if (fin) finalize_slot<DS>(d, P, st, i, v, vl, f);
            if (P.integrator == INTEG_DESCENT) {   // block-uniform
                const float3 g = descent_move(f, P.descent_step, P.descent_max);
                descend_component<DS>(r.x, rl.x, k.x, g.x, P.L[0], P.Linv[0]);
                descend_component<DS>(r.y, rl.y, k.y, g.y, P.L[1], P.Linv[1]);
                descend_component<DS>(r.z, rl.z, k.z, g.z, P.L[2], P.Linv[2]);
                d.pos[i] = r;
                if (DS) d.pos[d.S + i] = rl;
            } else {
                const float m = v.w;
                if (P.integrator == INTEG_HOOVER) {   // block-uniform: v *= scale first (verlet_nvt_hoover_kernel.cu)
                    const float sc = st.scale;
                    if (DS) {
                        ds_mul(v.x, vl.x, v.x, vl.x, sc, 0.0f);
                        ds_mul(v.y, vl.y, v.y, vl.y, sc, 0.0f);
                        ds_mul(v.z, vl.z, v.z, vl.z, sc, 0.0f);
                    } else {
                        v.x = __fmul_rn(v.x, sc); v.y = __fmul_rn(v.y, sc); v.z = __fmul_rn(v.z, sc);
                    }
                }
                const bool kick = P.integrator != INTEG_EULER;
                integrate_component<DS>(r.x, rl.x, v.x, vl.x, k.x, f.x, m, P.dt, P.dt_half, P.L[0], P.Linv[0], kick);
                integrate_component<DS>(r.y, rl.y, v.y, vl.y, k.y, f.y, m, P.dt, P.dt_half, P.L[1], P.Linv[1], kick);
                integrate_component<DS>(r.z, rl.z, v.z, vl.z, k.z, f.z, m, P.dt, P.dt_half, P.L[2], P.Linv[2], kick);
                d.pos[i] = r;
                d.vel[i] = v;
                if (DS) { d.pos[d.S + i] = rl; d.vel[d.S + i] = vl; }
            }
            if (k.x != 0.0f || k.y != 0.0f || k.z != 0.0f) {
                // image counters are read and written only on a wrap
                float4 im = d.img[i];
                im.x = __fadd_rn(im.x, k.x);
                im.y = __fadd_rn(im.y, k.y);
                im.z = __fadd_rn(im.z, k.z);
                d.img[i] = im;
            }
            const float4 q = d.r0[i];
            float dx = min_image(__fsub_rn(r.x, q.x), P.L[0], P.Linv[0]);
            float dy = min_image(__fsub_rn(r.y, q.y), P.L[1], P.Linv[1]);
            float dz = min_image(__fsub_rn(r.z, q.z), P.L[2], P.Linv[2]);
            rr = rr_exact(dx, dy, dz);
        }
    }
    __shared__ float s_max[8];
    __shared__ bool s_last;
    rr = warp_max(rr);
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = rr;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = s_max[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) b = fmaxf(b, s_max[w]);
        if (b > 0.0f) atomicMax(&st.disp2_bits, __float_as_uint(b));
        __threadfence();
        s_last = (atomicAdd(d.done, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const bool ok = (*(volatile uint32_t*)d.status == 0u);
    uint32_t any = 0;
    for (uint32_t q = threadIdx.x; q < d.nsys; q += blockDim.x) {
        SysState& t = d.st[q];
        const SysParam& Q = d.sys[q];
        const bool lv = ok && Q.active && t.steps_left != 0u;
        const float disp = __uint_as_float(atomicExch(&t.disp2_bits, 0u));
        const uint32_t rb = lv && (disp > Q.rr_half_skin || t.rebuild_request != 0u);
        t.rebuild = rb;
        t.live = lv;
        if (lv) {
            t.rebuild_request = 0u;
            t.step += 1ull;
            if (t.steps_left != 0xFFFFFFFFu) t.steps_left -= 1u;
            if (rb) t.rebuilds += 1ull;
        }
        any |= rb;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        *d.done = 0u;
        d.any_rebuild[0] = any ? 1u : 0u;
        d.any_rebuild[1] += any ? 1u : 0u;
        if (use_handle) cudaGraphSetConditional(h, any ? 1u : 0u);
    }
}

// Mark systems live for a force evaluation outside a step (set-up, or a
// force requested through the module interface); `rebuild_all` also flags
// every active system for a list rebuild.
__global__ void k_mark(Dev d, int rebuild_all)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < d.nsys; q += gridDim.x * blockDim.x) {
        SysState& t = d.st[q];
        const bool lv = d.sys[q].active != 0u;
        t.live = lv;
        t.rebuild = (lv && (rebuild_all || t.rebuild_request)) ? 1u : 0u;
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
    const float4 r = d.pos[i];
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

void launch_integrate(const Dev& d, bool ds, cudaGraphConditionalHandle h, bool use_handle, cudaStream_t st)
{
    const unsigned grid = d.S / 256;
    if (ds) k_integrate<true, false><<<grid, 256, 0, st>>>(d, h, use_handle ? 1 : 0);
    else k_integrate<false, false><<<grid, 256, 0, st>>>(d, h, use_handle ? 1 : 0);
}

void launch_finalize_integrate(const Dev& d, bool ds, cudaGraphConditionalHandle h, cudaStream_t st)
{
    const unsigned grid = d.S / 256;
    if (ds) k_integrate<true, true><<<grid, 256, 0, st>>>(d, h, 1);
    else k_integrate<false, true><<<grid, 256, 0, st>>>(d, h, 1);
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
    if (d.force_kinds == 0u) {
        launch_force_kind<FK_GENERIC>(d, aux, st);
        return;
    }
    if (d.force_kinds & (1u << FK_LJ1)) launch_force_kind<FK_LJ1>(d, aux, st);
    if (d.force_kinds & (1u << FK_SHIFTED)) launch_force_kind<FK_SHIFTED>(d, aux, st);
    if (d.force_kinds & (1u << FK_SMOOTH)) launch_force_kind<FK_SMOOTH>(d, aux, st);
    if (d.force_kinds & (1u << FK_FSHIFT)) launch_force_kind<FK_FSHIFT>(d, aux, st);
    if (d.force_kinds & (1u << FK_POT)) launch_force_kind<FK_POT>(d, aux, st);
}

// engines with a Nose-Hoover or Maxwell-Boltzmann system: the finalize
// writes the moments of the new velocities, one block per system runs the
// thermostat, and the velocities are rescaled or shifted
void launch_finalize(const Dev& d, bool ds, cudaStream_t st)
{
    const unsigned grid = d.S / 256;
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
    k_moments<<<d.S / 256, 256, 0, st>>>(d);
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
    k_thermo_partial<<<d.S / 256, 256, 0, st>>>(d);
    k_thermo_reduce<<<d.nsys, 256, 0, st>>>(d);
}

} // namespace hmd
