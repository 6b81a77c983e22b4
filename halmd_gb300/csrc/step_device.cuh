// step_device.cuh — the per-slot halves of a velocity-Verlet step used by
// the integrate kernels (kernels_step.cu): integrate (verlet_kernel.cu:38-72),
// finalize (verlet_kernel.cu:78-98, Andersen, Maxwell-Boltzmann draws),
// steepest descent, and the end-of-step decision.
#pragma once

#include "hmd_device.cuh"

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

// The words of one slot that a step reads.  None depends on the per-system
// parameters, so the step kernels load them first, unconditionally (every
// slot index is a valid address): one round of memory latency then covers
// both instead of the parameters' round followed by the slot's.
template <bool DS>
struct SlotIn {
    float4 r, rl, v, vl, f, q;   // position hi / lo, velocity hi / lo, force, r0
};

template <bool DS>
__device__ __forceinline__ SlotIn<DS> load_slot(const Dev& d, uint32_t i)
{
    SlotIn<DS> in;
    in.r = pos_hi(d.pos, i);
    in.rl = DS ? pos_lo(d.pos, i) : make_float4(0, 0, 0, 0);
    in.v = d.vel[i];
    in.vl = DS ? d.vel[d.S + i] : make_float4(0, 0, 0, 0);
    in.f = d.force[i];
    in.q = d.r0[i];
    return in;
}

// One slot of a step: the finalize of the previous step (FIN and fin: its
// force in.f) and the integrate of this one (live).  Only slots that
// finalize or integrate are written.  Returns |r - r0|^2 of an integrated
// slot, else 0.
template <bool DS, bool FIN>
__device__ __forceinline__ float step_slot(const Dev& d, const SysParam& P, const SysState& st, uint32_t i,
                                           const SlotIn<DS>& in, bool fin, bool live)
{
    float rr = 0.0f;
    float4 r = in.r;
    float4 rl = in.rl;
    const float4 f = in.f;
    const bool real = species_bits(r.w) != PLACEHOLDER;
    if (FIN && fin && !live && real) {
        // the system finished with the previous step: its last half-kick only
        float4 v = in.v;
        float4 vl = in.vl;
        finalize_slot<DS>(d, P, st, i, v, vl, f);
        d.vel[i] = v;
        if (DS) d.vel[d.S + i] = vl;
    }
    if (live && real) {
        float4 v = in.v;
        float4 k = make_float4(0, 0, 0, 0);   // box images crossed in this step
        float4 vl = in.vl;
        if (FIN && fin) finalize_slot<DS>(d, P, st, i, v, vl, f);
        if (P.integrator == INTEG_DESCENT) {   // block-uniform
            const float3 g = descent_move(f, P.descent_step, P.descent_max);
            descend_component<DS>(r.x, rl.x, k.x, g.x, P.L[0], P.Linv[0]);
            descend_component<DS>(r.y, rl.y, k.y, g.y, P.L[1], P.Linv[1]);
            descend_component<DS>(r.z, rl.z, k.z, g.z, P.L[2], P.Linv[2]);
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
            d.vel[i] = v;
            if (DS) d.vel[d.S + i] = vl;
        }
        pos_hi(d.pos, i) = r;
        if (DS) {
            pos_lo(d.pos, i) = rl;
            d.fpos[i] = fpos_encode(r, rl, P.lo_inv_scale);
        }
        if (k.x != 0.0f || k.y != 0.0f || k.z != 0.0f) {
            // image counters are read and written only on a wrap
            float4 im = d.img[i];
            im.x = __fadd_rn(im.x, k.x);
            im.y = __fadd_rn(im.y, k.y);
            im.z = __fadd_rn(im.z, k.z);
            d.img[i] = im;
        }
        const float4 q = in.q;
        float dx = min_image(__fsub_rn(r.x, q.x), P.L[0], P.Linv[0]);
        float dy = min_image(__fsub_rn(r.y, q.y), P.L[1], P.Linv[1]);
        float dz = min_image(__fsub_rn(r.z, q.z), P.L[2], P.Linv[2]);
        rr = rr_exact(dx, dy, dz);
    }
    return rr;
}

// End of a step, by every thread of every block: the block's largest
// |r - r0|^2 into its system (from_binning.cpp:130 via
// max_displacement.cpp:60-106), and in the last block to finish the
// per-system decision of the next step (rebuild, live, step counters),
// which also sets the conditional rebuild node of a captured step graph.
__device__ __forceinline__ void step_decision(const Dev& d, SysState& st, float rr, cudaGraphConditionalHandle h,
                                              int use_handle)
{
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
        const uint32_t rb = lv && Q.trunc != TRUNC_NONE && (disp > Q.rr_half_skin || t.rebuild_request != 0u);
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

} // namespace hmd
