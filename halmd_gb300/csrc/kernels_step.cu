// kernels_step.cu — per-step kernels: velocity-Verlet integrate (fused with the
// maximum-displacement reduction and the rebuild decision), truncated LJ pair
// force from the neighbour list, Verlet / Andersen finalize, FP64 reductions.
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

template <bool DS>
__device__ __forceinline__ void integrate_component(float& rh, float& rl, float& vh, float& vl, float& im,
                                                    float f, float m, float dt, float dt_half, float L, float Linv)
{
    float a = __fmul_rn(f, dt_half);
    if (m != 1.0f) a = __fdiv_rn(a, m);   // x / 1 == x exactly: skip the division for unit masses
    float k;
    if (DS) {
        float v0, v1, d0, d1, r0, r1;
        ds_add(v0, v1, vh, vl, a, 0.0f);
        ds_mul(d0, d1, v0, v1, dt, 0.0f);
        ds_add(r0, r1, rh, rl, d0, d1);
        k = rintf(__fmul_rn(r0, Linv));
        ds_sub(r0, r1, r0, r1, __fmul_rn(k, L), 0.0f);
        vh = v0; vl = v1; rh = r0; rl = r1;
    } else {
        float v = __fadd_rn(vh, a);
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

// the second half of step st.step of slot i, on velocities held in registers
template <bool DS>
__device__ __forceinline__ void finalize_slot(const Dev& d, const SysParam& P, const SysState& st, uint32_t i,
                                              float4& v, float4& vl, float4 f)
{
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

template <bool DS>
__global__ void __launch_bounds__(256) k_finalize(Dev d)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = d.chunk_sys[i / CHUNK];
    const SysParam& P = d.sys[s];
    const SysState& st = d.st[s];
    if (!P.active || !st.live || *d.status != 0u || P.integrator == INTEG_DESCENT) return;
    if (species_bits(d.pos[i].w) == PLACEHOLDER) return;
    float4 v = d.vel[i];
    float4 vl = make_float4(0, 0, 0, 0);
    if (DS) vl = d.vel[d.S + i];
    finalize_slot<DS>(d, P, st, i, v, vl, d.force[i]);
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
                integrate_component<DS>(r.x, rl.x, v.x, vl.x, k.x, f.x, m, P.dt, P.dt_half, P.L[0], P.Linv[0]);
                integrate_component<DS>(r.y, rl.y, v.y, vl.y, k.y, f.y, m, P.dt, P.dt_half, P.L[1], P.Linv[1]);
                integrate_component<DS>(r.z, rl.z, v.z, vl.z, k.z, f.z, m, P.dt, P.dt_half, P.L[2], P.Linv[2]);
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
// pair force (mdsim/gpu/forces/pair_trunc_kernel.cuh:165-255)
//   F_i = Σ_j fval(r_ij²) r_ij over list entries with r_ij² < r_c²;
//   aux: E_i = ½ Σ U, stress_i = ½ Σ fval r⊗r (full list, weight ½,
//   pair_trunc.hpp:291-294).
// FP32 math; each force component is accumulated with Knuth's TwoSum and
// a running compensation term, so the per-particle sum is as accurate as a
// double-single accumulator (the reference uses dsfloat, :194).
// The within-range test uses the same rounded squared distance as the list
// build, so the pair set is reproducible on the CPU.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void two_sum_acc(float& s, float& c, float x)
{
    const float t = __fadd_rn(s, x);
    const float z = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z));
    s = t;
    c = __fadd_rn(c, e);
}

// error of s = fl(a + b) (Knuth TwoSum)
__device__ __forceinline__ float two_sum_err(float a, float b, float s)
{
    const float bp = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// error of s = fl(a + b) for a, b >= 0 (Dekker's Fast2Sum on the ordered pair)
__device__ __forceinline__ float fast_err_pos(float a, float b, float s)
{
    return __fsub_rn(fminf(a, b), __fsub_rn(s, fmaxf(a, b)));
}

// LJ + truncation (lennard_jones_kernel.hpp:44-56, truncations/*_kernel.cuh).
// Compensated LJ for close pairs, whose forces can be an order of magnitude
// above the particle's net force: the squared distance arrives as a (hi, lo)
// pair, the reciprocal is refined against it, the float parameters sigma^2
// and 48 eps / sigma^2 carry their rounding errors, and every product of
// fval = 48 eps/sigma^2 rri^4 (rri^3 - 1/2) keeps its exact residual (FMA),
// so fval + flo is accurate to first order in the float roundings (the
// steep r^-14 law would otherwise amplify them seven-fold).  The smoothing
// factors (smooth_r4) and the force shift use approximate reciprocal /
// square-root intrinsics: their errors scale forces that are already small
// near r_c.
template <int TR>
__device__ __forceinline__ void pair_eval(const PairParam& p, float rr, float rrl, float rri_smooth,
                                          float& fval, float& flo, float& en)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(rr));
    const float res = __fmaf_rn(-rrl, y, __fmaf_rn(-rr, y, 1.0f));
    const float ylo = __fmul_rn(y, res);
    const float rri = __fmul_rn(p.sigma2, y);
    float rril = __fmaf_rn(p.sigma2, ylo, __fmaf_rn(p.sigma2, y, -rri));
    rril = __fmaf_rn(p.sigma2_lo, y, rril);
    const float t1 = __fmul_rn(rri, rri);
    const float ri6 = __fmul_rn(t1, rri);
    const float a = __fmul_rn(p.c48, rri);
    const float b = __fmul_rn(a, ri6);
    const float u = __fsub_rn(ri6, 0.5f);
    fval = __fmul_rn(b, u);
    // residuals: ri6 = rri^3, u = ri6 - 1/2, a = c48 rri, b = a ri6, fval = b u
    float ri6l = __fmaf_rn(__fmaf_rn(rri, rri, -t1), rri, __fmaf_rn(t1, rri, -ri6));
    ri6l = __fmaf_rn(__fmul_rn(3.0f, t1), rril, ri6l);
    const float ul = __fadd_rn(two_sum_err(ri6, -0.5f, u), ri6l);
    float al = __fmaf_rn(p.c48, rril, __fmaf_rn(p.c48, rri, -a));
    al = __fmaf_rn(p.c48_lo, rri, al);
    const float bl = __fmaf_rn(a, ri6l, __fmaf_rn(al, ri6, __fmaf_rn(a, ri6, -b)));
    flo = __fmaf_rn(b, ul, __fmaf_rn(bl, u, __fmaf_rn(b, u, -fval)));
    en = p.eps4 * ri6 * (ri6 - 1.0f) - p.en_cut;
    if (TR == TRUNC_SMOOTH_R4) {
        const float rinv = rsqrtf(rr);
        const float r = rr * rinv;
        const float dr = r - p.r_cut;
        const float x2 = dr * dr * rri_smooth;
        const float x4 = x2 * x2;
        const float x4i = __fdividef(1.0f, 1.0f + x4);
        const float h0 = x4 * x4i;
        const float h1 = 4.0f * dr * rri_smooth * x2 * x4i * x4i;
        fval = h0 * fval - h1 * (en * rinv);
        flo = h0 * flo;
        en = h0 * en;
    } else if (TR == TRUNC_FORCE_SHIFTED) {
        const float rinv = rsqrtf(rr);
        fval = fval - p.f_cut * rinv;
        en = en + (rr * rinv - p.r_cut) * p.f_cut;
    }
}

// plain FP32 evaluation for pairs that were farther than NEAR_SIGMA sigma at
// list build time (forces of order eps / sigma or less)
template <int TR>
__device__ __forceinline__ void pair_eval_fast(const PairParam& p, float rr, float rri_smooth, float& fval, float& en)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(rr));
    const float rri = p.sigma2 * y;
    const float ri6 = rri * rri * rri;
    fval = p.c48 * rri * ri6 * (ri6 - 0.5f);
    en = p.eps4 * ri6 * (ri6 - 1.0f) - p.en_cut;
    if (TR == TRUNC_SMOOTH_R4) {
        const float rinv = rsqrtf(rr);
        const float dr = rr * rinv - p.r_cut;
        const float x2 = dr * dr * rri_smooth;
        const float x4 = x2 * x2;
        const float x4i = __fdividef(1.0f, 1.0f + x4);
        const float h0 = x4 * x4i;
        const float h1 = 4.0f * dr * rri_smooth * x2 * x4i * x4i;
        fval = h0 * fval - h1 * (en * rinv);
        en = h0 * en;
    } else if (TR == TRUNC_FORCE_SHIFTED) {
        const float rinv = rsqrtf(rr);
        fval = fval - p.f_cut * rinv;
        en = en + (rr * rinv - p.r_cut) * p.f_cut;
    }
}

struct ForceAcc {
    float fx = 0, fy = 0, fz = 0, cx = 0, cy = 0, cz = 0;   // compensated (near pairs)
    float gx = 0, gy = 0, gz = 0;                           // plain sums (far pairs)
    float en = 0, s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0;
};

// TR >= ONE_SPECIES: single-species system, the pair table has one entry
constexpr int ONE_SPECIES = 16;

// Pair-parameter lookup for a neighbour of species b; false when b is not a
// species of the system (lists hold real particles only: this keeps the
// table lookup in bounds)
template <bool NS1>
__device__ __forceinline__ bool pair_of(const PairParam* row, const PairParam& p1, uint32_t ns, float w,
                                        const PairParam*& pp)
{
    if (NS1) { pp = &p1; return true; }
    const uint32_t b = species_bits(w);
    if (b >= ns) return false;
    pp = row + b;
    return true;
}

// one near pair: compensated separation, squared distance and LJ value;
// WRAP = false when no particle of the warp can see a neighbour across the
// box: then rint(s/L) = 0 for every pair and the minimum-image arithmetic is
// skipped without changing any result
// EXACT: every coordinate of every particle of the warp is at least
// SysParam::exact_min from zero, so each near partner (closer than that half
// distance per coordinate) has the same sign and lies within a factor of two:
// ri - rj is exact (Sterbenz) and its TwoSum error is zero, so the
// error terms are dropped without changing any bit of the result
template <int TR, bool AUX, bool WRAP, bool EXACT>
__device__ __forceinline__ void near_pair(const PairParam& p, const SysParam& P, float4 ri, float4 rj, ForceAcc& A)
{
    const float sx = __fsub_rn(ri.x, rj.x);
    const float sy = __fsub_rn(ri.y, rj.y);
    const float sz = __fsub_rn(ri.z, rj.z);
    const float dx = WRAP ? min_image(sx, P.L[0], P.Linv[0]) : sx;
    const float dy = WRAP ? min_image(sy, P.L[1], P.Linv[1]) : sy;
    const float dz = WRAP ? min_image(sz, P.L[2], P.Linv[2]) : sz;
    const float px = __fmul_rn(dx, dx), py = __fmul_rn(dy, dy), pz = __fmul_rn(dz, dz);
    const float pxy = __fadd_rn(px, py);
    const float rr = __fadd_rn(pxy, pz);   // == rr_exact(dx, dy, dz)
    if (!(rr < p.rr_cut)) return;
    // dx - k L is exact (k = 0, or Sterbenz for k = +-1): the difference
    // error is the TwoSum error of ri - rj
    float dxl = 0.0f, dyl = 0.0f, dzl = 0.0f;
    if (!EXACT) {
        dxl = two_sum_err(ri.x, -rj.x, sx);
        dyl = two_sum_err(ri.y, -rj.y, sy);
        dzl = two_sum_err(ri.z, -rj.z, sz);
    }
    float rrl = __fadd_rn(__fadd_rn(__fmaf_rn(dx, dx, -px), __fmaf_rn(dy, dy, -py)), __fmaf_rn(dz, dz, -pz));
    rrl = __fadd_rn(rrl, __fadd_rn(fast_err_pos(px, py, pxy), fast_err_pos(pxy, pz, rr)));
    if (!EXACT) rrl = __fmaf_rn(2.0f, __fmaf_rn(dx, dxl, __fmaf_rn(dy, dyl, __fmul_rn(dz, dzl))), rrl);
    float fval, flo, e;
    pair_eval<TR>(p, rr, rrl, P.rri_smooth, fval, flo, e);
    const float tx = __fmul_rn(fval, dx), ty = __fmul_rn(fval, dy), tz = __fmul_rn(fval, dz);
    two_sum_acc(A.fx, A.cx, tx);
    two_sum_acc(A.fy, A.cy, ty);
    two_sum_acc(A.fz, A.cz, tz);
    float cx = __fadd_rn(A.cx, __fmaf_rn(fval, dx, -tx));
    float cy = __fadd_rn(A.cy, __fmaf_rn(fval, dy, -ty));
    float cz = __fadd_rn(A.cz, __fmaf_rn(fval, dz, -tz));
    if (!EXACT) {
        cx = __fmaf_rn(fval, dxl, cx);
        cy = __fmaf_rn(fval, dyl, cy);
        cz = __fmaf_rn(fval, dzl, cz);
    }
    A.cx = __fmaf_rn(flo, dx, cx);
    A.cy = __fmaf_rn(flo, dy, cy);
    A.cz = __fmaf_rn(flo, dz, cz);
    if (AUX) {
        A.en += e;
        A.s0 += fval * dx * dx;
        A.s1 += fval * dy * dy;
        A.s2 += fval * dz * dz;
        A.s3 += fval * dx * dy;
        A.s4 += fval * dx * dz;
        A.s5 += fval * dy * dz;
    }
}

// one far pair: plain FP32 (forces of order eps / sigma or less)
template <int TR, bool AUX, bool WRAP>
__device__ __forceinline__ void far_pair(const PairParam& p, const SysParam& P, float4 ri, float4 rj, ForceAcc& A)
{
    const float sx = __fsub_rn(ri.x, rj.x);
    const float sy = __fsub_rn(ri.y, rj.y);
    const float sz = __fsub_rn(ri.z, rj.z);
    float dx = WRAP ? min_image(sx, P.L[0], P.Linv[0]) : sx;
    float dy = WRAP ? min_image(sy, P.L[1], P.Linv[1]) : sy;
    float dz = WRAP ? min_image(sz, P.L[2], P.Linv[2]) : sz;
    float rr = rr_exact(dx, dy, dz);
    if (!(rr < p.rr_cut)) return;
    if (WRAP) {
        // across the box ri - rj is of order L and its rounding error (up to
        // ulp(L)/2) would dominate the separation error: add the TwoSum error
        // back (the cut-off decision above keeps the rounded rr of the list
        // criterion)
        dx = __fadd_rn(dx, two_sum_err(ri.x, -rj.x, sx));
        dy = __fadd_rn(dy, two_sum_err(ri.y, -rj.y, sy));
        dz = __fadd_rn(dz, two_sum_err(ri.z, -rj.z, sz));
        rr = rr_exact(dx, dy, dz);
    }
    float fval, e;
    pair_eval_fast<TR>(p, rr, P.rri_smooth, fval, e);
    A.gx = __fmaf_rn(fval, dx, A.gx);
    A.gy = __fmaf_rn(fval, dy, A.gy);
    A.gz = __fmaf_rn(fval, dz, A.gz);
    if (AUX) {
        A.en += e;
        A.s0 += fval * dx * dx;
        A.s1 += fval * dy * dy;
        A.s2 += fval * dz * dz;
        A.s3 += fval * dx * dy;
        A.s4 += fval * dx * dz;
        A.s5 += fval * dy * dz;
    }
}

// E list entries per lane and block, read with one vector load
template <int E> struct IdxVec;
template <> struct IdxVec<1> { using T = uint32_t; };
template <> struct IdxVec<2> { using T = uint2; };
template <> struct IdxVec<4> { using T = uint4; };
__device__ __forceinline__ uint32_t idx_at(uint32_t v, int) { return v; }
__device__ __forceinline__ uint32_t idx_at(uint2 v, int e) { return e == 0 ? v.x : v.y; }
__device__ __forceinline__ uint32_t idx_at(uint4 v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }

// The list is stored in blocks of LB = W * E entries: entry k of slot i at
// ((k/LB)*S + i)*LB + k%LB, near entries from the front of the list, far
// entries from its back (entry k of the far part at list position cap-1-k).
// Lane q of the W lanes of a particle takes the E consecutive entries
// [q*E, q*E + E) of every block with one E-wide load, so a warp reads
// contiguous memory and each lane has E independent position gathers in
// flight.  Entries past the count are never dereferenced (the lane gathers
// its own position instead).
template <int W, int E, int TRX, bool AUX, bool WRAP, bool FAR, bool EXACT = false>
__device__ __forceinline__ void force_blocks(const Dev& d, uint32_t i, uint32_t q, uint32_t cnt, const SysParam& P,
                                             const PairParam* spp, float4 ri, uint32_t a, ForceAcc& A)
{
    constexpr bool NS1 = TRX >= ONE_SPECIES;
    constexpr int TR = TRX & (ONE_SPECIES - 1);
    constexpr uint32_t LB = W * E;
    using V = typename IdxVec<E>::T;
    const size_t bstride = (size_t)d.S;   // in V units: S * LB entries per block row / E
    const V* lst = reinterpret_cast<const V*>(d.nbr + (size_t)i * LB + q * E);
    if (FAR) lst += (size_t)(d.nbr_cap / LB - 1) * bstride * W;
    const ptrdiff_t step = FAR ? -(ptrdiff_t)(bstride * W) : (ptrdiff_t)(bstride * W);
    const uint32_t ns = P.ns;
    const PairParam* row = spp + a * ns;
    PairParam p1;
    if (NS1) p1 = spp[0];
    const uint32_t nblk = (cnt + LB - 1) / LB;
    for (uint32_t b = 0; b < nblk; ++b, lst += step) {
        const V jv = __ldg(lst);
        float4 rj[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t o = q * E + e;
            const uint32_t k = b * LB + (FAR ? LB - 1 - o : o);
            rj[e] = __ldg(d.pos + (k < cnt ? idx_at(jv, e) : i));
        }
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t o = q * E + e;
            const uint32_t k = b * LB + (FAR ? LB - 1 - o : o);
            const PairParam* pp;
            if (k >= cnt || !pair_of<NS1>(row, p1, ns, rj[e].w, pp)) continue;
            if (FAR) far_pair<TR, AUX, WRAP>(*pp, P, ri, rj[e], A);
            else near_pair<TR, AUX, WRAP, EXACT>(*pp, P, ri, rj[e], A);
        }
    }
}

template <int W, int E, int TR, bool AUX>
__device__ __forceinline__ void force_dispatch(const Dev& d, uint32_t i, uint32_t q, uint32_t nn, uint32_t nf,
                                               bool wrap, bool exact, const SysParam& P, const PairParam* spp,
                                               float4 ri, uint32_t a, ForceAcc& A)
{
    if (wrap) {
        force_blocks<W, E, TR, AUX, true, false>(d, i, q, nn, P, spp, ri, a, A);
        force_blocks<W, E, TR, AUX, true, true>(d, i, q, nf, P, spp, ri, a, A);
    } else {
        if (exact) force_blocks<W, E, TR, AUX, false, false, true>(d, i, q, nn, P, spp, ri, a, A);
        else force_blocks<W, E, TR, AUX, false, false>(d, i, q, nn, P, spp, ri, a, A);
        force_blocks<W, E, TR, AUX, false, true>(d, i, q, nf, P, spp, ri, a, A);
    }
    // fold the plain far-pair sums into the compensated accumulators
    two_sum_acc(A.fx, A.cx, A.gx);
    two_sum_acc(A.fy, A.cy, A.gy);
    two_sum_acc(A.fz, A.cz, A.gz);
}

// merge the compensated sums of the W lanes of a particle (fixed tree: deterministic)
template <int W>
__device__ __forceinline__ void lane_merge(float& s, float& c)
{
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xFFFFFFFFu, s, o, W);
        const float c2 = __shfl_xor_sync(0xFFFFFFFFu, c, o, W);
        const float t = __fadd_rn(s, s2);
        c = __fadd_rn(__fadd_rn(c, c2), two_sum_err(s, s2, t));
        s = t;
    }
}

template <int W>
__device__ __forceinline__ float lane_sum(float v)
{
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o, W);
    return v;
}

template <int W, int E, bool AUX>
__global__ void __launch_bounds__(128) k_force(Dev d)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t / W, q = t % W;
    const uint32_t s = d.chunk_sys[(blockIdx.x * (blockDim.x / W)) / CHUNK];
    const SysParam& P = d.sys[s];
    __shared__ PairParam spp[MAX_SPECIES * MAX_SPECIES];
    const uint32_t np = P.ns * P.ns;
    if (threadIdx.x < np) spp[threadIdx.x] = d.pair[P.pair_off + threadIdx.x];
    __syncthreads();
    if (!P.active || !d.st[s].live || *d.status != 0u) return;   // block-uniform
    const float4 ri = d.pos[i];
    const uint32_t a = species_bits(ri.w);
    const bool real = a != PLACEHOLDER;
    const uint32_t packed = real ? d.nbr_count[i] : 0u;
    const uint32_t nn = packed & 0xFFFFu, nf = packed >> 16;   // near / far list parts
    const bool inner = !real || (fabsf(ri.x) < P.inner[0] && fabsf(ri.y) < P.inner[1] && fabsf(ri.z) < P.inner[2]);
    const bool wrap = __any_sync(0xFFFFFFFFu, !inner);
    const bool far_from_zero = !real || (fabsf(ri.x) >= P.exact_min && fabsf(ri.y) >= P.exact_min &&
                                         fabsf(ri.z) >= P.exact_min);
    const bool exact = __all_sync(0xFFFFFFFFu, far_from_zero);
    ForceAcc A;
    if (real) {
        switch (P.trunc) {
        case TRUNC_SHARP:
        case TRUNC_SHIFTED:
            if (P.ns == 1) force_dispatch<W, E, ONE_SPECIES + TRUNC_SHIFTED, AUX>(d, i, q, nn, nf, wrap, exact, P, spp, ri, a, A);
            else force_dispatch<W, E, TRUNC_SHIFTED, AUX>(d, i, q, nn, nf, wrap, exact, P, spp, ri, a, A);
            break;
        case TRUNC_SMOOTH_R4: force_dispatch<W, E, TRUNC_SMOOTH_R4, AUX>(d, i, q, nn, nf, wrap, exact, P, spp, ri, a, A); break;
        default: force_dispatch<W, E, TRUNC_FORCE_SHIFTED, AUX>(d, i, q, nn, nf, wrap, exact, P, spp, ri, a, A); break;
        }
    }
    lane_merge<W>(A.fx, A.cx);
    lane_merge<W>(A.fy, A.cy);
    lane_merge<W>(A.fz, A.cz);
    if (AUX) {
        A.en = lane_sum<W>(A.en);
        A.s0 = lane_sum<W>(A.s0); A.s1 = lane_sum<W>(A.s1); A.s2 = lane_sum<W>(A.s2);
        A.s3 = lane_sum<W>(A.s3); A.s4 = lane_sum<W>(A.s4); A.s5 = lane_sum<W>(A.s5);
    }
    if (!real || q != 0) return;
    d.force[i] = make_float4(A.fx + A.cx, A.fy + A.cy, A.fz + A.cz, 0.0f);
    if (AUX) {
        const size_t stride = d.S;
        d.en_pot[i] = 0.5f * A.en;
        float* sp = d.stress + i;
        sp[0 * stride] = 0.5f * A.s0;
        sp[1 * stride] = 0.5f * A.s1;
        sp[2 * stride] = 0.5f * A.s2;
        sp[3 * stride] = 0.5f * A.s3;
        sp[4 * stride] = 0.5f * A.s4;
        sp[5 * stride] = 0.5f * A.s5;
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

template <int W, int E>
static void launch_force_w(const Dev& d, bool aux, cudaStream_t st)
{
    const unsigned grid = (unsigned)((size_t)d.S * W / 128);
    if (aux) k_force<W, E, true><<<grid, 128, 0, st>>>(d);
    else k_force<W, E, false><<<grid, 128, 0, st>>>(d);
}

// (lanes, list block) shapes the engine accepts: E = block / lanes entries per load
void launch_force(const Dev& d, bool aux, cudaStream_t st)
{
    const uint32_t lb = 1u << d.lb_log2;
    switch (d.lanes * 16u + lb) {
    case 1 * 16 + 4: launch_force_w<1, 4>(d, aux, st); break;
    case 2 * 16 + 4: launch_force_w<2, 2>(d, aux, st); break;
    case 2 * 16 + 8: launch_force_w<2, 4>(d, aux, st); break;
    case 4 * 16 + 4: launch_force_w<4, 1>(d, aux, st); break;
    case 4 * 16 + 8: launch_force_w<4, 2>(d, aux, st); break;
    default: launch_force_w<8, 1>(d, aux, st); break;
    }
}

void launch_finalize(const Dev& d, bool ds, cudaStream_t st)
{
    const unsigned grid = d.S / 256;
    if (ds) k_finalize<true><<<grid, 256, 0, st>>>(d);
    else k_finalize<false><<<grid, 256, 0, st>>>(d);
}

void launch_thermo(const Dev& d, cudaStream_t st)
{
    k_thermo_partial<<<d.S / 256, 256, 0, st>>>(d);
    k_thermo_reduce<<<d.nsys, 256, 0, st>>>(d);
}

} // namespace hmd
