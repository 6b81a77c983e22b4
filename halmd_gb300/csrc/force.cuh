// force.cuh — truncated Lennard-Jones pair force from the neighbour list
// (mdsim/gpu/forces/pair_trunc_kernel.cuh, potentials/pair/lennard_jones_kernel.hpp,
// truncations/*_kernel.cuh).  The kernel is a template over the kind of pair
// interaction; kernels_force_*.cu compile one kind each, so every kind gets
// its own register allocation, and kernels_step.cu launches the kinds an
// engine holds.
#pragma once

#include "hmd_device.cuh"
#include "kernels.h"

namespace hmd {

// Resident blocks of 128 threads per SM that the register allocation aims
// for: 7 (72 registers a thread).  The kernel is bound by the latency of the
// list stream and the position gathers; at LJ-1M (one lane, four entries per
// load) it measured 173 us with 7 blocks and the list prefetch below, 183-192
// us with 8 blocks (64 registers, more spills) or without the prefetch, and
// 211-286 us with 5 or 6 blocks and no spills.
#ifndef HMD_FORCE_MINB
#define HMD_FORCE_MINB 7
#endif
// threads per block of the force kernel (a multiple of 32 that divides 256:
// systems are padded to 256 slots, so a block never straddles two)
#ifndef HMD_FORCE_THREADS
#define HMD_FORCE_THREADS 128
#endif
static_assert(HMD_FORCE_THREADS % 32 == 0 && 256 % HMD_FORCE_THREADS == 0, "force block size");
// Resident blocks for the kernels of dsfloat engines, whose gathers carry
// the lo words (16-byte records, hmd_device.cuh fpos_encode): at LJ-1M
// 215 us with 5 blocks against 214 us with 6 and 216 us with 7; at KA-64k
// 40.5 us against 43.5 and 41.8 us.
#ifndef HMD_FORCE_MINB_DS
#define HMD_FORCE_MINB_DS 5
#endif
// 1: load a lane's next list block one iteration ahead (force_blocks2)
#ifndef HMD_FORCE_PREFETCH
#define HMD_FORCE_PREFETCH 1
#endif

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
    // the energy from rri^3 with its residual: rrl carries the lo words of
    // dsfloat positions, which can shift a close pair's r^-12 by far more
    // than the float rounding
    const float ri6c = __fadd_rn(ri6, ri6l);
    en = p.eps4 * ri6c * (ri6c - 1.0f) - p.en_cut;
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
template <bool NS1, bool LO = false>
__device__ __forceinline__ bool pair_of(const PairParam* row, const PairParam& p1, uint32_t ns, float w,
                                        const PairParam*& pp)
{
    if (NS1) { pp = &p1; return true; }
    const uint32_t b = LO ? fpos_species(w) : species_bits(w);
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
// LO: dsfloat positions; li / lj are the lo words of the two particles, and
// the separation carries their difference in its residual, so the force is
// that of the double-single state, not of its float hi part
template <int TR, bool AUX, bool WRAP, bool EXACT, bool LO = false>
__device__ __forceinline__ void near_pair(const PairParam& p, const SysParam& P, float4 ri, float4 rj, ForceAcc& A,
                                          float4 li = float4(), float4 lj = float4())
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
    if (LO) {
        dxl = __fadd_rn(dxl, __fsub_rn(li.x, lj.x));
        dyl = __fadd_rn(dyl, __fsub_rn(li.y, lj.y));
        dzl = __fadd_rn(dzl, __fsub_rn(li.z, lj.z));
    }
    float rrl = __fadd_rn(__fadd_rn(__fmaf_rn(dx, dx, -px), __fmaf_rn(dy, dy, -py)), __fmaf_rn(dz, dz, -pz));
    rrl = __fadd_rn(rrl, __fadd_rn(fast_err_pos(px, py, pxy), fast_err_pos(pxy, pz, rr)));
    if (!EXACT || LO) rrl = __fmaf_rn(2.0f, __fmaf_rn(dx, dxl, __fmaf_rn(dy, dyl, __fmul_rn(dz, dzl))), rrl);
    float fval, flo, e;
    pair_eval<TR>(p, rr, rrl, P.rri_smooth, fval, flo, e);
    const float tx = __fmul_rn(fval, dx), ty = __fmul_rn(fval, dy), tz = __fmul_rn(fval, dz);
    two_sum_acc(A.fx, A.cx, tx);
    two_sum_acc(A.fy, A.cy, ty);
    two_sum_acc(A.fz, A.cz, tz);
    float cx = __fadd_rn(A.cx, __fmaf_rn(fval, dx, -tx));
    float cy = __fadd_rn(A.cy, __fmaf_rn(fval, dy, -ty));
    float cz = __fadd_rn(A.cz, __fmaf_rn(fval, dz, -tz));
    if (!EXACT || LO) {
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
template <int TR, bool AUX, bool WRAP, bool LO = false>
__device__ __forceinline__ void far_pair(const PairParam& p, const SysParam& P, float4 ri, float4 rj, ForceAcc& A,
                                         float4 li = float4(), float4 lj = float4())
{
    const float sx = __fsub_rn(ri.x, rj.x);
    const float sy = __fsub_rn(ri.y, rj.y);
    const float sz = __fsub_rn(ri.z, rj.z);
    float dx = WRAP ? min_image(sx, P.L[0], P.Linv[0]) : sx;
    float dy = WRAP ? min_image(sy, P.L[1], P.Linv[1]) : sy;
    float dz = WRAP ? min_image(sz, P.L[2], P.Linv[2]) : sz;
    float rr = rr_exact(dx, dy, dz);
    if (!(rr < p.rr_cut)) return;
    if (WRAP || LO) {
        // across the box ri - rj is of order L and its rounding error (up to
        // ulp(L)/2) would dominate the separation error: add the TwoSum error
        // back; dsfloat positions add the difference of the lo words.  The
        // cut-off decision above keeps the rounded rr of the list criterion;
        // rr takes the residual e to first order (|e| << |d|)
        float ex = 0.0f, ey = 0.0f, ez = 0.0f;
        if (WRAP) {
            ex = two_sum_err(ri.x, -rj.x, sx);
            ey = two_sum_err(ri.y, -rj.y, sy);
            ez = two_sum_err(ri.z, -rj.z, sz);
        }
        if (LO) {
            ex = __fadd_rn(ex, __fsub_rn(li.x, lj.x));
            ey = __fadd_rn(ey, __fsub_rn(li.y, lj.y));
            ez = __fadd_rn(ez, __fsub_rn(li.z, lj.z));
        }
        rr = __fmaf_rn(2.0f, __fmaf_rn(dx, ex, __fmaf_rn(dy, ey, __fmul_rn(dz, ez))), rr);
        dx = __fadd_rn(dx, ex);
        dy = __fadd_rn(dy, ey);
        dz = __fadd_rn(dz, ez);
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

// ---------------------------------------------------------------------------
// Two list entries per instruction.  The SMs of this GPU issue FP32 add,
// multiply and FMA on register pairs (f32x2): entries e and e+1 of a lane's
// list load are evaluated together, lane .x of every float2 holding entry e
// and lane .y entry e+1.  Each lane of an f32x2 operation rounds exactly as
// the scalar operation, so a pair's force value equals that of the scalar
// path above bit for bit; the per-particle sums run as two interleaved
// accumulators (even and odd entries) that are merged at the end.  The
// evaluation is branch-free: entries past the count, pairs outside r_c and
// neighbours of no species of the system are masked by selecting zero for
// their force value (the lane still evaluates them, as the warp would).
// ---------------------------------------------------------------------------

__device__ __forceinline__ float2 sel2(bool ka, bool kb, float2 v)
{
    return make_float2(ka ? v.x : 0.0f, kb ? v.y : 0.0f);
}

// error of s = fl(a - b) per lane (Knuth TwoSum of a and -b), a shared
__device__ __forceinline__ float2 diff_err2(float a, float bA, float bB, float2 s)
{
    const float2 bp = sub2(s, bc2(a));
    const float2 e1 = sub2(bc2(a), sub2(s, bp));
    return add2(e1, f2(__fsub_rn(-bA, bp.x), __fsub_rn(-bB, bp.y)));
}

__device__ __forceinline__ float2 two_sum_err2(float2 a, float2 b, float2 s)
{
    const float2 bp = sub2(s, a);
    return add2(sub2(a, sub2(s, bp)), sub2(b, bp));
}

__device__ __forceinline__ float2 fast_err_pos2(float2 a, float2 b, float2 s)
{
    const float2 mn = f2(fminf(a.x, b.x), fminf(a.y, b.y));
    const float2 mx = f2(fmaxf(a.x, b.x), fmaxf(a.y, b.y));
    return sub2(mn, sub2(s, mx));
}

__device__ __forceinline__ void two_sum_acc2(float2& s, float2& c, float2 x)
{
    const float2 t = add2(s, x);
    const float2 z = sub2(t, s);
    const float2 e = add2(sub2(s, sub2(t, z)), sub2(x, z));
    s = t;
    c = add2(c, e);
}

// the parameters of two pairs, lane by lane
// (16-byte aligned, the fields a far pair reads first in pairs: a table of
// these in shared memory is read with 16-byte loads, each half of every
// field already in place)
struct alignas(16) PP2 {
    float2 sigma2, c48, rr_cut, rr_tie, eps4, en_cut, r_cut, f_cut, sigma2_lo, c48_lo;
};

__device__ __forceinline__ PP2 pack_params(const PairParam& a, const PairParam& b)
{
    PP2 p;
    p.eps4 = f2(a.eps4, b.eps4);
    p.c48 = f2(a.c48, b.c48);
    p.sigma2 = f2(a.sigma2, b.sigma2);
    p.rr_cut = f2(a.rr_cut, b.rr_cut);
    p.en_cut = f2(a.en_cut, b.en_cut);
    p.r_cut = f2(a.r_cut, b.r_cut);
    p.f_cut = f2(a.f_cut, b.f_cut);
    p.sigma2_lo = f2(a.sigma2_lo, b.sigma2_lo);
    p.c48_lo = f2(a.c48_lo, b.c48_lo);
    p.rr_tie = f2(a.rr_tie, b.rr_tie);
    return p;
}

struct ForceAcc2 {
    float2 fx = {0, 0}, fy = {0, 0}, fz = {0, 0}, cx = {0, 0}, cy = {0, 0}, cz = {0, 0};
    float2 gx = {0, 0}, gy = {0, 0}, gz = {0, 0};
    float2 en = {0, 0}, s0 = {0, 0}, s1 = {0, 0}, s2 = {0, 0}, s3 = {0, 0}, s4 = {0, 0}, s5 = {0, 0};
};

// energy (needed by smooth_r4 and the aux sums) and the truncation factors
// of the force value, as in pair_eval / pair_eval_fast
template <int TR, bool NEAR>
__device__ __forceinline__ void truncate2(const PP2& p, float2 rr, float2 ri6, float rri_smooth, float2& fval,
                                          float2& flo, float2& en)
{
    en = sub2(mul2(mul2(p.eps4, ri6), sub2(ri6, bc2(1.0f))), p.en_cut);
    if (TR == TRUNC_SMOOTH_R4) {
        const float2 rinv = f2(rsqrtf(rr.x), rsqrtf(rr.y));
        const float2 dr = sub2(mul2(rr, rinv), p.r_cut);
        const float2 x2 = mul2(mul2(dr, dr), bc2(rri_smooth));
        const float2 x4 = mul2(x2, x2);
        const float2 den = add2(bc2(1.0f), x4);
        const float2 x4i = f2(__fdividef(1.0f, den.x), __fdividef(1.0f, den.y));
        const float2 h0 = mul2(x4, x4i);
        const float2 h1 = mul2(mul2(mul2(bc2(4.0f * rri_smooth), dr), x2), mul2(x4i, x4i));
        fval = fma2(h0, fval, neg2(mul2(h1, mul2(en, rinv))));
        if (NEAR) flo = mul2(h0, flo);
        en = mul2(h0, en);
    } else if (TR == TRUNC_FORCE_SHIFTED) {
        const float2 rinv = f2(rsqrtf(rr.x), rsqrtf(rr.y));
        fval = fma2(neg2(p.f_cut), rinv, fval);
        en = fma2(sub2(mul2(rr, rinv), p.r_cut), p.f_cut, en);
    }
}

// compensated LJ of two close pairs (pair_eval, lane by lane)
template <int TR>
__device__ __forceinline__ void pair_eval2(const PP2& p, float2 rr, float2 rrl, float rri_smooth, float2& fval,
                                           float2& flo, float2& en)
{
    float ya, yb;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ya) : "f"(rr.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yb) : "f"(rr.y));
    const float2 y = f2(ya, yb);
    const float2 res = fma2(neg2(rrl), y, fma2(neg2(rr), y, bc2(1.0f)));
    const float2 ylo = mul2(y, res);
    const float2 rri = mul2(p.sigma2, y);
    float2 rril = fma2(p.sigma2, ylo, fma2(p.sigma2, y, neg2(rri)));
    rril = fma2(p.sigma2_lo, y, rril);
    const float2 t1 = mul2(rri, rri);
    const float2 ri6 = mul2(t1, rri);
    const float2 a = mul2(p.c48, rri);
    const float2 b = mul2(a, ri6);
    const float2 u = sub2(ri6, bc2(0.5f));
    fval = mul2(b, u);
    float2 ri6l = fma2(fma2(rri, rri, neg2(t1)), rri, fma2(t1, rri, neg2(ri6)));
    ri6l = fma2(mul2(bc2(3.0f), t1), rril, ri6l);
    const float2 ul = add2(two_sum_err2(ri6, bc2(-0.5f), u), ri6l);
    float2 al = fma2(p.c48, rril, fma2(p.c48, rri, neg2(a)));
    al = fma2(p.c48_lo, rri, al);
    const float2 bl = fma2(a, ri6l, fma2(al, ri6, fma2(a, ri6, neg2(b))));
    flo = fma2(b, ul, fma2(bl, u, fma2(b, u, neg2(fval))));
    // energy from rri^3 with its residual (pair_eval)
    truncate2<TR, true>(p, rr, add2(ri6, ri6l), rri_smooth, fval, flo, en);
}

template <bool AUX>
__device__ __forceinline__ void aux_acc2(ForceAcc2& A, float2 fval, float2 en, float2 dx, float2 dy, float2 dz)
{
    if (AUX) {
        A.en = add2(A.en, en);
        const float2 fx = mul2(fval, dx), fy = mul2(fval, dy);
        A.s0 = fma2(fx, dx, A.s0);
        A.s1 = fma2(fy, dy, A.s1);
        A.s2 = fma2(mul2(fval, dz), dz, A.s2);
        A.s3 = fma2(fx, dy, A.s3);
        A.s4 = fma2(fx, dz, A.s4);
        A.s5 = fma2(fy, dz, A.s5);
    }
}

// two near pairs (near_pair, lane by lane); va / vb: the entry is a real
// neighbour of a species of the system
// (LO: lx, ly, lz are the lo words' contribution li - lj to the two
// separations, record_dl2)
template <int TR, bool AUX, bool WRAP, bool EXACT, bool LO>
__device__ __forceinline__ void near_pair2(const PP2& p, const SysParam& P, float4 ri, float4 ra, float4 rb,
                                           bool va, bool vb, ForceAcc2& A, float2 lx, float2 ly, float2 lz)
{
    const float2 sx = f2(__fsub_rn(ri.x, ra.x), __fsub_rn(ri.x, rb.x));
    const float2 sy = f2(__fsub_rn(ri.y, ra.y), __fsub_rn(ri.y, rb.y));
    const float2 sz = f2(__fsub_rn(ri.z, ra.z), __fsub_rn(ri.z, rb.z));
    const float2 dx = WRAP ? min_image2(sx, P.L[0], P.Linv[0]) : sx;
    const float2 dy = WRAP ? min_image2(sy, P.L[1], P.Linv[1]) : sy;
    const float2 dz = WRAP ? min_image2(sz, P.L[2], P.Linv[2]) : sz;
    const float2 px = mul2(dx, dx), py = mul2(dy, dy), pz = mul2(dz, dz);
    const float2 pxy = add2(px, py);
    const float2 rr = add2(pxy, pz);
    // the cut-off test of the list criterion, in scalar arithmetic (add2 and
    // mul2 may come out contracted); a near pair can only reach r_c when
    // NEAR_SIGMA sigma + skin does
    bool ka = va, kb = vb;
    if (!P.near_in_range) {
        ka = ka && rr_exact(dx.x, dy.x, dz.x) < p.rr_cut.x;
        kb = kb && rr_exact(dx.y, dy.y, dz.y) < p.rr_cut.y;
    }
    float2 dxl = bc2(0.0f), dyl = bc2(0.0f), dzl = bc2(0.0f);
    if (!EXACT) {
        dxl = diff_err2(ri.x, ra.x, rb.x, sx);
        dyl = diff_err2(ri.y, ra.y, rb.y, sy);
        dzl = diff_err2(ri.z, ra.z, rb.z, sz);
    }
    if (LO) {
        if (EXACT) {
            dxl = lx; dyl = ly; dzl = lz;
        } else {
            dxl = add2(dxl, lx); dyl = add2(dyl, ly); dzl = add2(dzl, lz);
        }
    }
    float2 rrl = add2(add2(fma2(dx, dx, neg2(px)), fma2(dy, dy, neg2(py))), fma2(dz, dz, neg2(pz)));
    rrl = add2(rrl, add2(fast_err_pos2(px, py, pxy), fast_err_pos2(pxy, pz, rr)));
    if (!EXACT || LO) rrl = fma2(bc2(2.0f), fma2(dx, dxl, fma2(dy, dyl, mul2(dz, dzl))), rrl);
    float2 fval, flo, e;
    pair_eval2<TR>(p, rr, rrl, P.rri_smooth, fval, flo, e);
    fval = sel2(ka, kb, fval);
    flo = sel2(ka, kb, flo);
    const float2 tx = mul2(fval, dx), ty = mul2(fval, dy), tz = mul2(fval, dz);
    two_sum_acc2(A.fx, A.cx, tx);
    two_sum_acc2(A.fy, A.cy, ty);
    two_sum_acc2(A.fz, A.cz, tz);
    float2 cx = add2(A.cx, fma2(fval, dx, neg2(tx)));
    float2 cy = add2(A.cy, fma2(fval, dy, neg2(ty)));
    float2 cz = add2(A.cz, fma2(fval, dz, neg2(tz)));
    if (!EXACT || LO) {
        cx = fma2(fval, dxl, cx);
        cy = fma2(fval, dyl, cy);
        cz = fma2(fval, dzl, cz);
    }
    A.cx = fma2(flo, dx, cx);
    A.cy = fma2(flo, dy, cy);
    A.cz = fma2(flo, dz, cz);
    aux_acc2<AUX>(A, fval, sel2(ka, kb, e), dx, dy, dz);
}

// two far pairs (far_pair, lane by lane)
template <int TR, bool AUX, bool WRAP, bool LO>
__device__ __forceinline__ void far_pair2(const PP2& p, const SysParam& P, float4 ri, float4 ra, float4 rb,
                                          bool va, bool vb, ForceAcc2& A, float2 lx, float2 ly, float2 lz)
{
    const float2 sx = f2(__fsub_rn(ri.x, ra.x), __fsub_rn(ri.x, rb.x));
    const float2 sy = f2(__fsub_rn(ri.y, ra.y), __fsub_rn(ri.y, rb.y));
    const float2 sz = f2(__fsub_rn(ri.z, ra.z), __fsub_rn(ri.z, rb.z));
    float2 dx = WRAP ? min_image2(sx, P.L[0], P.Linv[0]) : sx;
    float2 dy = WRAP ? min_image2(sy, P.L[1], P.Linv[1]) : sy;
    float2 dz = WRAP ? min_image2(sz, P.L[2], P.Linv[2]) : sz;
    float2 rr = add2(add2(mul2(dx, dx), mul2(dy, dy)), mul2(dz, dz));
    // the cut-off test of the list criterion; add2 and mul2 may come out
    // contracted, which moves r^2 by at most an ulp or two, so pairs within
    // PairParam::rr_tie of r_c^2 are decided again in scalar arithmetic
    bool ka = va && rr.x < p.rr_cut.x;
    bool kb = vb && rr.y < p.rr_cut.y;
    const float2 gap = sub2(rr, p.rr_cut);
    if (fabsf(gap.x) <= p.rr_tie.x || fabsf(gap.y) <= p.rr_tie.y) {
        ka = va && rr_exact(dx.x, dy.x, dz.x) < p.rr_cut.x;
        kb = vb && rr_exact(dx.y, dy.y, dz.y) < p.rr_cut.y;
    }
    if (WRAP || LO) {
        // the separation's residual e: across the box the rounding error of
        // ri - rj, for dsfloat positions the difference of the lo words
        // (far_pair); rr takes it to first order
        float2 ex = bc2(0.0f), ey = bc2(0.0f), ez = bc2(0.0f);
        if (LO) {
            ex = lx;
            ey = ly;
            ez = lz;
        }
        if (WRAP) {
            ex = add2(ex, diff_err2(ri.x, ra.x, rb.x, sx));
            ey = add2(ey, diff_err2(ri.y, ra.y, rb.y, sy));
            ez = add2(ez, diff_err2(ri.z, ra.z, rb.z, sz));
        }
        rr = fma2(bc2(2.0f), fma2(dx, ex, fma2(dy, ey, mul2(dz, ez))), rr);
        dx = add2(dx, ex);
        dy = add2(dy, ey);
        dz = add2(dz, ez);
    }
    float ya, yb;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ya) : "f"(rr.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yb) : "f"(rr.y));
    const float2 rri = mul2(p.sigma2, f2(ya, yb));
    const float2 ri6 = mul2(mul2(rri, rri), rri);
    float2 fval = mul2(mul2(mul2(p.c48, rri), ri6), sub2(ri6, bc2(0.5f)));
    float2 flo, e = bc2(0.0f);
    if (AUX || TR == TRUNC_SMOOTH_R4 || TR == TRUNC_FORCE_SHIFTED)
        truncate2<TR, false>(p, rr, ri6, P.rri_smooth, fval, flo, e);
    fval = sel2(ka, kb, fval);
    A.gx = fma2(fval, dx, A.gx);
    A.gy = fma2(fval, dy, A.gy);
    A.gz = fma2(fval, dz, A.gz);
    aux_acc2<AUX>(A, fval, sel2(ka, kb, e), dx, dy, dz);
}

// merge the even and odd accumulators into one
template <bool AUX>
__device__ __forceinline__ void fold_lanes2(const ForceAcc2& B, ForceAcc& A)
{
    A.fx = B.fx.x; A.fy = B.fy.x; A.fz = B.fz.x;
    A.cx = __fadd_rn(B.cx.x, B.cx.y);
    A.cy = __fadd_rn(B.cy.x, B.cy.y);
    A.cz = __fadd_rn(B.cz.x, B.cz.y);
    two_sum_acc(A.fx, A.cx, B.fx.y);
    two_sum_acc(A.fy, A.cy, B.fy.y);
    two_sum_acc(A.fz, A.cz, B.fz.y);
    A.gx = __fadd_rn(B.gx.x, B.gx.y);
    A.gy = __fadd_rn(B.gy.x, B.gy.y);
    A.gz = __fadd_rn(B.gz.x, B.gz.y);
    if (AUX) {
        A.en = B.en.x + B.en.y;
        A.s0 = B.s0.x + B.s0.y; A.s1 = B.s1.x + B.s1.y; A.s2 = B.s2.x + B.s2.y;
        A.s3 = B.s3.x + B.s3.y; A.s4 = B.s4.x + B.s4.y; A.s5 = B.s5.x + B.s5.y;
    }
}

// The list is a stream read once per launch: it is loaded without
// allocating in L1, which then keeps the neighbour positions the gathers
// reuse (HMD_FORCE_LIST_NOALLOC 0: ordinary read-only loads)
#ifndef HMD_FORCE_LIST_NOALLOC
#define HMD_FORCE_LIST_NOALLOC 1
#endif
__device__ __forceinline__ uint4 ld_list(const uint4* p)
{
    if (!HMD_FORCE_LIST_NOALLOC) return __ldg(p);
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ld_list(const uint2* p)
{
    if (!HMD_FORCE_LIST_NOALLOC) return __ldg(p);
    uint2 v;
    asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ld_list(const uint32_t* p)
{
    if (!HMD_FORCE_LIST_NOALLOC) return __ldg(p);
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
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
// gather of a neighbour's position: its 16-byte record (hmd_device.cuh
// fpos_encode) in dsfloat engines (LO), else the hi word
template <bool LO>
__device__ __forceinline__ float4 gather_pos(const Dev& d, uint32_t j)
{
    return LO ? __ldg(d.fpos + j) : ldg_hi(d.pos, j);
}

// the lo words of a gathered record (exact multiples of the code unit s)
__device__ __forceinline__ float4 record_lo(float w, const SysParam& P)
{
    return make_float4(__fsub_rn(fpos_fx(w, P.lo_exp_bits), P.lo_bias),
                       __fsub_rn(fpos_fy(w, P.lo_exp_bits_y), P.lo_bias_y),
                       __fsub_rn(fpos_fz(w, P.lo_exp_bits), P.lo_bias), 0.0f);
}

// the own lo words in the binades of the records' decoded fields:
// lo + (2^23 + 512) s for x and z, the lo word rounded to the code unit s
// (as lo_code rounds it), and lo + (2^13 + 512) s for y, rounded to
// s / 1024
__device__ __forceinline__ float4 lo_anchor(float4 li, const SysParam& P)
{
    return make_float4(__fadd_rn(li.x, P.lo_bias), __fadd_rn(li.y, P.lo_bias_y), __fadd_rn(li.z, P.lo_bias), 0.0f);
}

// li - lj of two gathered records, per component, two entries per
// instruction: the separation residuals the lo words contribute.
// EXACT_LI (near pairs, whose forces are the most sensitive to the
// separation): the own lo word as it is, minus the neighbour's decoded one
// (lj = field - bias, exact).  Otherwise (far pairs): the anchor minus the
// field, one subtraction; both lie in one binade, so the difference is
// exact: (c_i - c_j) s with the own lo word rounded to the unit s as well
// (at most s/2 = ulp(L/2) / 2048 from the exact form; finer for y).
template <bool EXACT_LI>
__device__ __forceinline__ void record_dl2(float4 li, float4 anchor, float wa, float wb, const SysParam& P,
                                           float2& ex, float2& ey, float2& ez)
{
    const uint32_t eb = P.lo_exp_bits, eby = P.lo_exp_bits_y;
    const float2 fx = f2(fpos_fx(wa, eb), fpos_fx(wb, eb));
    const float2 fy = f2(fpos_fy(wa, eby), fpos_fy(wb, eby));
    const float2 fz = f2(fpos_fz(wa, eb), fpos_fz(wb, eb));
    if (EXACT_LI) {
        const float2 bias = bc2(P.lo_bias);
        ex = sub2(bc2(li.x), sub2(fx, bias));
        ey = sub2(bc2(li.y), sub2(fy, bc2(P.lo_bias_y)));
        ez = sub2(bc2(li.z), sub2(fz, bias));
    } else {
        ex = sub2(bc2(anchor.x), fx);
        ey = sub2(bc2(anchor.y), fy);
        ez = sub2(bc2(anchor.z), fz);
    }
}

// species of a gathered neighbour
template <bool LO>
__device__ __forceinline__ uint32_t nbr_species(float w)
{
    return LO ? fpos_species(w) : species_bits(w);
}

template <int W, int E, int TRX, bool AUX, bool WRAP, bool FAR, bool LO, bool EXACT = false>
__device__ __forceinline__ void force_blocks(const Dev& d, uint32_t i, uint32_t q, uint32_t cnt, const SysParam& P,
                                             const PairParam* spp, float4 ri, float4 li, uint32_t a, ForceAcc& A)
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
        const V jv = ld_list(lst);
        float4 rj[E], lj[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t o = q * E + e;
            const uint32_t k = b * LB + (FAR ? LB - 1 - o : o);
            rj[e] = gather_pos<LO>(d, k < cnt ? idx_at(jv, e) : i);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t o = q * E + e;
            const uint32_t k = b * LB + (FAR ? LB - 1 - o : o);
            lj[e] = LO ? record_lo(rj[e].w, P) : make_float4(0, 0, 0, 0);
            const PairParam* pp;
            if (k >= cnt || !pair_of<NS1, LO>(row, p1, ns, rj[e].w, pp)) continue;
            if (FAR) far_pair<TR, AUX, WRAP, LO>(*pp, P, ri, rj[e], A, li, lj[e]);
            else near_pair<TR, AUX, WRAP, EXACT, LO>(*pp, P, ri, rj[e], A, li, lj[e]);
        }
    }
}

// force_blocks with the E entries of a load taken two at a time (E even)
// pair2: the packed parameters of every (species, neighbour species,
// neighbour species) triple of the system in shared memory (several
// species; pack_params of the two rows), so a pair of entries reads its
// PP2 with four 16-byte loads instead of building it field by field
template <int W, int E, int TRX, bool AUX, bool WRAP, bool FAR, bool LO, bool EXACT = false>
__device__ __forceinline__ void force_blocks2(const Dev& d, uint32_t i, uint32_t q, uint32_t cnt, const SysParam& P,
                                              const PairParam* spp, const PP2* pair2, float4 ri, float4 li, uint32_t a,
                                              ForceAcc2& A)
{
    static_assert(E % 2 == 0, "entries are taken in pairs");
    constexpr bool NS1 = TRX >= ONE_SPECIES;
    constexpr int TR = TRX & (ONE_SPECIES - 1);
    constexpr uint32_t LB = W * E;
    using V = typename IdxVec<E>::T;
    const size_t bstride = (size_t)d.S;
    const V* lst = reinterpret_cast<const V*>(d.nbr + (size_t)i * LB + q * E);
    if (FAR) lst += (size_t)(d.nbr_cap / LB - 1) * bstride * W;
    const ptrdiff_t step = FAR ? -(ptrdiff_t)(bstride * W) : (ptrdiff_t)(bstride * W);
    const uint32_t ns = P.ns;
    const PP2* row2 = pair2 + a * ns * ns;
    PP2 p1;
    if (NS1) p1 = pack_params(spp[0], spp[0]);
    const float4 anchor = (LO && FAR) ? lo_anchor(li, P) : li;
    const uint32_t nblk = (cnt + LB - 1) / LB;
    V jv;
    if (HMD_FORCE_PREFETCH && nblk > 0) jv = ld_list(lst);
    for (uint32_t b = 0; b < nblk; ++b, lst += step) {
        // the list stream comes from HBM: the next block's indices are
        // loaded one iteration ahead of their gathers
        V jn;
        if (HMD_FORCE_PREFETCH) {
            jn = jv;
            if (b + 1 < nblk) jn = ld_list(lst + step);
        } else {
            jv = ld_list(lst);
        }
        float4 rj[E];
        bool in[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t o = q * E + e;
            const uint32_t k = b * LB + (FAR ? LB - 1 - o : o);
            in[e] = k < cnt;
            rj[e] = gather_pos<LO>(d, in[e] ? idx_at(jv, e) : i);
        }
#pragma unroll
        for (int e = 0; e < E; e += 2) {
            float2 lx = bc2(0.0f), ly = bc2(0.0f), lz = bc2(0.0f);
            if (LO) record_dl2<!FAR>(li, anchor, rj[e].w, rj[e + 1].w, P, lx, ly, lz);
            PP2 pp;
            bool va = in[e], vb = in[e + 1];
            if (NS1) {
                pp = p1;
            } else {
                // a neighbour of no species of the system (lists hold real
                // particles only) reads row entry 0 and is masked
                const uint32_t ba = nbr_species<LO>(rj[e].w), bb = nbr_species<LO>(rj[e + 1].w);
                va = va && ba < ns;
                vb = vb && bb < ns;
                pp = row2[(ba < ns ? ba : 0u) * ns + (bb < ns ? bb : 0u)];
            }
            if (FAR) far_pair2<TR, AUX, WRAP, LO>(pp, P, ri, rj[e], rj[e + 1], va, vb, A, lx, ly, lz);
            else near_pair2<TR, AUX, WRAP, EXACT, LO>(pp, P, ri, rj[e], rj[e + 1], va, vb, A, lx, ly, lz);
        }
        if (HMD_FORCE_PREFETCH) jv = jn;
    }
}

template <int W, int E, int TR, bool AUX, bool LO>
__device__ __forceinline__ void force_dispatch(const Dev& d, uint32_t i, uint32_t q, uint32_t nn, uint32_t nf,
                                               bool wrap, bool exact, const SysParam& P, const PairParam* spp,
                                               const PP2* pair2, float4 ri, float4 li, uint32_t a, ForceAcc& A)
{
    if constexpr (E % 2 == 0) {
        ForceAcc2 B;
        if (wrap) {
            force_blocks2<W, E, TR, AUX, true, false, LO>(d, i, q, nn, P, spp, pair2, ri, li, a, B);
            force_blocks2<W, E, TR, AUX, true, true, LO>(d, i, q, nf, P, spp, pair2, ri, li, a, B);
        } else {
            if (exact) force_blocks2<W, E, TR, AUX, false, false, LO, true>(d, i, q, nn, P, spp, pair2, ri, li, a, B);
            else force_blocks2<W, E, TR, AUX, false, false, LO>(d, i, q, nn, P, spp, pair2, ri, li, a, B);
            force_blocks2<W, E, TR, AUX, false, true, LO>(d, i, q, nf, P, spp, pair2, ri, li, a, B);
        }
        fold_lanes2<AUX>(B, A);
    } else if (wrap) {
        force_blocks<W, E, TR, AUX, true, false, LO>(d, i, q, nn, P, spp, ri, li, a, A);
        force_blocks<W, E, TR, AUX, true, true, LO>(d, i, q, nf, P, spp, ri, li, a, A);
    } else {
        if (exact) force_blocks<W, E, TR, AUX, false, false, LO, true>(d, i, q, nn, P, spp, ri, li, a, A);
        else force_blocks<W, E, TR, AUX, false, false, LO>(d, i, q, nn, P, spp, ri, li, a, A);
        force_blocks<W, E, TR, AUX, false, true, LO>(d, i, q, nf, P, spp, ri, li, a, A);
    }
    // fold the plain far-pair sums into the compensated accumulators
    two_sum_acc(A.fx, A.cx, A.gx);
    two_sum_acc(A.fy, A.cy, A.gy);
    two_sum_acc(A.fz, A.cz, A.gz);
}

// ---------------------------------------------------------------------------
// The other pair potentials (mie, morse, power_law) with any truncation.
// The geometry runs two entries per FP32x2 instruction as above; each half
// then evaluates the potential in scalar FP32 (per-pair exponents), the
// reference's GPU formulas (mie_kernel.hpp, morse_kernel.hpp,
// power_law_kernel.hpp) with the parameter products precomputed on the host.
// Near pairs carry the separation's rounding error and are accumulated with
// compensation, far pairs with plain FMAs.
// ---------------------------------------------------------------------------

// integer power by repeated squaring, exponent per pair (numeric/pow.hpp)
__device__ __forceinline__ float ipowf(float x, uint32_t n)
{
    float y = 1.0f;
    for (; n; n >>= 1, x *= x)
        if (n & 1u) y *= x;
    return y;
}

// bare -U'(r)/r and U(r); PairParam::q0..q3 as documented there
template <int POT>
__device__ __forceinline__ void pot_eval(const PairParam& p, float rr, float& fval, float& en)
{
    if (POT == POT_MIE) {
        const float rri = __fdiv_rn(p.sigma2, rr);
        const uint32_t m2 = (uint32_t)p.q2, n2 = (uint32_t)p.q3;
        const float rni = ipowf(rri, n2);
        const float rmni = (m2 - n2 == n2) ? rni : ipowf(rri, m2 - n2);
        const float eps_rni = p.q0 * rni;
        fval = p.q1 * rri * eps_rni * (p.q2 * rmni - p.q3);
        en = eps_rni * (rmni - 1.0f);
    } else if (POT == POT_MORSE) {
        const float r_sigma_B = sqrtf(rr) * p.q2;
        const float dr = p.q3 - r_sigma_B;
        const float e = expf(dr);
        const float eA = (p.q1 == 1.0f) ? e : expf(p.q1 * dr);
        const float eps_e = p.q0 * e;
        fval = __fdiv_rn((p.q1 + 1.0f) * eps_e * (eA - 1.0f) * r_sigma_B, rr);
        en = eps_e * (eA - p.q1 - 1.0f);
    } else {
        const float rri = __fdiv_rn(p.sigma2, rr);
        float rni = ipowf(rri, (uint32_t)p.q2);
        if (p.q3 != 0.0f) rni *= sqrtf(rri);
        const float eps_rni = p.q0 * rni;
        fval = __fdiv_rn(p.q1 * eps_rni, rr);
        en = eps_rni;
    }
}

// truncations/{sharp,shifted,smooth_r4,force_shifted}_kernel.cuh on a bare
// (fval, en); en_cut = 0 for sharp.  rrl: the rounding residual of rr.  The
// smooth_r4 factors vary on the scale h near r_c, so r - r_c is formed from
// the correctly rounded root plus the residual's first-order term (r and r_c
// are within a factor two there: the difference is exact)
__device__ __forceinline__ void truncate_any(const PairParam& p, uint32_t trunc, float rr, float rrl, float rri_smooth,
                                             float& fval, float& en)
{
    en -= p.en_cut;
    if (trunc == TRUNC_SMOOTH_R4) {
        const float r = sqrtf(rr);
        const float rinv = __fdiv_rn(1.0f, r);
        const float dr = __fmaf_rn(0.5f * rrl, rinv, __fsub_rn(r, p.r_cut));
        const float x2 = dr * dr * rri_smooth;
        const float x4 = x2 * x2;
        const float x4i = __fdiv_rn(1.0f, 1.0f + x4);
        const float h0 = x4 * x4i;
        const float h1 = 4.0f * dr * rri_smooth * x2 * x4i * x4i;
        fval = h0 * fval - h1 * (en * rinv);
        en = h0 * en;
    } else if (trunc == TRUNC_FORCE_SHIFTED) {
        const float rinv = rsqrtf(rr);
        fval = fval - p.f_cut * rinv;
        en = en + (rr * rinv - p.r_cut) * p.f_cut;
    }
}

template <int POT, bool AUX, bool WRAP, bool NEAR, bool LO>
__device__ __forceinline__ void pot_pair2(const PairParam& pa, const PairParam& pb, const SysParam& P, float4 ri,
                                          float4 ra, float4 rb, bool va, bool vb, ForceAcc2& A, float4 li,
                                          float4 la, float4 lb)
{
    const float2 sx = f2(__fsub_rn(ri.x, ra.x), __fsub_rn(ri.x, rb.x));
    const float2 sy = f2(__fsub_rn(ri.y, ra.y), __fsub_rn(ri.y, rb.y));
    const float2 sz = f2(__fsub_rn(ri.z, ra.z), __fsub_rn(ri.z, rb.z));
    float2 dx = WRAP ? min_image2(sx, P.L[0], P.Linv[0]) : sx;
    float2 dy = WRAP ? min_image2(sy, P.L[1], P.Linv[1]) : sy;
    float2 dz = WRAP ? min_image2(sz, P.L[2], P.Linv[2]) : sz;
    float2 rr = rr_exact2(dx, dy, dz);
    // the cut-off test in scalar arithmetic (far_pair2)
    const bool ka = va && rr_exact(dx.x, dy.x, dz.x) < pa.rr_cut;
    const bool kb = vb && rr_exact(dx.y, dy.y, dz.y) < pb.rr_cut;
    const bool smooth = P.trunc == TRUNC_SMOOTH_R4;   // block-uniform
    float2 rrl = bc2(0.0f);
    if (WRAP || NEAR || LO || smooth) {
        // the separation's rounding error and, for dsfloat positions, the
        // difference of the lo words back in (the cut-off decision above
        // keeps the rounded squared distance of the list criterion)
        float2 ex = diff_err2(ri.x, ra.x, rb.x, sx);
        float2 ey = diff_err2(ri.y, ra.y, rb.y, sy);
        float2 ez = diff_err2(ri.z, ra.z, rb.z, sz);
        if (LO) {
            ex = add2(ex, f2(__fsub_rn(li.x, la.x), __fsub_rn(li.x, lb.x)));
            ey = add2(ey, f2(__fsub_rn(li.y, la.y), __fsub_rn(li.y, lb.y)));
            ez = add2(ez, f2(__fsub_rn(li.z, la.z), __fsub_rn(li.z, lb.z)));
        }
        dx = add2(dx, ex);
        dy = add2(dy, ey);
        dz = add2(dz, ez);
        const float2 px = mul2(dx, dx), py = mul2(dy, dy), pz = mul2(dz, dz);
        const float2 pxy = add2(px, py);
        rr = add2(pxy, pz);
        if (smooth) {
            rrl = add2(add2(fma2(dx, dx, neg2(px)), fma2(dy, dy, neg2(py))), fma2(dz, dz, neg2(pz)));
            rrl = add2(rrl, add2(two_sum_err2(px, py, pxy), two_sum_err2(pxy, pz, rr)));
        }
    }
    float fa, ea, fb, eb;
    pot_eval<POT>(pa, rr.x, fa, ea);
    pot_eval<POT>(pb, rr.y, fb, eb);
    truncate_any(pa, P.trunc, rr.x, rrl.x, P.rri_smooth, fa, ea);
    truncate_any(pb, P.trunc, rr.y, rrl.y, P.rri_smooth, fb, eb);
    const float2 fval = sel2(ka, kb, f2(fa, fb));
    if (NEAR) {
        const float2 tx = mul2(fval, dx), ty = mul2(fval, dy), tz = mul2(fval, dz);
        two_sum_acc2(A.fx, A.cx, tx);
        two_sum_acc2(A.fy, A.cy, ty);
        two_sum_acc2(A.fz, A.cz, tz);
        A.cx = add2(A.cx, fma2(fval, dx, neg2(tx)));
        A.cy = add2(A.cy, fma2(fval, dy, neg2(ty)));
        A.cz = add2(A.cz, fma2(fval, dz, neg2(tz)));
    } else {
        A.gx = fma2(fval, dx, A.gx);
        A.gy = fma2(fval, dy, A.gy);
        A.gz = fma2(fval, dz, A.gz);
    }
    aux_acc2<AUX>(A, fval, sel2(ka, kb, f2(ea, eb)), dx, dy, dz);
}

// force_blocks2 for the other potentials; an odd E pairs the last entry of
// a load with a masked copy of the particle itself
template <int W, int E, int POT, bool AUX, bool WRAP, bool FAR, bool LO>
__device__ __forceinline__ void force_blocks_pot(const Dev& d, uint32_t i, uint32_t q, uint32_t cnt,
                                                 const SysParam& P, const PairParam* spp, float4 ri, float4 li,
                                                 uint32_t a, ForceAcc2& A)
{
    constexpr uint32_t LB = W * E;
    using V = typename IdxVec<E>::T;
    const size_t bstride = (size_t)d.S;
    const V* lst = reinterpret_cast<const V*>(d.nbr + (size_t)i * LB + q * E);
    if (FAR) lst += (size_t)(d.nbr_cap / LB - 1) * bstride * W;
    const ptrdiff_t step = FAR ? -(ptrdiff_t)(bstride * W) : (ptrdiff_t)(bstride * W);
    const uint32_t ns = P.ns;
    const PairParam* row = spp + a * ns;
    const uint32_t nblk = (cnt + LB - 1) / LB;
    for (uint32_t b = 0; b < nblk; ++b, lst += step) {
        const V jv = ld_list(lst);
        float4 rj[E], lj[E];
        bool in[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t o = q * E + e;
            const uint32_t k = b * LB + (FAR ? LB - 1 - o : o);
            in[e] = k < cnt;
            rj[e] = gather_pos<LO>(d, in[e] ? idx_at(jv, e) : i);
        }
#pragma unroll
        for (int e = 0; e < E; ++e)
            lj[e] = LO ? record_lo(rj[e].w, P) : make_float4(0, 0, 0, 0);
#pragma unroll
        for (int e = 0; e < E; e += 2) {
            const bool two = e + 1 < E;
            const float4 ra = rj[e], rb = two ? rj[e + 1 < E ? e + 1 : e] : ri;
            const float4 la = lj[e], lb = two ? lj[e + 1 < E ? e + 1 : e] : li;
            const uint32_t ba = nbr_species<LO>(ra.w), bb = two ? nbr_species<LO>(rb.w) : species_bits(rb.w);
            const bool va = in[e] && ba < ns;
            const bool vb = two && in[e + 1 < E ? e + 1 : e] && bb < ns;
            const PairParam& pa = row[ba < ns ? ba : 0u];
            const PairParam& pb = row[vb ? bb : 0u];
            pot_pair2<POT, AUX, WRAP, !FAR, LO>(pa, pb, P, ri, ra, rb, va, vb, A, li, la, lb);
        }
    }
}

template <int W, int E, int POT, bool AUX, bool LO>
__device__ __forceinline__ void force_dispatch_pot(const Dev& d, uint32_t i, uint32_t q, uint32_t nn, uint32_t nf,
                                                   bool wrap, const SysParam& P, const PairParam* spp, float4 ri,
                                                   float4 li, uint32_t a, ForceAcc& A)
{
    ForceAcc2 B;
    if (wrap) {
        force_blocks_pot<W, E, POT, AUX, true, false, LO>(d, i, q, nn, P, spp, ri, li, a, B);
        force_blocks_pot<W, E, POT, AUX, true, true, LO>(d, i, q, nf, P, spp, ri, li, a, B);
    } else {
        force_blocks_pot<W, E, POT, AUX, false, false, LO>(d, i, q, nn, P, spp, ri, li, a, B);
        force_blocks_pot<W, E, POT, AUX, false, true, LO>(d, i, q, nf, P, spp, ri, li, a, B);
    }
    fold_lanes2<AUX>(B, A);
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

// kind of pair interaction of a system (FK_*), the template selector of k_force
__device__ __forceinline__ int force_kind_of(const SysParam& P)
{
    if (P.trunc == TRUNC_NONE) return FK_FULL;
    if (P.pot != POT_LJ) return FK_POT;
    if (P.trunc == TRUNC_SHARP || P.trunc == TRUNC_SHIFTED) return P.ns == 1 ? FK_LJ1 : FK_SHIFTED;
    return P.trunc == TRUNC_SMOOTH_R4 ? FK_SMOOTH : FK_FSHIFT;
}

template <int W, int E, bool AUX, bool LO>
__device__ __forceinline__ void force_pot(const Dev& d, uint32_t i, uint32_t q, uint32_t nn, uint32_t nf, bool wrap,
                                          const SysParam& P, const PairParam* spp, float4 ri, float4 li, uint32_t a,
                                          ForceAcc& A)
{
    switch (P.pot) {
    case POT_MIE: force_dispatch_pot<W, E, POT_MIE, AUX, LO>(d, i, q, nn, nf, wrap, P, spp, ri, li, a, A); break;
    case POT_MORSE: force_dispatch_pot<W, E, POT_MORSE, AUX, LO>(d, i, q, nn, nf, wrap, P, spp, ri, li, a, A); break;
    default: force_dispatch_pot<W, E, POT_POWER_LAW, AUX, LO>(d, i, q, nn, nf, wrap, P, spp, ri, li, a, A); break;
    }
}

// LO: the engine holds dsfloat positions (the separations carry the lo words)
template <int W, int E, int KIND, bool AUX, bool LO>
__global__ void __launch_bounds__(HMD_FORCE_THREADS, (LO ? HMD_FORCE_MINB_DS : HMD_FORCE_MINB) * 128 / HMD_FORCE_THREADS)
k_force(Dev d)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t / W, q = t % W;
    // the particle's own words first (every slot index is a valid address):
    // their latency overlaps the system parameters' and the pair table's
    float4 ri, li = make_float4(0, 0, 0, 0);
    if (LO) ldg_pos2(d.pos, i, ri, li);
    else ri = ldg_hi(d.pos, i);
    const uint32_t counts = __ldg(d.nbr_count + i);
    const uint32_t s = d.chunk_sys[(blockIdx.x * (blockDim.x / W)) / CHUNK];
    const SysParam& P = d.sys[s];
    __shared__ PairParam spp[MAX_SPECIES * MAX_SPECIES];
    // packed pair parameters per (species, neighbour, neighbour) for the
    // several-species kinds of the two-entry path (force_blocks2)
    constexpr bool PACKED2 = (E % 2 == 0) && KIND != FK_LJ1 && KIND != FK_POT;
    __shared__ PP2 s_pair2[PACKED2 ? MAX_SPECIES * MAX_SPECIES * MAX_SPECIES : 1];
    const uint32_t np = P.ns * P.ns;
    if (threadIdx.x < np) spp[threadIdx.x] = d.pair[P.pair_off + threadIdx.x];
    __syncthreads();
    if (!P.active || !d.st[s].live || *d.status != 0u) return;   // block-uniform
    if (KIND != FK_GENERIC && force_kind_of(P) != KIND) return;      // another kind's launch
    if (KIND == FK_GENERIC && force_kind_of(P) == FK_FULL) return;   // no list: k_force_full
    if (PACKED2) {
        for (uint32_t k = threadIdx.x; k < np * P.ns; k += blockDim.x) {
            const uint32_t sa = k / np, ba = (k / P.ns) % P.ns, bb = k % P.ns;
            s_pair2[k] = pack_params(spp[sa * P.ns + ba], spp[sa * P.ns + bb]);
        }
        __syncthreads();
    }
    const uint32_t a = species_bits(ri.w);
    const bool real = a != PLACEHOLDER;
    const uint32_t packed = real ? counts : 0u;
    const uint32_t nn = packed & 0xFFFFu, nf = packed >> 16;   // near / far list parts
    const bool inner = !real || (fabsf(ri.x) < P.inner[0] && fabsf(ri.y) < P.inner[1] && fabsf(ri.z) < P.inner[2]);
    const bool wrap = __any_sync(0xFFFFFFFFu, !inner);
    const bool far_from_zero = !real || (fabsf(ri.x) >= P.exact_min && fabsf(ri.y) >= P.exact_min &&
                                         fabsf(ri.z) >= P.exact_min);
    const bool exact = __all_sync(0xFFFFFFFFu, far_from_zero);
    ForceAcc A;
    if (real) {
        if constexpr (KIND == FK_LJ1) {
            force_dispatch<W, E, ONE_SPECIES + TRUNC_SHIFTED, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A);
        } else if constexpr (KIND == FK_SHIFTED) {
            force_dispatch<W, E, TRUNC_SHIFTED, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A);
        } else if constexpr (KIND == FK_SMOOTH) {
            force_dispatch<W, E, TRUNC_SMOOTH_R4, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A);
        } else if constexpr (KIND == FK_FSHIFT) {
            force_dispatch<W, E, TRUNC_FORCE_SHIFTED, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A);
        } else if constexpr (KIND == FK_POT) {
            force_pot<W, E, AUX, LO>(d, i, q, nn, nf, wrap, P, spp, ri, li, a, A);
        } else {
            switch (force_kind_of(P)) {
            case FK_LJ1: force_dispatch<W, E, ONE_SPECIES + TRUNC_SHIFTED, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A); break;
            case FK_SHIFTED: force_dispatch<W, E, TRUNC_SHIFTED, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A); break;
            case FK_SMOOTH: force_dispatch<W, E, TRUNC_SMOOTH_R4, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A); break;
            case FK_POT: force_pot<W, E, AUX, LO>(d, i, q, nn, nf, wrap, P, spp, ri, li, a, A); break;
            default: force_dispatch<W, E, TRUNC_FORCE_SHIFTED, AUX, LO>(d, i, q, nn, nf, wrap, exact, P, spp, s_pair2, ri, li, a, A); break;
            }
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

template <int W, int E, int KIND>
static void launch_force_shape(const Dev& d, bool aux, cudaStream_t st)
{
    constexpr unsigned T = HMD_FORCE_THREADS;
    const unsigned grid = (unsigned)((size_t)d.S_grid * W / T);
    if (d.ds) {
        if (aux) k_force<W, E, KIND, true, true><<<grid, T, 0, st>>>(d);
        else k_force<W, E, KIND, false, true><<<grid, T, 0, st>>>(d);
    } else {
        if (aux) k_force<W, E, KIND, true, false><<<grid, T, 0, st>>>(d);
        else k_force<W, E, KIND, false, false><<<grid, T, 0, st>>>(d);
    }
}

// (lanes, list block) shapes the engine accepts: E = block / lanes entries per load
template <int KIND>
void launch_force_kind(const Dev& d, bool aux, cudaStream_t st)
{
    const uint32_t lb = 1u << d.lb_log2;
    switch (d.lanes * 16u + lb) {
    case 1 * 16 + 4: launch_force_shape<1, 4, KIND>(d, aux, st); break;
    case 2 * 16 + 4: launch_force_shape<2, 2, KIND>(d, aux, st); break;
    case 2 * 16 + 8: launch_force_shape<2, 4, KIND>(d, aux, st); break;
    case 4 * 16 + 4: launch_force_shape<4, 1, KIND>(d, aux, st); break;
    case 4 * 16 + 8: launch_force_shape<4, 2, KIND>(d, aux, st); break;
    default: launch_force_shape<8, 1, KIND>(d, aux, st); break;
    }
}

} // namespace hmd
