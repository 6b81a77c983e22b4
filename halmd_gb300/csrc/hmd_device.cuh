// hmd_device.cuh — device-side types and arithmetic shared by the MD kernels.
//
// Layout (HBM, flat over all systems of an engine):
//   slots      every system s owns slots [off_s, off_s + A_s), A_s = n_s rounded
//              up to SLOT_ALIGN; slots past n_s are ghosts (species 0xFFFFFFFF),
//              following mdsim/gpu/particle.cpp:67-88 (ghost padding).
//   position   float4 [2*S], the two words of a slot side by side: slot i
//              holds its hi word (x, y, z, species bits) at 2i and its lo
//              word (the dsfloat split, mdsim/gpu/particle.hpp:56-88) at
//              2i + 1, so the force kernel gathers a neighbour's full
//              position with one 32-byte load.  FP32 engines keep the lo
//              words at zero.
//   velocity   float4 [2*S]: (vx, vy, vz, mass) hi, then lo.
//   image      float4 [S]; force float4 [S]; en_pot float [S];
//              stress float [6*S] column-major (mdsim/force_kernel.hpp:64-80).
//   neighbours uint32 [cap * S] transposed: entry k of slot i at k*S + i
//              (from_binning_kernel.cu:154-158), plus a count per slot.
//
// All float arithmetic that must agree bit-for-bit with the CPU oracle
// (minimum image, squared distance, cell index, Hilbert key, dsfloat
// integrator) uses the __f*_rn intrinsics so nvcc cannot contract it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hmd {

constexpr uint32_t PLACEHOLDER = 0xFFFFFFFFu;
constexpr int MAX_SPECIES = 4;
constexpr int SLOT_ALIGN = 256;   // slots per system are a multiple of this
// units of the rebuild list: slots / 256, sorting slots / 256, sort tiles,
// cells / 256, cells / 4
constexpr uint32_t RB_UNITS = 5;
// The shared list scan does a warp's 32 particles in one serial pass over the
// cells around them; it pays off once a rebuild has enough warps per SM to
// hide that pass's latency (measured: 1M particles 1.8x faster, 64k
// particles 1.4x slower), so by default systems of at least this many
// particles use it
constexpr uint32_t NBR_SHARED_MIN_N = 1u << 18;
constexpr int CHUNK = 64;         // granularity of the slot -> system map

// default entries per block of the neighbour-list layout for a force kernel
// with w threads per particle (each thread reads block / w entries at once;
// the engine also accepts 8 for w = 2 and w = 4)
__host__ __device__ constexpr uint32_t list_block(uint32_t w) { return w < 4u ? 4u : w; }

// TRUNC_NONE: untruncated potential over all pairs (forces/pair_full.hpp)
enum Trunc : uint32_t { TRUNC_SHARP = 0, TRUNC_SHIFTED = 1, TRUNC_SMOOTH_R4 = 2, TRUNC_FORCE_SHIFTED = 3, TRUNC_NONE = 4 };
enum Pot : uint32_t { POT_LJ = 0, POT_MIE = 1, POT_MORSE = 2, POT_POWER_LAW = 3 };
// INTEG_DESCENT: steepest-descent energy minimisation (positions only);
// INTEG_HOOVER: Nose-Hoover chain of two; INTEG_BOLTZMANN: Verlet with
// Maxwell-Boltzmann velocities drawn every `interval` steps; INTEG_EULER:
// r += v dt only
enum Integrator : uint32_t {
    INTEG_VERLET = 0, INTEG_ANDERSEN = 1, INTEG_DESCENT = 2, INTEG_HOOVER = 3, INTEG_BOLTZMANN = 4, INTEG_EULER = 5
};
enum Status : uint32_t {
    ST_CELL_OVERFLOW = 1u,
    ST_NBR_OVERFLOW = 2u,
};

// per species pair of one system (LJ parameters + truncation constants)
struct PairParam {
    float eps4;        // 4 eps
    float c48;         // 48 eps / sigma^2
    float sigma2;
    float rr_cut;      // (float)(r_c^2)
    float en_cut;      // U(r_c) (0 for sharp)
    float r_cut;
    float rr_cut_skin; // (float)((r_c + skin)^2)
    float f_cut;       // force_shifted: F_c = fval(r_c) r_c
    float rr_near;     // (float)((NEAR_SIGMA sigma)^2): list pairs closer at build time get the compensated path
    float sigma2_lo;   // sigma^2 - sigma2 (the rounding error of the float parameter)
    float c48_lo;      // 48 eps / sigma^2 - c48
    // parameters of the other potentials (SysParam::pot):
    //   mie:       q0 = eps C(m, n), q1 = 2 / sigma^2, q2 = m/2, q3 = n/2 (integers as float)
    //   morse:     q0 = eps / A, q1 = A = 2 B^2 - 1, q2 = 1 / (sigma B), q3 = r_min / (sigma B)
    //   power_law: q0 = eps, q1 = n, q2 = n/2 (integer as float), q3 = 1 for odd n else 0
    float q0, q1, q2, q3;
    float rr_tie;      // 8 ulp of rr_cut: packed squared distances this close to it are tested again in scalar
};

// a force in double (FP64 variant), 32-byte aligned
struct alignas(32) Force64 {
    double x, y, z, w;
};

// the pair parameters in double for the FP64 variant (kernels_fp64.cu)
struct PairParam64 {
    double eps4, c48, sigma2, rr_cut, en_cut, r_cut, f_cut, pad;
};

// pairs closer than NEAR_SIGMA sigma at list build time are evaluated with
// the compensated arithmetic; the rest (|F| below ~2 eps / sigma even after
// closing in by the skin) in plain FP32
constexpr double NEAR_SIGMA = 1.5;

struct SysParam {
    uint32_t off, n, A;        // slot range and real particle count
    uint32_t ns, trunc, pair_off;
    float L[3], Linv[3];
    int32_t ncell[3];
    float cell_len[3];
    uint32_t cell_off;         // first cell of this system in the cell arrays
    uint32_t cell_size;        // slots per cell (multiple of 32)
    uint32_t ncells;
    uint32_t cell_word_off;    // first word of this system's cell contents
    float rri_smooth;          // h^-2 for smooth_r4
    float dt, dt_half;
    float rr_half_skin;        // (skin/2)^2 rebuild threshold on squared displacement
    uint32_t depth;            // Hilbert recursion depth
    uint32_t integrator;
    float sqrt_T;
    uint32_t coll_threshold;   // collision iff philox word < threshold
    uint32_t seed_lo, seed_hi;
    uint32_t active;           // 0: all slots are ghosts, kernels skip
    uint32_t sort_enable;      // Hilbert reorder on rebuild
    float inner[3];            // |r| below this in every dimension: no list pair wraps the box
    uint32_t sort_hist_off;    // first word of this system's digit histograms
    uint32_t sort_ntiles;      // sort tiles covering the slot range
    float exact_min;           // |coordinate| from which near-pair differences are exact (k_force)
    float descent_step;        // INTEG_DESCENT: move = descent_step * F ...
    float descent_max;         // ... capped at this length per particle and step
    uint32_t near_in_range;    // 1: a near pair (NEAR_SIGMA sigma + skin apart at most) is always inside r_c
    float lo_scale;            // unit s of the lo-word codes of Dev::fpos (a power of two)
    float lo_inv_scale;        // 1 / s
    uint32_t lo_exp_bits;      // bits of the float 2^23 s (the x or z field ORed in gives (2^23 + field) s)
    float lo_bias;             // (2^23 + 512) s
    uint32_t lo_exp_bits_y;    // bits of the float 2^13 s (the y field in place gives (2^13 + field) s)
    float lo_bias_y;           // (2^13 + 512) s
    uint32_t pot;              // pair potential (Pot)
    uint32_t interval;         // INTEG_BOLTZMANN: steps between velocity draws
    double dt64;               // the time step in double (FP64 variant)
    double rri_smooth64;       // h^-2 in double (FP64 variant)
    // INTEG_HOOVER (verlet_nvt_hoover.cpp:58-84): chain masses, dim N T, T, dt
    double nhc_mass[2];
    double nhc_target2;
    double nhc_T;
    double nhc_dt;
};

// mutable per-system device state
struct SysState {
    uint32_t disp2_bits;       // running max |r - r0|^2 (float bits, >= 0)
    uint32_t rebuild;          // 1: rebuild lists in this step
    uint32_t max_nbr;          // largest neighbour count of the last build
    uint32_t max_cell;         // largest cell occupancy of the last build
    unsigned long long step;   // completed integration steps
    unsigned long long rebuilds;
    uint32_t steps_left;       // integration steps still to do (0: frozen, ~0u: unbounded)
    uint32_t live;             // 1: the system advances in the current step
    uint32_t rebuild_request;  // host-set: rebuild at the next opportunity
    uint32_t pad;
    // thermostat state (INTEG_HOOVER: chain positions and velocities, the
    // velocity scale of the current half step; INTEG_BOLTZMANN: the
    // centre-of-mass velocity of the last draw)
    double xi[2], v_xi[2];
    double vcm[3];
    float scale;
    uint32_t pad2;
};

// device pointers of one engine (passed by value to every kernel)
struct Dev {
    float4* pos;               // [2S] slot i: hi at 2i, lo at 2i + 1
    float4* vel;               // [2S] hi | lo
    float4* img;               // [S]
    float4* force;             // [S]
    float4* r0;                // [S] hi positions at the last list build
    float4* fpos;              // [S] dsfloat engines: the force kernel's gather records (fpos_encode)
    Force64* force64;          // [S] FP64 variant: forces in double
    const PairParam64* pair64; // FP64 variant: the pair table in double
    float* en_pot;             // [S]
    float* stress;             // [6S]
    uint32_t* id;              // [S] tag of the particle within its system
    uint32_t* rid;             // [S] slot of (off + tag)
    uint32_t* nbr;             // [nbr_cap * S], blocked: entry k of slot i at ((k/LB)*S + i)*LB + k%LB, LB = 1 << lb_log2
    uint32_t* nbr_count;       // [S] near count | far count << 16 (near entries from the front, far from the back)
    uint32_t nbr_cap;          // multiple of 8
    uint32_t lanes;            // threads per particle in the force kernel (1, 2, 4, 8)
    uint32_t lb_log2;          // log2 of the list block width LB (4 or 8)
    uint32_t nbr_scan;         // list build: 0 by system size, 1 per lane, 2 shared per warp of 32 particles
    uint32_t force_kinds;      // bit k: a system of force kind k (kernels.h ForceKind); 0: unknown, one kernel for all
    uint32_t integ_kinds;      // bit k: a system with integrator k (Integrator)
    uint32_t* cell;            // cell contents
    uint32_t* cell_count;      // [total_cells]
    const uint32_t* cell_sys;  // [total_cells] owning system
    uint32_t total_cells;
    const SysParam* sys;
    SysState* st;
    const PairParam* pair;
    const uint32_t* chunk_sys; // [S / CHUNK]
    uint32_t S, nsys;
    uint32_t ds;               // 1: dsfloat positions and velocities (lo words in use)
    uint32_t fp64;             // 1: the FP64 variant (kernels_fp64.cu) runs the step
    uint32_t float_cutoff;     // FP64 variant: pair set by the float list criterion on the hi words
    // extents the launch grids cover (fixed layout: everything; capacity
    // mode: the slots, sort tiles and cells below the high-water mark of the
    // systems present, rounded up to a power of two)
    uint32_t S_grid, cells_grid, tiles_grid;
    uint32_t sm_count;         // SMs of the device (grids of one resident wave)
    // work list of the rebuild chain (k_rebuild_list): [0] count, then the
    // rebuilding systems and the prefix sums of their virtual blocks
    uint32_t* rb;
    uint32_t* status;          // ST_* bits
    uint32_t* done;            // last-block ticket counter
    uint32_t* any_rebuild;      // [0] this step rebuilds, [1] count of steps that ran the rebuild chain
    // sort scratch
    uint32_t* key[2];
    uint32_t* val[2];
    uint32_t* hist;
    uint32_t* dtot;            // [nsys * 256] digit totals of a system's keys in the current radix pass
    const uint2* tiles;        // (system, first slot) of every sort tile
    uint32_t ntiles;
    // rearrange temporaries
    float4* tpos;
    float4* tvel;
    float4* timg;
    uint32_t* tid;
    // reductions
    double* partial;           // [S / 256 * NTHERMO]
    double* thermo;            // [nsys * NTHERMO]
};

constexpr int NTHERMO = 14;    // see k_thermo_partial

__device__ __forceinline__ uint32_t species_bits(float w) { return __float_as_uint(w); }

// hi / lo position word of slot i in an interleaved position array
__device__ __forceinline__ float4& pos_hi(float4* p, uint32_t i) { return p[2 * (size_t)i]; }
__device__ __forceinline__ float4& pos_lo(float4* p, uint32_t i) { return p[2 * (size_t)i + 1]; }
__device__ __forceinline__ const float4& pos_hi(const float4* p, uint32_t i) { return p[2 * (size_t)i]; }
__device__ __forceinline__ const float4& pos_lo(const float4* p, uint32_t i) { return p[2 * (size_t)i + 1]; }
__device__ __forceinline__ float4 ldg_hi(const float4* p, uint32_t i) { return __ldg(p + 2 * (size_t)i); }

// The force kernel's gather record of a dsfloat slot, 16 bytes: the hi
// word's x, y, z and in w the lo words as multiples c of the system's
// lo_scale s = ulp(L/2) / 1024, stored as the 10-bit fields c + 512 (x in
// bits 0-9, y in bits 10-19, z in bits 22-31), and the species (bits
// 20-21).  |lo| <= ulp(L/2)/2 = 512 s, so c = lo / s rounded (clamped to
// +-511) is within s/2 of it (s a power of two: the scaling is exact).  The
// full double-single word pair is 32 bytes; the gathers of the force kernel
// are bound by the L1 data path, and half the bytes halve that traffic.  The
// x field ORed into the mantissa of 2^23 s gives the float (2^23 + c + 512) s,
// the y field left in place (mantissa bits 10-19) in that of 2^13 s gives
// (2^13 + c + 512) s, and the z field shifted down like x: c s costs one
// subtraction (record_lo), no integer conversion, and x and y no shift.
__device__ __forceinline__ uint32_t lo_code(float lo, float inv_s)
{
    const int c = __float2int_rn(__fmul_rn(lo, inv_s));
    return (uint32_t)(min(max(c, -511), 511) + 512);
}

__device__ __forceinline__ float4 fpos_encode(float4 hi, float4 lo, float inv_s)
{
    const uint32_t w = lo_code(lo.x, inv_s) | (lo_code(lo.y, inv_s) << 10) | ((species_bits(hi.w) & 3u) << 20) |
                       (lo_code(lo.z, inv_s) << 22);
    return make_float4(hi.x, hi.y, hi.z, __uint_as_float(w));
}

// species of a record's w word, and its three code fields as the floats
// (2^23 + c + 512) s for x and z (exp_bits: SysParam::lo_exp_bits) and
// (2^13 + c + 512) s for y (SysParam::lo_exp_bits_y)
__device__ __forceinline__ uint32_t fpos_species(float w) { return (__float_as_uint(w) >> 20) & 3u; }
__device__ __forceinline__ float fpos_fx(float w, uint32_t exp_bits)
{
    return __uint_as_float((__float_as_uint(w) & 0x3FFu) | exp_bits);
}
__device__ __forceinline__ float fpos_fy(float w, uint32_t exp_bits_y)
{
    return __uint_as_float((__float_as_uint(w) & 0xFFC00u) | exp_bits_y);
}
__device__ __forceinline__ float fpos_fz(float w, uint32_t exp_bits)
{
    return __uint_as_float((__float_as_uint(w) >> 22) | exp_bits);
}

// both words of slot i with one 256-bit read-only load (32-byte aligned:
// the array comes from cudaMalloc and a slot spans 32 bytes)
__device__ __forceinline__ void ldg_pos2(const float4* p, uint32_t i, float4& hi, float4& lo)
{
    const float4* a = p + 2 * (size_t)i;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(hi.x), "=f"(hi.y), "=f"(hi.z), "=f"(hi.w), "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w)
        : "l"(a));
}

// minimum image: k = rint(dr / L) via dr * (1/L); dr - k L (box_kernel.cuh:37-47)
// dr - rint(dr / L) L for dr = ri - rj of two in-box positions: |dr| <= L,
// so k is -1, 0 or 1, k L is exact, and the fused form rounds once exactly
// like dr - fl(k L)
__device__ __forceinline__ float min_image(float dr, float L, float Linv)
{
    const float k = rintf(__fmul_rn(dr, Linv));
    return __fmaf_rn(-k, L, dr);
}

__device__ __forceinline__ float rr_exact(float dx, float dy, float dz)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// ---- FP32x2: two values per instruction, each half rounded as the scalar
// operation (__fadd_rn, __fmul_rn, __fmaf_rn) -------------------------------

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
// Products and sums of register pairs can come out contracted: on this GPU
// a squared distance written as (x^2 + y^2) + z^2 with f32x2 multiply and
// add (builtins or PTX with an explicit rounding modifier alike) measured
// as fma(z, z, x^2 + y^2) for some inputs.  Decisions that must round as
// the oracle's float restatement (the cut-off test) therefore use the
// scalar __fmul_rn / __fadd_rn form, rr_exact.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// min_image of each half
__device__ __forceinline__ float2 min_image2(float2 s, float L, float Linv)
{
    const float2 q = mul2(s, bc2(Linv));
    return fma2(f2(-rintf(q.x), -rintf(q.y)), bc2(L), s);
}

// rr_exact of each half
__device__ __forceinline__ float2 rr_exact2(float2 dx, float2 dy, float2 dz)
{
    return add2(add2(mul2(dx, dx), mul2(dy, dy)), mul2(dz, dz));
}

// ---- double-single arithmetic: Knuth TwoSum / Dekker split (DSFUN) --------

__device__ __forceinline__ void ds_add(float& c0, float& c1, float a0, float a1, float b0, float b1)
{
    float t1 = __fadd_rn(a0, b0);
    float e = __fsub_rn(t1, a0);
    float t2 = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(b0, e), __fsub_rn(a0, __fsub_rn(t1, e))), a1), b1);
    e = __fadd_rn(t1, t2);
    c0 = e;
    c1 = __fsub_rn(t2, __fsub_rn(e, t1));
}

__device__ __forceinline__ void ds_sub(float& c0, float& c1, float a0, float a1, float b0, float b1)
{
    float t1 = __fsub_rn(a0, b0);
    float e = __fsub_rn(t1, a0);
    float t2 = __fsub_rn(__fadd_rn(__fadd_rn(__fsub_rn(-b0, e), __fsub_rn(a0, __fsub_rn(t1, e))), a1), b1);
    e = __fadd_rn(t1, t2);
    c0 = e;
    c1 = __fsub_rn(t2, __fsub_rn(e, t1));
}

__device__ __forceinline__ void ds_mul(float& c0, float& c1, float a0, float a1, float b0, float b1)
{
    float cona = __fmul_rn(a0, 8193.0f);
    float conb = __fmul_rn(b0, 8193.0f);
    float sa1 = __fsub_rn(cona, __fsub_rn(cona, a0));
    float sb1 = __fsub_rn(conb, __fsub_rn(conb, b0));
    float sa2 = __fsub_rn(a0, sa1);
    float sb2 = __fsub_rn(b0, sb1);
    float c11 = __fmul_rn(a0, b0);
    float c21 = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fmul_rn(sa1, sb1), c11), __fmul_rn(sa1, sb2)),
                                    __fmul_rn(sa2, sb1)), __fmul_rn(sa2, sb2));
    float c2 = __fadd_rn(__fmul_rn(a0, b1), __fmul_rn(a1, b0));
    float t1 = __fadd_rn(c11, c2);
    float e = __fsub_rn(t1, c11);
    float t2 = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(c2, e), __fsub_rn(c11, __fsub_rn(t1, e))), c21),
                         __fmul_rn(a1, b1));
    e = __fadd_rn(t1, t2);
    c0 = e;
    c1 = __fsub_rn(t2, __fsub_rn(e, t1));
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ---------------------

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = 0xD2511F53u * c.x;
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        uint32_t lo1 = 0xCD9E8D57u * c.z;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// uniform in (0, 1) from the top 24 bits
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f) + (0.5f / 16777216.0f); }

// ---- warp / block helpers -------------------------------------------------

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

} // namespace hmd
