// kernels_rebuild.cu — neighbour-list rebuild chain, run for the systems whose
// maximum displacement exceeded skin/2 (SysState::rebuild):
//   Hilbert keys -> stable LSD radix sort -> rearrange (mdsim/gpu/sorts/hilbert.cpp:71-117,
//   particle.cpp:173-218) -> cell binning (binning.cpp:166-221) -> full Verlet
//   list (neighbours/from_binning_kernel.cu:99-267).
#include "hmd_device.cuh"
#include "kernels.h"

namespace hmd {

// ---------------------------------------------------------------------------
// Hilbert key (mdsim/sorts/hilbert_kernel.hpp:70-230; Wang & Shan, 2005):
// the position, scaled to the unit cube, is snapped to the centre of its cell
// on a 2^depth grid and descended vertex by vertex.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void hswap(uint32_t& v, uint32_t& a, uint32_t& b)
{
    const uint32_t va = (v >> a) & 7u;
    const uint32_t vb = (v >> b) & 7u;
    v = v ^ (va << a) ^ (vb << b) ^ (va << b) ^ (vb << a);
    const uint32_t t = a; a = b; b = t;
}

__device__ uint32_t hilbert_key(float x0, float x1, float x2, uint32_t depth)
{
    const float n = (float)(1u << depth);
    float r[3] = {x0, x1, x2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        r[q] = __fmul_rn(__fsub_rn(r[q], floorf(r[q])), n);
        r[q] = __fsub_rn(__fdiv_rn(__fadd_rn(floorf(r[q]), 0.5f), n), 0.5f);
    }
    uint32_t a = 21, b = 18, c = 12, d = 15, e = 3, f = 0, g = 6, h = 9;
    uint32_t vc = (1u << b) ^ (2u << c) ^ (3u << d) ^ (4u << e) ^ (5u << f) ^ (6u << g) ^ (7u << h);
    uint32_t code = 0;
    for (uint32_t i = 0; i < depth; ++i) {
        const uint32_t x = signbit(r[0]) ? 1u : 0u;
        const uint32_t y = signbit(r[1]) ? 1u : 0u;
        const uint32_t z = signbit(r[2]) ? 1u : 0u;
        const uint32_t v = (vc >> (3u * (x + (y << 1) + (z << 2)))) & 7u;
        r[0] = __fsub_rn(__fadd_rn(__fmul_rn(r[0], 2.0f), (float)x), 0.5f);
        r[1] = __fsub_rn(__fadd_rn(__fmul_rn(r[1], 2.0f), (float)y), 0.5f);
        r[2] = __fsub_rn(__fadd_rn(__fmul_rn(r[2], 2.0f), (float)z), 0.5f);
        if (v == 0) { hswap(vc, b, h); hswap(vc, c, e); }
        else if (v == 1 || v == 2) { hswap(vc, c, g); hswap(vc, d, h); }
        else if (v == 3 || v == 4) { hswap(vc, a, c); hswap(vc, f, h); }
        else if (v == 5 || v == 6) { hswap(vc, a, e); hswap(vc, b, f); }
        else { hswap(vc, a, g); hswap(vc, d, f); }
        code = (code << 3) + v;
    }
    return code;
}

// Hilbert sort key of a slot; ghosts get the largest key of the 3*depth-bit
// range so the (stable) sort keeps them behind every real particle
__device__ __forceinline__ uint32_t slot_key(const Dev& d, const SysParam& P, uint32_t i)
{
    const float4 r = pos_hi(d.pos, i);
    const uint32_t bits = 3u * P.depth;
    if (species_bits(r.w) == PLACEHOLDER) return (1u << bits) - 1u;
    return hilbert_key(__fdiv_rn(r.x, P.L[0]), __fdiv_rn(r.y, P.L[1]), __fdiv_rn(r.z, P.L[2]), P.depth);
}

// Hilbert keys of all real particles of every system (module interface)
__global__ void k_hilbert_keys(Dev d, uint32_t* keys)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.S) return;
    const SysParam& P = d.sys[d.chunk_sys[i / CHUNK]];
    const float4 r = pos_hi(d.pos, i);
    keys[i] = (species_bits(r.w) == PLACEHOLDER)
        ? PLACEHOLDER
        : hilbert_key(__fdiv_rn(r.x, P.L[0]), __fdiv_rn(r.y, P.L[1]), __fdiv_rn(r.z, P.L[2]), P.depth);
}

// ---------------------------------------------------------------------------
// Work list of the rebuild chain.  The chain runs whenever any system
// rebuilds; in an engine of many systems only a few do, so instead of a grid
// over every slot (and cell) whose blocks mostly exit, k_rebuild_list
// compacts the rebuilding systems and the prefix sums of their virtual blocks
// in each unit the chain's kernels use, and those kernels loop over the
// virtual blocks with a grid of at most RB_WAVE blocks per SM (an engine of one
// system, with nothing to compact, launches a block per virtual block).  A
// virtual block covers the same slots (or cells) as one block of a launch
// over everything, so results do not change.
// ---------------------------------------------------------------------------

constexpr unsigned RB_WAVE = 8;   // blocks per SM of a capped rebuild-chain grid

struct RbList {
    uint32_t n;
    const uint32_t* sys;
    const uint32_t* p[RB_UNITS];   // prefix sums, n + 1 entries each
};

__device__ __forceinline__ RbList rb_list(const Dev& d)
{
    RbList L;
    L.n = d.rb[0];
    L.sys = d.rb + 1;
    for (uint32_t u = 0; u < RB_UNITS; ++u) L.p[u] = d.rb + 1 + d.nsys + u * (d.nsys + 1);
    return L;
}

// the list entry k with p[k] <= v < p[k + 1] (entries of zero width are skipped)
__device__ __forceinline__ uint32_t rb_find(const uint32_t* p, uint32_t n, uint32_t v)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (p[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

// one block: compact the active systems that rebuild, in system order
__global__ void __launch_bounds__(1024) k_rebuild_list(Dev d)
{
    __shared__ uint32_t s_warp[32][RB_UNITS + 1];
    __shared__ uint32_t s_carry[RB_UNITS + 1];
    uint32_t* sys = d.rb + 1;
    uint32_t* pre[RB_UNITS];
    for (uint32_t u = 0; u < RB_UNITS; ++u) pre[u] = d.rb + 1 + d.nsys + u * (d.nsys + 1);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x <= RB_UNITS) s_carry[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t base = 0; base < d.nsys; base += blockDim.x) {
        const uint32_t s = base + threadIdx.x;
        uint32_t c[RB_UNITS + 1] = {0, 0, 0, 0, 0, 0};   // [0]: rebuilds, then the units
        if (s < d.nsys) {
            const SysParam& P = d.sys[s];
            if (P.active && d.st[s].rebuild) {
                c[0] = 1;
                c[1] = P.A / 256;
                if (P.sort_enable) { c[2] = P.A / 256; c[3] = P.sort_ntiles; }
                c[4] = (P.ncells + 255) / 256;
                c[5] = (P.ncells + 3) / 4;
            }
        }
        uint32_t incl[RB_UNITS + 1];
#pragma unroll
        for (uint32_t u = 0; u <= RB_UNITS; ++u) {
            uint32_t x = c[u];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= (uint32_t)o) x += y;
            }
            incl[u] = x;
            if (lane == 31) s_warp[warp][u] = x;
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (uint32_t u = 0; u <= RB_UNITS; ++u) {
                const uint32_t v = lane < nw ? s_warp[lane][u] : 0u;
                uint32_t x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (lane >= (uint32_t)o) x += y;
                }
                if (lane < nw) s_warp[lane][u] = x - v;   // exclusive over warps
            }
        }
        __syncthreads();
        if (c[0]) {
            const uint32_t k = s_carry[0] + s_warp[warp][0] + incl[0] - 1u;
            sys[k] = s;
#pragma unroll
            for (uint32_t u = 0; u < RB_UNITS; ++u) pre[u][k] = s_carry[u + 1] + s_warp[warp][u + 1] + incl[u + 1] - c[u + 1];
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1)
            for (uint32_t u = 0; u <= RB_UNITS; ++u) s_carry[u] += s_warp[warp][u] + incl[u];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const uint32_t n = s_carry[0];
        for (uint32_t u = 0; u < RB_UNITS; ++u) pre[u][n] = s_carry[u + 1];
        d.rb[0] = n;
    }
}

// ---------------------------------------------------------------------------
// Segmented stable LSD radix sort, 8-bit digits (algorithm/gpu/radix_sort_kernel.cu:76-230
// restated per system): the slot range of every system is cut into tiles of
// 2048 keys that never straddle two systems (tile table d.tiles); each pass
// is one launch over all tiles (digit histograms and per-system digit
// totals), one launch with a warp per (system, digit) (digit-major exclusive
// scan of its tiles) and one launch over all tiles (stable scatter with
// warp-match ranking).  Only systems that rebuild with
// sorting on do work; the permutation ends in val[passes % 2].
// ---------------------------------------------------------------------------

// A tile of 2048 keys is taken by one block of 1024 threads in two rounds:
// a small system has few tiles (KA-64k: 32), so the rounds a block runs
// one after the other, each a dependent chain of load, rank and store, set
// the time of the pass.
constexpr int RADIX_THREADS = 1024;
constexpr int RADIX_ROUNDS = 2;
constexpr int RADIX_WARPS = RADIX_THREADS / 32;
constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;
static_assert(RADIX_TILE == SORT_TILE, "tile table and kernels disagree");

__device__ __forceinline__ bool sort_live(const Dev& d, uint32_t s)
{
    const SysParam& P = d.sys[s];
    return P.active && P.sort_enable && d.st[s].rebuild;
}

// keys (Hilbert code, ghosts last) and identity values of the sorting systems
__global__ void __launch_bounds__(256) k_seg_keys(Dev d)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[1][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[1], L.n, v);
        const SysParam& P = d.sys[L.sys[k]];
        const uint32_t i = P.off + (v - L.p[1][k]) * 256u + threadIdx.x;
        d.key[0][i] = slot_key(d, P, i);
        d.val[0][i] = i;
        // digit totals of the first pass start from zero
        if (v == L.p[1][k]) d.dtot[(size_t)L.sys[k] * 256u + threadIdx.x] = 0u;
    }
}

__global__ void __launch_bounds__(RADIX_THREADS) k_seg_hist(Dev d, const uint32_t* keys, uint32_t shift)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[2][L.n];
    __shared__ uint32_t h[256];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[2], L.n, v);
        const uint32_t s = L.sys[k];
        const SysParam& P = d.sys[s];
        const uint32_t local = v - L.p[2][k];
        const uint32_t first = P.off + local * RADIX_TILE;
        const uint32_t end = min(first + (uint32_t)RADIX_TILE, P.off + P.A);
        if (threadIdx.x < 256) h[threadIdx.x] = 0;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RADIX_ROUNDS; ++r) {
            const uint32_t idx = first + r * RADIX_THREADS + threadIdx.x;
            if (idx < end) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 256) {
            const uint32_t c = h[threadIdx.x];
            d.hist[P.sort_hist_off + threadIdx.x * P.sort_ntiles + local] = c;
            if (c) atomicAdd(&d.dtot[(size_t)s * 256u + threadIdx.x], c);
        }
        __syncthreads();
    }
}

// Exclusive scan of a system's histogram, digit-major over its tiles, one
// warp per digit: the digit's base is the sum of the totals of the smaller
// digits (Dev::dtot, accumulated by k_seg_hist), its row of tile counts is
// scanned lane-strided with warp shuffles and a running carry.  A grid of
// (systems, 32) blocks of 8 warps covers the 256 digits of every system at
// once; offsets come out as absolute slots.
__global__ void __launch_bounds__(256) k_seg_scan(Dev d)
{
    const RbList L = rb_list(d);
    const uint32_t lane = threadIdx.x & 31u, g = blockIdx.y * 8u + (threadIdx.x >> 5);
    for (uint32_t k = blockIdx.x; k < L.n; k += gridDim.x) {
        const uint32_t s = L.sys[k];
        if (!sort_live(d, s)) continue;   // warp-uniform
        const SysParam& P = d.sys[s];
        const uint32_t* tot = d.dtot + (size_t)s * 256u;
        uint32_t base = 0;
        for (uint32_t q = lane; q < g; q += 32) base += tot[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) base += __shfl_xor_sync(0xFFFFFFFFu, base, o);
        uint32_t carry = P.off + base;
        const uint32_t nt = P.sort_ntiles;
        uint32_t* row = d.hist + P.sort_hist_off + g * nt;
        for (uint32_t t0 = 0; t0 < nt; t0 += 32) {
            const uint32_t t = t0 + lane;
            const uint32_t v = (t < nt) ? row[t] : 0u;
            uint32_t incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= (uint32_t)o) incl += x;
            }
            if (t < nt) row[t] = carry + incl - v;
            carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
        }
    }
}

__device__ __forceinline__ void seg_scatter_tile(const Dev& d, uint32_t s, uint32_t local, const uint32_t* kin,
                                                 const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t shift);

__global__ void __launch_bounds__(RADIX_THREADS) k_seg_scatter(Dev d, const uint32_t* kin, const uint32_t* vin,
                                                               uint32_t* kout, uint32_t* vout, uint32_t shift)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[2][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[2], L.n, v);
        seg_scatter_tile(d, L.sys[k], v - L.p[2][k], kin, vin, kout, vout, shift);
        __syncthreads();
    }
}

// one tile of 2048 keys of a system: stable scatter by the current digit
__device__ __forceinline__ void seg_scatter_tile(const Dev& d, uint32_t s, uint32_t local, const uint32_t* kin,
                                                 const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t shift)
{
    const SysParam& P = d.sys[s];
    const uint32_t th = threadIdx.x, lane = th & 31u, warp = th >> 5;
    // the scan of this pass has read the digit totals: the next pass's
    // histograms accumulate from zero
    if (local == 0 && th < 256) d.dtot[(size_t)s * 256u + th] = 0u;
    const uint32_t first = P.off + local * RADIX_TILE;
    const uint32_t end = min(first + (uint32_t)RADIX_TILE, P.off + P.A);
    __shared__ uint32_t s_w[RADIX_WARPS][256];   // per warp and digit: count, then exclusive offset
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_goff[256];
    uint32_t* s_flat = &s_w[0][0];
    if (th < 256) {
        s_base[th] = 0;
        s_goff[th] = d.hist[P.sort_hist_off + th * P.sort_ntiles + local];
    }
    for (uint32_t k = th; k < RADIX_WARPS * 256u; k += RADIX_THREADS) s_flat[k] = 0;
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const uint32_t idx = first + r * RADIX_THREADS + th;
        const bool valid = idx < end;
        uint32_t key = 0, val = 0, dg = 256u;
        if (valid) { key = kin[idx]; val = vin[idx]; dg = (key >> shift) & 255u; }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dg);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) s_w[warp][dg] = __popc(peers);
        __syncthreads();
        if (th < 256) {
            uint32_t run = s_base[th];
#pragma unroll 8
            for (int w = 0; w < RADIX_WARPS; ++w) {
                const uint32_t c = s_w[w][th];
                s_w[w][th] = run;
                run += c;
            }
            s_base[th] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = s_goff[dg] + s_w[warp][dg] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        for (uint32_t k = th; k < RADIX_WARPS * 256u; k += RADIX_THREADS) s_flat[k] = 0;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// rearrange (particle.cpp:173-218, particle_kernel.cu:45): gather phase space
// by the sort permutation into temporaries, then copy back, for the systems
// that rebuild; reverse ids follow.
// ---------------------------------------------------------------------------

template <bool DS>
__device__ __forceinline__ void rearrange_slot(const Dev& d, const SysParam& P, uint32_t i, const uint32_t* perm);

template <bool DS>
__global__ void __launch_bounds__(256) k_rearrange(Dev d, const uint32_t* perm)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[1][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[1], L.n, v);
        const SysParam& P = d.sys[L.sys[k]];
        rearrange_slot<DS>(d, P, P.off + (v - L.p[1][k]) * 256u + threadIdx.x, perm);
    }
}

template <bool DS>
__device__ __forceinline__ void rearrange_slot(const Dev& d, const SysParam& P, uint32_t i, const uint32_t* perm)
{
    const uint32_t src = perm[i];
    pos_hi(d.tpos, i) = pos_hi(d.pos, src);
    d.tvel[i] = d.vel[src];
    if (DS) {
        pos_lo(d.tpos, i) = pos_lo(d.pos, src);
        d.tvel[d.S + i] = d.vel[d.S + src];
    }
    d.timg[i] = d.img[src];
    const uint32_t tag = d.id[src];
    d.tid[i] = tag;
    if (tag != PLACEHOLDER) d.rid[P.off + tag] = i;
}

template <bool DS>
__global__ void __launch_bounds__(256) k_copyback(Dev d)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[1][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[1], L.n, v);
        const uint32_t i = d.sys[L.sys[k]].off + (v - L.p[1][k]) * 256u + threadIdx.x;
        pos_hi(d.pos, i) = pos_hi(d.tpos, i);
        d.vel[i] = d.tvel[i];
        if (DS) {
            pos_lo(d.pos, i) = pos_lo(d.tpos, i);
            d.vel[d.S + i] = d.tvel[d.S + i];
        }
        d.img[i] = d.timg[i];
        d.id[i] = d.tid[i];
    }
}

// ---------------------------------------------------------------------------
// cell binning: cell index (binning_kernel.cu:36-75) -> atomic slot in
// fixed-capacity cells -> each cell sorted ascending (the same contents as
// the reference's stable radix sort + assign_cells, binning_kernel.cu:94-123)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void cell_coords(const SysParam& P, float4 r, int& cx, int& cy, int& cz)
{
    const float x = __fadd_rn(__fdiv_rn(r.x, P.cell_len[0]), (float)P.ncell[0]);
    const float y = __fadd_rn(__fdiv_rn(r.y, P.cell_len[1]), (float)P.ncell[1]);
    const float z = __fadd_rn(__fdiv_rn(r.z, P.cell_len[2]), (float)P.ncell[2]);
    cx = (int)(((uint32_t)x) % (uint32_t)P.ncell[0]);
    cy = (int)(((uint32_t)y) % (uint32_t)P.ncell[1]);
    cz = (int)(((uint32_t)z) % (uint32_t)P.ncell[2]);
}

__global__ void __launch_bounds__(256) k_cell_clear(Dev d)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[3][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[3], L.n, v);
        const SysParam& P = d.sys[L.sys[k]];
        const uint32_t local = (v - L.p[3][k]) * 256u + threadIdx.x;
        if (local < P.ncells) d.cell_count[P.cell_off + local] = 0;
    }
}

__global__ void __launch_bounds__(256) k_bin(Dev d)
{
    const RbList L = rb_list(d);
    const uint32_t total = L.p[0][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[0], L.n, v);
        const SysParam& P = d.sys[L.sys[k]];
        const uint32_t i = P.off + (v - L.p[0][k]) * 256u + threadIdx.x;
        const float4 r = pos_hi(d.pos, i);
        if (species_bits(r.w) == PLACEHOLDER) continue;
        int cx, cy, cz;
        cell_coords(P, r, cx, cy, cz);
        const uint32_t c = ((uint32_t)cz * P.ncell[1] + cy) * P.ncell[0] + cx;
        const uint32_t q = atomicAdd(&d.cell_count[P.cell_off + c], 1u);
        if (q < P.cell_size) d.cell[P.cell_word_off + c * P.cell_size + q] = i;
    }
}

__device__ __forceinline__ void cell_sort_one(const Dev& d, uint32_t s, uint32_t c, uint32_t* buf, uint32_t lane);

// one warp per cell: sort the occupied slots ascending, pad with placeholders
__global__ void __launch_bounds__(128) k_cell_sort(Dev d)
{
    __shared__ uint32_t s_buf[4][256];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const RbList L = rb_list(d);
    const uint32_t total = L.p[4][L.n];
    for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
        const uint32_t k = rb_find(L.p[4], L.n, v);
        const uint32_t s = L.sys[k];
        const SysParam& P = d.sys[s];
        const uint32_t local = (v - L.p[4][k]) * 4u + warp;
        if (local < P.ncells) cell_sort_one(d, s, P.cell_off + local, s_buf[warp], lane);
        __syncwarp();
    }
}

__device__ __forceinline__ void cell_sort_one(const Dev& d, uint32_t s, uint32_t c, uint32_t* buf, uint32_t lane)
{
    const SysParam& P = d.sys[s];
    const uint32_t cs = P.cell_size;
    const uint32_t cnt = d.cell_count[c];
    if (lane == 0) {
        atomicMax(&d.st[s].max_cell, cnt);
        if (cnt > cs) atomicOr(d.status, ST_CELL_OVERFLOW);
    }
    const uint32_t n = min(cnt, cs);
    uint32_t* cell = d.cell + P.cell_word_off + (c - P.cell_off) * cs;
    for (uint32_t k = lane; k < n; k += 32) buf[k] = cell[k];
    __syncwarp();
    uint32_t mine[8];
    uint32_t rk[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint32_t k = lane + 32u * q;
        mine[q] = (k < n) ? buf[k] : PLACEHOLDER;
        rk[q] = 0;
    }
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t x = buf[k];
#pragma unroll
        for (int q = 0; q < 8; ++q) rk[q] += (x < mine[q]) ? 1u : 0u;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint32_t k = lane + 32u * q;
        if (k < n) cell[rk[q]] = mine[q];
        else if (k < cs) cell[k] = PLACEHOLDER;
    }
}

// ---------------------------------------------------------------------------
// Full Verlet list (from_binning_kernel.cu:144-163): every j != i with
// rr <= (r_c + skin)^2 in float, minimum image; blocked layout (Dev::nbr),
// near pairs (closer than NEAR_SIGMA sigma) from the front, far pairs from
// the back.  Also stores r0 = r for the displacement check
// (max_displacement.cpp:60-72).
//
// Shared scan (Dev::nbr_scan = 2; by default systems of at least
// NBR_SHARED_MIN_N particles): one warp per 32 consecutive slots.  After the
// Hilbert sort these are spatially compact, so the warp scans the cells
// around their bounding box once for all 32 particles: lanes load 32
// candidates of a cell at a time, drop those farther than r_c + skin from the
// box and buffer the rest in shared memory; every lane tests each batch of
// 32 buffered candidates against its own particle into bit masks and then
// appends its neighbours in batch order (cluster_batch).  Smaller systems, and warps whose box spans too many cells (an
// unsorted system, a tiny box), scan per lane instead: the 27 cells around each particle (each
// distinct cell once when a dimension has fewer than 3 cells).  Both scans
// test the same float criterion, so the pair sets are identical; entries are
// appended in cell order and, within a cell, in slot order (deterministic).
// ---------------------------------------------------------------------------

// Resident blocks of 128 threads per SM of the list build (64 registers).
// Both scans run without spills at this budget as long as the one-system
// variant recomputes its slot from the block index (held in a register, it
// pushed spill traffic into the shared scan's inner loop: 14 % more
// instructions, and 72 registers without spills measured 1 % slower than 64).
constexpr int NBR_MINB = 8;
// A one-system engine whose grid fills at most NBR_SMALL_MINB blocks per SM
// (KA-64k: 500 blocks on 152 SMs) gains nothing from 8 resident blocks; its
// build runs with 4, and up to 128 registers, which the compiler spends on
// more loads in flight (KA-64k chain 0.30 against 0.32 ms with the per-lane
// scan, 0.29 against 0.33 ms with the shared scan; at LJ-1M, whose grid is
// 13 waves, 4 blocks measured 1.20 against 0.99 ms).
constexpr int NBR_SMALL_MINB = 4;

constexpr uint32_t NBR_CLUSTER_MAX_CELLS = 150;   // larger cell ranges: per-lane scan
struct NbrOut {
    uint32_t* out;        // this slot's row in the blocked list
    size_t bstride;       // words between list blocks
    uint32_t lw, lmask;   // log2 of the block width, width - 1
    uint32_t cap;         // a multiple of the block width
    uint32_t nn = 0, nf = 0;
    __device__ __forceinline__ void add(uint32_t j, bool near)
    {
        const uint32_t e = near ? nn : cap - 1u - nf;
        if (nn + nf < cap) out[(e >> lw) * bstride + (e & lmask)] = j;
        if (near) ++nn; else ++nf;
    }
};

// The per-lane scan's writer: the same layout, with pn and pf following the
// next near and far entry incrementally, so an append costs no 64-bit
// multiply (the shared scan keeps NbrOut: its register budget is tighter).
// Entry e sits at (e / LB) * bstride + e % LB; nothing is stored once the two
// parts meet (the counts still grow: overflow is detected).
struct NbrOutInc {
    NbrOut& o;
    uint32_t* pn;
    uint32_t* pf;
    __device__ __forceinline__ explicit NbrOutInc(NbrOut& base) : o(base)
    {
        pn = o.out + (o.nn >> o.lw) * o.bstride + (o.nn & o.lmask);
        const uint32_t e = o.cap - 1u - o.nf;
        pf = o.out + (e >> o.lw) * o.bstride + (e & o.lmask);
    }
    __device__ __forceinline__ void add(uint32_t j, bool near)
    {
        if (near) add_near(j);
        else add_far(j);
    }
    __device__ __forceinline__ void add_near(uint32_t j)
    {
        if (o.nn + o.nf < o.cap) *pn = j;
        ++o.nn;
        pn += (o.nn & o.lmask) ? (ptrdiff_t)1 : (ptrdiff_t)(o.bstride - o.lmask);   // to the next block
    }
    __device__ __forceinline__ void add_far(uint32_t j)
    {
        if (o.nn + o.nf < o.cap) *pf = j;
        const uint32_t e = o.cap - 1u - o.nf;
        ++o.nf;
        pf -= (e & o.lmask) ? (ptrdiff_t)1 : (ptrdiff_t)(o.bstride - o.lmask);
    }
};

// box and species count in registers: the list stores of the scan loops
// could alias SysParam in global memory and would force a reload per pair
struct NbrBox {
    float L[3], Linv[3];
    uint32_t ns;
    __device__ __forceinline__ explicit NbrBox(const SysParam& P)
        : L{P.L[0], P.L[1], P.L[2]}, Linv{P.Linv[0], P.Linv[1], P.Linv[2]}, ns(P.ns) {}
};

// Pair cut-offs of the lane's particle for the list scans: held in
// registers for one or two species, read from shared memory per pair above
template <int NS>
struct LaneCut {
    float c0, c1, n0, n1;
    const float* rc;
    const float* rn;
    uint32_t ns;
    __device__ __forceinline__ LaneCut(const float* rrcs, const float* rrnear, uint32_t ns_)
        : c0(rrcs[0]), c1(NS == 2 ? rrcs[1] : 0.0f), n0(rrnear[0]), n1(NS == 2 ? rrnear[1] : 0.0f), rc(rrcs),
          rn(rrnear), ns(ns_) {}
    // false for a slot of no species of the system
    __device__ __forceinline__ bool get(uint32_t b, float& c, float& n) const
    {
        if (NS == 1) { c = c0; n = n0; return b == 0u; }
        if (NS == 2) { c = b ? c1 : c0; n = b ? n1 : n0; return b < 2u; }
        const bool ok = b < ns;
        c = rc[ok ? b : 0u];
        n = rn[ok ? b : 0u];
        return ok;
    }
};

// nbr_test (below) of the per-lane scan: the same criterion, in the same order
template <bool WRAP, int NS>
__device__ __forceinline__ void lane_test(const NbrBox& B, float4 ri, uint32_t i, float4 rj, uint32_t j,
                                          const LaneCut<NS>& cut, NbrOutInc& o)
{
    const float sx = __fsub_rn(ri.x, rj.x), sy = __fsub_rn(ri.y, rj.y), sz = __fsub_rn(ri.z, rj.z);
    const float dx = WRAP ? min_image(sx, B.L[0], B.Linv[0]) : sx;
    const float dy = WRAP ? min_image(sy, B.L[1], B.Linv[1]) : sy;
    const float dz = WRAP ? min_image(sz, B.L[2], B.Linv[2]) : sz;
    const float rr = rr_exact(dx, dy, dz);
    float c, n;
    const bool ok = cut.get(species_bits(rj.w), c, n);
    if (ok && rr <= c && j != i) o.add(j, rr < n);
}

// Positions are canonical, |x| <= L/2, and the binning maps x and x + L to
// one cell (cells are anchored at x = 0, so the periodic seam of the box
// may run through a cell).  A particle farther than 2.5 cell lengths from
// every face therefore sees, in its 27 cells, only particles of the same
// periodic image within two cell lengths (plus rounding) in each coordinate;
// that distance is below L/2 (the condition implies at least 6 cells), where
// min_image returns the separation unchanged (rint of a ratio below 1/2 is
// zero), so the minimum-image arithmetic is skipped without changing any
// result.  The cell indices still wrap.
__device__ __forceinline__ bool far_from_faces(const SysParam& P, float4 r)
{
    return fabsf(r.x) + 2.5f * P.cell_len[0] < 0.5f * P.L[0] && fabsf(r.y) + 2.5f * P.cell_len[1] < 0.5f * P.L[1] &&
           fabsf(r.z) + 2.5f * P.cell_len[2] < 0.5f * P.L[2];
}

// the 27 cells around the particle, for one lane (each distinct cell once
// when a dimension has fewer than 3 cells); WRAP = false only when every
// lane of the warp is far from the faces (far_from_faces)
template <bool WRAP, int NS>
__device__ __forceinline__ void lane_scan(const SysParam& P, const float4* pos, const uint32_t* cells,
                                          const uint32_t* counts, float4 ri, uint32_t i, int cx, int cy, int cz,
                                          const LaneCut<NS>& cut, NbrOut& base)
{
    NbrOutInc o(base);
    const NbrBox B(P);
    const int nx = P.ncell[0], ny = P.ncell[1], nz = P.ncell[2];
    const int lox = nx >= 3 ? -1 : 0, hix = nx >= 2 ? 1 : 0;
    const int loy = ny >= 3 ? -1 : 0, hiy = ny >= 2 ? 1 : 0;
    const int loz = nz >= 3 ? -1 : 0, hiz = nz >= 2 ? 1 : 0;
    const uint32_t cs = P.cell_size;
    for (int oz = loz; oz <= hiz; ++oz) {
        const int z = (cz + oz + nz) % nz;
        for (int oy = loy; oy <= hiy; ++oy) {
            const int y = (cy + oy + ny) % ny;
            for (int ox = lox; ox <= hix; ++ox) {
                const int x = (cx + ox + nx) % nx;
                const uint32_t c = (uint32_t)(z * ny + y) * nx + x;
                // occupied slots of the cell (ascending), four at a time so the
                // position gathers are independent of one another; a cell holds
                // a multiple of 32 words, so the last group's load stays inside
                const uint32_t nc = min(counts[c], cs);
                const uint4* cell4 = reinterpret_cast<const uint4*>(cells + c * cs);
                uint32_t k = 0;
                for (; k + 4 <= nc; k += 4) {
                    const uint4 jj = __ldg(cell4 + (k >> 2));
                    const float4 r0 = ldg_hi(pos, jj.x), r1 = ldg_hi(pos, jj.y);
                    const float4 r2 = ldg_hi(pos, jj.z), r3 = ldg_hi(pos, jj.w);
                    lane_test<WRAP, NS>(B, ri, i, r0, jj.x, cut, o);
                    lane_test<WRAP, NS>(B, ri, i, r1, jj.y, cut, o);
                    lane_test<WRAP, NS>(B, ri, i, r2, jj.z, cut, o);
                    lane_test<WRAP, NS>(B, ri, i, r3, jj.w, cut, o);
                }
                if (k < nc) {
                    const uint4 jj = __ldg(cell4 + (k >> 2));
                    const uint32_t jv[3] = {jj.x, jj.y, jj.z};
                    float4 rv[3];
#pragma unroll
                    for (int u = 0; u < 3; ++u) rv[u] = (k + u < nc) ? ldg_hi(pos, jv[u]) : make_float4(0, 0, 0, 0);
#pragma unroll
                    for (int u = 0; u < 3; ++u)
                        if (k + u < nc) lane_test<WRAP, NS>(B, ri, i, rv[u], jv[u], cut, o);
                }
            }
        }
    }
}

// The per-lane scan of one particle, out of line: it then gets its own
// register allocation instead of sharing the shared scan's (inlined
// together, the two spilled, and the rebuild chains measured 1-2 % slower).  Pointers are passed by value, not the kernel
// parameter block; the list counts come back as (near, far).
template <bool WRAP>
__device__ __noinline__ uint2 lane_scan_call(const SysParam* Pp, const float4* pos, const uint32_t* cell,
                                             const uint32_t* cell_count, float4 ri, uint32_t i, const float* rrcs,
                                             const float* rrnear, uint32_t* out, size_t bstride, uint32_t lw,
                                             uint32_t cap)
{
    const SysParam& P = *Pp;
    NbrOut o;
    o.out = out;
    o.bstride = bstride;
    o.lw = lw;
    o.lmask = (1u << lw) - 1u;
    o.cap = cap;
    int cx, cy, cz;
    cell_coords(P, ri, cx, cy, cz);
    const uint32_t* cells = cell + P.cell_word_off;
    const uint32_t* counts = cell_count + P.cell_off;
    if (P.ns == 1) lane_scan<WRAP, 1>(P, pos, cells, counts, ri, i, cx, cy, cz, LaneCut<1>(rrcs, rrnear, 1u), o);
    else if (P.ns == 2) lane_scan<WRAP, 2>(P, pos, cells, counts, ri, i, cx, cy, cz, LaneCut<2>(rrcs, rrnear, 2u), o);
    else lane_scan<WRAP, 0>(P, pos, cells, counts, ri, i, cx, cy, cz, LaneCut<0>(rrcs, rrnear, P.ns), o);
    return make_uint2(o.nn, o.nf);
}

// Per-warp shared memory of the cluster scan: a buffer of staged candidates
// (a batch of 32 plus the up to 31 a cell adds beyond it), and per particle
// of the cluster the batch position of the candidate that is the particle
// itself
struct ClusterSmem {
    float4 pos[64];
    uint32_t j[64];
    uint32_t self[32];
};

// One batch of cnt <= 32 staged candidates (FULL: cnt = 32) against the
// lane's particle: the list criterion of each candidate goes into bit u of
// a keep mask and a near mask (no branch per candidate), then the lane
// appends its neighbours in batch order (ascending u).  A particle meets
// itself at r^2 = 0; that bit is cleared through ClusterSmem::self (the
// list criterion's j != i).
template <bool WRAP, int NS, bool FULL>
__device__ __forceinline__ void cluster_batch(const NbrBox& B, ClusterSmem& sm, uint32_t cnt, uint32_t i0, float4 ri,
                                              const LaneCut<NS>& cut, uint32_t lane, bool real, NbrOutInc& o)
{
    sm.self[lane] = 32u;
    __syncwarp();
    if (lane < cnt) {
        const uint32_t j = sm.j[lane];
        if (j - i0 < 32u) sm.self[j - i0] = lane;
    }
    __syncwarp();
    if (real) {
        uint32_t keep = 0, near = 0;
#pragma unroll
        for (uint32_t u = 0; u < 32u; ++u) {
            if (!FULL && u >= cnt) break;
            const float4 rj = sm.pos[u];
            const float sx = __fsub_rn(ri.x, rj.x), sy = __fsub_rn(ri.y, rj.y), sz = __fsub_rn(ri.z, rj.z);
            const float dx = WRAP ? min_image(sx, B.L[0], B.Linv[0]) : sx;
            const float dy = WRAP ? min_image(sy, B.L[1], B.Linv[1]) : sy;
            const float dz = WRAP ? min_image(sz, B.L[2], B.Linv[2]) : sz;
            const float rr = rr_exact(dx, dy, dz);
            float c, n;
            const bool ok = cut.get(species_bits(rj.w), c, n);
            if (ok && rr <= c) keep |= 1u << u;
            if (rr < n) near |= 1u << u;
        }
        const uint32_t self = sm.self[lane];
        if (self < 32u) keep &= ~(1u << self);
        near &= keep;
        uint32_t far = keep & ~near;
        // near entries, then far entries: each loop without a branch on the
        // part (the parts grow from the two ends of the list independently)
        while (near) {
            const uint32_t u = __ffs(near) - 1u;
            near &= near - 1u;
            o.add_near(sm.j[u]);
        }
        while (far) {
            const uint32_t u = __ffs(far) - 1u;
            far &= far - 1u;
            o.add_far(sm.j[u]);
        }
    }
    __syncwarp();
}

// The cells around the bounding box [lo, hi] of the warp's 32 particles
// (cell ranges c0 + [0, nc) per dimension, wrapped): lanes load 32
// candidates of a cell at a time and buffer those within r_c + skin of the
// box (in cell order, ascending slots within a cell); every full batch of
// 32, and the rest at the end, goes through cluster_batch.
template <bool WRAP, int NS>
__device__ __forceinline__ void cluster_scan(const Dev& d, const SysParam& P, float4 ri, uint32_t i, bool real,
                                             const LaneCut<NS>& cut, NbrOut& base, const float* lo, const float* hi,
                                             const int* c0, const int* ncr, float rcs2, ClusterSmem& sm,
                                             uint32_t lane)
{
    const NbrBox B(P);
    NbrOutInc o(base);
    const float cxb = 0.5f * (lo[0] + hi[0]), cyb = 0.5f * (lo[1] + hi[1]), czb = 0.5f * (lo[2] + hi[2]);
    const float hxb = 0.5f * (hi[0] - lo[0]), hyb = 0.5f * (hi[1] - lo[1]), hzb = 0.5f * (hi[2] - lo[2]);
    const int nx = P.ncell[0], ny = P.ncell[1], nz = P.ncell[2];
    const uint32_t cs = P.cell_size;
    // the system's cell tables, read once (the list stores could alias SysParam)
    const uint32_t* counts = d.cell_count + P.cell_off;
    const uint32_t* cells = d.cell + P.cell_word_off;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t i0 = i - lane;   // the warp's slots are consecutive
    uint32_t nb = 0;   // buffered candidates (warp-uniform)
    int z = c0[2];
    for (int kz = 0; kz < ncr[2]; ++kz, z = (z + 1 == nz) ? 0 : z + 1) {
        int y = c0[1];
        for (int ky = 0; ky < ncr[1]; ++ky, y = (y + 1 == ny) ? 0 : y + 1) {
            int x = c0[0];
            for (int kx = 0; kx < ncr[0]; ++kx, x = (x + 1 == nx) ? 0 : x + 1) {
                const uint32_t c = (uint32_t)(z * ny + y) * nx + x;
                const uint32_t nc = min(counts[c], cs);
                const uint32_t* cell = cells + c * cs;
                for (uint32_t k = 0; k < nc; k += 32) {
                    const bool have = k + lane < nc;
                    const uint32_t j = have ? __ldg(cell + k + lane) : 0u;
                    const float4 rj = have ? ldg_hi(d.pos, j) : make_float4(0, 0, 0, 0);
                    bool keep = false;
                    if (have) {
                        // distance from the candidate to the bounding box
                        float ex = __fsub_rn(rj.x, cxb), ey = __fsub_rn(rj.y, cyb), ez = __fsub_rn(rj.z, czb);
                        if (WRAP) {
                            ex = min_image(ex, B.L[0], B.Linv[0]);
                            ey = min_image(ey, B.L[1], B.Linv[1]);
                            ez = min_image(ez, B.L[2], B.Linv[2]);
                        }
                        const float qx = fmaxf(fabsf(ex) - hxb, 0.0f);
                        const float qy = fmaxf(fabsf(ey) - hyb, 0.0f);
                        const float qz = fmaxf(fabsf(ez) - hzb, 0.0f);
                        keep = qx * qx + qy * qy + qz * qz <= rcs2;
                    }
                    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, keep);
                    if (keep) {
                        const uint32_t at = nb + __popc(ballot & lt_mask);
                        sm.pos[at] = rj;
                        sm.j[at] = j;
                    }
                    nb += __popc(ballot);
                    __syncwarp();
                    if (nb >= 32u) {
                        cluster_batch<WRAP, NS, true>(B, sm, 32u, i0, ri, cut, lane, real, o);
                        // the candidates beyond the batch move to the front
                        const uint32_t rest = nb - 32u;
                        float4 tp = make_float4(0, 0, 0, 0);
                        uint32_t tj = 0;
                        if (lane < rest) { tp = sm.pos[32u + lane]; tj = sm.j[32u + lane]; }
                        __syncwarp();
                        if (lane < rest) { sm.pos[lane] = tp; sm.j[lane] = tj; }
                        nb = rest;
                        __syncwarp();
                    }
                }
            }
        }
    }
    if (nb > 0u) cluster_batch<WRAP, NS, false>(B, sm, nb, i0, ri, cut, lane, real, o);
}

template <bool WRAP>
__device__ __forceinline__ void cluster_scan_ns(const Dev& d, const SysParam& P, float4 ri, uint32_t i, bool real,
                                                const float* rrcs, const float* rrnear, NbrOut& o, const float* lo,
                                                const float* hi, const int* c0, const int* ncr, float rcs2,
                                                ClusterSmem& sm, uint32_t lane)
{
    if (P.ns == 1)
        cluster_scan<WRAP, 1>(d, P, ri, i, real, LaneCut<1>(rrcs, rrnear, 1u), o, lo, hi, c0, ncr, rcs2, sm, lane);
    else if (P.ns == 2)
        cluster_scan<WRAP, 2>(d, P, ri, i, real, LaneCut<2>(rrcs, rrnear, 2u), o, lo, hi, c0, ncr, rcs2, sm, lane);
    else
        cluster_scan<WRAP, 0>(d, P, ri, i, real, LaneCut<0>(rrcs, rrnear, P.ns), o, lo, hi, c0, ncr, rcs2, sm,
                              lane);
}

__device__ __forceinline__ void neighbour_slot(const Dev& d, uint32_t s, uint32_t i, const float* s_rrcs,
                                               const float* s_rrnear, ClusterSmem& sm, uint32_t lane);

// two virtual blocks of 128 slots per 256-slot unit of a rebuilding system.
// Only v stays live across the scan: the list bounds are read again each
// round (the list stores may alias them, so they are not kept in
// registers) and the pair table is staged again per virtual block.
// LOOP = false: the grid has a block per virtual block (one-system engines).
template <bool LOOP, int MINB = NBR_MINB>
__global__ void __launch_bounds__(128, MINB) k_neighbour(Dev d)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __shared__ float s_rrcs[MAX_SPECIES * MAX_SPECIES];
    __shared__ float s_rrnear[MAX_SPECIES * MAX_SPECIES];
    __shared__ ClusterSmem s_cl[4];
    for (uint32_t v = blockIdx.x;; v += gridDim.x) {
        const RbList L = rb_list(d);
        if (v >= 2u * L.p[0][L.n]) break;
        // one system (LOOP = false): system 0 at slot 0, so the slot is
        // recomputed from the block index instead of held in a register
        const uint32_t k = LOOP ? rb_find(L.p[0], L.n, v >> 1) : 0u;
        const uint32_t s = LOOP ? L.sys[k] : 0u;
        const SysParam& P = d.sys[s];
        const uint32_t i = LOOP ? P.off + (v - 2u * L.p[0][k]) * 128u + threadIdx.x : blockIdx.x * 128u + threadIdx.x;
        __syncthreads();
        if (threadIdx.x < P.ns * P.ns) {
            s_rrcs[threadIdx.x] = d.pair[P.pair_off + threadIdx.x].rr_cut_skin;
            s_rrnear[threadIdx.x] = d.pair[P.pair_off + threadIdx.x].rr_near;
        }
        __syncthreads();
        neighbour_slot(d, s, i, s_rrcs, s_rrnear, s_cl[warp], lane);
        if (!LOOP) break;
    }
}

// the Verlet list of slot i (one lane; the warp's 32 slots scan together)
__device__ __forceinline__ void neighbour_slot(const Dev& d, uint32_t s, uint32_t i, const float* s_rrcs,
                                               const float* s_rrnear, ClusterSmem& sm, uint32_t lane)
{
    const SysParam& P = d.sys[s];
    const float4 ri = pos_hi(d.pos, i);
    const uint32_t a = species_bits(ri.w);
    const bool real = a != PLACEHOLDER;
    NbrOut o;
    o.lw = d.lb_log2;
    o.lmask = (1u << o.lw) - 1u;
    o.bstride = (size_t)d.S << o.lw;
    o.out = d.nbr + ((size_t)i << o.lw);
    o.cap = d.nbr_cap;
    if (real) {
        d.r0[i] = ri;
        if (d.ds) d.fpos[i] = fpos_encode(ri, pos_lo(d.pos, i), P.lo_inv_scale);
    }
    // bounding box of the warp's real particles
    float lo[3] = {real ? ri.x : INFINITY, real ? ri.y : INFINITY, real ? ri.z : INFINITY};
    float hi[3] = {real ? ri.x : -INFINITY, real ? ri.y : -INFINITY, real ? ri.z : -INFINITY};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
#pragma unroll
        for (int w = 16; w > 0; w >>= 1) {
            lo[q] = fminf(lo[q], __shfl_xor_sync(0xFFFFFFFFu, lo[q], w));
            hi[q] = fmaxf(hi[q], __shfl_xor_sync(0xFFFFFFFFu, hi[q], w));
        }
    }
    if (__any_sync(0xFFFFFFFFu, real)) {
        float rcs2 = 0.0f;
        for (uint32_t q = 0; q < P.ns * P.ns; ++q) rcs2 = fmaxf(rcs2, s_rrcs[q]);
        const float rcs = sqrtf(rcs2) * (1.0f + 1e-4f);   // margin: a superset of the cells is harmless
        // cell range per dimension, with the binning's own float formula (monotonic in x)
        int c0[3], ncr[3];
        bool wrap = false;
        uint32_t ncells = 1;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int n = P.ncell[q];
            float ul = __fadd_rn(__fdiv_rn(__fsub_rn(lo[q], rcs), P.cell_len[q]), (float)n);
            float uh = __fadd_rn(__fdiv_rn(__fadd_rn(hi[q], rcs), P.cell_len[q]), (float)n);
            // positions lie in [-L/2, L/2]: u in [n/2 - 1, 3n/2 + 1]; the clamp only
            // guards the integer conversion against non-finite positions
            ul = fminf(fmaxf(ul, 0.0f), 4.0f * n);
            uh = fminf(fmaxf(uh, 0.0f), 4.0f * n);
            const int a0 = (int)floorf(ul), a1 = (int)floorf(uh);
            if (!(a1 >= a0) || a1 - a0 + 1 >= n) { c0[q] = 0; ncr[q] = n; }
            else { c0[q] = a0 % n; ncr[q] = a1 - a0 + 1; }
            ncells *= (uint32_t)ncr[q];
            const float half = 0.5f * P.L[q];
            // no pair of the scan reaches |s| >= L/2 and no cell range crosses the box
            wrap |= !(__fsub_rn(lo[q], rcs) > -half && __fadd_rn(hi[q], rcs) < half &&
                      (hi[q] - lo[q]) + 2.0f * rcs < 0.49f * P.L[q]);
        }
        // by default a system of at least NBR_SHARED_MIN_N particles uses the shared
        // scan: a decision of the system alone, so its lists (and their order) do
        // not depend on the other systems of the engine
        const bool shared = d.nbr_scan == 2u || (d.nbr_scan == 0u && P.n >= NBR_SHARED_MIN_N);
        const float* rrcs = s_rrcs + (real ? a : 0u) * P.ns;
        const float* rrnear = s_rrnear + (real ? a : 0u) * P.ns;
        if (shared && ncells <= NBR_CLUSTER_MAX_CELLS) {
            if (wrap)
                cluster_scan_ns<true>(d, P, ri, i, real, rrcs, rrnear, o, lo, hi, c0, ncr, rcs * rcs, sm, lane);
            else
                cluster_scan_ns<false>(d, P, ri, i, real, rrcs, rrnear, o, lo, hi, c0, ncr, rcs * rcs, sm, lane);
        } else {
            const bool lwrap = __any_sync(0xFFFFFFFFu, real && !far_from_faces(P, ri));
            if (real) {
                const uint2 c = lwrap ? lane_scan_call<true>(d.sys + s, d.pos, d.cell, d.cell_count, ri, i, rrcs,
                                                             rrnear, o.out, o.bstride, o.lw, o.cap)
                                      : lane_scan_call<false>(d.sys + s, d.pos, d.cell, d.cell_count, ri, i, rrcs,
                                                              rrnear, o.out, o.bstride, o.lw, o.cap);
                o.nn = c.x;
                o.nf = c.y;
            }
        }
    }
    uint32_t count = 0;
    if (real) {
        count = o.nn + o.nf;
        const uint32_t sn = min(o.nn, o.cap);
        const uint32_t sf = min(o.nf, o.cap - sn);   // stored regions never overlap
        d.nbr_count[i] = sn | (sf << 16);
    }
    // warp-aggregated maximum and overflow flag (all lanes of the warp are here)
    uint32_t m = count;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, w));
    if (lane == 0) {
        if (m > 0) atomicMax(&d.st[s].max_nbr, m);
        if (m > d.nbr_cap) atomicOr(d.status, ST_NBR_OVERFLOW);
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

int radix_passes(uint32_t key_bits) { return (int)((key_bits + 7) / 8); }

// Sort the slot ranges of the systems that rebuild; the permutation ends in
// val[passes % 2]
// Launch grids of the rebuild chain: the kernels loop over the virtual blocks
// of the rebuild list, so a grid never needs more blocks than the work the
// engine could hold (one block per unit of every system).  An engine of
// several systems caps the grid at RB_WAVE blocks per SM, so the systems
// that do not rebuild cost no blocks; an engine of one system (nothing to
// compact) launches one block per unit, which the block scheduler balances
// better than a fixed share per block.
static unsigned rb_grid(const Dev& d, uint32_t upper)
{
    return std::max(1u, d.nsys == 1 ? upper : std::min(upper, RB_WAVE * d.sm_count));
}

void launch_rebuild_list(const Dev& d, cudaStream_t st)
{
    k_rebuild_list<<<1, 1024, 0, st>>>(d);
}

void launch_sort(const Dev& d, int passes, cudaStream_t st)
{
    k_seg_keys<<<rb_grid(d, d.S_grid / 256), 256, 0, st>>>(d);
    for (int p = 0; p < passes; ++p) {
        const uint32_t shift = 8u * p;
        const int cur = p & 1;
        k_seg_hist<<<rb_grid(d, d.tiles_grid), RADIX_THREADS, 0, st>>>(d, d.key[cur], shift);
        k_seg_scan<<<dim3(rb_grid(d, d.nsys), 32), 256, 0, st>>>(d);
        k_seg_scatter<<<rb_grid(d, d.tiles_grid), RADIX_THREADS, 0, st>>>(d, d.key[cur], d.val[cur], d.key[1 - cur],
                                                                       d.val[1 - cur], shift);
    }
}

int sort_kernel_count(int passes) { return 1 + 3 * passes; }

void launch_rearrange(const Dev& d, bool ds, const uint32_t* perm, cudaStream_t st)
{
    const unsigned grid = rb_grid(d, d.S_grid / 256);
    if (ds) { k_rearrange<true><<<grid, 256, 0, st>>>(d, perm); k_copyback<true><<<grid, 256, 0, st>>>(d); }
    else { k_rearrange<false><<<grid, 256, 0, st>>>(d, perm); k_copyback<false><<<grid, 256, 0, st>>>(d); }
}

void launch_binning(const Dev& d, cudaStream_t st)
{
    k_cell_clear<<<rb_grid(d, (d.cells_grid + 255) / 256 + d.nsys), 256, 0, st>>>(d);
    k_bin<<<rb_grid(d, d.S_grid / 256), 256, 0, st>>>(d);
    k_cell_sort<<<rb_grid(d, (d.cells_grid + 3) / 4 + d.nsys), 128, 0, st>>>(d);
}

void launch_neighbour(const Dev& d, cudaStream_t st)
{
    // one-system engines launch a block per virtual block; otherwise one
    // wave of resident blocks loops over the virtual blocks
    const unsigned all = std::max(1u, d.S_grid / 128);
    if (d.nsys == 1 && all <= d.sm_count * NBR_SMALL_MINB) k_neighbour<false, NBR_SMALL_MINB><<<all, 128, 0, st>>>(d);
    else if (d.nsys == 1) k_neighbour<false><<<all, 128, 0, st>>>(d);
    else k_neighbour<true><<<std::min(all, d.sm_count * NBR_MINB), 128, 0, st>>>(d);
}

void launch_hilbert_keys(const Dev& d, uint32_t* keys, cudaStream_t st)
{
    k_hilbert_keys<<<(d.S_grid + 255) / 256, 256, 0, st>>>(d, keys);
}

} // namespace hmd
