// kernels_force_full.cu — untruncated pair forces over all pairs
// (mdsim/gpu/forces/pair_full_kernel.cuh:49-130, pair_full.hpp:192-270): the
// module the reference's force constructor picks when the potential has no
// cutoff (lua/halmd/mdsim/forces/pair.lua.in:78-83).  No binning and no list:
//   F_i = Σ_{j≠i} fval(r_ij²) r_ij,  r_ij the minimum image,
//   aux: E_i = ½ Σ U, stress_i = ½ Σ fval r⊗r (the weight is halved because
//   both particles of a pair belong to the same instance, pair_full.hpp:249-252).
// The pair arithmetic is that of the list kernels (force.cuh) with an
// infinite cutoff: compensated separation and accumulation, so the sum over
// all N - 1 partners is as accurate as the reference's dsfloat accumulator.
#include "force.cuh"

namespace hmd {

// lanes per particle: a block of 128 threads covers 32 particles, and each
// lane takes every FULL_LANES-th partner of a staged tile
constexpr uint32_t FULL_LANES = 4;
constexpr uint32_t FULL_TILE = 128;

// s_r holds the tile's hi and lo words side by side (slot u at 2u, 2u + 1)
template <int POT, bool AUX>
__device__ __forceinline__ void full_tile_pot(const SysParam& P, const PairParam* row, float4 ri, float4 li,
                                              uint32_t i, uint32_t base, const float4* s_r, uint32_t q, ForceAcc2& B)
{
    // entries u and u + FULL_LANES of the lane's share evaluated together
    for (uint32_t u = q; u < FULL_TILE; u += 2 * FULL_LANES) {
        const float4 ra = s_r[2 * u], rb = s_r[2 * (u + FULL_LANES)];
        const float4 la = s_r[2 * u + 1], lb = s_r[2 * (u + FULL_LANES) + 1];
        const uint32_t ba = species_bits(ra.w), bb = species_bits(rb.w);
        const bool va = ba < P.ns && base + u != i;
        const bool vb = bb < P.ns && base + u + FULL_LANES != i;
        pot_pair2<POT, AUX, true, true, true>(row[va ? ba : 0u], row[vb ? bb : 0u], P, ri, ra, rb, va, vb, B, li,
                                              la, lb);
    }
}

template <bool AUX>
__global__ void __launch_bounds__(128) k_force_full(Dev d)
{
    constexpr uint32_t W = FULL_LANES;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t / W, q = t % W;
    const uint32_t s = d.chunk_sys[(blockIdx.x * (blockDim.x / W)) / CHUNK];
    const SysParam& P = d.sys[s];
    __shared__ PairParam spp[MAX_SPECIES * MAX_SPECIES];
    __shared__ float4 s_r[2 * FULL_TILE];
    if (threadIdx.x < P.ns * P.ns) spp[threadIdx.x] = d.pair[P.pair_off + threadIdx.x];
    __syncthreads();
    if (!P.active || !d.st[s].live || *d.status != 0u) return;   // block-uniform
    if (force_kind_of(P) != FK_FULL) return;                       // a list kind's block
    const float4 ri = pos_hi(d.pos, i), li = pos_lo(d.pos, i);   // lo words 0 in FP32 engines
    const uint32_t a = species_bits(ri.w);
    const bool real = a != PLACEHOLDER;
    const PairParam* row = spp + (real ? a : 0u) * P.ns;
    ForceAcc A;
    ForceAcc2 B;
    for (uint32_t base = P.off; base < P.off + P.A; base += FULL_TILE) {
        __syncthreads();
        s_r[2 * threadIdx.x] = pos_hi(d.pos, base + threadIdx.x);
        s_r[2 * threadIdx.x + 1] = pos_lo(d.pos, base + threadIdx.x);
        __syncthreads();
        if (!real) continue;
        switch (P.pot) {
        case POT_LJ:
            for (uint32_t u = q; u < FULL_TILE; u += W) {
                const float4 rj = s_r[2 * u];
                const uint32_t b = species_bits(rj.w);
                if (b < P.ns && base + u != i)
                    near_pair<TRUNC_SHARP, AUX, true, false, true>(row[b], P, ri, rj, A, li, s_r[2 * u + 1]);
            }
            break;
        case POT_MIE: full_tile_pot<POT_MIE, AUX>(P, row, ri, li, i, base, s_r, q, B); break;
        case POT_MORSE: full_tile_pot<POT_MORSE, AUX>(P, row, ri, li, i, base, s_r, q, B); break;
        default: full_tile_pot<POT_POWER_LAW, AUX>(P, row, ri, li, i, base, s_r, q, B); break;
        }
    }
    if (P.pot != POT_LJ) {
        fold_lanes2<AUX>(B, A);
        two_sum_acc(A.fx, A.cx, A.gx);
        two_sum_acc(A.fy, A.cy, A.gy);
        two_sum_acc(A.fz, A.cz, A.gz);
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

void launch_force_full(const Dev& d, bool aux, cudaStream_t st)
{
    const unsigned grid = (unsigned)((size_t)d.S_grid * FULL_LANES / 128);
    if (aux) k_force_full<true><<<grid, 128, 0, st>>>(d);
    else k_force_full<false><<<grid, 128, 0, st>>>(d);
}

} // namespace hmd
