/*
 * oracle.cpp — CPU restatement of HALMD's molecular-dynamics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product in
 * halmd_gb300/csrc: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py may load it.  Nothing in the product links it.
 *
 * Two families of functions live here:
 *
 *  1. FP64 restatements of the reference's host backend (mdsim/host/...),
 *     which serve as the accuracy oracle and as the timed single-core CPU
 *     baseline (the reference host backend itself needs Boost, Lua and HDF5
 *     and cannot be built here):
 *       - Lennard-Jones + truncations   mdsim/host/potentials/pair/lennard_jones.hpp:56-66,
 *                                        .../truncations/{sharp,shifted,smooth_r4,force_shifted}.hpp
 *       - periodic box                  mdsim/box.hpp:115-140
 *       - cell binning                  mdsim/host/binning.cpp:47-116
 *       - half neighbour list           mdsim/host/neighbours/from_binning.cpp:118-229
 *       - truncated pair force (+aux)   mdsim/host/forces/pair_trunc.hpp:219-344
 *       - velocity Verlet               mdsim/host/integrators/verlet.cpp:59-101
 *       - max displacement              mdsim/host/max_displacement.cpp:67-87, skin/2 rule
 *                                        mdsim/gpu/neighbours/from_binning.cpp:130
 *       - accumulator                   numeric/accumulator.hpp:83-119
 *       - MSD / density modes / ISF      observables/dynamics/mean_square_displacement.hpp:36-42,
 *                                        observables/gpu/density_mode_kernel.cu:46-82 (+ sign
 *                                        convention density_mode.cpp:128),
 *                                        observables/dynamics/intermediate_scattering_function.hpp:89-113
 *       - wavevector shells             algorithm/host/pick_lattice_points.hpp:74-160
 *       - fcc lattice                   mdsim/host/positions/lattice.cpp:64-120
 *
 *  2. Bit-exact restatements of the FP32 / double-single conventions that
 *     the GPU path adopts from the reference's GPU backend (mdsim/gpu/...):
 *       - float minimum image            mdsim/gpu/box_kernel.cuh:37-47
 *       - full-list criterion rr <= rc_skin^2 in float
 *                                        mdsim/gpu/neighbours/from_binning_kernel.cu:144-163
 *       - cell index / cell contents     mdsim/gpu/binning_kernel.cu:60-123, binning.cpp:81-116
 *       - Hilbert key                    mdsim/sorts/hilbert_kernel.hpp:70-230,
 *                                        mdsim/gpu/sorts/hilbert_kernel.cu:39-66, hilbert.cpp:51-54
 *       - DSFUN add/sub/mul              numeric/mp/dsfun.hpp:124-210
 *       - dsfloat velocity Verlet        mdsim/gpu/integrators/verlet_kernel.cu:38-98
 *       - float max displacement         mdsim/gpu/max_displacement_kernel.cu:37-68
 *       - Andersen thermostat             mdsim/host/integrators/verlet_nvt_andersen.cpp:111-137
 *         (per-particle collisions; random numbers from Philox4x32-10,
 *          J. K. Salmon et al., "Parallel random numbers: as easy as 1, 2, 3",
 *          SC'11 — the reference's rand48 / Boost mt19937 streams have no KAT,
 *          so RNG-dependent parity is statistical against the reference and
 *          exact against this restatement for the collision decisions)
 *
 * Compile with -ffp-contract=off: the float functions must round every
 * operation exactly as the CUDA kernels' __f*_rn intrinsics do.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#define ORC_API extern "C" __attribute__((visibility("default")))

typedef uint32_t u32;
static const u32 PLACEHOLDER = 0xFFFFFFFFu;

/* ------------------------------------------------------------------------ */
/* Lennard-Jones potential with truncations (FP64)                           */
/* ------------------------------------------------------------------------ */

/* TRUNC_NONE: the untruncated potential (host/forces/pair_full.hpp): an
 * infinite cutoff, so the half list below holds every pair i < j exactly
 * once, as pair_full.hpp:237-239 loops j from i + 1 */
enum { TRUNC_SHARP = 0, TRUNC_SHIFTED = 1, TRUNC_SMOOTH_R4 = 2, TRUNC_FORCE_SHIFTED = 3, TRUNC_NONE = 4 };
enum { ORC_MAX_SPECIES = 8 };

enum { POT_LJ = 0, POT_MIE = 1, POT_MORSE = 2, POT_POWER_LAW = 3 };

struct orc_pot {
    int ns;
    int trunc;
    int pot;
    double h;
    double rri_smooth;
    double eps[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double sigma2[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double rcut[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double rrcut[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double encut[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double fcut[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    /* mie: m, n and eps C(m, n); power_law: index; morse: r_min / sigma, B */
    unsigned idx_m[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    unsigned idx_n[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double eps_C[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double sigma[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double rmin_sigma[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    double distortion[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
};

ORC_API size_t orc_pot_sizeof(void) { return sizeof(orc_pot); }

/* mdsim/host/potentials/pair/lennard_jones.hpp:56-66 */
static inline void lj_bare(const orc_pot* p, double rr, int ab, double* fval, double* en)
{
    double sigma2 = p->sigma2[ab];
    double rri = sigma2 / rr;
    double r6i = rri * rri * rri;
    double eps_r6i = p->eps[ab] * r6i;
    *fval = 48 * rri * eps_r6i * (r6i - 0.5) / sigma2;
    *en = 4 * eps_r6i * (r6i - 1);
}

/* integer power (numeric/pow.hpp) */
static inline double ipow_d(double x, unsigned n)
{
    double y = 1;
    for (; n; n >>= 1, x *= x)
        if (n & 1) y *= x;
    return y;
}

/* mdsim/host/potentials/pair/mie.hpp:63-73 (prefactor mie.cpp:85-92) */
static inline void mie_bare(const orc_pot* p, double rr, int ab, double* fval, double* en)
{
    const double sigma2 = p->sigma2[ab];
    const unsigned m_2 = p->idx_m[ab] / 2, n_2 = p->idx_n[ab] / 2;
    const double rri = sigma2 / rr;
    const double rni = ipow_d(rri, n_2);
    const double rmni = (m_2 - n_2 == n_2) ? rni : ipow_d(rri, m_2 - n_2);
    const double eps_rni = p->eps_C[ab] * rni;
    *fval = 2 * rri * eps_rni * (m_2 * rmni - n_2) / sigma2;
    *en = eps_rni * (rmni - 1);
}

/* mdsim/host/potentials/pair/morse.hpp:64-77 */
static inline void morse_bare(const orc_pot* p, double rr, int ab, double* fval, double* en)
{
    const double B = p->distortion[ab];
    const double r_sigma_B = std::sqrt(rr) / p->sigma[ab] / B;
    const double dr = p->rmin_sigma[ab] / B - r_sigma_B;
    const double exp_dr = std::exp(dr);
    const double A = 2 * B * B - 1;
    const double exp_A_dr = (A == 1) ? exp_dr : std::exp(A * dr);
    const double eps_exp_dr = p->eps[ab] * exp_dr / A;
    *fval = (A + 1) * eps_exp_dr * (exp_A_dr - 1) * r_sigma_B / rr;
    *en = eps_exp_dr * (exp_A_dr - A - 1);
}

/* mdsim/host/potentials/pair/power_law.hpp:129-148 */
static inline void power_law_bare(const orc_pot* p, double rr, int ab, double* fval, double* en)
{
    const unsigned n = p->idx_m[ab];
    const double rri = p->sigma2[ab] / rr;
    double rni = ipow_d(rri, n / 2);
    if (n % 2) rni *= std::sqrt(rri);
    const double eps_rni = p->eps[ab] * rni;
    *fval = n * eps_rni / rr;
    *en = eps_rni;
}

static inline void pot_bare(const orc_pot* p, double rr, int ab, double* fval, double* en)
{
    switch (p->pot) {
    case POT_MIE: mie_bare(p, rr, ab, fval, en); break;
    case POT_MORSE: morse_bare(p, rr, ab, fval, en); break;
    case POT_POWER_LAW: power_law_bare(p, rr, ab, fval, en); break;
    default: lj_bare(p, rr, ab, fval, en); break;
    }
}

/* host/potentials/pair/{lennard_jones.hpp:56-66, mie.cpp:72-92, morse.hpp:64-77,
 * power_law.hpp:129-148}; truncation constants as truncations/{shifted,
 * force_shifted,smooth_r4}.hpp */
/* any potential: idx_m = mie m or power_law index, idx_n = mie n; r_min and
 * distortion for morse (r_min in absolute units); null where unused */
ORC_API int orc_pot_init_any(orc_pot* p, int pot, int ns, const double* eps, const double* sigma,
                             const double* rcut_sigma, int trunc, double h, const unsigned* idx_m,
                             const unsigned* idx_n, const double* r_min, const double* distortion)
{
    if (ns < 1 || ns > ORC_MAX_SPECIES) return -1;
    if (trunc < 0 || trunc > TRUNC_NONE || pot < 0 || pot > 3) return -1;
    std::memset(p, 0, sizeof(*p));
    p->ns = ns;
    p->trunc = trunc;
    p->pot = pot;
    p->h = h;
    p->rri_smooth = (trunc == TRUNC_SMOOTH_R4) ? std::pow(h, -2) : 0;
    for (int ab = 0; ab < ns * ns; ++ab) {
        p->eps[ab] = eps[ab];
        p->sigma[ab] = sigma[ab];
        p->sigma2[ab] = sigma[ab] * sigma[ab];
        p->rcut[ab] = (trunc == TRUNC_NONE) ? INFINITY : sigma[ab] * rcut_sigma[ab];
        p->rrcut[ab] = p->rcut[ab] * p->rcut[ab];
        if (pot == POT_MIE) {
            const unsigned m = idx_m[ab], n = idx_n[ab];
            if ((m & 1) || (n & 1) || m <= n || n == 0) return -2;   /* mie.cpp:72-83 */
            p->idx_m[ab] = m;
            p->idx_n[ab] = n;
            const double md = m, nd = n;
            p->eps_C[ab] = eps[ab] * (md / (md - nd) * std::pow(md / nd, nd / (md - nd)));
        } else if (pot == POT_POWER_LAW) {
            p->idx_m[ab] = idx_m[ab];
        } else if (pot == POT_MORSE) {
            p->rmin_sigma[ab] = r_min[ab] / sigma[ab];
            p->distortion[ab] = distortion[ab];
        }
        double f = 0, e = 0;
        if (trunc != TRUNC_NONE) pot_bare(p, p->rrcut[ab], ab, &f, &e);
        p->encut[ab] = (trunc == TRUNC_SHARP) ? 0 : e;
        /* force_shifted.hpp:63-64 stores F_c = fval(rc) * rc */
        p->fcut[ab] = (trunc == TRUNC_FORCE_SHIFTED) ? f * p->rcut[ab] : 0;
    }
    return 0;
}

/* rcut_sigma: cutoff in units of sigma (as the reference's `cutoff` matrix) */
ORC_API int orc_pot_init(orc_pot* p, int ns, const double* eps, const double* sigma,
                         const double* rcut_sigma, int trunc, double h)
{
    return orc_pot_init_any(p, POT_LJ, ns, eps, sigma, rcut_sigma, trunc, h, nullptr, nullptr, nullptr, nullptr);
}

/* truncations/{sharp,shifted,smooth_r4,force_shifted}.hpp operator() */
ORC_API void orc_pot_eval(const orc_pot* p, double rr, int a, int b, double* fval, double* en)
{
    int ab = a * p->ns + b;
    double f, e;
    pot_bare(p, rr, ab, &f, &e);
    switch (p->trunc) {
    case TRUNC_SHARP:
    case TRUNC_NONE:
        break;
    case TRUNC_SHIFTED:
        e = e - p->encut[ab];
        break;
    case TRUNC_SMOOTH_R4: {
        e = e - p->encut[ab];
        double r = std::sqrt(rr);
        double dr = r - p->rcut[ab];
        double x2 = dr * dr * p->rri_smooth;
        double x4 = x2 * x2;
        double x4i = 1 / (1 + x4);
        double h0_r = x4 * x4i;
        double h1_r = 4 * dr * p->rri_smooth * x2 * x4i * x4i;
        f = h0_r * f - h1_r * (e / r);
        e = h0_r * e;
        break;
    }
    case TRUNC_FORCE_SHIFTED: {
        double r = std::sqrt(rr);
        f -= p->fcut[ab] / r;
        e = e - p->encut[ab] + (r - p->rcut[ab]) * p->fcut[ab];
        break;
    }
    }
    *fval = f;
    *en = e;
}

/* ------------------------------------------------------------------------ */
/* accumulator (numeric/accumulator.hpp:83-119)                              */
/* ------------------------------------------------------------------------ */

struct orc_acc { double n, m, v; };

static inline void acc_add(orc_acc& a, double x)
{
    double t = x - a.m;
    a.n += 1;
    a.m += t / a.n;
    a.v += t * (x - a.m);
}

static inline void acc_merge(orc_acc& a, orc_acc const& b)
{
    if (b.n > 0) {
        double count = a.n + b.n;
        a.v += b.v;
        double diff = a.m - b.m;
        a.v += diff * diff * a.n * b.n / count;
        a.m = (a.n * a.m + b.n * b.m) / count;
        a.n = count;
    }
}

/* numeric/accumulator.hpp:83-119 */
/* out[0..4] = count, mean, variance, sigma, error_of_mean, sum */
ORC_API void orc_accumulate(int n, const double* x, double* out)
{
    orc_acc a = {0, 0, 0};
    for (int i = 0; i < n; ++i) acc_add(a, x[i]);
    out[0] = a.n;
    out[1] = a.m;
    out[2] = a.v / a.n;
    out[3] = std::sqrt(a.v / a.n);
    out[4] = std::sqrt((a.v / a.n) / (a.n - 1));
    out[5] = a.m * a.n;
}

/* ------------------------------------------------------------------------ */
/* periodic box (mdsim/box.hpp:115-140): host convention                     */
/* ------------------------------------------------------------------------ */

static inline double reduce_periodic_d(double& r, double L)
{
    double half = 0.5 * L;
    if (r > half) { r -= L; return 1; }
    if (r < -half) { r += L; return -1; }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* FP32 conventions shared with the CUDA kernels (bit-exact)                  */
/* ------------------------------------------------------------------------ */

/* mdsim/gpu/box_kernel.cuh:37-59 */
/* minimum image in float: k = rint(dr * (1/L)); dr -= k * L */
static inline float min_image_f(float dr, float L, float Linv)
{
    float k = std::rint(dr * Linv);
    return dr - k * L;
}

/* the list criterion of from_binning_kernel.cu:144-163 */
/* squared distance in float, fixed evaluation order, no contraction */
static inline float rr_f(float dx, float dy, float dz)
{
    float xx = dx * dx;
    float yy = dy * dy;
    float zz = dz * dz;
    return (xx + yy) + zz;
}

/* species stored as the bits of position.w (mdsim/gpu/particle.hpp:56-88) */
static inline u32 species_of(const float* pos4, int i)
{
    u32 s;
    std::memcpy(&s, pos4 + 4 * i + 3, 4);
    return s;
}

/* ------------------------------------------------------------------------ */
/* cell binning — GPU convention (binning.cpp:47-116, binning_kernel.cu:60)  */
/* ------------------------------------------------------------------------ */

/* sizing, binning.cpp:81-101: returns cell_size; ncell[3] filled */
ORC_API int orc_binning_sizing(int n, const double* L, double r_cut_max, double skin,
                               double occupancy, int* ncell)
{
    const double warp = 32;
    double nwarps = n / (occupancy * warp);
    double volume = L[0] * L[1] * L[2];
    size_t ncells = 1;
    for (int d = 0; d < 3; ++d) {
        int nmax = (int)(L[d] / (r_cut_max + skin));
        int nc = (int)std::ceil(L[d] * std::pow(nwarps / volume, 1. / 3));
        ncell[d] = std::min(nc, nmax);
        if (ncell[d] < 1) return -1;
        ncells *= ncell[d];
    }
    return (int)(warp * std::ceil(nwarps / ncells));
}

/* mdsim/gpu/binning_kernel.cu:36-75 */
/* cell index of a float position: (uint)(r / cell_length + ncell) % ncell */
static inline u32 cell_index_f(const float* r, const float* cell_len, const int* ncell)
{
    u32 idx[3];
    for (int d = 0; d < 3; ++d) {
        float x = r[d] / cell_len[d] + (float)ncell[d];
        idx[d] = ((u32)x) % (u32)ncell[d];
    }
    return (idx[2] * ncell[1] + idx[1]) * ncell[0] + idx[0];
}

/* mdsim/gpu/binning_kernel.cu:60-139 (compute_cell, gen_index, find_cell_offset, assign_cells) */
/*
 * Fill `cells` [ncells * cell_size] with the particle indices of every cell
 * in ascending order, padded with 0xFFFFFFFF (same contents as the
 * reference's stable radix sort + assign_cells).  Ghosts (species -1U) are
 * skipped.  Returns the largest cell occupancy (overflow iff > cell_size).
 */
ORC_API int orc_binning_f32(int n, const float* pos4, const int* ncell, const float* cell_len,
                            int cell_size, u32* cells, u32* cell_of)
{
    size_t ncells = (size_t)ncell[0] * ncell[1] * ncell[2];
    std::vector<u32> count(ncells, 0);
    for (size_t k = 0; k < ncells * cell_size; ++k) cells[k] = PLACEHOLDER;
    int maxocc = 0;
    for (int i = 0; i < n; ++i) {
        if (species_of(pos4, i) == PLACEHOLDER) { if (cell_of) cell_of[i] = PLACEHOLDER; continue; }
        u32 c = cell_index_f(pos4 + 4 * i, cell_len, ncell);
        if (cell_of) cell_of[i] = c;
        u32 k = count[c]++;
        if ((int)k < cell_size) cells[(size_t)c * cell_size + k] = (u32)i;
        maxocc = std::max(maxocc, (int)count[c]);
    }
    return maxocc;
}

/* ------------------------------------------------------------------------ */
/* full neighbour list with the GPU's float criterion                        */
/* (from_binning_kernel.cu:144-163: rr <= rr_cut_skin(type1, type2))         */
/* ------------------------------------------------------------------------ */

/*
 * counts[i] = number of j != i with float rr(i,j) <= rr_cut_skin[a*ns+b];
 * lists[i*maxn + k] = those j in ascending order (PLACEHOLDER padded).
 * Candidate pairs are enumerated with a cell grid whose cells are at least
 * (1 + 1e-4) * sqrt(max rr_cut_skin) wide, so no pair is missed.
 * Returns the largest count (lists truncated beyond maxn).
 */
ORC_API int orc_neighbour_full_f32(int n, const float* pos4, const float* Lf, int ns,
                                   const float* rr_cut_skin, int maxn, u32* counts, u32* lists)
{
    float Linv[3];
    for (int d = 0; d < 3; ++d) Linv[d] = (float)(1.0 / (double)Lf[d]);
    float rrmax = 0;
    for (int ab = 0; ab < ns * ns; ++ab) rrmax = std::max(rrmax, rr_cut_skin[ab]);
    double rmax = std::sqrt((double)rrmax) * (1 + 1e-4);
    int nc[3];
    for (int d = 0; d < 3; ++d) nc[d] = std::max(1, (int)((double)Lf[d] / rmax));
    size_t ncells = (size_t)nc[0] * nc[1] * nc[2];
    std::vector<std::vector<int>> cell(ncells);
    auto cidx = [&](int i, int* c) {
        for (int d = 0; d < 3; ++d) {
            double s = (double)pos4[4 * i + d] / (double)Lf[d] + 0.5;
            s -= std::floor(s);
            int k = (int)(s * nc[d]);
            c[d] = std::min(std::max(k, 0), nc[d] - 1);
        }
    };
    for (int i = 0; i < n; ++i) {
        if (species_of(pos4, i) == PLACEHOLDER) continue;
        int c[3];
        cidx(i, c);
        cell[((size_t)c[2] * nc[1] + c[1]) * nc[0] + c[0]].push_back(i);
    }
    int maxcount = 0;
    std::vector<u32> tmp;
    for (int i = 0; i < n; ++i) {
        counts[i] = 0;
        for (int k = 0; k < maxn; ++k) lists[(size_t)i * maxn + k] = PLACEHOLDER;
        u32 a = species_of(pos4, i);
        if (a == PLACEHOLDER) continue;
        int c[3];
        cidx(i, c);
        tmp.clear();
        /* distinct neighbour-cell offsets per dimension */
        int off[3][3], noff[3];
        for (int d = 0; d < 3; ++d) {
            if (nc[d] >= 3) { off[d][0] = -1; off[d][1] = 0; off[d][2] = 1; noff[d] = 3; }
            else if (nc[d] == 2) { off[d][0] = 0; off[d][1] = 1; noff[d] = 2; }
            else { off[d][0] = 0; noff[d] = 1; }
        }
        for (int oz = 0; oz < noff[2]; ++oz)
        for (int oy = 0; oy < noff[1]; ++oy)
        for (int ox = 0; ox < noff[0]; ++ox) {
            int cx = (c[0] + off[0][ox] + nc[0]) % nc[0];
            int cy = (c[1] + off[1][oy] + nc[1]) % nc[1];
            int cz = (c[2] + off[2][oz] + nc[2]) % nc[2];
            for (int j : cell[((size_t)cz * nc[1] + cy) * nc[0] + cx]) {
                if (j == i) continue;
                u32 b = species_of(pos4, j);
                float dx = min_image_f(pos4[4 * i + 0] - pos4[4 * j + 0], Lf[0], Linv[0]);
                float dy = min_image_f(pos4[4 * i + 1] - pos4[4 * j + 1], Lf[1], Linv[1]);
                float dz = min_image_f(pos4[4 * i + 2] - pos4[4 * j + 2], Lf[2], Linv[2]);
                float rr = rr_f(dx, dy, dz);
                if (rr <= rr_cut_skin[a * ns + b]) tmp.push_back((u32)j);
            }
        }
        std::sort(tmp.begin(), tmp.end());
        counts[i] = (u32)tmp.size();
        maxcount = std::max(maxcount, (int)tmp.size());
        for (size_t k = 0; k < tmp.size() && (int)k < maxn; ++k) lists[(size_t)i * maxn + k] = tmp[k];
    }
    return maxcount;
}

/* ------------------------------------------------------------------------ */
/* FP64 host backend: binning + half list + pair force                        */
/* ------------------------------------------------------------------------ */

struct half_list {
    std::vector<std::vector<int>> nb;
};

/* host/binning.cpp:91-116 and host/neighbours/from_binning.cpp:118-229 */
static void build_half_list(int n, const double* r, const u32* sp, const double* L,
                            const orc_pot* p, double skin, half_list& hl)
{
    int ns = p->ns;
    double rcs_max = 0;
    std::vector<double> rr_cut_skin(ns * ns);
    for (int ab = 0; ab < ns * ns; ++ab) {
        double rcs = p->rcut[ab] + skin;
        rr_cut_skin[ab] = rcs * rcs;
        rcs_max = std::max(rcs_max, rcs);
    }
    int nc[3];
    double cl[3];
    for (int d = 0; d < 3; ++d) {
        nc[d] = std::max((int)(L[d] / rcs_max), 1);
        cl[d] = L[d] / nc[d];
    }
    size_t ncells = (size_t)nc[0] * nc[1] * nc[2];
    std::vector<std::vector<int>> cell(ncells);
    auto cid = [&](int i, int* c) {
        for (int d = 0; d < 3; ++d) {
            long k = (long)(r[3 * i + d] / cl[d] + nc[d]);
            c[d] = (int)(k % nc[d]);
        }
    };
    for (int i = 0; i < n; ++i) {
        int c[3];
        cid(i, c);
        cell[((size_t)c[2] * nc[1] + c[1]) * nc[0] + c[0]].push_back(i);
    }
    hl.nb.assign(n, std::vector<int>());
    /* visit 13 of the 26 neighbour cells (lexicographically before the
     * centre) and the own cell with j > i; when a dimension has fewer than 3
     * cells the offsets alias, so distinct cells are visited once each and
     * pairs are deduplicated by index order instead */
    bool small = nc[0] < 3 || nc[1] < 3 || nc[2] < 3;
    for (int cz = 0; cz < nc[2]; ++cz)
    for (int cy = 0; cy < nc[1]; ++cy)
    for (int cx = 0; cx < nc[0]; ++cx) {
        const std::vector<int>& c1 = cell[((size_t)cz * nc[1] + cy) * nc[0] + cx];
        for (int i : c1) {
            auto visit = [&](const std::vector<int>& c2, bool same_or_small) {
                for (int j : c2) {
                    if (same_or_small && j <= i) continue;
                    double dr[3];
                    for (int d = 0; d < 3; ++d) {
                        dr[d] = r[3 * i + d] - r[3 * j + d];
                        reduce_periodic_d(dr[d], L[d]);
                    }
                    double rr = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
                    if (rr >= rr_cut_skin[sp[i] * ns + sp[j]]) continue;
                    hl.nb[i].push_back(j);
                }
            };
            if (!small) {
                /* the reference loops j[0] (x offset) outermost; reaching
                 * (0,0,0) ends the half shell */
                int done = 0;
                for (int j0 = -1; j0 <= 1 && !done; ++j0)
                for (int j1 = -1; j1 <= 1 && !done; ++j1)
                for (int j2 = -1; j2 <= 1 && !done; ++j2) {
                    if (j0 == 0 && j1 == 0 && j2 == 0) { done = 1; break; }
                    int kx = (cx + j0 + nc[0]) % nc[0];
                    int ky = (cy + j1 + nc[1]) % nc[1];
                    int kz = (cz + j2 + nc[2]) % nc[2];
                    visit(cell[((size_t)kz * nc[1] + ky) * nc[0] + kx], false);
                }
                visit(c1, true);
            } else {
                /* all distinct cells, each pair once by index order */
                std::vector<size_t> seen;
                for (int j0 = -1; j0 <= 1; ++j0)
                for (int j1 = -1; j1 <= 1; ++j1)
                for (int j2 = -1; j2 <= 1; ++j2) {
                    int kx = (cx + j0 + nc[0]) % nc[0];
                    int ky = (cy + j1 + nc[1]) % nc[1];
                    int kz = (cz + j2 + nc[2]) % nc[2];
                    size_t k = ((size_t)kz * nc[1] + ky) * nc[0] + kx;
                    if (std::find(seen.begin(), seen.end(), k) != seen.end()) continue;
                    seen.push_back(k);
                    visit(cell[k], true);
                }
            }
        }
    }
}

/*
 * Force evaluation over a half list with Newton's third law
 * (host/forces/pair_trunc.hpp:219-344).  en_pot/stress receive half of each
 * pair's contribution per particle (weight 1/2, pair_trunc.hpp:302-305).
 *
 * decide_f32 != 0: the within_range decision is taken on the float squared
 * distance computed from pos4 exactly as the CUDA force kernel does, so the
 * pair set matches the GPU and the comparison isolates arithmetic error.
 * The force value itself is always evaluated in double.
 */
static void force_half(int n, const double* r, const u32* sp, const double* L, const orc_pot* p,
                       const half_list& hl, int decide_f32, const float* pos4, const float* Lf,
                       double* f, double* en, double* stress, double* totals)
{
    int ns = p->ns;
    float Linv[3] = {0, 0, 0};
    float rrcut_f[ORC_MAX_SPECIES * ORC_MAX_SPECIES];
    if (decide_f32) {
        for (int d = 0; d < 3; ++d) Linv[d] = (float)(1.0 / (double)Lf[d]);
        for (int ab = 0; ab < ns * ns; ++ab) rrcut_f[ab] = (float)p->rrcut[ab];
    }
    std::fill(f, f + 3 * n, 0.0);
    if (en) std::fill(en, en + n, 0.0);
    if (stress) std::fill(stress, stress + 6 * n, 0.0);
    double epot = 0, vir = 0;
    for (int i = 0; i < n; ++i) {
        for (int j : hl.nb[i]) {
            double dr[3];
            for (int d = 0; d < 3; ++d) {
                dr[d] = r[3 * i + d] - r[3 * j + d];
                reduce_periodic_d(dr[d], L[d]);
            }
            int ab = sp[i] * ns + sp[j];
            double rr = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
            bool in;
            if (decide_f32) {
                float dx = min_image_f(pos4[4 * i + 0] - pos4[4 * j + 0], Lf[0], Linv[0]);
                float dy = min_image_f(pos4[4 * i + 1] - pos4[4 * j + 1], Lf[1], Linv[1]);
                float dz = min_image_f(pos4[4 * i + 2] - pos4[4 * j + 2], Lf[2], Linv[2]);
                in = rr_f(dx, dy, dz) < rrcut_f[ab];
            } else {
                in = rr < p->rrcut[ab];
            }
            if (!in) continue;
            double fval, e;
            orc_pot_eval(p, rr, sp[i], sp[j], &fval, &e);
            for (int d = 0; d < 3; ++d) {
                f[3 * i + d] += dr[d] * fval;
                f[3 * j + d] -= dr[d] * fval;
            }
            double w = 0.5;
            if (en) { en[i] += w * e; en[j] += w * e; }
            double s[6] = {dr[0] * dr[0], dr[1] * dr[1], dr[2] * dr[2],
                           dr[0] * dr[1], dr[0] * dr[2], dr[1] * dr[2]};
            if (stress) {
                for (int k = 0; k < 6; ++k) {
                    stress[6 * i + k] += w * fval * s[k];
                    stress[6 * j + k] += w * fval * s[k];
                }
            }
            epot += e;
            vir += fval * rr;
        }
    }
    if (totals) { totals[0] = epot; totals[1] = vir; }
}

/* host/forces/pair_trunc.hpp:219-344 over host/neighbours/from_binning.cpp:118-229 */
/*
 * Pair forces of a snapshot in FP64 (cell list + half list, complete for
 * pairs inside r_cut).  totals[0] = total potential energy, totals[1] =
 * Σ_pairs r·F (pair virial).  Returns the number of interacting pairs.
 */
ORC_API long orc_forces(int n, const double* r, const u32* sp, const double* L, const orc_pot* p,
                        int decide_f32, const float* pos4, const float* Lf,
                        double* f, double* en, double* stress, double* totals)
{
    half_list hl;
    /* with the float decision, candidates slightly beyond r_c in FP64 can be
     * inside it in float: the candidate list reaches 1e-3 r_c further */
    double reach = 0.0;
    if (decide_f32)
        for (int ab = 0; ab < p->ns * p->ns; ++ab)
            if (std::isfinite(p->rcut[ab])) reach = std::max(reach, 1e-3 * p->rcut[ab]);
    build_half_list(n, r, sp, L, p, reach, hl);
    force_half(n, r, sp, L, p, hl, decide_f32, pos4, Lf, f, en, stress, totals);
    long np = 0;
    for (auto& v : hl.nb) np += (long)v.size();
    return np;
}

/* ------------------------------------------------------------------------ */
/* DSFUN arithmetic (numeric/mp/dsfun.hpp:124-210): Knuth TwoSum, Dekker     */
/* ------------------------------------------------------------------------ */

static inline void dsadd(float& c0, float& c1, float a0, float a1, float b0, float b1)
{
    float t1 = a0 + b0;
    float e = t1 - a0;
    float t2 = ((b0 - e) + (a0 - (t1 - e))) + a1 + b1;
    c0 = e = t1 + t2;
    c1 = t2 - (e - t1);
}

static inline void dssub(float& c0, float& c1, float a0, float a1, float b0, float b1)
{
    float t1 = a0 - b0;
    float e = t1 - a0;
    float t2 = ((-b0 - e) + (a0 - (t1 - e))) + a1 - b1;
    c0 = e = t1 + t2;
    c1 = t2 - (e - t1);
}

static inline void dsmul(float& c0, float& c1, float a0, float a1, float b0, float b1)
{
    float cona = a0 * 8193.0f;
    float conb = b0 * 8193.0f;
    float sa1 = cona - (cona - a0);
    float sb1 = conb - (conb - b0);
    float sa2 = a0 - sa1;
    float sb2 = b0 - sb1;
    float c11 = a0 * b0;
    float c21 = (((sa1 * sb1 - c11) + sa1 * sb2) + sa2 * sb1) + sa2 * sb2;
    float c2 = a0 * b1 + a1 * b0;
    float t1 = c11 + c2;
    float e = t1 - c11;
    float t2 = ((c2 - e) + (c11 - (t1 - e))) + c21 + a1 * b1;
    c0 = e = t1 + t2;
    c1 = t2 - (e - t1);
}

/* op: 0 add, 1 sub, 2 mul; a, b, c are (hi, lo) pairs */
ORC_API void orc_dsfun(int op, int n, const float* a, const float* b, float* c)
{
    for (int i = 0; i < n; ++i) {
        float c0, c1;
        if (op == 0) dsadd(c0, c1, a[2 * i], a[2 * i + 1], b[2 * i], b[2 * i + 1]);
        else if (op == 1) dssub(c0, c1, a[2 * i], a[2 * i + 1], b[2 * i], b[2 * i + 1]);
        else dsmul(c0, c1, a[2 * i], a[2 * i + 1], b[2 * i], b[2 * i + 1]);
        c[2 * i] = c0;
        c[2 * i + 1] = c1;
    }
}

/* ------------------------------------------------------------------------ */
/* dsfloat velocity Verlet, GPU convention (verlet_kernel.cu:38-98)          */
/* ------------------------------------------------------------------------ */

/*
 * r4 = [hi float4 x n | lo float4 x n], same for v4 (w of v hi = mass);
 * img4 float4 image counters; f4 float4 forces.  dt_half = (float)(dt/2).
 * Ghosts (species -1U) are skipped.  For precision == 0 (float) the lo
 * words are ignored and plain float arithmetic is used.
 */
ORC_API void orc_integrate_f32(int n, int ds, float* r4, float* v4, float* img4, const float* f4,
                               float dt, float dt_half, const float* Lf)
{
    float Linv[3];
    for (int d = 0; d < 3; ++d) Linv[d] = (float)(1.0 / (double)Lf[d]);
    float* rlo = r4 + 4 * (size_t)n;
    float* vlo = v4 + 4 * (size_t)n;
    for (int i = 0; i < n; ++i) {
        if (species_of(r4, i) == PLACEHOLDER) continue;
        float m = v4[4 * i + 3];
        for (int d = 0; d < 3; ++d) {
            float a = (f4[4 * i + d] * dt_half) / m;
            float k;
            if (ds) {
                float v0, v1, d0, d1, r0, r1;
                dsadd(v0, v1, v4[4 * i + d], vlo[4 * i + d], a, 0.0f);
                dsmul(d0, d1, v0, v1, dt, 0.0f);
                dsadd(r0, r1, r4[4 * i + d], rlo[4 * i + d], d0, d1);
                k = std::rint(r0 * Linv[d]);
                dssub(r0, r1, r0, r1, k * Lf[d], 0.0f);
                v4[4 * i + d] = v0; vlo[4 * i + d] = v1;
                r4[4 * i + d] = r0; rlo[4 * i + d] = r1;
            } else {
                float v = v4[4 * i + d] + a;
                float r = r4[4 * i + d] + v * dt;
                k = std::rint(r * Linv[d]);
                r = r - k * Lf[d];
                v4[4 * i + d] = v;
                r4[4 * i + d] = r;
            }
            img4[4 * i + d] = img4[4 * i + d] + k;
        }
    }
}

/* second half-kick in float / dsfloat (gpu/integrators/verlet_kernel.cu:78-98) */
ORC_API void orc_finalize_f32(int n, int ds, const float* r4, float* v4, const float* f4, float dt_half)
{
    float* vlo = v4 + 4 * (size_t)n;
    for (int i = 0; i < n; ++i) {
        if (species_of(r4, i) == PLACEHOLDER) continue;
        float m = v4[4 * i + 3];
        for (int d = 0; d < 3; ++d) {
            float a = (f4[4 * i + d] * dt_half) / m;
            if (ds) {
                float v0, v1;
                dsadd(v0, v1, v4[4 * i + d], vlo[4 * i + d], a, 0.0f);
                v4[4 * i + d] = v0; vlo[4 * i + d] = v1;
            } else {
                v4[4 * i + d] = v4[4 * i + d] + a;
            }
        }
    }
}

/* float max displacement (max_displacement_kernel.cu:37-68): max |Δr|² */
ORC_API float orc_max_displacement2_f32(int n, const float* r4, const float* r04, const float* Lf)
{
    float Linv[3];
    for (int d = 0; d < 3; ++d) Linv[d] = (float)(1.0 / (double)Lf[d]);
    float m = 0;
    for (int i = 0; i < n; ++i) {
        if (species_of(r4, i) == PLACEHOLDER) continue;
        float dx = min_image_f(r4[4 * i + 0] - r04[4 * i + 0], Lf[0], Linv[0]);
        float dy = min_image_f(r4[4 * i + 1] - r04[4 * i + 1], Lf[1], Linv[1]);
        float dz = min_image_f(r4[4 * i + 2] - r04[4 * i + 2], Lf[2], Linv[2]);
        m = std::max(m, rr_f(dx, dy, dz));
    }
    return m;
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al., SC'11)                                      */
/* ------------------------------------------------------------------------ */

static inline void mulhilo(u32 a, u32 b, u32& hi, u32& lo)
{
    uint64_t p = (uint64_t)a * b;
    hi = (u32)(p >> 32);
    lo = (u32)p;
}

/* the engine's keyed stream; it replaces the reference's rand48
 * (random/gpu/rand48_kernel.cuh:61-78), whose state is per thread */
ORC_API void orc_philox4x32_10(const u32* ctr_in, const u32* key_in, u32* out)
{
    u32 c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    u32 k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        u32 hi0, lo0, hi1, lo1;
        mulhilo(0xD2511F53u, c0, hi0, lo0);
        mulhilo(0xCD9E8D57u, c2, hi1, lo1);
        u32 n0 = hi1 ^ c1 ^ k0;
        u32 n1 = lo1;
        u32 n2 = hi0 ^ c3 ^ k1;
        u32 n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* uniform float in (0, 1) from the top 24 bits */
static inline double u01(u32 x) { return ((double)(x >> 8) + 0.5) * (1.0 / 16777216.0); }

/*
 * Andersen finalize (per-particle collisions, host convention
 * verlet_nvt_andersen.cpp:111-137).  The collision of particle i at step
 * `step` happens iff philox(id, step, 'ANDR')[0] < threshold; resampled
 * velocity components are sigma * N(0,1) from Box–Muller of the second
 * Philox block (id, step, 'ANDS').  Velocity hi/lo layout as above.
 * collided[i] is set to 1 for particles that collided.
 */
ORC_API void orc_andersen_finalize_f32(int n, int ds, const float* r4, float* v4, const float* f4,
                                       const u32* id, float dt_half, float sqrt_temperature,
                                       u32 threshold, uint64_t seed, uint64_t step,
                                       unsigned char* collided)
{
    float* vlo = v4 + 4 * (size_t)n;
    u32 key[2] = {(u32)seed, (u32)(seed >> 32)};
    for (int i = 0; i < n; ++i) {
        collided[i] = 0;
        if (species_of(r4, i) == PLACEHOLDER) continue;
        u32 ctr[4] = {id[i], (u32)step, (u32)(step >> 32), 0x414E4452u};
        u32 u[4];
        orc_philox4x32_10(ctr, key, u);
        if (u[0] >= threshold) {
            float m = v4[4 * i + 3];
            for (int d = 0; d < 3; ++d) {
                float a = (f4[4 * i + d] * dt_half) / m;
                if (ds) {
                    float v0, v1;
                    dsadd(v0, v1, v4[4 * i + d], vlo[4 * i + d], a, 0.0f);
                    v4[4 * i + d] = v0; vlo[4 * i + d] = v1;
                } else {
                    v4[4 * i + d] = v4[4 * i + d] + a;
                }
            }
        } else {
            collided[i] = 1;
            ctr[3] = 0x414E4453u;
            u32 w[4];
            orc_philox4x32_10(ctr, key, w);
            double rad0 = std::sqrt(-2 * std::log(u01(w[0])));
            double rad1 = std::sqrt(-2 * std::log(u01(w[2])));
            double g[3] = {rad0 * std::cos(2 * M_PI * u01(w[1])), rad0 * std::sin(2 * M_PI * u01(w[1])),
                           rad1 * std::cos(2 * M_PI * u01(w[3]))};
            for (int d = 0; d < 3; ++d) {
                v4[4 * i + d] = (float)(sqrt_temperature * g[d]);
                if (ds) vlo[4 * i + d] = 0.0f;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Hilbert curve keys (mdsim/sorts/hilbert_kernel.hpp:70-230)                */
/* ------------------------------------------------------------------------ */

/* gpu/sorts/hilbert.cpp:51-54 */
ORC_API unsigned orc_hilbert_depth(double max_length)
{
    unsigned depth = (unsigned)std::ceil(std::log(max_length) / M_LN2);
    return std::min(10u, depth);
}

static inline void hswap(u32& v, u32& a, u32& b, u32 mask)
{
    u32 va = (v >> a) & mask;
    u32 vb = (v >> b) & mask;
    v = v ^ (va << a) ^ (vb << b) ^ (va << b) ^ (vb << a);
    std::swap(a, b);
}

/* mdsim/sorts/hilbert_kernel.hpp:70-230 */
/* r: coordinates already divided by the box length */
static u32 hilbert_map3(float x0, float x1, float x2, unsigned depth)
{
    float n = (float)(1UL << depth);
    float r[3] = {x0, x1, x2};
    for (int d = 0; d < 3; ++d) {
        r[d] = (r[d] - std::floor(r[d])) * n;
        r[d] = (std::floor(r[d]) + 0.5f) / n;
        r[d] -= 0.5f;
    }
    u32 hcode = 0;
    u32 a = 21, b = 18, c = 12, d = 15, e = 3, f = 0, g = 6, h = 9;
    u32 vc = 1U << b ^ 2U << c ^ 3U << d ^ 4U << e ^ 5U << f ^ 6U << g ^ 7U << h;
    const u32 mask = 7;
    for (unsigned i = 0; i < depth; ++i) {
        u32 x = std::signbit(r[0]) & 1;
        u32 y = std::signbit(r[1]) & 1;
        u32 z = std::signbit(r[2]) & 1;
        u32 v = (vc >> (3 * (x + (y << 1) + (z << 2))) & mask);
        r[0] *= 2; r[1] *= 2; r[2] *= 2;
        r[0] += x; r[0] -= 0.5f;
        r[1] += y; r[1] -= 0.5f;
        r[2] += z; r[2] -= 0.5f;
        if (v == 0) { hswap(vc, b, h, mask); hswap(vc, c, e, mask); }
        else if (v == 1 || v == 2) { hswap(vc, c, g, mask); hswap(vc, d, h, mask); }
        else if (v == 3 || v == 4) { hswap(vc, a, c, mask); hswap(vc, f, h, mask); }
        else if (v == 5 || v == 6) { hswap(vc, a, e, mask); hswap(vc, b, f, mask); }
        else if (v == 7) { hswap(vc, a, g, mask); hswap(vc, d, f, mask); }
        hcode = (hcode << 3) + v;
    }
    return hcode;
}

/* unit-cube coordinates in, keys out (used to pin against the reference's own map) */
ORC_API void orc_hilbert_map_unit(int n, const float* s3, unsigned depth, u32* keys)
{
    for (int i = 0; i < n; ++i) keys[i] = hilbert_map3(s3[3 * i], s3[3 * i + 1], s3[3 * i + 2], depth);
}

/* hilbert_kernel.cu:39-66 with IEEE division r / L; ghosts → 0xFFFFFFFF */
ORC_API void orc_hilbert_keys_f32(int n, const float* pos4, const float* Lf, unsigned depth, u32* keys)
{
    for (int i = 0; i < n; ++i) {
        if (species_of(pos4, i) == PLACEHOLDER) { keys[i] = PLACEHOLDER; continue; }
        keys[i] = hilbert_map3(pos4[4 * i] / Lf[0], pos4[4 * i + 1] / Lf[1], pos4[4 * i + 2] / Lf[2], depth);
    }
}

/* permutation of a stable ascending sort (radix_sort key/value semantics) */
ORC_API void orc_stable_argsort_u32(int n, const u32* keys, u32* perm)
{
    std::vector<u32> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](u32 a, u32 b) { return keys[a] < keys[b]; });
    std::copy(idx.begin(), idx.end(), perm);
}

/* ------------------------------------------------------------------------ */
/* observables                                                               */
/* ------------------------------------------------------------------------ */

/* observables/gpu/thermodynamics.cpp:68-190, thermodynamics_kernel.cu:35-106 */
/*
 * Σ m v², Σ m v (3), Σ e_pot, Σ virial trace in double; out[0] = 0.5 Σ m v²,
 * out[1..3] = Σ m v, out[4] = Σ m.
 */
ORC_API void orc_kinetic(int n, const double* v, const double* m, double* out)
{
    double ek = 0, p[3] = {0, 0, 0}, mt = 0;
    for (int i = 0; i < n; ++i) {
        double vv = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
        ek += m[i] * vv;
        for (int d = 0; d < 3; ++d) p[d] += m[i] * v[3 * i + d];
        mt += m[i];
    }
    out[0] = 0.5 * ek;
    out[1] = p[0]; out[2] = p[1]; out[3] = p[2];
    out[4] = mt;
}

/*
 * MSD of two unwrapped samples (mean_square_displacement.hpp:36-42) over the
 * index range [first, last): out = count, mean, variance (accumulator).
 */
ORC_API void orc_msd(int first, int last, const double* r1, const double* r2, double* out)
{
    orc_acc a = {0, 0, 0};
    for (int i = first; i < last; ++i) {
        double dd = 0;
        for (int d = 0; d < 3; ++d) {
            double x = r2[3 * i + d] - r1[3 * i + d];
            dd += x * x;
        }
        acc_add(a, dd);
    }
    out[0] = a.n; out[1] = a.m; out[2] = a.n > 0 ? a.v / a.n : 0;
}

/*
 * mean quartic displacement (observables/dynamics/mean_quartic_displacement.hpp:34-41):
 * |r2 - r1|^4, and velocity autocorrelation
 * (observables/dynamics/velocity_autocorrelation.hpp:34-38): v1 . v2, both
 * accumulated like the MSD.  kind 0: MSD, 2: MQD, 3: VACF.
 */
ORC_API void orc_tcf(int kind, int first, int last, const double* a, const double* b, double* out)
{
    orc_acc acc = {0, 0, 0};
    for (int i = first; i < last; ++i) {
        double x = 0;
        if (kind == 3) {
            for (int d = 0; d < 3; ++d) x += a[3 * i + d] * b[3 * i + d];
        } else {
            for (int d = 0; d < 3; ++d) {
                const double dx = b[3 * i + d] - a[3 * i + d];
                x += dx * dx;
            }
            if (kind == 2) x = x * x;
        }
        acc_add(acc, x);
    }
    out[0] = acc.n; out[1] = acc.m; out[2] = acc.n > 0 ? acc.v / acc.n : 0;
}

/*
 * density modes ρ(q) = Σ_j exp(i q·r_j) over particles [first,last) with the
 * reference's sign convention (imaginary part negated, density_mode.cpp:128).
 * q·r is evaluated in float as (qx*x + qy*y) + qz*z (the GPU's rounding); the
 * trigonometric functions and the sum are FP64.  out: nq x (re, im).
 */
ORC_API void orc_density_modes(int first, int last, const float* pos4, int nq, const float* q3, double* out)
{
    for (int k = 0; k < nq; ++k) {
        double re = 0, im = 0;
        for (int j = first; j < last; ++j) {
            float qr = (q3[3 * k] * pos4[4 * j] + q3[3 * k + 1] * pos4[4 * j + 1]) + q3[3 * k + 2] * pos4[4 * j + 2];
            re += std::cos((double)qr);
            im += std::sin((double)qr);
        }
        out[2 * k] = re;
        out[2 * k + 1] = -im;
    }
}

/*
 * ISF of two density-mode samples (intermediate_scattering_function.hpp:89-113):
 * per shell [shell[2s], shell[2s+1]) the accumulator of Re[ρ1 ρ2*]/norm.
 * out: nshell x (count, mean, variance).
 */
ORC_API void orc_isf(int nshell, const int* shell, const double* rho1, const double* rho2, double norm, double* out)
{
    for (int s = 0; s < nshell; ++s) {
        orc_acc a = {0, 0, 0};
        for (int i = shell[2 * s]; i < shell[2 * s + 1]; ++i) {
            double re = rho1[2 * i] * rho2[2 * i] + rho1[2 * i + 1] * rho2[2 * i + 1];
            acc_add(a, re / norm);
        }
        out[3 * s] = a.n; out[3 * s + 1] = a.m; out[3 * s + 2] = a.n > 0 ? a.v / a.n : 0;
    }
}

/* part of pick_lattice_points_from_shell (algorithm/host/pick_lattice_points.hpp:74-160) */
static bool is_coprime3(const unsigned* h)
{
    auto gcd = [](unsigned a, unsigned b) { while (b) { unsigned t = a % b; a = b; b = t; } return a; };
    unsigned g = gcd(gcd(h[0], h[1]), h[2]);
    return g == 1;
}

/*
 * pick_lattice_points_from_shell (algorithm/host/pick_lattice_points.hpp:74-160)
 * for 3D; the output is grouped per radius in input order (as the
 * multimap iteration of wavevector.cpp:98-120).  out_q holds up to
 * max_out vectors; shell[2*i], shell[2*i+1] index ranges per radius (empty
 * shells give equal bounds).  Returns the number of vectors.
 */
ORC_API int orc_wavevectors(int nr, const double* radius, const double* unit_cell, double tolerance,
                            int max_count, const int* filter, int max_out, double* out_q, int* shell)
{
    std::vector<std::vector<double>> per(nr);
    double rmax = *std::max_element(radius, radius + nr) * (1 + tolerance);
    unsigned msum[3];
    for (int j = 0; j < 3; ++j) msum[j] = unit_cell[j] == 0 ? 0 : (unsigned)(rmax / unit_cell[j]);
    msum[1] += msum[0];
    msum[2] += msum[1];
    std::vector<unsigned> count(nr, 0);
    unsigned idx[3] = {0, 0, 0};
    while (idx[2] <= msum[2]) {
        unsigned hkl[3] = {idx[0], idx[1] - idx[0], idx[2] - idx[1]};
        bool pass = true;
        for (int j = 0; j < 3; ++j) if (hkl[j] * filter[j] != hkl[j]) pass = false;
        if (pass && is_coprime3(hkl)) {
            double r0[3] = {unit_cell[0] * hkl[0], unit_cell[1] * hkl[1], unit_cell[2] * hkl[2]};
            double r0n = std::sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
            for (int i = 0; i < nr; ++i) {
                if ((int)count[i] < max_count) {
                    unsigned nn = (unsigned)std::floor(radius[i] / r0n + 0.5);
                    if (nn > 0 && std::fabs(nn * r0n - radius[i]) <= radius[i] * tolerance) {
                        per[i].push_back(nn * r0[0]);
                        per[i].push_back(nn * r0[1]);
                        per[i].push_back(nn * r0[2]);
                        ++count[i];
                    }
                }
            }
        }
        ++idx[0];
        for (int j = 0; j < 2; ++j) {
            if (idx[j] <= msum[j]) break;
            idx[j] = 0;
            ++idx[j + 1];
        }
    }
    int total = 0;
    for (int i = 0; i < nr; ++i) {
        shell[2 * i] = total;
        for (size_t k = 0; k < per[i].size(); k += 3) {
            if (total < max_out) {
                out_q[3 * total] = per[i][k];
                out_q[3 * total + 1] = per[i][k + 1];
                out_q[3 * total + 2] = per[i][k + 2];
            }
            ++total;
        }
        shell[2 * i + 1] = total;
    }
    return total;
}

/* ------------------------------------------------------------------------ */
/* fcc lattice (host/positions/lattice.cpp:64-120, lattice_primitive.hpp)    */
/* ------------------------------------------------------------------------ */

/*
 * n = 4 * ncell^3 points of an fcc lattice filling a cubic box of edge L
 * centred at the origin: cell (i,j,k) + basis {0, (½,½,0), (½,0,½), (0,½,½)},
 * shifted by a quarter cell so no point lies on a box face.
 */
ORC_API void orc_fcc_lattice(int ncell, double L, double* r)
{
    double a = L / ncell;
    const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    size_t p = 0;
    for (int k = 0; k < ncell; ++k)
    for (int j = 0; j < ncell; ++j)
    for (int i = 0; i < ncell; ++i)
    for (int b = 0; b < 4; ++b) {
        r[3 * p + 0] = (i + basis[b][0] + 0.25) * a - 0.5 * L;
        r[3 * p + 1] = (j + basis[b][1] + 0.25) * a - 0.5 * L;
        r[3 * p + 2] = (k + basis[b][2] + 0.25) * a - 0.5 * L;
        ++p;
    }
}

/*
 * positions.lattice set() (mdsim/host/positions/lattice.cpp:63-175 with
 * mdsim/positions/lattice_primitive.hpp close_packed_lattice): fcc sites in
 * the slab (fractions of the box edges) at the centre of the box, the smallest
 * lattice distance with enough sites, a vacancy every `skip` sites.
 * out[3 n]; returns the number of sites.
 */
ORC_API long orc_lattice(int n, const double* box, const double* slab, double* out)
{
    double length[3], offset[3];
    for (int q = 0; q < 3; ++q) {
        length[q] = box[q] * slab[q];
        offset[q] = -length[q] / 2;
    }
    const double u = 4;
    double V = length[0] * length[1] * length[2] / std::ceil(n / u);
    double a = std::pow(V, 1.0 / 3);
    unsigned c[3];
    for (int q = 0; q < 3; ++q) c[q] = (unsigned)(length[q] / a);
    while (n > u * c[0] * c[1] * c[2]) {
        double t[3];
        for (int q = 0; q < 3; ++q) t[q] = length[q] / (c[q] + 1);
        a = *std::max_element(t, t + 3);
        unsigned m[3] = {c[0], c[1], c[2]};
        for (int q = 0; q < 3; ++q) c[q] = std::max(m[q], (unsigned)(length[q] / a));
        if (m[0] == c[0] && m[1] == c[1] && m[2] == c[2])
            for (int q = 0; q < 3; ++q) c[q] += 1;
    }
    const unsigned long N = 4ul * c[0] * c[1] * c[2];
    const unsigned long skip = (N > (unsigned long)n) ? (unsigned long)std::ceil((double)N / (N - n)) : 0;
    unsigned long i = 0;
    for (int t = 0; t < n; ++t, ++i) {
        if (skip && i % skip == skip - 1) ++i;
        const unsigned long cell = i >> 2, b = i & 3;
        const double r[3] = {(double)(cell % c[0]) + (double)((((b ^ (b >> 1)) & 1) * 2 + 1)) / 4,
                             (double)((cell / c[0]) % c[1]) + (double)(((b & 1) * 2 + 1)) / 4,
                             (double)(cell / ((unsigned long)c[0] * c[1])) + (double)(((b & 2) + 1)) / 4};
        for (int q = 0; q < 3; ++q) out[3 * t + q] = r[q] * a + offset[q];
    }
    return (long)N;
}

/*
 * velocities.boltzmann set() as the engine draws it: each component
 * N(0, sqrt(T)) / sqrt(m) by Box-Muller in FP64 on the Philox4x32-10 words of
 * (tag, 0, 0, 'BOLT') under the seed, then the centre-of-mass velocity
 * removed (gpu/velocities/boltzmann_kernel.cu:47-140 draws from rand48).
 */
ORC_API void orc_boltzmann(int n, const double* mass, double T, uint64_t seed, double* out)
{
    const u32 key[2] = {(u32)seed, (u32)(seed >> 32)};
    double mv[3] = {0, 0, 0}, msum = 0;
    for (int t = 0; t < n; ++t) {
        u32 ctr[4] = {(u32)t, 0u, 0u, 0x424F4C54u}, w[4];
        orc_philox4x32_10(ctr, key, w);
        const double inv = 1.0 / 4294967296.0;
        const double u0 = (w[0] + 0.5) * inv, u1 = (w[1] + 0.5) * inv, u2 = (w[2] + 0.5) * inv, u3 = (w[3] + 0.5) * inv;
        const double r0 = std::sqrt(-2.0 * std::log(u0)), r1 = std::sqrt(-2.0 * std::log(u2));
        const double f = std::sqrt(T / mass[t]);
        out[3 * t + 0] = f * r0 * std::cos(2 * M_PI * u1);
        out[3 * t + 1] = f * r0 * std::sin(2 * M_PI * u1);
        out[3 * t + 2] = f * r1 * std::cos(2 * M_PI * u3);
        for (int q = 0; q < 3; ++q) mv[q] += mass[t] * out[3 * t + q];
        msum += mass[t];
    }
    for (int t = 0; t < n; ++t)
        for (int q = 0; q < 3; ++q) out[3 * t + q] -= mv[q] / msum;
}

/* ------------------------------------------------------------------------ */
/* the host backend's MD loop in FP64 (the timed CPU baseline)                */
/* ------------------------------------------------------------------------ */

/*
 * velocity Verlet NVE (or Andersen NVT when coll_rate > 0) with a half
 * Verlet list rebuilt when the maximum displacement exceeds skin/2
 * (host/integrators/verlet.cpp:59-101, host/neighbours/from_binning.cpp,
 * host/max_displacement.cpp:67-87, host/forces/pair_trunc.hpp:219-260).
 * Particles are reordered by Hilbert key at every rebuild (the reference's
 * default sort).  Single thread, as the reference host backend.
 * r, v, image are updated in place; stats[0] = number of rebuilds,
 * stats[1] = final potential energy, stats[2] = final kinetic energy.
 */
/*
 * Nose-Hoover chain of two, one half step (host/integrators/verlet_nvt_hoover.cpp
 * propagate_chain, the same algorithm as the GPU module's
 * gpu/integrators/verlet_nvt_hoover.cpp:141-185); en_kin_2 = sum m v^2.
 * Returns the velocity scale.
 */
struct orc_chain {
    double xi[2], v_xi[2], mass[2], target2, T;
};

static double chain_half_step(orc_chain& c, double en_kin_2, double dt)
{
    c.v_xi[1] += (c.mass[0] * c.v_xi[0] * c.v_xi[0] - c.T) / c.mass[1] * (dt / 4);
    const double t = std::exp(-c.v_xi[1] * (dt / 8));
    c.v_xi[0] *= t;
    c.v_xi[0] += (en_kin_2 - c.target2) / c.mass[0] * (dt / 4);
    c.v_xi[0] *= t;
    for (int k = 0; k < 2; ++k) c.xi[k] += c.v_xi[k] * (dt / 2);
    const double s = std::exp(-c.v_xi[0] * (dt / 2));
    en_kin_2 *= s * s;
    c.v_xi[0] *= t;
    c.v_xi[0] += (en_kin_2 - c.target2) / c.mass[0] * (dt / 4);
    c.v_xi[0] *= t;
    c.v_xi[1] += (c.mass[0] * c.v_xi[0] * c.v_xi[0] - c.T) / c.mass[1] * (dt / 4);
    return s;
}

/* host/integrators/{verlet.cpp:59-101, verlet_nvt_andersen.cpp:96-137,
 * verlet_nvt_hoover.cpp, euler.cpp} with the skin/2 rule of from_binning.cpp:130 */
enum { ORC_VERLET = 0, ORC_ANDERSEN = 1, ORC_HOOVER = 2, ORC_BOLTZMANN = 3, ORC_EULER = 4 };

ORC_API int orc_md_run_any(int n, double* r, double* v, double* image, const u32* sp_in, const double* mass_in,
                           const double* L, const orc_pot* p, double skin, double dt, int nsteps, int integrator,
                           double temperature, double coll_rate, double resonance_frequency, uint64_t seed,
                           double* stats, double* chain_out);

ORC_API int orc_md_run(int n, double* r, double* v, double* image, const u32* sp_in, const double* mass_in,
                       const double* L, const orc_pot* p, double skin, double dt, int nsteps,
                       double temperature, double coll_rate, uint64_t seed, double* stats)
{
    return orc_md_run_any(n, r, v, image, sp_in, mass_in, L, p, skin, dt, nsteps,
                          coll_rate > 0 ? ORC_ANDERSEN : ORC_VERLET, temperature, coll_rate, 0, seed, stats, nullptr);
}

/*
 * FP64 MD run with the host integrators: velocity Verlet
 * (host/integrators/verlet.cpp:59-101), Andersen (verlet_nvt_andersen.cpp:96-137,
 * collisions from the engine's Philox stream), Nose-Hoover chain
 * (verlet_nvt_hoover.cpp), Maxwell-Boltzmann draws every
 * max(1, round(1 / (rate dt))) steps (verlet_nvt_boltzmann.lua.in with
 * velocities/boltzmann: N(0, sqrt T) / sqrt(m), centre-of-mass velocity
 * removed), Euler (host/integrators/euler.cpp: r += v dt).
 * chain_out (Nose-Hoover): xi[2], v_xi[2], energy per particle.
 */
ORC_API int orc_md_run_any(int n, double* r, double* v, double* image, const u32* sp_in, const double* mass_in,
                           const double* L, const orc_pot* p, double skin, double dt, int nsteps, int integrator,
                           double temperature, double coll_rate, double resonance_frequency, uint64_t seed,
                           double* stats, double* chain_out)
{
    std::vector<u32> sp(sp_in, sp_in + n);
    std::vector<double> m(mass_in, mass_in + n);
    std::vector<u32> id(n);
    std::iota(id.begin(), id.end(), 0u);
    std::vector<double> f(3 * (size_t)n), r0(3 * (size_t)n);
    half_list hl;
    double Lmax = std::max(L[0], std::max(L[1], L[2]));
    unsigned depth = orc_hilbert_depth(Lmax);
    int rebuilds = 0;
    double totals[2] = {0, 0};
    double sqrtT = std::sqrt(temperature);
    u32 thresh = (integrator == ORC_ANDERSEN)
                     ? (u32)std::min(4294967295.0, std::floor(coll_rate * dt * 4294967296.0)) : 0u;
    u32 key[2] = {(u32)seed, (u32)(seed >> 32)};
    const uint64_t interval = (integrator == ORC_BOLTZMANN)
                                  ? (uint64_t)std::max(1.0, std::floor(1.0 / (coll_rate * dt) + 0.5)) : 1u;
    orc_chain chain = {};
    if (integrator == ORC_HOOVER) {
        const double omega_sq = std::pow(2 * M_PI * resonance_frequency, 2);
        const double dof = 3.0 * n;
        chain.mass[0] = dof * temperature / omega_sq;
        chain.mass[1] = temperature / omega_sq;
        chain.target2 = dof * temperature;
        chain.T = temperature;
    }
    auto en_kin_2 = [&]() {
        double e = 0;
        for (int i = 0; i < n; ++i)
            e += m[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
        return e;
    };

    auto rebuild = [&]() {
        /* Hilbert reorder (host/sorts/hilbert.cpp:91-111 orders by cell; the
         * key here is the particle's own Hilbert code) */
        std::vector<u32> keys(n), perm(n);
        for (int i = 0; i < n; ++i)
            keys[i] = hilbert_map3((float)(r[3 * i] / L[0]), (float)(r[3 * i + 1] / L[1]),
                                   (float)(r[3 * i + 2] / L[2]), depth);
        orc_stable_argsort_u32(n, keys.data(), perm.data());
        std::vector<double> tr(r, r + 3 * (size_t)n), tv(v, v + 3 * (size_t)n), ti(image, image + 3 * (size_t)n);
        std::vector<u32> ts(sp), tid(id);
        std::vector<double> tm(m);
        for (int i = 0; i < n; ++i) {
            u32 q = perm[i];
            for (int d = 0; d < 3; ++d) {
                r[3 * i + d] = tr[3 * q + d];
                v[3 * i + d] = tv[3 * q + d];
                image[3 * i + d] = ti[3 * q + d];
            }
            sp[i] = ts[q]; id[i] = tid[q]; m[i] = tm[q];
        }
        build_half_list(n, r, sp.data(), L, p, skin, hl);
        std::copy(r, r + 3 * (size_t)n, r0.begin());
        ++rebuilds;
    };
    auto max_disp_exceeded = [&]() {
        double rr_max = 0;
        for (int i = 0; i < n; ++i) {
            double dr[3];
            for (int d = 0; d < 3; ++d) {
                dr[d] = r[3 * i + d] - r0[3 * i + d];
                reduce_periodic_d(dr[d], L[d]);
            }
            rr_max = std::max(rr_max, dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        }
        return std::sqrt(rr_max) > skin / 2;
    };

    rebuild();
    force_half(n, r, sp.data(), L, p, hl, 0, nullptr, nullptr, f.data(), nullptr, nullptr, totals);
    for (int s = 0; s < nsteps; ++s) {
        const uint64_t step = (uint64_t)s + 1;   /* 1-based step of this integration */
        if (integrator == ORC_HOOVER) {
            const double sc = chain_half_step(chain, en_kin_2(), dt);
            for (int k = 0; k < 3 * n; ++k) v[k] *= sc;
        }
        for (int i = 0; i < n; ++i) {
            for (int d = 0; d < 3; ++d) {
                if (integrator != ORC_EULER) v[3 * i + d] += f[3 * i + d] * (dt / 2) / m[i];
                r[3 * i + d] += v[3 * i + d] * dt;
                image[3 * i + d] += reduce_periodic_d(r[3 * i + d], L[d]);
            }
        }
        if (max_disp_exceeded()) rebuild();
        force_half(n, r, sp.data(), L, p, hl, 0, nullptr, nullptr, f.data(), nullptr, nullptr, totals);
        if (integrator == ORC_EULER) continue;
        if (integrator == ORC_BOLTZMANN && step % interval == 0) {
            double mv[3] = {0, 0, 0}, msum = 0;
            for (int i = 0; i < n; ++i) {
                u32 ctr[4] = {id[i], (u32)step, (u32)(step >> 32), 0x424F4C5Au}, w[4];
                orc_philox4x32_10(ctr, key, w);
                const double rad0 = std::sqrt(-2 * std::log(u01(w[0])));
                const double rad1 = std::sqrt(-2 * std::log(u01(w[2])));
                const double q = std::sqrt(m[i]);
                v[3 * i + 0] = sqrtT * rad0 * std::cos(2 * M_PI * u01(w[1])) / q;
                v[3 * i + 1] = sqrtT * rad0 * std::sin(2 * M_PI * u01(w[1])) / q;
                v[3 * i + 2] = sqrtT * rad1 * std::cos(2 * M_PI * u01(w[3])) / q;
                for (int d = 0; d < 3; ++d) mv[d] += m[i] * v[3 * i + d];
                msum += m[i];
            }
            for (int i = 0; i < n; ++i)
                for (int d = 0; d < 3; ++d) v[3 * i + d] -= mv[d] / msum;
            continue;
        }
        if (integrator == ORC_HOOVER) {
            for (int i = 0; i < n; ++i)
                for (int d = 0; d < 3; ++d) v[3 * i + d] += f[3 * i + d] * (dt / 2) / m[i];
            const double sc = chain_half_step(chain, en_kin_2(), dt);
            for (int k = 0; k < 3 * n; ++k) v[k] *= sc;
            continue;
        }
        for (int i = 0; i < n; ++i) {
            bool collide = false;
            if (coll_rate > 0) {
                u32 ctr[4] = {id[i], (u32)s, 0u, 0x414E4452u}, u[4];
                orc_philox4x32_10(ctr, key, u);
                collide = u[0] < thresh;
                if (collide) {
                    ctr[3] = 0x414E4453u;
                    u32 w[4];
                    orc_philox4x32_10(ctr, key, w);
                    double rad0 = std::sqrt(-2 * std::log(u01(w[0])));
                    double rad1 = std::sqrt(-2 * std::log(u01(w[2])));
                    v[3 * i + 0] = sqrtT * rad0 * std::cos(2 * M_PI * u01(w[1]));
                    v[3 * i + 1] = sqrtT * rad0 * std::sin(2 * M_PI * u01(w[1]));
                    v[3 * i + 2] = sqrtT * rad1 * std::cos(2 * M_PI * u01(w[3]));
                }
            }
            if (!collide)
                for (int d = 0; d < 3; ++d) v[3 * i + d] += f[3 * i + d] * (dt / 2) / m[i];
        }
    }
    /* restore the caller's particle order (by id) */
    {
        std::vector<double> tr(r, r + 3 * (size_t)n), tv(v, v + 3 * (size_t)n), ti(image, image + 3 * (size_t)n);
        for (int i = 0; i < n; ++i) {
            u32 q = id[i];
            for (int d = 0; d < 3; ++d) {
                r[3 * q + d] = tr[3 * i + d];
                v[3 * q + d] = tv[3 * i + d];
                image[3 * q + d] = ti[3 * i + d];
            }
        }
    }
    double ek = 0;
    for (int i = 0; i < n; ++i)
        ek += 0.5 * m[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
    if (stats) { stats[0] = rebuilds; stats[1] = totals[0]; stats[2] = ek; }
    if (chain_out) {
        /* verlet_nvt_hoover.cpp:134-140 */
        double en = chain.T * (3.0 * n * chain.xi[0] + chain.xi[1]);
        for (int k = 0; k < 2; ++k) en += chain.mass[k] * chain.v_xi[k] * chain.v_xi[k] / 2;
        chain_out[0] = chain.xi[0]; chain_out[1] = chain.xi[1];
        chain_out[2] = chain.v_xi[0]; chain_out[3] = chain.v_xi[1];
        chain_out[4] = en / n;
    }
    return 0;
}

/*
 * Steepest-descent minimisation in FP64: the restatement of the engine's
 * minimiser (the reference has none).  Each step moves particle i by
 * step * F_i, shortened to max_move when longer; a NaN force component
 * leaves the particle in place, infinite components move it by max_move
 * along them.  Lists follow the usual skin rule.  stats[0] = potential
 * energy and stats[1] = max_i |F_i| of the final positions.
 */
ORC_API int orc_minimize(int n, double* r, double* image, const u32* sp, const double* L, const orc_pot* p,
                         double skin, int nsteps, double step, double max_move, double* stats)
{
    std::vector<double> f(3 * (size_t)n), r0(r, r + 3 * (size_t)n);
    half_list hl;
    double totals[2] = {0, 0};
    build_half_list(n, r, sp, L, p, skin, hl);
    force_half(n, r, sp, L, p, hl, 0, nullptr, nullptr, f.data(), nullptr, nullptr, totals);
    for (int s = 0; s < nsteps; ++s) {
        double rr_max = 0;
        for (int i = 0; i < n; ++i) {
            double g[3];
            bool nan = false, inf = false;
            for (int d = 0; d < 3; ++d) {
                g[d] = f[3 * i + d] * step;
                nan |= std::isnan(g[d]);
                inf |= std::isinf(g[d]);
            }
            if (nan) continue;
            if (inf)
                for (int d = 0; d < 3; ++d) g[d] = std::isinf(g[d]) ? std::copysign(1.0, g[d]) : 0.0;
            const double len = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            const double c = (inf || len > max_move) ? max_move / len : 1.0;
            double dr[3];
            for (int d = 0; d < 3; ++d) {
                r[3 * i + d] += c * g[d];
                image[3 * i + d] += reduce_periodic_d(r[3 * i + d], L[d]);
                dr[d] = r[3 * i + d] - r0[3 * i + d];
                reduce_periodic_d(dr[d], L[d]);
            }
            rr_max = std::max(rr_max, dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        }
        if (std::sqrt(rr_max) > skin / 2) {
            build_half_list(n, r, sp, L, p, skin, hl);
            std::copy(r, r + 3 * (size_t)n, r0.begin());
        }
        force_half(n, r, sp, L, p, hl, 0, nullptr, nullptr, f.data(), nullptr, nullptr, totals);
    }
    double fmax = 0;
    for (int i = 0; i < n; ++i)
        fmax = std::max(fmax, std::sqrt(f[3 * i] * f[3 * i] + f[3 * i + 1] * f[3 * i + 1] + f[3 * i + 2] * f[3 * i + 2]));
    if (stats) { stats[0] = totals[0]; stats[1] = fmax; }
    return 0;
}
