// engine.cu — host runtime: layout, buffers, step graph, overflow recovery.
#include "engine.h"
#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace hmd {

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error(HMD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

static uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }
static float f32_from_bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t bits_of(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

Engine::Engine(int precision, int device) : precision_(precision), device_(device)
{
    if (precision != HMD_PRECISION_FLOAT && precision != HMD_PRECISION_DSFLOAT && precision != HMD_PRECISION_DOUBLE)
        throw Error(HMD_ERR_INVALID, "precision must be HMD_PRECISION_FLOAT, _DSFLOAT or _DOUBLE");
    int ndev = 0;
    HMD_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) throw Error(HMD_ERR_INVALID, "no such CUDA device");
    HMD_CUDA(cudaSetDevice(device));
    int sms = 0;
    HMD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    sm_count_ = (uint32_t)std::max(sms, 1);
    HMD_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    HMD_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
}

Engine::~Engine()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    destroy_graphs();
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
    if (side_) cudaStreamDestroy(side_);
}

void Engine::check_committed() const
{
    if (!committed_) throw Error(HMD_ERR_STATE, "engine is not committed");
}

void Engine::check_sys(uint32_t s) const
{
    check_committed();
    if (s >= table_size_ || !sys_[s].used) throw Error(HMD_ERR_INVALID, "no such system");
}

const SysHost& Engine::system(uint32_t s) const
{
    check_sys(s);
    return sys_[s];
}

void Engine::sync() { HMD_CUDA(cudaStreamSynchronize(stream_)); }

// LJ in double for the cut-off constants (lennard_jones.hpp:56-66)
static void lj_double(double eps, double sigma2, double rr, double& fval, double& en)
{
    const double rri = sigma2 / rr;
    const double r6i = rri * rri * rri;
    const double eps_r6i = eps * r6i;
    fval = 48 * rri * eps_r6i * (r6i - 0.5) / sigma2;
    en = 4 * eps_r6i * (r6i - 1);
}

// Mie prefactor C(m, n) = m / (m - n) (m / n)^(n / (m - n)) (mdsim/host/potentials/pair/mie.cpp:85-92)
static double mie_prefactor(double m, double n) { return m / (m - n) * std::pow(m / n, n / (m - n)); }

// integer power by repeated multiplication (numeric/pow.hpp)
static double ipow(double x, unsigned n)
{
    double y = 1;
    for (; n; n >>= 1, x *= x)
        if (n & 1) y *= x;
    return y;
}

// the bare pair potential in double for species pair ab: -U'(r)/r and U(r)
// (host potentials lennard_jones.hpp:56-66, mie.hpp:63-73, morse.hpp:64-77,
// power_law.hpp:129-148), for the truncation constants at r_c
static void pot_double(const hmd_system_desc& d, uint32_t ab, double rr, double& fval, double& en)
{
    const double eps = d.epsilon[ab], sigma = d.sigma[ab], sigma2 = sigma * sigma;
    switch (d.potential) {
    case HMD_POTENTIAL_MIE: {
        const unsigned m2 = d.index_repulsion[ab] / 2, n2 = d.index_attraction[ab] / 2;
        const double epsC = eps * mie_prefactor(d.index_repulsion[ab], d.index_attraction[ab]);
        const double rri = sigma2 / rr;
        const double rni = ipow(rri, n2);
        const double rmni = ipow(rri, m2 - n2);
        const double eps_rni = epsC * rni;
        fval = 2 * rri * eps_rni * (m2 * rmni - n2) / sigma2;
        en = eps_rni * (rmni - 1);
        return;
    }
    case HMD_POTENTIAL_MORSE: {
        const double B = d.distortion[ab];
        const double r_sigma_B = std::sqrt(rr) / sigma / B;
        const double dr = d.r_min[ab] / sigma / B - r_sigma_B;
        const double A = 2 * B * B - 1;
        const double exp_dr = std::exp(dr), exp_A_dr = std::exp(A * dr);
        const double eps_exp_dr = eps * exp_dr / A;
        fval = (A + 1) * eps_exp_dr * (exp_A_dr - 1) * r_sigma_B / rr;
        en = eps_exp_dr * (exp_A_dr - A - 1);
        return;
    }
    case HMD_POTENTIAL_POWER_LAW: {
        const unsigned n = d.index[ab];
        const double rri = sigma2 / rr;
        double rni = ipow(rri, n / 2);
        if (n % 2) rni *= std::sqrt(rri);
        const double eps_rni = eps * rni;
        fval = n * eps_rni / rr;
        en = eps_rni;
        return;
    }
    default:
        lj_double(eps, sigma2, rr, fval, en);
    }
}

// HMD_INTEGRATOR_* -> Integrator
static uint32_t integrator_of(int32_t k)
{
    switch (k) {
    case HMD_INTEGRATOR_ANDERSEN: return INTEG_ANDERSEN;
    case HMD_INTEGRATOR_HOOVER: return INTEG_HOOVER;
    case HMD_INTEGRATOR_BOLTZMANN: return INTEG_BOLTZMANN;
    case HMD_INTEGRATOR_EULER: return INTEG_EULER;
    default: return INTEG_VERLET;
    }
}

uint32_t Engine::add_system(const hmd_system_desc& d)
{
    if (committed_ && !capacity_) throw Error(HMD_ERR_STATE, "systems must be added before commit");
    if (d.nparticle == 0) throw Error(HMD_ERR_INVALID, "nparticle must be positive");
    if (d.nspecies < 1 || d.nspecies > HMD_MAX_SPECIES) throw Error(HMD_ERR_INVALID, "nspecies out of range [1, 4]");
    if (d.truncation < HMD_TRUNC_SHARP || d.truncation > HMD_TRUNC_NONE) throw Error(HMD_ERR_INVALID, "unknown truncation");
    const bool full = d.truncation == HMD_TRUNC_NONE;
    if (capacity_ && full)
        throw Error(HMD_ERR_INVALID, "engines with a reserved capacity take truncated potentials");
    if (d.integrator < HMD_INTEGRATOR_VERLET || d.integrator > HMD_INTEGRATOR_EULER)
        throw Error(HMD_ERR_INVALID, "unknown integrator");
    if (capacity_ && d.integrator != HMD_INTEGRATOR_VERLET && d.integrator != HMD_INTEGRATOR_ANDERSEN)
        throw Error(HMD_ERR_INVALID, "engines with a reserved capacity take verlet and verlet_nvt_andersen systems");
    if (!(d.timestep > 0)) throw Error(HMD_ERR_INVALID, "timestep must be positive");
    if (!(d.skin >= 0)) throw Error(HMD_ERR_INVALID, "skin must be non-negative");
    if (!(d.cell_occupancy > 0) || !(d.neighbour_occupancy > 0)) throw Error(HMD_ERR_INVALID, "occupancy must be positive");
    if (d.truncation == HMD_TRUNC_SMOOTH_R4 && !(d.smoothing > 0)) throw Error(HMD_ERR_INVALID, "smooth_r4 needs h > 0");
    const uint32_t ns = d.nspecies;
    if (d.potential < HMD_POTENTIAL_LENNARD_JONES || d.potential > HMD_POTENTIAL_POWER_LAW)
        throw Error(HMD_ERR_INVALID, "unknown potential");
    if (fp64() && (d.potential != HMD_POTENTIAL_LENNARD_JONES || full || d.integrator != HMD_INTEGRATOR_VERLET))
        throw Error(HMD_ERR_INVALID, "the FP64 variant takes truncated Lennard-Jones potentials and verlet");
    for (uint32_t ab = 0; ab < ns * ns; ++ab) {
        if (!(d.sigma[ab] > 0) || !(full || d.r_cut[ab] > 0) || !(d.epsilon[ab] >= 0))
            throw Error(HMD_ERR_INVALID, "bad potential parameters");
        if (d.potential == HMD_POTENTIAL_MIE) {
            const uint32_t m = d.index_repulsion[ab], n = d.index_attraction[ab];
            // mdsim/host/potentials/pair/mie.cpp:72-83
            if ((m & 1u) || (n & 1u)) throw Error(HMD_ERR_STATE, "power law indices of potential must be even");
            if (m <= n) throw Error(HMD_ERR_STATE, "repulsive part of potential must be stronger than attraction");
            if (n == 0 || m > 96) throw Error(HMD_ERR_INVALID, "mie indices out of range [2, 96]");
        }
        if (d.potential == HMD_POTENTIAL_MORSE && (!(d.r_min[ab] > 0) || !(d.distortion[ab] > 0) ||
                                                   2 * d.distortion[ab] * d.distortion[ab] - 1 == 0))
            throw Error(HMD_ERR_INVALID, "morse needs r_min > 0 and a distortion B > 0 with 2 B^2 != 1");
        if (d.potential == HMD_POTENTIAL_POWER_LAW && (d.index[ab] < 1 || d.index[ab] > 96))
            throw Error(HMD_ERR_INVALID, "power_law index out of range [1, 96]");
    }
    for (int q = 0; q < 3; ++q)
        if (!(d.box[q] > 0)) throw Error(HMD_ERR_INVALID, "box edges must be positive");
    if (d.integrator == HMD_INTEGRATOR_ANDERSEN && (!(d.temperature >= 0) || !(d.collision_rate >= 0)))
        throw Error(HMD_ERR_INVALID, "bad thermostat parameters");
    if (d.integrator == HMD_INTEGRATOR_HOOVER && (!(d.temperature > 0) || !(d.resonance_frequency > 0)))
        throw Error(HMD_ERR_INVALID, "verlet_nvt_hoover needs a temperature and a resonance frequency > 0");
    if (d.integrator == HMD_INTEGRATOR_BOLTZMANN && (!(d.temperature >= 0) || !(d.collision_rate > 0)))
        throw Error(HMD_ERR_INVALID, "verlet_nvt_boltzmann needs a temperature >= 0 and a rate > 0");
    if (committed_) return add_live_system(d);   // joins a running engine with a reserved capacity
    if (sys_.size() >= 65536) throw Error(HMD_ERR_INVALID, "too many systems");
    if (capacity_ && sys_.size() >= cap_systems_) throw Error(HMD_ERR_NOMEM, "system table full");
    SysHost h;
    std::memset(&h.P, 0, sizeof(h.P));
    h.desc = d;
    h.used = true;
    sys_.push_back(h);
    return (uint32_t)(sys_.size() - 1);
}

void Engine::layout_system(SysHost& h, uint32_t rank, uint32_t align)
{
    const hmd_system_desc& d = h.desc;
    SysParam& P = h.P;
    const uint32_t ns = d.nspecies;
    P.n = d.nparticle;
    P.A = round_up(std::max<uint32_t>(d.nparticle, 1), align);
    P.ns = ns;
    P.trunc = (uint32_t)d.truncation;
    P.pot = (uint32_t)d.potential;
    P.active = 1;
    const bool full = d.truncation == HMD_TRUNC_NONE;
    P.sort_enable = (d.sort && !full) ? 1u : 0u;
    P.integrator = integrator_of(d.integrator);
    double rc_max = 0, rcs_max = 0;
    h.pairs.resize(ns * ns);
    h.pairs64.resize(ns * ns);
    for (uint32_t ab = 0; ab < ns * ns; ++ab) {
        const double sigma = d.sigma[ab], eps = d.epsilon[ab];
        const double sigma2 = sigma * sigma;
        // untruncated (pair_full): every pair is in range and nothing is shifted
        const double rc = full ? INFINITY : sigma * d.r_cut[ab];
        const double rcs = rc + d.skin;
        double fc = 0, ec = 0;
        if (!full) pot_double(d, ab, rc * rc, fc, ec);
        PairParam& p = h.pairs[ab];
        p.eps4 = (float)(4 * eps);
        p.c48 = (float)(48 * eps / sigma2);
        p.sigma2 = (float)sigma2;
        p.rr_cut = (float)(rc * rc);
        p.r_cut = (float)rc;
        p.rr_cut_skin = full ? 0.0f : (float)(rcs * rcs);
        p.en_cut = (d.truncation == HMD_TRUNC_SHARP) ? 0.0f : (float)ec;
        p.f_cut = (d.truncation == HMD_TRUNC_FORCE_SHIFTED) ? (float)(fc * rc) : 0.0f;
        p.rr_near = (float)(NEAR_SIGMA * NEAR_SIGMA * sigma2);
        p.sigma2_lo = (float)(sigma2 - (double)p.sigma2);
        p.c48_lo = (float)(48 * eps / sigma2 - (double)p.c48);
        p.q0 = p.q1 = p.q2 = p.q3 = 0.0f;
        if (d.potential == HMD_POTENTIAL_MIE) {
            p.q0 = (float)(eps * mie_prefactor(d.index_repulsion[ab], d.index_attraction[ab]));
            p.q1 = (float)(2 / sigma2);
            p.q2 = (float)(d.index_repulsion[ab] / 2);
            p.q3 = (float)(d.index_attraction[ab] / 2);
        } else if (d.potential == HMD_POTENTIAL_MORSE) {
            const double B = d.distortion[ab], A = 2 * B * B - 1;
            p.q0 = (float)(eps / A);
            p.q1 = (float)A;
            p.q2 = (float)(1 / (sigma * B));
            p.q3 = (float)(d.r_min[ab] / (sigma * B));
        } else if (d.potential == HMD_POTENTIAL_POWER_LAW) {
            p.q0 = (float)eps;
            p.q1 = (float)d.index[ab];
            p.q2 = (float)(d.index[ab] / 2);
            p.q3 = (float)(d.index[ab] % 2);
        }
        p.rr_tie = 8.0f * (std::nextafter(p.rr_cut, INFINITY) - p.rr_cut);
        PairParam64& q = h.pairs64[ab];
        q.eps4 = 4 * eps;
        q.c48 = 48 * eps / sigma2;
        q.sigma2 = sigma2;
        q.rr_cut = rc * rc;
        q.r_cut = rc;
        q.en_cut = (d.truncation == HMD_TRUNC_SHARP) ? 0.0 : ec;
        q.f_cut = (d.truncation == HMD_TRUNC_FORCE_SHIFTED) ? fc * rc : 0.0;
        q.pad = 0.0;
        if (full) continue;
        rc_max = std::max(rc_max, rc);
        rcs_max = std::max(rcs_max, rcs);
    }
    P.rri_smooth = (d.truncation == HMD_TRUNC_SMOOTH_R4) ? (float)std::pow(d.smoothing, -2) : 0.0f;
    P.rri_smooth64 = (d.truncation == HMD_TRUNC_SMOOTH_R4) ? std::pow(d.smoothing, -2) : 0.0;
    P.dt64 = d.timestep;
    P.dt = (float)d.timestep;
    P.dt_half = (float)(d.timestep / 2);
    P.rr_half_skin = full ? INFINITY : (float)(0.25 * d.skin * d.skin);   // pair_full never rebuilds
    P.sqrt_T = (float)std::sqrt(d.temperature);
    {
        const double q = d.collision_rate * d.timestep;
        P.coll_threshold = (d.integrator == HMD_INTEGRATOR_ANDERSEN)
                               ? (uint32_t)std::min(4294967295.0, std::floor(q * 4294967296.0)) : 0u;
    }
    P.seed_lo = (uint32_t)d.seed;
    P.seed_hi = (uint32_t)(d.seed >> 32);
    // verlet_nvt_boltzmann.lua.in: coupling interval max(1, round(1 / (rate dt)))
    P.interval = (d.integrator == HMD_INTEGRATOR_BOLTZMANN)
                     ? (uint32_t)std::max(1.0, std::floor(1.0 / (d.collision_rate * d.timestep) + 0.5)) : 1u;
    if (d.integrator == HMD_INTEGRATOR_HOOVER) {
        // verlet_nvt_hoover.cpp:58-84: masses of the heat-bath variables after
        // Martyna et al., J. Chem. Phys. 97, 2635 (1992)
        const double omega_sq = std::pow(2 * M_PI * d.resonance_frequency, 2);
        const double dof = 3.0 * d.nparticle;
        P.nhc_mass[0] = dof * d.temperature / omega_sq;
        P.nhc_mass[1] = d.temperature / omega_sq;
        P.nhc_target2 = dof * d.temperature;
        P.nhc_T = d.temperature;
        P.nhc_dt = d.timestep;
    }
    {
        // a near pair (closer than NEAR_SIGMA sigma at the build) is within
        // NEAR_SIGMA sigma + skin at force time in every coordinate; from twice
        // that distance to zero on, a coordinate and its partner's differ exactly
        double near_max = 0;
        for (uint32_t ab = 0; ab < ns * ns; ++ab) near_max = std::max(near_max, NEAR_SIGMA * d.sigma[ab] + d.skin);
        P.exact_min = (float)(2.0 * near_max * (1.0 + 1e-6));
        // near pairs never reach r_c when NEAR_SIGMA sigma + skin stays below it
        bool in_range = true;
        for (uint32_t ab = 0; ab < ns * ns; ++ab)
            in_range = in_range && NEAR_SIGMA * d.sigma[ab] + d.skin < d.sigma[ab] * d.r_cut[ab] * (1.0 - 1e-6);
        P.near_in_range = (in_range && !full) ? 1u : 0u;
    }
    for (int q = 0; q < 3; ++q) {
        // a list pair is within r_c + skin of each other at force time (each
        // particle moved < skin/2 since the build); particles farther than
        // that from every face have no partner across the box
        const double in = 0.5 * d.box[q] - (rcs_max + d.skin) - 1e-4 * d.box[q];
        P.inner[q] = (in > 0 && !full) ? (float)in : 0.0f;
    }
    float Lmax = 0;
    for (int q = 0; q < 3; ++q) {
        const float Lf = (float)d.box[q];
        P.L[q] = Lf;
        P.Linv[q] = (float)(1.0 / (double)Lf);
        Lmax = std::max(Lmax, Lf);
        if (!(d.box[q] > 2 * rc_max))
            throw Error(HMD_ERR_INVALID, "box edge must exceed twice the largest cutoff (minimum image)");
    }
    {
        // unit of the lo-word codes of the force kernel's gather records:
        // ulp of the binade of L_max / 2 (the largest |coordinate|) / 1024
        int e = 0;
        std::frexp(0.5 * (double)Lmax, &e);              // 0.5 Lmax in [2^(e-1), 2^e)
        const int es = e - 1 - 23 - 10;                   // s = 2^es
        P.lo_scale = (float)std::ldexp(1.0, es);
        P.lo_inv_scale = (float)std::ldexp(1.0, -es);
        P.lo_exp_bits = (uint32_t)(es + 23 + 127) << 23;  // the float 2^23 s
        P.lo_bias = (float)std::ldexp(8388608.0 + 512.0, es);
        P.lo_exp_bits_y = (uint32_t)(es + 13 + 127) << 23;   // the float 2^13 s
        P.lo_bias_y = (float)std::ldexp(8192.0 + 512.0, es);
    }
    // Hilbert depth (gpu/sorts/hilbert.cpp:51-54)
    P.depth = std::min(10u, (uint32_t)std::ceil(std::log((double)Lmax) / M_LN2));
    if (full) {
        // no binning and no list; one placeholder cell keeps the tables uniform
        for (int q = 0; q < 3; ++q) {
            P.ncell[q] = 1;
            P.cell_len[q] = P.L[q];
        }
        P.ncells = 1;
        P.cell_size = 32;
        h.nbr_size = 8;
        return;
    }
    // binning sizing (gpu/binning.cpp:81-101)
    const double warp = 32;
    const double nwarps = d.nparticle / (d.cell_occupancy * warp);
    const double volume = d.box[0] * d.box[1] * d.box[2];
    uint32_t ncells = 1;
    for (int q = 0; q < 3; ++q) {
        const int nmax = (int)(d.box[q] / rcs_max);
        const int nc = (int)std::ceil(d.box[q] * std::pow(nwarps / volume, 1.0 / 3));
        P.ncell[q] = std::max(1, std::min(nc, nmax));
        P.cell_len[q] = P.L[q] / (float)P.ncell[q];
        ncells *= (uint32_t)P.ncell[q];
    }
    P.ncells = ncells;
    P.cell_size = (uint32_t)(warp * std::ceil(nwarps / ncells));
    P.cell_size = std::max<uint32_t>(32, P.cell_size);
    if (P.cell_size > 256) throw Error(HMD_ERR_INVALID, "cell size above 256 slots; lower the density or occupancy");
    // neighbour list capacity (from_binning.cpp:96-119)
    const float sphere = (float)(4 * M_PI / 3) * std::pow((float)rcs_max, 3.0f);
    const float density = (float)(d.nparticle / volume);
    h.nbr_size = (uint32_t)std::ceil(sphere * (density / (float)d.neighbour_occupancy));
    h.nbr_size = std::max<uint32_t>(h.nbr_size, 32);
}

// ---- layout ---------------------------------------------------------------
//
// Fixed engines lay their systems out back to back (slot ranges padded to
// SLOT_ALIGN).  Engines with a reserved capacity keep slots, cells and cell
// words in first-fit arenas so systems can join and leave between steps: slot
// ranges are then SORT_TILE-aligned, free ranges belong to an inert "null
// system" at the last table index, and every kernel reads all per-system state
// from device tables, so captured step graphs stay valid while the set of
// systems changes.

bool Arena::alloc(uint32_t n, uint32_t& at)
{
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            at = it->first;
            const uint32_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[at + n] = rest;
            used_ += n;
            return true;
        }
    }
    return false;
}

void Arena::release(uint32_t at, uint32_t n)
{
    if (n == 0) return;
    used_ -= n;
    auto next = free_.lower_bound(at);
    uint32_t start = at, len = n;
    if (next != free_.begin()) {
        auto prev = std::prev(next);
        if (prev->first + prev->second == at) {
            start = prev->first;
            len += prev->second;
            free_.erase(prev);
        }
    }
    next = free_.lower_bound(at);
    if (next != free_.end() && next->first == at + n) {
        len += next->second;
        free_.erase(next);
    }
    free_[start] = len;
}

void Engine::reserve(uint32_t slots, uint32_t systems, uint32_t neighbour_capacity)
{
    if (committed_) throw Error(HMD_ERR_STATE, "capacity must be reserved before commit");
    if (fp64()) throw Error(HMD_ERR_INVALID, "the FP64 variant runs fixed engines only");
    if (slots == 0 || systems == 0) throw Error(HMD_ERR_INVALID, "capacity must be positive");
    for (const SysHost& h : sys_)
        if (h.desc.integrator != HMD_INTEGRATOR_VERLET && h.desc.integrator != HMD_INTEGRATOR_ANDERSEN)
            throw Error(HMD_ERR_INVALID, "engines with a reserved capacity take verlet and verlet_nvt_andersen systems");
    capacity_ = true;
    cap_slots_ = round_up(slots, SORT_TILE);
    cap_systems_ = systems;
    cap_nbr_ = neighbour_capacity;
}

// place system s in the arenas (capacity mode); false if it does not fit
bool Engine::place(uint32_t s)
{
    SysParam& P = sys_[s].P;
    uint32_t at_slot, at_cell, at_word;
    if (!slot_arena_.alloc(P.A / SORT_TILE, at_slot)) return false;
    if (!cell_arena_.alloc(P.ncells, at_cell)) {
        slot_arena_.release(at_slot, P.A / SORT_TILE);
        return false;
    }
    if (!word_arena_.alloc(P.ncells * P.cell_size / 32, at_word)) {
        slot_arena_.release(at_slot, P.A / SORT_TILE);
        cell_arena_.release(at_cell, P.ncells);
        return false;
    }
    P.off = at_slot * SORT_TILE;
    P.cell_off = at_cell;
    P.cell_word_off = at_word * 32;
    P.sort_ntiles = P.A / SORT_TILE;
    P.sort_hist_off = 256u * at_slot;
    return true;
}

void Engine::unplace(uint32_t s)
{
    const SysParam& P = sys_[s].P;
    slot_arena_.release(P.off / SORT_TILE, P.A / SORT_TILE);
    cell_arena_.release(P.cell_off, P.ncells);
    word_arena_.release(P.cell_word_off / 32, P.ncells * P.cell_size / 32);
}

// kind of pair interaction of a system (kernels.h ForceKind; the device
// counterpart is force_kind_of in force.cuh)
static int force_kind(const SysParam& P)
{
    if (P.trunc == TRUNC_NONE) return FK_FULL;
    if (P.pot != POT_LJ) return FK_POT;
    if (P.trunc == TRUNC_SHARP || P.trunc == TRUNC_SHIFTED) return P.ns == 1 ? FK_LJ1 : FK_SHIFTED;
    return P.trunc == TRUNC_SMOOTH_R4 ? FK_SMOOTH : FK_FSHIFT;
}

void Engine::commit()
{
    if (committed_) throw Error(HMD_ERR_STATE, "engine already committed");
    if (sys_.empty() && !capacity_) throw Error(HMD_ERR_STATE, "no systems");
    HMD_CUDA(cudaSetDevice(device_));
    uint32_t cell_words = 0;
    uint32_t hist_words = 0;
    std::vector<uint2> tiles;
    nbr_cap_ = 0;
    any_sort_ = false;
    uint32_t shift = 0;
    force_kinds_ = 0;
    integ_kinds_ = 0;
    if (!capacity_) {
        table_size_ = (uint32_t)sys_.size();
        null_sys_ = PLACEHOLDER;
        S_ = 0;
        total_cells_ = 0;
        for (uint32_t s = 0; s < sys_.size(); ++s) {
            SysHost& h = sys_[s];
            layout_system(h, s, SLOT_ALIGN);
            h.P.off = S_;
            S_ += h.P.A;
            h.P.cell_off = total_cells_;
            h.P.cell_word_off = cell_words;
            total_cells_ += h.P.ncells;
            cell_words += h.P.ncells * h.P.cell_size;
            nbr_cap_ = std::max(nbr_cap_, round_up(h.nbr_size, 8));
            shift = std::max(shift, 3 * h.P.depth);
            any_sort_ = any_sort_ || h.P.sort_enable;
            force_kinds_ |= 1u << force_kind(h.P);
            integ_kinds_ |= 1u << h.P.integrator;
        }
        // each system sorts its own slot range with 3*depth-bit Hilbert keys,
        // in tiles that never straddle two systems
        for (uint32_t s = 0; s < sys_.size(); ++s) {
            SysParam& P = sys_[s].P;
            P.sort_ntiles = (P.A + SORT_TILE - 1) / SORT_TILE;
            P.sort_hist_off = hist_words;
            if (!P.sort_enable) continue;
            hist_words += 256u * P.sort_ntiles;
            for (uint32_t t = 0; t < P.sort_ntiles; ++t) tiles.push_back(make_uint2(s, P.off + t * SORT_TILE));
        }
    } else {
        table_size_ = cap_systems_ + 1;
        null_sys_ = cap_systems_;
        S_ = cap_slots_;
        // cells: at most one per 8 slots on average, 32-word cells (grown on demand)
        total_cells_ = std::max<uint32_t>(S_ / 8, 64);
        cell_words = 64u * total_cells_;
        slot_arena_.init(S_ / SORT_TILE);
        cell_arena_.init(total_cells_);
        word_arena_.init(cell_words / 32);
        std::vector<SysHost> pre = sys_;
        sys_.assign(table_size_, SysHost());
        for (uint32_t s = 0; s < pre.size(); ++s) {
            sys_[s] = pre[s];
            layout_system(sys_[s], s, SORT_TILE);
            if (!place(s)) throw Error(HMD_ERR_NOMEM, "reserved capacity too small for the systems");
            sys_[s].used = true;
        }
        for (auto& h : sys_) nbr_cap_ = std::max(nbr_cap_, h.used ? round_up(h.nbr_size, 8) : 0u);
        nbr_cap_ = std::max(nbr_cap_, round_up(cap_nbr_, 8));
        shift = 30;           // any depth up to 10
        any_sort_ = true;
        hist_words = 256u * (S_ / SORT_TILE);
        tiles.resize(S_ / SORT_TILE);
        for (uint32_t t = 0; t < tiles.size(); ++t) tiles[t] = make_uint2(null_sys_, t * SORT_TILE);
        for (uint32_t s = 0; s < pre.size(); ++s)
            for (uint32_t t = 0; t < sys_[s].P.sort_ntiles; ++t)
                tiles[sys_[s].P.off / SORT_TILE + t] = make_uint2(s, sys_[s].P.off + t * SORT_TILE);
    }
    if (nbr_cap_ == 0) nbr_cap_ = 64;
    key_bits_ = shift;
    sort_passes_ = radix_passes(key_bits_);
    ntiles_ = (uint32_t)tiles.size();
    tiles_.alloc(std::max<size_t>(tiles.size(), 1));
    if (!tiles.empty())
        HMD_CUDA(cudaMemcpy(tiles_.p, tiles.data(), tiles.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    hist_.alloc(std::max<uint32_t>(hist_words, 1));
    dtot_.alloc((size_t)table_size_ * 256);
    // force-kernel shape when not set (the autotuner refines it): small
    // engines need several lanes per particle to fill 152 SMs (measured best
    // at 64k particles: 4 lanes, 2 entries per load); large ones one lane
    // with 4 entries per load (measured best at 1M)
    if (lanes_ == 0) {
        const bool small = S_ <= (1u << 19);
        lanes_ = small ? 4u : 1u;
        if (lb_ == 0 && small) lb_ = 8u;
    }

    const size_t S = S_;
    pos_.alloc(2 * S); vel_.alloc(2 * S); img_.alloc(S); force_.alloc(S); r0_.alloc(S);
    if (ds()) fpos_.alloc(S);
    if (fp64()) force64_.alloc(S);
    tpos_.alloc(2 * S); tvel_.alloc(2 * S); timg_.alloc(S); tid_.alloc(S);
    en_pot_.alloc(S); stress_.alloc(6 * S);
    id_.alloc(S); rid_.alloc(S);
    nbr_.alloc((size_t)nbr_cap_ * S); nbr_count_.alloc(S);
    cell_.alloc(std::max<uint32_t>(cell_words, 1));
    cell_count_.alloc(std::max<uint32_t>(total_cells_, 1));
    cell_sys_.alloc(std::max<uint32_t>(total_cells_, 1));
    chunk_sys_.alloc(S / CHUNK);
    key0_.alloc(S); key1_.alloc(S); val0_.alloc(S); val1_.alloc(S);
    // done_: [0] last-block ticket counter, [1] flag of launch_check_finite;
    // any_rebuild_: [0] this step rebuilds, [1] rebuild chains run
    status_.alloc(1); done_.alloc(2); any_rebuild_.alloc(2);
    // rebuild list: count, systems, and RB_UNITS prefix sums of n + 1 entries
    rb_.alloc(1 + table_size_ + (size_t)RB_UNITS * (table_size_ + 1));
    dsys_.alloc(table_size_); dst_.alloc(table_size_);
    dpair_.alloc((size_t)table_size_ * MAX_SPECIES * MAX_SPECIES);
    if (fp64()) dpair64_.alloc((size_t)table_size_ * MAX_SPECIES * MAX_SPECIES);
    partial_.alloc((S / 256) * NTHERMO + 1); thermo_.alloc((size_t)table_size_ * NTHERMO);

    // everything starts as ghosts owned by the null system (capacity mode)
    {
        std::vector<float4> hpos(2 * S, make_float4(0, 0, 0, 0));
        for (size_t k = 0; k < S; ++k) hpos[2 * k].w = f32_from_bits(PLACEHOLDER);   // hi words: ghosts
        HMD_CUDA(cudaMemcpyAsync(pos_.p, hpos.data(), 2 * S * sizeof(float4), cudaMemcpyHostToDevice, stream_));
        sync();
        for (size_t k = 0; k < S; ++k) hpos[k] = make_float4(0, 0, 0, f32_from_bits(PLACEHOLDER));
        HMD_CUDA(cudaMemcpyAsync(r0_.p, hpos.data(), S * sizeof(float4), cudaMemcpyHostToDevice, stream_));
        sync();   // the staging vector goes out of scope
        HMD_CUDA(cudaMemsetAsync(vel_.p, 0, vel_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(img_.p, 0, img_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(force_.p, 0, force_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(en_pot_.p, 0, en_pot_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(stress_.p, 0, stress_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(nbr_count_.p, 0, nbr_count_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(cell_count_.p, 0, cell_count_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(status_.p, 0, status_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(done_.p, 0, done_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(any_rebuild_.p, 0, any_rebuild_.bytes(), stream_));
        HMD_CUDA(cudaMemsetAsync(id_.p, 0xFF, id_.bytes(), stream_));
        std::vector<uint32_t> iota(S);
        for (size_t k = 0; k < S; ++k) iota[k] = (uint32_t)k;
        HMD_CUDA(cudaMemcpyAsync(rid_.p, iota.data(), rid_.bytes(), cudaMemcpyHostToDevice, stream_));
        const uint32_t owner = capacity_ ? null_sys_ : 0u;
        std::vector<uint32_t> hchunk(S / CHUNK, owner), hcs(std::max<uint32_t>(total_cells_, 1), owner);
        HMD_CUDA(cudaMemcpyAsync(chunk_sys_.p, hchunk.data(), chunk_sys_.bytes(), cudaMemcpyHostToDevice, stream_));
        HMD_CUDA(cudaMemcpyAsync(cell_sys_.p, hcs.data(), cell_sys_.bytes(), cudaMemcpyHostToDevice, stream_));
        std::vector<SysState> st(table_size_);
        for (auto& t : st) std::memset(&t, 0, sizeof(t));
        HMD_CUDA(cudaMemcpyAsync(dst_.p, st.data(), dst_.bytes(), cudaMemcpyHostToDevice, stream_));
        std::vector<SysParam> P(table_size_);
        for (auto& p : P) std::memset(&p, 0, sizeof(p));
        HMD_CUDA(cudaMemcpyAsync(dsys_.p, P.data(), dsys_.bytes(), cudaMemcpyHostToDevice, stream_));
        sync();
    }
    committed_ = true;
    grid_slots_ = grid_cells_ = 0;
    update_grid_extent();
    for (uint32_t s = 0; s < table_size_; ++s)
        if (!capacity_ || sys_[s].used) install(s);
    sync();
}

// write one system's slots, maps, tables and state to the device
void Engine::install(uint32_t s)
{
    SysHost& h = sys_[s];
    h.used = true;
    SysParam& P = h.P;
    P.pair_off = s * (uint32_t)(MAX_SPECIES * MAX_SPECIES);
    P.active = 1;
    const size_t S = S_;
    std::vector<float4> hp(P.A), hv(P.A, make_float4(0, 0, 0, 0));
    std::vector<uint32_t> ids(P.A), rids(P.A);
    for (uint32_t t = 0; t < P.A; ++t) {
        const bool real = t < P.n;
        hp[t] = make_float4(0, 0, 0, real ? 0.0f : f32_from_bits(PLACEHOLDER));   // species 0
        hv[t].w = real ? 1.0f : 0.0f;                                           // unit mass (particle.cpp:56-160)
        ids[t] = real ? t : PLACEHOLDER;
        rids[t] = P.off + t;
    }
    upload_pos(false, P.off, P.A, hp.data());
    HMD_CUDA(cudaMemcpyAsync(r0_.p + P.off, hp.data(), P.A * sizeof(float4), cudaMemcpyHostToDevice, stream_));
    HMD_CUDA(cudaMemset2DAsync(pos_.p + 2 * (size_t)P.off + 1, 2 * sizeof(float4), 0, sizeof(float4), P.A, stream_));
    HMD_CUDA(cudaMemcpyAsync(vel_.p + P.off, hv.data(), P.A * sizeof(float4), cudaMemcpyHostToDevice, stream_));
    HMD_CUDA(cudaMemsetAsync(vel_.p + S + P.off, 0, P.A * sizeof(float4), stream_));
    HMD_CUDA(cudaMemsetAsync(img_.p + P.off, 0, P.A * sizeof(float4), stream_));
    HMD_CUDA(cudaMemsetAsync(force_.p + P.off, 0, P.A * sizeof(float4), stream_));
    HMD_CUDA(cudaMemsetAsync(en_pot_.p + P.off, 0, P.A * sizeof(float), stream_));
    for (int c = 0; c < 6; ++c) HMD_CUDA(cudaMemsetAsync(stress_.p + c * S + P.off, 0, P.A * sizeof(float), stream_));
    HMD_CUDA(cudaMemsetAsync(nbr_count_.p + P.off, 0, P.A * sizeof(uint32_t), stream_));
    HMD_CUDA(cudaMemcpyAsync(id_.p + P.off, ids.data(), P.A * 4, cudaMemcpyHostToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(rid_.p + P.off, rids.data(), P.A * 4, cudaMemcpyHostToDevice, stream_));
    std::vector<uint32_t> own(std::max<uint32_t>(P.A / CHUNK, P.ncells), s);
    HMD_CUDA(cudaMemcpyAsync(chunk_sys_.p + P.off / CHUNK, own.data(), (P.A / CHUNK) * 4, cudaMemcpyHostToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(cell_sys_.p + P.cell_off, own.data(), P.ncells * 4, cudaMemcpyHostToDevice, stream_));
    HMD_CUDA(cudaMemsetAsync(cell_count_.p + P.cell_off, 0, P.ncells * 4, stream_));
    if (capacity_) {
        std::vector<uint2> tl(P.sort_ntiles);
        for (uint32_t t = 0; t < P.sort_ntiles; ++t) tl[t] = make_uint2(P.sort_enable ? s : null_sys_, P.off + t * SORT_TILE);
        HMD_CUDA(cudaMemcpyAsync(tiles_.p + P.off / SORT_TILE, tl.data(), tl.size() * sizeof(uint2),
                                 cudaMemcpyHostToDevice, stream_));
    }
    SysState st;
    std::memset(&st, 0, sizeof(st));
    st.steps_left = 0xFFFFFFFFu;
    st.rebuild_request = 1u;
    HMD_CUDA(cudaMemcpyAsync(dst_.p + s, &st, sizeof(st), cudaMemcpyHostToDevice, stream_));
    upload_system(s);
    sync();
    forces_valid_ = false;
}

void Engine::upload_system(uint32_t s)
{
    const SysHost& h = sys_[s];
    HMD_CUDA(cudaMemcpyAsync(dsys_.p + s, &h.P, sizeof(SysParam), cudaMemcpyHostToDevice, stream_));
    if (!h.pairs.empty())
        HMD_CUDA(cudaMemcpyAsync(dpair_.p + h.P.pair_off, h.pairs.data(), h.pairs.size() * sizeof(PairParam),
                                 cudaMemcpyHostToDevice, stream_));
    if (fp64() && !h.pairs64.empty())
        HMD_CUDA(cudaMemcpyAsync(dpair64_.p + h.P.pair_off, h.pairs64.data(), h.pairs64.size() * sizeof(PairParam64),
                                 cudaMemcpyHostToDevice, stream_));
    sync();
}

void Engine::upload_tables()
{
    for (uint32_t s = 0; s < table_size_; ++s)
        if (sys_[s].used) upload_system(s);
}

uint32_t Engine::add_live_system(const hmd_system_desc& d)
{
    if (!capacity_) throw Error(HMD_ERR_STATE, "systems join a committed engine only with a reserved capacity");
    uint32_t s = PLACEHOLDER;
    for (uint32_t k = 0; k < cap_systems_; ++k)
        if (!sys_[k].used) { s = k; break; }
    if (s == PLACEHOLDER) throw Error(HMD_ERR_NOMEM, "system table full");
    SysHost h;
    std::memset(&h.P, 0, sizeof(h.P));
    h.desc = d;
    sys_[s] = h;
    layout_system(sys_[s], s, SORT_TILE);
    if (round_up(sys_[s].nbr_size, 8) > nbr_cap_) {
        sys_[s] = SysHost();
        throw Error(HMD_ERR_NOMEM, "system needs more neighbour-list slots than the engine reserved");
    }
    if (!place(s)) {
        sys_[s] = SysHost();
        throw Error(HMD_ERR_NOMEM, "no room in the reserved capacity");
    }
    install(s);
    update_grid_extent();
    return s;
}

void Engine::remove_system(uint32_t s)
{
    check_sys(s);
    if (!capacity_) throw Error(HMD_ERR_STATE, "systems leave only engines with a reserved capacity");
    SysParam P = sys_[s].P;
    std::vector<float4> ghost(P.A, make_float4(0, 0, 0, f32_from_bits(PLACEHOLDER)));
    upload_pos(false, P.off, P.A, ghost.data());
    HMD_CUDA(cudaMemsetAsync(id_.p + P.off, 0xFF, P.A * 4, stream_));
    std::vector<uint32_t> own(std::max<uint32_t>(P.A / CHUNK, P.ncells), null_sys_);
    HMD_CUDA(cudaMemcpyAsync(chunk_sys_.p + P.off / CHUNK, own.data(), (P.A / CHUNK) * 4, cudaMemcpyHostToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(cell_sys_.p + P.cell_off, own.data(), P.ncells * 4, cudaMemcpyHostToDevice, stream_));
    std::vector<uint2> tl(P.sort_ntiles);
    for (uint32_t t = 0; t < P.sort_ntiles; ++t) tl[t] = make_uint2(null_sys_, P.off + t * SORT_TILE);
    HMD_CUDA(cudaMemcpyAsync(tiles_.p + P.off / SORT_TILE, tl.data(), tl.size() * sizeof(uint2),
                             cudaMemcpyHostToDevice, stream_));
    SysParam z;
    std::memset(&z, 0, sizeof(z));
    HMD_CUDA(cudaMemcpyAsync(dsys_.p + s, &z, sizeof(z), cudaMemcpyHostToDevice, stream_));
    SysState st;
    std::memset(&st, 0, sizeof(st));
    HMD_CUDA(cudaMemcpyAsync(dst_.p + s, &st, sizeof(st), cudaMemcpyHostToDevice, stream_));
    sync();
    unplace(s);
    sys_[s] = SysHost();
    update_grid_extent();
}

// Launch-grid extents (Dev::S_grid, cells_grid, tiles_grid).  A fixed layout
// covers everything.  With a reserved capacity the grids cover the slots and
// cells below the high-water mark of the systems present (first-fit
// placement keeps them low), rounded up to a power of two, instead of the
// whole reservation: they grow as soon as a system needs it and shrink once
// the mark falls below a quarter, and the captured step graphs, which carry
// the grid sizes, are recaptured on a change.
void Engine::update_grid_extent()
{
    uint32_t slots = S_, cells = total_cells_;
    if (capacity_) {
        uint32_t hs = SORT_TILE, hc = 64;
        for (const SysHost& h : sys_) {
            if (!h.used) continue;
            hs = std::max(hs, h.P.off + h.P.A);
            hc = std::max(hc, h.P.cell_off + h.P.ncells);
        }
        auto bucket = [](uint32_t need, uint32_t cur, uint32_t full) {
            uint32_t b = 1;
            while (b < need) b <<= 1;
            b = std::min(b, full);
            return (need > cur || (uint64_t)need * 4 <= cur) ? b : cur;
        };
        slots = bucket(hs, grid_slots_, S_);
        cells = bucket(hc, grid_cells_, total_cells_);
    }
    if (slots != grid_slots_ || cells != grid_cells_) {
        grid_slots_ = slots;
        grid_cells_ = cells;
        destroy_graphs();
    }
}

void Engine::capacity_info(uint64_t* out) const
{
    out[0] = S_;
    out[1] = capacity_ ? (uint64_t)slot_arena_.used() * SORT_TILE : S_;
    out[2] = total_cells_;
    out[3] = capacity_ ? cell_arena_.used() : total_cells_;
    out[4] = nbr_cap_;
    uint32_t n = 0;
    for (uint32_t s = 0; s < table_size_; ++s) n += sys_[s].used ? 1u : 0u;
    out[5] = n;
    out[6] = capacity_ ? cap_systems_ : table_size_;
    out[7] = bytes_per_slot();
}

void Engine::progress(uint64_t* step, uint32_t* steps_left, uint32_t n)
{
    check_committed();
    std::vector<SysState> st = read_state();
    for (uint32_t s = 0; s < n && s < table_size_; ++s) {
        if (step) step[s] = st[s].step;
        if (steps_left) steps_left[s] = st[s].steps_left;
    }
}

uint64_t Engine::bytes_per_slot() const
{
    // device bytes that scale with the slot count
    return 2 * 16 + 2 * 16 + 16 + 16 + 16 + 2 * 16 + 2 * 16 + 16 + 4 + 4 + 24 + 4 + 4 + 4 + 16 + 4ull * nbr_cap_ +
           2 * 16 + 2 * 16 + 16 + 16 + 8;
}

Dev Engine::dev() const
{
    Dev d;
    std::memset(&d, 0, sizeof(d));
    d.pos = pos_.p; d.vel = vel_.p; d.img = img_.p; d.force = force_.p; d.r0 = r0_.p;
    d.fpos = fpos_.p;
    d.force64 = force64_.p;
    d.pair64 = dpair64_.p;
    d.fp64 = fp64() ? 1u : 0u;
    d.float_cutoff = float_cutoff_ ? 1u : 0u;
    d.en_pot = en_pot_.p; d.stress = stress_.p; d.id = id_.p; d.rid = rid_.p;
    d.nbr = nbr_.p; d.nbr_count = nbr_count_.p; d.nbr_cap = nbr_cap_;
    d.lanes = lanes_;
    d.lb_log2 = block() == 8u ? 3u : 2u;
    d.nbr_scan = nbr_scan_;   // 0: each system by its own size (k_neighbour)
    d.force_kinds = force_kinds_;
    d.integ_kinds = integ_kinds_;
    d.cell = cell_.p; d.cell_count = cell_count_.p; d.cell_sys = cell_sys_.p; d.total_cells = total_cells_;
    d.sys = dsys_.p; d.st = dst_.p; d.pair = dpair_.p; d.chunk_sys = chunk_sys_.p;
    d.S = S_; d.nsys = table_size_;
    d.ds = ds() ? 1u : 0u;
    d.S_grid = grid_slots_ ? grid_slots_ : S_;
    d.cells_grid = grid_cells_ ? grid_cells_ : total_cells_;
    d.tiles_grid = capacity_ ? d.S_grid / SORT_TILE : ntiles_;
    d.sm_count = sm_count_;
    d.status = status_.p; d.done = done_.p; d.any_rebuild = any_rebuild_.p;
    d.key[0] = key0_.p; d.key[1] = key1_.p; d.val[0] = val0_.p; d.val[1] = val1_.p; d.hist = hist_.p; d.dtot = dtot_.p;
    d.tiles = tiles_.p; d.ntiles = ntiles_; d.rb = rb_.p;
    d.tpos = tpos_.p; d.tvel = tvel_.p; d.timg = timg_.p; d.tid = tid_.p;
    d.partial = partial_.p; d.thermo = thermo_.p;
    return d;
}

template <typename T>
void Engine::download(const DevBuf<T>& b, size_t first, size_t count, T* host)
{
    if (count == 0) return;
    HMD_CUDA(cudaMemcpyAsync(host, b.p + first, count * sizeof(T), cudaMemcpyDeviceToHost, stream_));
    sync();
}

template <typename T>
void Engine::upload(DevBuf<T>& b, size_t first, size_t count, const T* host)
{
    if (count == 0) return;
    HMD_CUDA(cudaMemcpyAsync(b.p + first, host, count * sizeof(T), cudaMemcpyHostToDevice, stream_));
    sync();
}

void Engine::download_pos(bool lo, size_t first, size_t count, float4* host)
{
    if (count == 0) return;
    HMD_CUDA(cudaMemcpy2DAsync(host, sizeof(float4), pos_.p + 2 * first + (lo ? 1 : 0), 2 * sizeof(float4),
                               sizeof(float4), count, cudaMemcpyDeviceToHost, stream_));
    sync();
}

void Engine::upload_pos(bool lo, size_t first, size_t count, const float4* host)
{
    if (count == 0) return;
    HMD_CUDA(cudaMemcpy2DAsync(pos_.p + 2 * first + (lo ? 1 : 0), 2 * sizeof(float4), host, sizeof(float4),
                               sizeof(float4), count, cudaMemcpyHostToDevice, stream_));
    sync();
}

std::vector<SysState> Engine::read_state()
{
    std::vector<SysState> st(table_size_);
    download(dst_, 0, st.size(), st.data());
    return st;
}

void Engine::write_state(const std::vector<SysState>& st) { upload(dst_, 0, st.size(), st.data()); }

std::vector<uint32_t> Engine::slots_of(uint32_t s)
{
    const SysParam& P = sys_[s].P;
    std::vector<uint32_t> r(P.n);
    download(rid_, P.off, P.n, r.data());
    return r;
}

// positions.lattice (mdsim/host/positions/lattice.cpp:63-175): fcc sites in
// the slab (fraction of each box edge) at the centre of the box, with the
// smallest lattice constant that gives enough sites, the vacancies spread
// evenly; the image counters are zeroed.  Sites are generated on the device.
void Engine::lattice(uint32_t s, const double* slab_in)
{
    check_sys(s);
    const SysHost& h = sys_[s];
    const uint32_t n = h.P.n;
    double slab[3] = {1.0, 1.0, 1.0};
    if (slab_in)
        for (int q = 0; q < 3; ++q) slab[q] = slab_in[q];
    for (int q = 0; q < 3; ++q)   // lattice.cpp:52-57
        if (!(slab[q] > 0 && slab[q] <= 1)) throw Error(HMD_ERR_STATE, "slab extents must be a fraction between 0 and 1");
    double length[3], offset[3];
    for (int q = 0; q < 3; ++q) {
        length[q] = h.desc.box[q] * slab[q];
        offset[q] = -length[q] / 2;
    }
    // lattice.cpp:124-146: the smallest lattice distance a with
    // 4 prod floor(L_i / a) >= n, growing the cell counts from the cube root
    const double u = 4;
    double a = std::pow(length[0] * length[1] * length[2] / std::ceil(n / u), 1.0 / 3);
    uint32_t c[3];
    for (int q = 0; q < 3; ++q) c[q] = (uint32_t)(length[q] / a);
    while ((double)n > u * (double)c[0] * c[1] * c[2]) {
        double t = 0;
        for (int q = 0; q < 3; ++q) t = std::max(t, length[q] / (c[q] + 1));
        a = t;
        bool same = true;
        for (int q = 0; q < 3; ++q) {
            const uint32_t m = std::max(c[q], (uint32_t)(length[q] / a));
            same = same && m == c[q];
            c[q] = m;
        }
        if (same)
            for (int q = 0; q < 3; ++q) c[q] += 1;
    }
    const uint64_t N = 4ull * c[0] * c[1] * c[2];
    // lattice.cpp:150-165: a vacancy every `skip` sites
    const uint32_t skip = (N > n) ? (uint32_t)std::ceil((double)N / (double)(N - n)) : 0u;
    HMD_CUDA(cudaMemsetAsync(img_.p + h.P.off, 0, h.P.A * sizeof(float4), stream_));
    stage(3 * (size_t)n);
    launch_lattice(io_.p, n, c, a, offset, skip, stream_);
    launch_set_vector(dev(), s, n, 0, ds(), io_.p, stream_);
    HMD_CUDA(cudaGetLastError());
    sync();
    forces_valid_ = false;
    request_rebuild(s);
}

// velocities.boltzmann set() (mdsim/gpu/velocities/boltzmann.cpp): each
// component N(0, sqrt(T)) / sqrt(m), then the centre-of-mass velocity
// removed; drawn on the device from a Philox stream keyed by (seed, tag)
void Engine::boltzmann(uint32_t s, double temperature, uint64_t seed)
{
    check_sys(s);
    if (!(temperature >= 0)) throw Error(HMD_ERR_INVALID, "temperature must be non-negative");
    const uint32_t n = sys_[s].P.n;
    const size_t blocks = (n + 255) / 256;
    stage(3 * (size_t)n + 4 * blocks + 3);
    launch_boltzmann(dev(), s, n, temperature, seed, io_.p, io_.p + 3 * (size_t)n, stream_);
    launch_set_vector(dev(), s, n, 1, ds(), io_.p, stream_);
    HMD_CUDA(cudaGetLastError());
    sync();
}

// staging buffer of the device-side set / get conversions (grows on demand)
void Engine::stage(size_t doubles)
{
    if (io_.n < doubles) io_.alloc(doubles);
}

void Engine::set(uint32_t s, const std::string& name, const void* host, size_t count)
{
    check_sys(s);
    const SysParam& P = sys_[s].P;
    const uint32_t n = P.n;
    auto need = [&](size_t k) {
        if (count != k) throw Error(HMD_ERR_INVALID, "array '" + name + "' needs " + std::to_string(k) + " elements");
    };
    if (name == "position" || name == "velocity") {
        // one copy into the staging buffer, then the conversion on the device
        need(3 * (size_t)n);
        const double* x = static_cast<const double*>(host);
        stage(3 * (size_t)n);
        HMD_CUDA(cudaMemcpyAsync(io_.p, x, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, stream_));
        if (name == "position") {
            // checked on the device copy, before anything is stored
            launch_check_finite(io_.p, 3 * (size_t)n, done_.p + 1, stream_);
            uint32_t bad = 0;
            download(done_, 1, 1, &bad);
            if (bad) throw Error(HMD_ERR_INVALID, "positions must be finite");
        }
        launch_set_vector(dev(), s, n, name == "position" ? 0 : 1, ds(), io_.p, stream_);
        HMD_CUDA(cudaGetLastError());
        sync();
        if (name == "position") {
            forces_valid_ = false;
            request_rebuild(s);
        }
        return;
    }
    std::vector<uint32_t> slot = slots_of(s);
    if (name == "mass") {
        need(n);
        const double* x = static_cast<const double*>(host);
        std::vector<float4> hi(P.A);
        download(vel_, P.off, P.A, hi.data());
        for (uint32_t t = 0; t < n; ++t) {
            if (!(x[t] > 0)) throw Error(HMD_ERR_INVALID, "mass must be positive");
            hi[slot[t] - P.off].w = (float)x[t];
        }
        upload(vel_, P.off, P.A, hi.data());
    } else if (name == "species") {
        need(n);
        const uint32_t* x = static_cast<const uint32_t*>(host);
        std::vector<float4> hi(P.A);
        download_pos(false, P.off, P.A, hi.data());
        for (uint32_t t = 0; t < n; ++t) {
            if (x[t] >= P.ns) throw Error(HMD_ERR_INVALID, "species out of range");
            hi[slot[t] - P.off].w = f32_from_bits(x[t]);
        }
        upload_pos(false, P.off, P.A, hi.data());
        forces_valid_ = false;
        request_rebuild(s);
    } else if (name == "image") {
        need(3 * (size_t)n);
        const double* x = static_cast<const double*>(host);
        std::vector<float4> im(P.A);
        download(img_, P.off, P.A, im.data());
        for (uint32_t t = 0; t < n; ++t) {
            float* g = &im[slot[t] - P.off].x;
            for (int q = 0; q < 3; ++q) g[q] = (float)x[3 * t + q];
        }
        upload(img_, P.off, P.A, im.data());
    } else {
        throw Error(HMD_ERR_INVALID, "unknown or read-only array '" + name + "'");
    }
}

void Engine::get(uint32_t s, const std::string& name, void* host, size_t count)
{
    check_sys(s);
    const SysParam& P = sys_[s].P;
    const uint32_t n = P.n;
    const size_t S = S_;
    auto need = [&](size_t k) {
        if (count != k) throw Error(HMD_ERR_INVALID, "array '" + name + "' needs " + std::to_string(k) + " elements");
    };
    static const char* const vec_names[] = {"position", "unwrapped_position", "velocity", "force", "image"};
    for (int w = 0; w < 5; ++w) {
        if (name != vec_names[w]) continue;
        need(3 * (size_t)n);
        stage(3 * (size_t)n);
        launch_get_vector(dev(), s, n, w, io_.p, stream_);
        HMD_CUDA(cudaGetLastError());
        HMD_CUDA(cudaMemcpyAsync(host, io_.p, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
        sync();
        return;
    }
    if (name == "id") {
        need(P.A);
        download(id_, P.off, P.A, static_cast<uint32_t*>(host));
        return;
    }
    std::vector<uint32_t> slot = slots_of(s);
    if (name == "reverse_id") {
        need(n);
        uint32_t* o = static_cast<uint32_t*>(host);
        for (uint32_t t = 0; t < n; ++t) o[t] = slot[t] - P.off;
    } else if (name == "position" || name == "unwrapped_position") {
        need(3 * (size_t)n);
        std::vector<float4> hi(P.A), lo(P.A), im(P.A);
        download_pos(false, P.off, P.A, hi.data());
        download_pos(true, P.off, P.A, lo.data());
        download(img_, P.off, P.A, im.data());
        double* o = static_cast<double*>(host);
        const bool unwrap = name == "unwrapped_position";
        for (uint32_t t = 0; t < n; ++t) {
            const uint32_t k = slot[t] - P.off;
            const float* h = &hi[k].x;
            const float* l = &lo[k].x;
            const float* g = &im[k].x;
            for (int q = 0; q < 3; ++q)
                o[3 * t + q] = (double)h[q] + (double)l[q] + (unwrap ? (double)g[q] * (double)P.L[q] : 0.0);
        }
    } else if (name == "velocity") {
        need(3 * (size_t)n);
        std::vector<float4> hi(P.A), lo(P.A);
        download(vel_, P.off, P.A, hi.data());
        download(vel_, S + P.off, P.A, lo.data());
        double* o = static_cast<double*>(host);
        for (uint32_t t = 0; t < n; ++t) {
            const uint32_t k = slot[t] - P.off;
            const float* h = &hi[k].x;
            const float* l = &lo[k].x;
            for (int q = 0; q < 3; ++q) o[3 * t + q] = (double)h[q] + (double)l[q];
        }
    } else if (name == "mass" || name == "species") {
        need(n);
        std::vector<float4> b(P.A);
        if (name == "mass") download(vel_, P.off, P.A, b.data());
        else download_pos(false, P.off, P.A, b.data());
        for (uint32_t t = 0; t < n; ++t) {
            const float w = b[slot[t] - P.off].w;
            if (name == "mass") static_cast<double*>(host)[t] = w;
            else static_cast<uint32_t*>(host)[t] = bits_of(w);
        }
    } else if (name == "image" || name == "force") {
        need(3 * (size_t)n);
        std::vector<float4> b(P.A);
        download(name == "image" ? img_ : force_, P.off, P.A, b.data());
        double* o = static_cast<double*>(host);
        for (uint32_t t = 0; t < n; ++t) {
            const float* g = &b[slot[t] - P.off].x;
            for (int q = 0; q < 3; ++q) o[3 * t + q] = g[q];
        }
    } else if (name == "potential_energy") {
        need(n);
        std::vector<float> b(P.A);
        download(en_pot_, P.off, P.A, b.data());
        double* o = static_cast<double*>(host);
        for (uint32_t t = 0; t < n; ++t) o[t] = b[slot[t] - P.off];
    } else if (name == "stress_pot") {
        need(6 * (size_t)n);
        double* o = static_cast<double*>(host);
        std::vector<float> b(P.A);
        for (int c = 0; c < 6; ++c) {
            download(stress_, (size_t)c * S + P.off, P.A, b.data());
            for (uint32_t t = 0; t < n; ++t) o[6 * t + c] = b[slot[t] - P.off];
        }
    } else {
        throw Error(HMD_ERR_INVALID, "unknown array '" + name + "'");
    }
}

void Engine::get_raw(uint32_t s, const std::string& name, void* host, size_t bytes)
{
    check_sys(s);
    const SysParam& P = sys_[s].P;
    const size_t S = S_;
    auto need = [&](size_t b) {
        if (bytes != b) throw Error(HMD_ERR_INVALID, "raw array '" + name + "' has " + std::to_string(b) + " bytes");
    };
    if (name == "cells") {
        need((size_t)P.ncells * P.cell_size * 4);
        uint32_t* o = static_cast<uint32_t*>(host);
        download(cell_, P.cell_word_off, (size_t)P.ncells * P.cell_size, o);
        for (size_t k = 0; k < (size_t)P.ncells * P.cell_size; ++k)
            if (o[k] != PLACEHOLDER) o[k] -= P.off;
        return;
    }
    need((size_t)P.A * 16);
    float4* o = static_cast<float4*>(host);
    if (name == "position_hi") download_pos(false, P.off, P.A, o);
    else if (name == "position_lo") download_pos(true, P.off, P.A, o);
    else if (name == "velocity_hi") download(vel_, P.off, P.A, o);
    else if (name == "velocity_lo") download(vel_, S + P.off, P.A, o);
    else if (name == "image") download(img_, P.off, P.A, o);
    else if (name == "force") download(force_, P.off, P.A, o);
    else if (name == "r0") download(r0_, P.off, P.A, o);
    else throw Error(HMD_ERR_INVALID, "unknown raw array '" + name + "'");
}

void Engine::info(uint32_t s, hmd_system_info* out)
{
    check_sys(s);
    const SysHost& h = sys_[s];
    std::vector<SysState> st = read_state();
    std::memset(out, 0, sizeof(*out));
    out->nparticle = h.P.n;
    out->nspecies = h.P.ns;
    out->slot_offset = h.P.off;
    out->slots = h.P.A;
    for (int q = 0; q < 3; ++q) { out->ncell[q] = h.P.ncell[q]; out->box_f32[q] = h.P.L[q]; }
    out->cell_size = h.P.cell_size;
    out->neighbour_capacity = nbr_cap_;
    out->hilbert_depth = h.P.depth;
    out->max_neighbours = st[s].max_nbr;
    out->max_cell_occupancy = st[s].max_cell;
    out->step = st[s].step;
    out->rebuilds = st[s].rebuilds;
    out->sort_key_bits = key_bits_;
    out->rebuild_kernels = rebuild_kernel_count();
    for (size_t ab = 0; ab < h.pairs.size(); ++ab) {
        out->rr_cut_skin[ab] = h.pairs[ab].rr_cut_skin;
        out->rr_cut[ab] = h.pairs[ab].rr_cut;
    }
}

void Engine::request_rebuild(uint32_t s)
{
    check_sys(s);
    std::vector<SysState> st = read_state();
    st[s].rebuild_request = 1u;
    write_state(st);
    forces_valid_ = false;
}

// list block width: the option when it fits the lane count (1 lane: 4;
// 8 lanes: 8; 2 or 4 lanes: 4 or 8), else the default for the lanes
uint32_t Engine::block() const
{
    const uint32_t w = lanes_ ? lanes_ : 4u;
    if (lb_ == 8u && (w == 2u || w == 4u)) return 8u;
    if (lb_ == 4u && w <= 4u) return 4u;
    return list_block(w);
}

void Engine::set_option(const std::string& name, int64_t value)
{
    if (name == "force_lanes") {
        if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
            throw Error(HMD_ERR_INVALID, "force_lanes must be 0 (auto), 1, 2, 4 or 8");
        if (!committed_) {
            lanes_ = (uint32_t)value;
            return;
        }
        const uint32_t w = value == 0 ? 4u : (uint32_t)value;
        if (w == lanes_) return;
        lanes_ = w;   // the list layout changes: rebuild every list before the next force
        destroy_graphs();
        std::vector<SysState> st = read_state();
        for (auto& t : st) t.rebuild_request = 1u;
        write_state(st);
        forces_valid_ = false;
        return;
    }
    if (name == "list_block") {
        if (value != 0 && value != 4 && value != 8) throw Error(HMD_ERR_INVALID, "list_block must be 0 (auto), 4 or 8");
        if ((uint32_t)value == lb_) return;
        lb_ = (uint32_t)value;
        if (committed_) {   // the list layout changes: rebuild every list before the next force
            destroy_graphs();
            std::vector<SysState> st = read_state();
            for (auto& t : st) t.rebuild_request = 1u;
            write_state(st);
            forces_valid_ = false;
        }
        return;
    }
    if (name == "float_cutoff") {
        // FP64 variant: take the pair set of the float list criterion (the
        // other engines' cut-off test) instead of r^2 < r_c^2 in double
        float_cutoff_ = value != 0;
        if (committed_) destroy_graphs();
        forces_valid_ = false;
        return;
    }
    if (name == "fuse_steps") {
        const bool f = value != 0;
        if (f == fuse_) return;
        fuse_ = f;
        if (committed_) destroy_graphs();
        return;
    }
    if (name == "neighbour_scan") {
        if (value < 0 || value > 2)
            throw Error(HMD_ERR_INVALID, "neighbour_scan must be 0 (auto), 1 (per lane) or 2 (shared per warp)");
        if (nbr_scan_ == (uint32_t)value) return;
        nbr_scan_ = (uint32_t)value;
        if (committed_) destroy_graphs();   // captured launches carry the old setting
        return;
    }
    throw Error(HMD_ERR_INVALID, "unknown option '" + name + "'");
}

int64_t Engine::get_option(const std::string& name) const
{
    if (name == "force_lanes") return lanes_;
    if (name == "list_block") return block();
    if (name == "neighbour_scan") return nbr_scan_;
    if (name == "step_kernels") return (int64_t)step_kernels_;
    if (name == "fuse_steps") return fuse_ ? 1 : 0;
    if (name == "float_cutoff") return float_cutoff_ ? 1 : 0;
    if (name == "neighbour_capacity") return nbr_cap_;
    if (name == "rebuild_chains") {
        uint32_t v[2];
        const_cast<Engine*>(this)->download(any_rebuild_, 0, 2, v);
        return v[1];
    }
    throw Error(HMD_ERR_INVALID, "unknown option '" + name + "'");
}

void Engine::set_steps_left(uint32_t s, uint32_t steps)
{
    check_sys(s);
    std::vector<SysState> st = read_state();
    st[s].steps_left = steps;
    write_state(st);
}

// Steepest-descent minimisation of one system's potential energy (set-up
// of a start configuration from random positions; no counterpart in the
// reference).  The system runs `steps` steps of the captured step graph
// with its integrator switched to INTEG_DESCENT; the other systems are held
// (steps_left = 0) meanwhile.  Velocities are not touched; the step counter
// is restored afterwards, so minimisation does not count as MD time.
void Engine::minimize(uint32_t s, uint32_t steps, double step_size, double max_move)
{
    check_committed();
    check_sys(s);
    if (!(step_size > 0) || !(max_move > 0) || !std::isfinite(step_size) || !std::isfinite(max_move))
        throw Error(HMD_ERR_INVALID, "minimize: step_size and max_move must be positive");
    if (steps == 0) return;
    if (steps == 0xFFFFFFFFu) throw Error(HMD_ERR_INVALID, "minimize: too many steps");
    SysHost& h = sys_[s];
    const SysParam saved = h.P;
    const std::vector<SysState> before = read_state();
    std::vector<SysState> st = before;
    for (uint32_t q = 0; q < (uint32_t)st.size(); ++q) st[q].steps_left = (q == s) ? steps : 0u;
    write_state(st);
    h.P.integrator = INTEG_DESCENT;
    h.P.descent_step = (float)step_size;
    h.P.descent_max = (float)max_move;
    upload_system(s);
    auto put_back = [&] {
        std::vector<SysState> now = read_state();
        for (uint32_t q = 0; q < (uint32_t)now.size(); ++q) now[q].steps_left = before[q].steps_left;
        now[s].step = before[s].step;
        write_state(now);
        h.P = saved;
        upload_system(s);
    };
    try {
        step(steps, false);
    } catch (...) {
        put_back();
        throw;
    }
    put_back();
}

// ---- the step --------------------------------------------------------------

void Engine::rebuild_chain(cudaStream_t st)
{
    const Dev d = dev();
    launch_rebuild_list(d, st);
    if (any_sort_) {
        launch_sort(d, sort_passes_, st);
        launch_rearrange(d, ds(), d.val[sort_passes_ & 1], st);   // pass p writes val[1 - p % 2]
    }
    launch_binning(d, st);
    launch_neighbour(d, st);
}

void Engine::ensure_forces(bool aux)
{
    if (forces_valid_ && (!aux || aux_valid_)) return;
    const Dev d = dev();
    launch_mark(d, false, stream_);
    rebuild_chain(stream_);
    launch_pack_fpos(d, stream_);
    launch_force(d, aux, stream_);
    HMD_CUDA(cudaGetLastError());
    uint32_t status = 0;
    download(status_, 0, 1, &status);
    if (status != 0) {
        if (!grow_after_overflow(status)) throw Error(HMD_ERR_OVERFLOW, "capacity overflow in the initial list build");
        HMD_CUDA(cudaMemsetAsync(status_.p, 0, 4, stream_));
        std::vector<SysState> st = read_state();
        for (auto& t : st) t.rebuild_request = 1u;
        write_state(st);
        forces_valid_ = false;
        ensure_forces(aux);
        return;
    }
    forces_valid_ = true;
    aux_valid_ = aux;
    integrated_ = false;
}

cudaGraphExec_t Engine::capture(int nsteps, bool aux_last)
{
    const Dev d = dev();
    cudaGraph_t g;
    HMD_CUDA(cudaGraphCreate(&g, 0));
    HMD_CUDA(cudaStreamBeginCaptureToGraph(stream_, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    try {
        // step k: [integrate k] -> IF(rebuild k) -> force k -> [finalize k + integrate k+1];
        // the fused kernel sets the conditional of step k+1, so the handles exist up front
        std::vector<cudaGraphConditionalHandle> hs(nsteps);
        for (int k = 0; k < nsteps; ++k)
            HMD_CUDA(cudaGraphConditionalHandleCreate(&hs[k], g, 0, cudaGraphCondAssignDefault));
        launch_integrate_prepare(d, stream_);
        launch_integrate(d, ds(), hs[0], true, stream_);
        for (int k = 0; k < nsteps; ++k) {
            const cudaGraphConditionalHandle h = hs[k];
            cudaStreamCaptureStatus cs;
            cudaGraph_t cg;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            HMD_CUDA(cudaStreamGetCaptureInfo(stream_, &cs, nullptr, &cg, &deps, nullptr, &nd));
            cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            cudaGraphNode_t cn;
            HMD_CUDA(cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            HMD_CUDA(cudaStreamUpdateCaptureDependencies(stream_, &cn, nullptr, 1, cudaStreamSetCaptureDependencies));
            HMD_CUDA(cudaStreamBeginCaptureToGraph(side_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            rebuild_chain(side_);
            cudaGraph_t body_out;
            HMD_CUDA(cudaStreamEndCapture(side_, &body_out));
            launch_force(d, aux_last && k == nsteps - 1, stream_);
            if (k + 1 < nsteps && fused()) {
                launch_finalize_integrate(d, ds(), hs[k + 1], stream_);
            } else {
                launch_finalize(d, ds(), stream_);
                if (k + 1 < nsteps) {
                    launch_integrate_prepare(d, stream_);
                    launch_integrate(d, ds(), hs[k + 1], true, stream_);
                }
            }
        }
    } catch (...) {
        cudaGraph_t tmp;
        cudaStreamEndCapture(stream_, &tmp);
        cudaGraphDestroy(g);
        throw;
    }
    cudaGraph_t out;
    HMD_CUDA(cudaStreamEndCapture(stream_, &out));
    cudaGraphExec_t exec;
    HMD_CUDA(cudaGraphInstantiate(&exec, out, 0));
    HMD_CUDA(cudaGraphDestroy(out));
    return exec;
}

void Engine::destroy_graphs()
{
    if (g_chunk_) cudaGraphExecDestroy(g_chunk_);
    if (g_short_) cudaGraphExecDestroy(g_short_);
    if (g_one_) cudaGraphExecDestroy(g_one_);
    if (g_one_aux_) cudaGraphExecDestroy(g_one_aux_);
    g_chunk_ = g_short_ = g_one_ = g_one_aux_ = nullptr;
}

void Engine::build_graphs()
{
    destroy_graphs();
    g_chunk_ = capture(CHUNK_STEPS, false);
    g_short_ = capture(SHORT_STEPS, false);
    g_one_ = capture(1, false);
    g_one_aux_ = capture(1, true);
}

void Engine::snapshot()
{
    const size_t S = S_;
    if (!snap_pos_.p) {
        snap_pos_.alloc(2 * S); snap_vel_.alloc(2 * S); snap_img_.alloc(S); snap_force_.alloc(S);
        snap_id_.alloc(S); snap_rid_.alloc(S); snap_st_.alloc(table_size_);
    }
    HMD_CUDA(cudaMemcpyAsync(snap_pos_.p, pos_.p, pos_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(snap_vel_.p, vel_.p, vel_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(snap_img_.p, img_.p, img_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(snap_force_.p, force_.p, force_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    if (fp64()) {
        if (!snap_force64_.p) snap_force64_.alloc(S_);
        HMD_CUDA(cudaMemcpyAsync(snap_force64_.p, force64_.p, force64_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    }
    HMD_CUDA(cudaMemcpyAsync(snap_id_.p, id_.p, id_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(snap_rid_.p, rid_.p, rid_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(snap_st_.p, dst_.p, dst_.bytes(), cudaMemcpyDeviceToDevice, stream_));
}

void Engine::restore()
{
    HMD_CUDA(cudaMemcpyAsync(pos_.p, snap_pos_.p, pos_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(vel_.p, snap_vel_.p, vel_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(img_.p, snap_img_.p, img_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(force_.p, snap_force_.p, force_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    if (fp64())
        HMD_CUDA(cudaMemcpyAsync(force64_.p, snap_force64_.p, force64_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(id_.p, snap_id_.p, id_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(rid_.p, snap_rid_.p, rid_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemcpyAsync(dst_.p, snap_st_.p, dst_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    HMD_CUDA(cudaMemsetAsync(status_.p, 0, 4, stream_));
    HMD_CUDA(cudaMemsetAsync(done_.p, 0, 4, stream_));
    sync();
}

// grow cell or list capacity from the occupancies the failed build recorded
bool Engine::grow_after_overflow(uint32_t status)
{
    std::vector<SysState> st = read_state();
    bool changed = false;
    if (status & ST_CELL_OVERFLOW) {
        if (!capacity_) {
            uint32_t words = 0;
            for (uint32_t s = 0; s < table_size_; ++s) {
                SysParam& P = sys_[s].P;
                if (st[s].max_cell > P.cell_size) {
                    const uint32_t want = round_up((uint32_t)std::ceil(st[s].max_cell * 1.25), 32);
                    if (want > 256 || want <= P.cell_size) return false;
                    P.cell_size = want;
                    changed = true;
                }
                P.cell_word_off = words;
                words += P.ncells * P.cell_size;
            }
            cell_.alloc(std::max<uint32_t>(words, 1));
            upload_tables();
        } else {
            // move each crowded system's cell contents to a larger word range
            for (uint32_t s = 0; s < table_size_; ++s) {
                SysParam& P = sys_[s].P;
                if (!sys_[s].used || st[s].max_cell <= P.cell_size) continue;
                const uint32_t want = round_up((uint32_t)std::ceil(st[s].max_cell * 1.25), 32);
                if (want > 256 || want <= P.cell_size) return false;
                word_arena_.release(P.cell_word_off / 32, P.ncells * P.cell_size / 32);
                uint32_t at;
                if (!word_arena_.alloc(P.ncells * want / 32, at)) {
                    word_arena_.alloc(P.ncells * P.cell_size / 32, at);   // the range just freed
                    P.cell_word_off = at * 32;
                    return false;
                }
                P.cell_size = want;
                P.cell_word_off = at * 32;
                upload_system(s);
                changed = true;
            }
        }
    }
    if (status & ST_NBR_OVERFLOW) {
        uint32_t m = 0;
        for (auto& t : st) m = std::max(m, t.max_nbr);
        const uint32_t want = round_up((uint32_t)std::ceil(m * 1.2) + 8, 8);
        if (want <= nbr_cap_) return false;
        nbr_cap_ = want;
        nbr_.alloc((size_t)nbr_cap_ * S_);
        changed = true;
    }
    for (auto& t : st) { t.max_cell = 0; t.max_nbr = 0; }
    write_state(st);
    if (changed) destroy_graphs();
    return changed;
}

// captured chunks fuse the finalize of step k with the integrate of step
// k + 1 unless a thermostat runs between them (Nose-Hoover, Maxwell-Boltzmann)
bool Engine::fused() const
{
    return fuse_ && !(integ_kinds_ & ((1u << INTEG_HOOVER) | (1u << INTEG_BOLTZMANN)));
}

// step kernels of a captured chunk of n steps (rebuild chains not included):
// fused, integrate + n force launches + (n - 1) fused finalize + integrate +
// finalize; otherwise n times the kernels of one step
uint64_t Engine::chunk_kernels(int n) const
{
    const Dev d = dev();
    if (fused()) {
        const int nforce = d.force_kinds ? __builtin_popcount(d.force_kinds) : 1;
        return (uint64_t)n * (nforce + 1) + 1;
    }
    return (uint64_t)n * step_kernel_count(d);
}

void Engine::run_steps(uint64_t nsteps, bool aux_last)
{
    if (!g_chunk_) build_graphs();
    // a captured chunk of n steps launches 2n + 1 step kernels (integrate, n
    // forces, n - 1 fused finalize + integrate, finalize), plus the
    // conditional rebuild chains
    uint64_t left = nsteps;
    while (left > 0) {
        if (left >= (uint64_t)CHUNK_STEPS && !(aux_last && left == (uint64_t)CHUNK_STEPS)) {
            HMD_CUDA(cudaGraphLaunch(g_chunk_, stream_));
            left -= CHUNK_STEPS;
            step_kernels_ += chunk_kernels(CHUNK_STEPS);
        } else if (left >= (uint64_t)SHORT_STEPS && !(aux_last && left == (uint64_t)SHORT_STEPS)) {
            HMD_CUDA(cudaGraphLaunch(g_short_, stream_));
            left -= SHORT_STEPS;
            step_kernels_ += chunk_kernels(SHORT_STEPS);
        } else if (left == 1 && aux_last) {
            HMD_CUDA(cudaGraphLaunch(g_one_aux_, stream_));
            left -= 1;
            step_kernels_ += chunk_kernels(1);
        } else {
            HMD_CUDA(cudaGraphLaunch(g_one_, stream_));
            left -= 1;
            step_kernels_ += chunk_kernels(1);
        }
    }
}

void Engine::step(uint64_t nsteps, bool aux_last)
{
    check_committed();
    if (nsteps == 0) return;
    ensure_forces(false);
    uint64_t left = nsteps;
    while (left > 0) {
        const uint64_t seg = std::min(left, SEGMENT_STEPS);
        const bool aux = aux_last && seg == left;
        snapshot();
        int tries = 0;
        for (;;) {
            run_steps(seg, aux);
            uint32_t status = 0;
            download(status_, 0, 1, &status);
            if (status == 0) break;
            if (++tries > 6 || !grow_after_overflow(status))
                throw Error(HMD_ERR_OVERFLOW, "neighbour or cell capacity overflow could not be resolved");
            restore();
            std::vector<SysState> st = read_state();
            for (auto& t : st) t.rebuild_request = 1u;
            write_state(st);
        }
        left -= seg;
    }
    aux_valid_ = aux_last;
    forces_valid_ = true;
    integrated_ = false;
}

void Engine::tic()
{
    if (!profile_) return;
    HMD_CUDA(cudaEventRecord(ev0_, stream_));
}

void Engine::toc(const char* phase)
{
    if (!profile_) return;
    HMD_CUDA(cudaEventRecord(ev1_, stream_));
    HMD_CUDA(cudaEventSynchronize(ev1_));
    float ms = 0;
    HMD_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
    for (auto& t : timers_)
        if (t.first == phase) { t.second.ms += ms; t.second.count += 1; return; }
    timers_.push_back({phase, Timer{ms, 1}});
}

void Engine::profile_enable(bool on)
{
    if (on && !ev0_) {
        HMD_CUDA(cudaEventCreate(&ev0_));
        HMD_CUDA(cudaEventCreate(&ev1_));
    }
    profile_ = on;
    if (on) timers_.clear();
}

void Engine::profile_get(const std::string& phase, double* total_ms, uint64_t* count)
{
    *total_ms = 0;
    *count = 0;
    for (auto& t : timers_)
        if (t.first == phase) { *total_ms = t.second.ms; *count = t.second.count; }
}

uint32_t Engine::rebuild_kernel_count() const
{
    // rebuild list; sort keys + (hist, scan, scatter) per pass + rearrange + copy back; cell clear, bin,
    // sort; list build
    return 1u + (any_sort_ ? (uint32_t)sort_kernel_count(sort_passes_) + 2u : 0u) + 3u + 1u;
}

void Engine::integrate()
{
    check_committed();
    ensure_forces(false);
    tic();
    launch_integrate_prepare(dev(), stream_);
    launch_integrate(dev(), ds(), 0, false, stream_);
    HMD_CUDA(cudaGetLastError());
    toc("integrate");
    integrated_ = true;
    forces_valid_ = false;
}

// pair_trunc::apply (forces/pair_trunc.hpp:192-216): always evaluates; the
// lists are rebuilt first where a step flagged it or a rebuild is pending
void Engine::force(bool aux)
{
    check_committed();
    const Dev d = dev();
    bool need = true;
    if (!integrated_) {
        launch_mark(d, false, stream_);
    } else {
        // the integrate kernel's last block decided on the device; one word
        // comes back (the reference reads its displacement maxima every step,
        // max_displacement.cpp:96)
        uint32_t any = 0;
        download(any_rebuild_, 0, 1, &any);
        need = any != 0;
    }
    if (need) {
        tic();
        rebuild_chain(stream_);
        toc("rebuild");
    }
    tic();
    launch_pack_fpos(d, stream_);
    launch_force(d, aux, stream_);
    HMD_CUDA(cudaGetLastError());
    toc(aux ? "force_aux" : "force");
    uint32_t status = 0;
    download(status_, 0, 1, &status);
    // A cell overflow also hides list lengths (the lists were built from
    // truncated cells), so capacities can grow in stages: rebuild until the
    // build fits.  Each round grows a capacity strictly (cells up to 256
    // slots, lists until an allocation fails) or gives up, so this ends.
    while (status != 0) {
        if (!grow_after_overflow(status)) throw Error(HMD_ERR_OVERFLOW, "capacity overflow in list rebuild");
        HMD_CUDA(cudaMemsetAsync(status_.p, 0, 4, stream_));
        const Dev d2 = dev();
        launch_mark(d2, true, stream_);
        rebuild_chain(stream_);
        launch_pack_fpos(d2, stream_);
        launch_force(d2, aux, stream_);
        download(status_, 0, 1, &status);
    }
    forces_valid_ = true;
    aux_valid_ = aux;
    integrated_ = false;
}

void Engine::finalize()
{
    check_committed();
    tic();
    launch_finalize(dev(), ds(), stream_);
    HMD_CUDA(cudaGetLastError());
    toc("finalize");
    sync();
}

// verlet_nvt_hoover.cpp:134-140 (en_nhc per particle) and the chain state;
// the last Maxwell-Boltzmann draw's centre-of-mass velocity
void Engine::integrator_state(uint32_t s, double* out)
{
    check_sys(s);
    sync();
    const SysState t = read_state()[s];
    const SysParam& P = sys_[s].P;
    for (int k = 0; k < 8; ++k) out[k] = 0.0;
    if (P.integrator == INTEG_HOOVER) {
        const double dof = 3.0 * P.n;
        double en = P.nhc_T * (dof * t.xi[0] + t.xi[1]);
        for (int k = 0; k < 2; ++k) en += P.nhc_mass[k] * t.v_xi[k] * t.v_xi[k] / 2;
        out[0] = t.xi[0]; out[1] = t.xi[1];
        out[2] = t.v_xi[0]; out[3] = t.v_xi[1];
        out[4] = en / P.n;
    } else if (P.integrator == INTEG_BOLTZMANN) {
        out[5] = t.vcm[0]; out[6] = t.vcm[1]; out[7] = t.vcm[2];
    }
}

double Engine::max_displacement(uint32_t s)
{
    check_sys(s);
    const SysParam& P = sys_[s].P;
    // on the device (k_max_displacement); the done_ word 1 is free outside
    // launch_check_finite, which the host reads before it returns
    launch_max_displacement(dev(), s, P.A, done_.p + 1, stream_);
    HMD_CUDA(cudaGetLastError());
    uint32_t bits = 0;
    download(done_, 1, 1, &bits);
    float m;
    std::memcpy(&m, &bits, sizeof(m));
    return std::sqrt((double)m);
}

void Engine::thermo(uint32_t s, double* out)
{
    check_sys(s);
    launch_thermo(dev(), stream_);
    HMD_CUDA(cudaGetLastError());
    download(thermo_, (size_t)s * NTHERMO, NTHERMO, out);
}

void Engine::neighbour_lists(uint32_t s, uint32_t* counts, uint32_t* lists, uint32_t maxn)
{
    check_sys(s);
    if (sys_[s].P.trunc == TRUNC_NONE)
        throw Error(HMD_ERR_STATE, "an untruncated potential (pair_full) has no neighbour list");
    ensure_forces(false);
    const SysParam& P = sys_[s].P;
    std::vector<uint32_t> slot = slots_of(s);
    std::vector<uint32_t> cnt(P.A), id(P.A);
    download(nbr_count_, P.off, P.A, cnt.data());
    download(id_, P.off, P.A, id.data());
    // counts are packed (near | far << 16): near entries from the front of a
    // list, far entries from its back
    for (uint32_t t = 0; t < P.n; ++t) {
        const uint32_t k = slot[t] - P.off;
        if ((cnt[k] & 0xFFFFu) + (cnt[k] >> 16) > maxn) throw Error(HMD_ERR_INVALID, "maxn smaller than a neighbour count");
    }
    // blocked layout: block b holds entries [b*W, b*W + W) of every slot
    const uint32_t W = block();
    const uint32_t nblk = nbr_cap_ / W;
    std::vector<uint32_t> all((size_t)nbr_cap_ * P.A);
    for (uint32_t b = 0; b < nblk; ++b)
        download(nbr_, ((size_t)b * S_ + P.off) * W, (size_t)P.A * W, all.data() + (size_t)b * P.A * W);
    for (uint32_t t = 0; t < P.n; ++t) {
        const uint32_t k = slot[t] - P.off;
        const uint32_t nn = cnt[k] & 0xFFFFu, nf = cnt[k] >> 16;
        counts[t] = nn + nf;
        std::vector<uint32_t> v(nn + nf);
        for (uint32_t q = 0; q < nn + nf; ++q) {
            const uint32_t e = q < nn ? q : nbr_cap_ - 1u - (q - nn);
            v[q] = id[all[((size_t)(e / W) * P.A + k) * W + e % W] - P.off];
        }
        std::sort(v.begin(), v.end());
        for (uint32_t q = 0; q < maxn; ++q) lists[(size_t)t * maxn + q] = q < counts[t] ? v[q] : PLACEHOLDER;
    }
}

void Engine::hilbert_keys(uint32_t s, uint32_t* keys)
{
    check_sys(s);
    const SysParam& P = sys_[s].P;
    launch_hilbert_keys(dev(), key0_.p, stream_);
    HMD_CUDA(cudaGetLastError());
    std::vector<uint32_t> k(P.A);
    download(key0_, P.off, P.A, k.data());
    std::vector<uint32_t> slot = slots_of(s);
    for (uint32_t t = 0; t < P.n; ++t) keys[t] = k[slot[t] - P.off];
}

} // namespace hmd
