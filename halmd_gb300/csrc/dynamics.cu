// dynamics.cu — blocking scheme, correlation and the MSD / ISF functions.
#include "dynamics.h"
#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <map>

namespace hmd {

// Knuth / Welford update and pairwise merge (numeric/accumulator.hpp:83-119)
void Accum::add(double x)
{
    const double t = x - m;
    n += 1;
    m += t / n;
    v += t * (x - m);
}

void Accum::merge(double n2, double m2, double v2)
{
    if (n2 > 0) {
        const double c = n + n2;
        v += v2;
        const double diff = m - m2;
        v += diff * diff * n * n2 / c;
        m = (n * m + n2 * m2) / c;
        n = c;
    }
}

Dynamics::Dynamics(Engine& e, uint32_t sys, double max_lag_time, double resolution, uint32_t block_size,
                   uint32_t shift, uint32_t separation)
    : e_(e), sys_(sys), block_size_(block_size), separation_(separation)
{
    const SysHost& h = e.system(sys);
    dt_ = h.desc.timestep;
    if (block_size < 2) throw Error(HMD_ERR_INVALID, "Minimum size of coarse-graining blocks is 2.");
    if (shift == 0) throw Error(HMD_ERR_INVALID, "Coarse-graining shift must be non-zero.");
    if (shift >= block_size) throw Error(HMD_ERR_INVALID, "Coarse-graining shift must be less than block size.");
    if (!(resolution > 0)) throw Error(HMD_ERR_INVALID, "Resolution must be a positive value.");
    const uint64_t max_interval = (uint64_t)std::llround(max_lag_time / dt_);
    uint64_t s = (uint64_t)std::llround(resolution / dt_);
    if (s == 0) throw Error(HMD_ERR_INVALID, "Resolution is below the time step.");
    while (s <= max_interval) {
        interval_.push_back(s);
        if (shift > 1) {
            const uint64_t s_odd = s * shift;
            if (s_odd <= max_interval) interval_.push_back(s_odd);
        }
        s *= block_size;
    }
    if (interval_.empty()) throw Error(HMD_ERR_INVALID, "Sampling interval of dynamic correlations is too large.");
    origin_.assign(interval_.size(), current_step());
    blocks_.resize(interval_.size());
}

uint64_t Dynamics::current_step()
{
    hmd_system_info info;
    e_.info(sys_, &info);
    return info.step;
}

void Dynamics::time(double* out) const
{
    for (size_t i = 0; i < interval_.size(); ++i)
        for (uint32_t j = 0; j < block_size_; ++j) out[i * block_size_ + j] = (double)(interval_[i] * j) * dt_;
}

void Dynamics::setup_blocks(Tcf& t, uint32_t begin, uint32_t end, uint32_t chunk)
{
    std::vector<uint32_t> range = {begin, end}, br, bb;
    for (uint32_t k = begin; k < end; k += chunk) {
        br.push_back(0);
        bb.push_back(k);
    }
    t.nblk = (uint32_t)br.size();
    t.range.alloc(2);
    t.blk_range.alloc(std::max<size_t>(1, br.size()));
    t.blk_begin.alloc(std::max<size_t>(1, bb.size()));
    HMD_CUDA(cudaMemcpy(t.range.p, range.data(), 8, cudaMemcpyHostToDevice));
    if (!br.empty()) {
        HMD_CUDA(cudaMemcpy(t.blk_range.p, br.data(), br.size() * 4, cudaMemcpyHostToDevice));
        HMD_CUDA(cudaMemcpy(t.blk_begin.p, bb.data(), bb.size() * 4, cudaMemcpyHostToDevice));
    }
}

// MSD (kind 0), MQD (2) or VACF (3) of the particles with tag in [first, last)
int32_t Dynamics::add_particle_tcf(int kind, uint32_t first, uint32_t last)
{
    if (started_) throw Error(HMD_ERR_STATE, "correlations must be added before the first sample");
    const SysHost& h = e_.system(sys_);
    if (first >= last || last > h.P.n) throw Error(HMD_ERR_INVALID, "bad particle range");
    auto t = std::make_unique<Tcf>();
    t->kind = kind;
    t->first = first;
    t->last = last;
    t->nshell = 1;
    t->res.resize(interval_.size() * block_size_);
    setup_blocks(*t, first, last, 8192);
    t->partial.alloc(3 * std::max<uint32_t>(t->nblk, 1));
    t->out.alloc(3);
    tcf_.push_back(std::move(t));
    return (int32_t)tcf_.size() - 1;
}

static bool coprime3(const uint32_t* h)
{
    auto gcd = [](uint32_t a, uint32_t b) { while (b) { uint32_t t = a % b; a = b; b = t; } return a; };
    return gcd(gcd(h[0], h[1]), h[2]) == 1;
}

int32_t Dynamics::add_isf(const double* wavenumber, uint32_t nk, double tolerance, uint32_t max_count,
                          uint32_t first, uint32_t last, double norm)
{
    if (started_) throw Error(HMD_ERR_STATE, "correlations must be added before the first sample");
    const SysHost& h = e_.system(sys_);
    if (first >= last || last > h.P.n) throw Error(HMD_ERR_INVALID, "bad particle range");
    if (!(norm > 0)) throw Error(HMD_ERR_INVALID, "norm must be positive");
    auto t = std::make_unique<Tcf>();
    t->kind = 1;
    t->first = first;
    t->last = last;
    t->norm = norm;
    // lattice points of the reciprocal lattice on shells |q| ~ k (pick_lattice_points.hpp:74-160)
    double unit[3];
    for (int q = 0; q < 3; ++q) unit[q] = 2 * M_PI / (double)h.P.L[q];
    const double rmax = *std::max_element(wavenumber, wavenumber + nk) * (1 + tolerance);
    uint32_t msum[3];
    for (int q = 0; q < 3; ++q) msum[q] = (uint32_t)(rmax / unit[q]);
    msum[1] += msum[0];
    msum[2] += msum[1];
    std::vector<std::vector<double>> per(nk);
    std::vector<uint32_t> count(nk, 0);
    uint32_t idx[3] = {0, 0, 0};
    while (idx[2] <= msum[2]) {
        const uint32_t hkl[3] = {idx[0], idx[1] - idx[0], idx[2] - idx[1]};
        if (coprime3(hkl)) {
            const double r0[3] = {unit[0] * hkl[0], unit[1] * hkl[1], unit[2] * hkl[2]};
            const double r0n = std::sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
            for (uint32_t i = 0; i < nk; ++i) {
                if (count[i] >= max_count) continue;
                const uint32_t m = (uint32_t)std::floor(wavenumber[i] / r0n + 0.5);
                if (m > 0 && std::fabs(m * r0n - wavenumber[i]) <= wavenumber[i] * tolerance) {
                    for (int q = 0; q < 3; ++q) per[i].push_back(m * r0[q]);
                    ++count[i];
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
    std::vector<float4> qs;
    for (uint32_t i = 0; i < nk; ++i) {
        if (per[i].empty()) continue;   // wavevector.cpp:121-127: empty shells are discarded
        t->wavenumber.push_back(wavenumber[i]);
        t->shell.push_back((uint32_t)qs.size());
        for (size_t k = 0; k < per[i].size(); k += 3)
            qs.push_back(make_float4((float)per[i][k], (float)per[i][k + 1], (float)per[i][k + 2], 0.0f));
        t->shell.push_back((uint32_t)qs.size());
    }
    if (qs.empty()) throw Error(HMD_ERR_STATE, "Constraints on wavevectors are incompatible with geometry of simulation box.");
    t->nshell = (uint32_t)t->wavenumber.size();
    t->nq = (uint32_t)qs.size();
    t->q.alloc(qs.size());
    HMD_CUDA(cudaMemcpy(t->q.p, qs.data(), qs.size() * sizeof(float4), cudaMemcpyHostToDevice));
    t->res.resize(interval_.size() * block_size_ * t->nshell);
    setup_blocks(*t, h.P.off + first, h.P.off + last, 2048);
    t->partial.alloc(2 * (size_t)t->nq * std::max<uint32_t>(t->nblk, 1));
    t->out.alloc(2 * (size_t)t->nq);
    int n_isf = 0;
    for (auto& x : tcf_) n_isf += x->kind == 1;
    t->isf = n_isf;
    tcf_.push_back(std::move(t));
    return (int32_t)tcf_.size() - 1;
}

std::shared_ptr<Dynamics::Sample> Dynamics::acquire(uint64_t step)
{
    if (last_ && last_->step == step) return last_;
    auto s = std::make_shared<Sample>();
    s->step = step;
    const Dev d = e_.dev();
    const SysParam& P = e_.system(sys_).P;
    bool need_pos = false, need_vel = false;
    for (auto& t : tcf_) {
        need_pos = need_pos || t->kind == 0 || t->kind == 2;
        need_vel = need_vel || t->kind == 3;
    }
    if (need_pos) {
        s->pos = std::make_shared<PosSample>();
        s->pos->r.alloc(3 * (size_t)P.n);
        launch_sample_position(d, P.off, P.A, s->pos->r.p, e_.stream());
        HMD_CUDA(cudaGetLastError());
    }
    if (need_vel) {
        s->vel = std::make_shared<PosSample>();
        s->vel->r.alloc(3 * (size_t)P.n);
        launch_sample_velocity(d, P.off, P.A, s->vel->r.p, e_.stream());
        HMD_CUDA(cudaGetLastError());
    }
    for (auto& t : tcf_) {
        if (t->kind != 1) continue;
        launch_density_modes(d, t->range.p, 1, t->blk_range.p, t->blk_begin.p, t->nblk, t->q.p, t->nq, t->partial.p,
                             t->out.p, e_.stream());
        HMD_CUDA(cudaGetLastError());
        auto r = std::make_shared<Rho>();
        r->v.resize(2 * (size_t)t->nq);
        HMD_CUDA(cudaMemcpyAsync(r->v.data(), t->out.p, r->v.size() * 8, cudaMemcpyDeviceToHost, e_.stream()));
        s->rho.push_back(r);
    }
    e_.sync();
    last_ = s;
    return s;
}

void Dynamics::sample()
{
    started_ = true;
    const uint64_t step = current_step();
    for (uint32_t i = 0; i < interval_.size(); ++i) {
        if (step >= origin_[i] && (step - origin_[i]) % interval_[i] == 0) {
            blocks_[i].push_back(acquire(step));
            if (blocks_[i].size() == block_size_) process(i);
        }
    }
}

void Dynamics::finalise()
{
    for (uint32_t i = 0; i < interval_.size(); ++i)
        while (!blocks_[i].empty()) process(i);
}

void Dynamics::correlate(Tcf& t, const Sample& a, const Sample& b, Accum* out)
{
    if (t.kind != 1) {
        const bool vel = t.kind == 3;
        launch_tcf(t.kind, vel ? a.vel->r.p : a.pos->r.p, vel ? b.vel->r.p : b.pos->r.p, t.range.p, 1, t.blk_range.p,
                   t.blk_begin.p, t.nblk, t.partial.p, t.out.p, e_.stream());
        HMD_CUDA(cudaGetLastError());
        double r[3];
        HMD_CUDA(cudaMemcpyAsync(r, t.out.p, 24, cudaMemcpyDeviceToHost, e_.stream()));
        e_.sync();
        out[0].merge(r[0], r[1], r[2] * r[0]);
    } else {
        const std::vector<double>& r1 = a.rho[t.isf]->v;
        const std::vector<double>& r2 = b.rho[t.isf]->v;
        for (uint32_t sh = 0; sh < t.nshell; ++sh) {
            Accum acc;
            for (uint32_t i = t.shell[2 * sh]; i < t.shell[2 * sh + 1]; ++i)
                acc.add((r1[2 * i] * r2[2 * i] + r1[2 * i + 1] * r2[2 * i + 1]) / t.norm);
            out[sh].merge(acc.n, acc.m, acc.v);
        }
    }
}

void Dynamics::process(uint32_t level)
{
    auto& blk = blocks_[level];
    for (auto& t : tcf_) {
        const Sample& first = *blk.front();
        for (size_t j = 0; j < blk.size(); ++j)
            correlate(*t, first, *blk[j], &t->res[((size_t)level * block_size_ + j) * t->nshell]);
    }
    const uint64_t iv = interval_[level];
    const uint64_t skip = std::max<uint64_t>((separation_ + iv - 1) / iv, 1);
    origin_[level] += skip * iv;
    for (uint64_t k = 0; k < skip && !blk.empty(); ++k) blk.pop_front();
}

void Dynamics::result(int32_t k, double* mean, double* error, uint64_t* count) const
{
    if (k < 0 || k >= (int32_t)tcf_.size()) throw Error(HMD_ERR_INVALID, "no such correlation");
    const Tcf& t = *tcf_[k];
    for (size_t i = 0; i < t.res.size(); ++i) {
        const Accum& a = t.res[i];
        if (mean) mean[i] = a.m;
        if (error) error[i] = a.n > 1 ? std::sqrt((a.v / a.n) / (a.n - 1)) : 0.0;
        if (count) count[i] = (uint64_t)a.n;
    }
}

void Dynamics::shells(int32_t k, uint32_t* nshell, double* wavenumber) const
{
    if (k < 0 || k >= (int32_t)tcf_.size()) throw Error(HMD_ERR_INVALID, "no such correlation");
    const Tcf& t = *tcf_[k];
    if (nshell) *nshell = t.nshell;
    if (wavenumber) for (uint32_t s = 0; s < t.wavenumber.size(); ++s) wavenumber[s] = t.wavenumber[s];
}

} // namespace hmd
