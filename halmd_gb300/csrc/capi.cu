// capi.cu — extern "C" entry points of include/halmd_gb300.h.
#include <cstring>
#include <string>

#include "dynamics.h"
#include "engine.h"

using hmd::Engine;
using hmd::Error;

struct hmd_engine {
    Engine* e;
};

static thread_local std::string g_last_error;

template <typename F>
static int guard(hmd_engine* h, F&& f)
{
    try {
        f();
        return HMD_OK;
    } catch (const Error& x) {
        if (h && h->e) h->e->err = x.what();
        g_last_error = x.what();
        return x.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        if (h && h->e) h->e->err = g_last_error;
        return HMD_ERR_NOMEM;
    } catch (const std::exception& x) {
        g_last_error = x.what();
        if (h && h->e) h->e->err = g_last_error;
        return HMD_ERR_STATE;
    }
}

#define ENGINE_OR_FAIL(h)                                                    \
    do {                                                                     \
        if (!(h) || !(h)->e) {                                               \
            g_last_error = "null engine";                                    \
            return HMD_ERR_INVALID;                                          \
        }                                                                    \
    } while (0)

extern "C" {

void hmd_system_desc_init(hmd_system_desc* d)
{
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->nparticle = 0;
    d->nspecies = 1;
    for (int k = 0; k < HMD_MAX_SPECIES * HMD_MAX_SPECIES; ++k) {
        d->epsilon[k] = 1.0;
        d->sigma[k] = 1.0;
        d->r_cut[k] = 2.5;
    }
    d->truncation = HMD_TRUNC_SHIFTED;
    d->smoothing = 0.005;
    d->skin = 0.5;
    d->cell_occupancy = 0.5;
    d->neighbour_occupancy = 0.4;
    d->timestep = 0.001;
    d->integrator = HMD_INTEGRATOR_VERLET;
    d->temperature = 1.0;
    d->collision_rate = 0.0;
    d->seed = 0;
    d->sort = 1;
    d->potential = HMD_POTENTIAL_LENNARD_JONES;
    for (int k = 0; k < HMD_MAX_SPECIES * HMD_MAX_SPECIES; ++k) {
        d->index_repulsion[k] = 12;
        d->index_attraction[k] = 6;
        d->index[k] = 12;
        d->r_min[k] = 0.0;
        d->distortion[k] = 1.0;
    }
    d->resonance_frequency = 0.0;   /* required for verlet_nvt_hoover (verlet_nvt_hoover.lua.in:176) */
}

int hmd_last_error(const hmd_engine* h, char* buf, size_t size)
{
    const std::string& m = (h && h->e) ? h->e->err : g_last_error;
    if (buf && size) {
        std::strncpy(buf, m.c_str(), size - 1);
        buf[size - 1] = 0;
    }
    return (int)m.size();
}

int hmd_engine_create(int precision, int device, hmd_engine** out)
{
    if (!out) return HMD_ERR_INVALID;
    *out = nullptr;
    hmd_engine* h = new hmd_engine{nullptr};
    int rc = guard(nullptr, [&] { h->e = new Engine(precision, device); });
    if (rc != HMD_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return HMD_OK;
}

int hmd_engine_destroy(hmd_engine* h)
{
    if (!h) return HMD_OK;
    delete h->e;
    delete h;
    return HMD_OK;
}

int hmd_engine_add_system(hmd_engine* h, const hmd_system_desc* d, uint32_t* index)
{
    ENGINE_OR_FAIL(h);
    if (!d) return HMD_ERR_INVALID;
    return guard(h, [&] {
        uint32_t k = h->e->add_system(*d);
        if (index) *index = k;
    });
}

int hmd_engine_commit(hmd_engine* h)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->commit(); });
}

int hmd_engine_reserve(hmd_engine* h, uint32_t slots, uint32_t systems, uint32_t neighbour_capacity)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->reserve(slots, systems, neighbour_capacity); });
}

int hmd_engine_remove_system(hmd_engine* h, uint32_t sys)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->remove_system(sys); });
}

int hmd_engine_capacity(hmd_engine* h, uint64_t* out)
{
    ENGINE_OR_FAIL(h);
    if (!out) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->capacity_info(out); });
}

int hmd_engine_progress(hmd_engine* h, uint64_t* step, uint32_t* steps_left, uint32_t n)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->progress(step, steps_left, n); });
}

int hmd_engine_set_option(hmd_engine* h, const char* name, int64_t value)
{
    ENGINE_OR_FAIL(h);
    if (!name) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->set_option(name, value); });
}

int hmd_engine_get_option(hmd_engine* h, const char* name, int64_t* value)
{
    ENGINE_OR_FAIL(h);
    if (!name || !value) return HMD_ERR_INVALID;
    return guard(h, [&] { *value = h->e->get_option(name); });
}

int hmd_engine_stream(hmd_engine* h, void** stream)
{
    ENGINE_OR_FAIL(h);
    if (!stream) return HMD_ERR_INVALID;
    *stream = (void*)h->e->stream();
    return HMD_OK;
}

int hmd_info(hmd_engine* h, uint32_t sys, hmd_system_info* info)
{
    ENGINE_OR_FAIL(h);
    if (!info) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->info(sys, info); });
}

int hmd_set(hmd_engine* h, uint32_t sys, const char* name, const void* host, size_t count)
{
    ENGINE_OR_FAIL(h);
    if (!name || !host) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->set(sys, name, host, count); });
}

int hmd_get(hmd_engine* h, uint32_t sys, const char* name, void* host, size_t count)
{
    ENGINE_OR_FAIL(h);
    if (!name || !host) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->get(sys, name, host, count); });
}

int hmd_get_raw(hmd_engine* h, uint32_t sys, const char* name, void* host, size_t bytes)
{
    ENGINE_OR_FAIL(h);
    if (!name || !host) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->get_raw(sys, name, host, bytes); });
}

int hmd_step(hmd_engine* h, uint64_t nsteps, int aux_last)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->step(nsteps, aux_last != 0); });
}

int hmd_integrate(hmd_engine* h)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->integrate(); });
}

int hmd_force(hmd_engine* h, int aux)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->force(aux != 0); });
}

int hmd_finalize(hmd_engine* h)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->finalize(); });
}

int hmd_request_rebuild(hmd_engine* h, uint32_t sys)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->request_rebuild(sys); });
}

int hmd_set_steps_left(hmd_engine* h, uint32_t sys, uint32_t steps)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->set_steps_left(sys, steps); });
}

int hmd_minimize(hmd_engine* h, uint32_t sys, uint32_t steps, double step_size, double max_move)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->minimize(sys, steps, step_size, max_move); });
}

int hmd_max_displacement(hmd_engine* h, uint32_t sys, double* displacement)
{
    ENGINE_OR_FAIL(h);
    if (!displacement) return HMD_ERR_INVALID;
    return guard(h, [&] { *displacement = h->e->max_displacement(sys); });
}

int hmd_thermo(hmd_engine* h, uint32_t sys, double* out)
{
    ENGINE_OR_FAIL(h);
    if (!out) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->thermo(sys, out); });
}

int hmd_positions_lattice(hmd_engine* h, uint32_t sys, const double* slab)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->lattice(sys, slab); });
}

int hmd_velocities_boltzmann(hmd_engine* h, uint32_t sys, double temperature, uint64_t seed)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->boltzmann(sys, temperature, seed); });
}

int hmd_integrator_state(hmd_engine* h, uint32_t sys, double* out)
{
    ENGINE_OR_FAIL(h);
    if (!out) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->integrator_state(sys, out); });
}

int hmd_neighbour_lists(hmd_engine* h, uint32_t sys, uint32_t* counts, uint32_t* lists, uint32_t maxn)
{
    ENGINE_OR_FAIL(h);
    if (!counts || !lists) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->neighbour_lists(sys, counts, lists, maxn); });
}

int hmd_profile_enable(hmd_engine* h, int enable)
{
    ENGINE_OR_FAIL(h);
    return guard(h, [&] { h->e->profile_enable(enable != 0); });
}

int hmd_profile_get(hmd_engine* h, const char* phase, double* total_ms, uint64_t* count)
{
    ENGINE_OR_FAIL(h);
    if (!phase || !total_ms || !count) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->profile_get(phase, total_ms, count); });
}

int hmd_hilbert_keys(hmd_engine* h, uint32_t sys, uint32_t* keys)
{
    ENGINE_OR_FAIL(h);
    if (!keys) return HMD_ERR_INVALID;
    return guard(h, [&] { h->e->hilbert_keys(sys, keys); });
}

// ---- dynamics ---------------------------------------------------------------

struct hmd_dynamics {
    hmd_engine* owner;
    hmd::Dynamics* d;
};

#define DYN_OR_FAIL(x)                                                       \
    do {                                                                     \
        if (!(x) || !(x)->d) {                                               \
            g_last_error = "null dynamics handle";                           \
            return HMD_ERR_INVALID;                                          \
        }                                                                    \
    } while (0)

int hmd_dynamics_create(hmd_engine* h, uint32_t sys, double max_lag_time, double resolution, uint32_t block_size,
                        uint32_t shift, uint32_t separation, hmd_dynamics** out)
{
    ENGINE_OR_FAIL(h);
    if (!out) return HMD_ERR_INVALID;
    *out = nullptr;
    hmd::Dynamics* d = nullptr;
    int rc = guard(h, [&] { d = new hmd::Dynamics(*h->e, sys, max_lag_time, resolution, block_size, shift, separation); });
    if (rc != HMD_OK) return rc;
    *out = new hmd_dynamics{h, d};
    return HMD_OK;
}

int hmd_dynamics_destroy(hmd_dynamics* x)
{
    if (!x) return HMD_OK;
    delete x->d;
    delete x;
    return HMD_OK;
}

int hmd_dynamics_levels(hmd_dynamics* x, uint32_t* levels, uint32_t* block_size)
{
    DYN_OR_FAIL(x);
    if (levels) *levels = x->d->levels();
    if (block_size) *block_size = x->d->block_size();
    return HMD_OK;
}

int hmd_dynamics_time(hmd_dynamics* x, double* time)
{
    DYN_OR_FAIL(x);
    if (!time) return HMD_ERR_INVALID;
    return guard(x->owner, [&] { x->d->time(time); });
}

int hmd_dynamics_add_msd(hmd_dynamics* x, uint32_t first, uint32_t last, int32_t* tcf)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] {
        int32_t k = x->d->add_msd(first, last);
        if (tcf) *tcf = k;
    });
}

int hmd_dynamics_add_mqd(hmd_dynamics* x, uint32_t first, uint32_t last, int32_t* tcf)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] {
        int32_t k = x->d->add_mqd(first, last);
        if (tcf) *tcf = k;
    });
}

int hmd_dynamics_add_vacf(hmd_dynamics* x, uint32_t first, uint32_t last, int32_t* tcf)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] {
        int32_t k = x->d->add_vacf(first, last);
        if (tcf) *tcf = k;
    });
}

int hmd_dynamics_add_isf(hmd_dynamics* x, const double* wavenumber, uint32_t nk, double tolerance, uint32_t max_count,
                         uint32_t first, uint32_t last, double norm, int32_t* tcf)
{
    DYN_OR_FAIL(x);
    if (!wavenumber || nk == 0) return HMD_ERR_INVALID;
    return guard(x->owner, [&] {
        int32_t k = x->d->add_isf(wavenumber, nk, tolerance, max_count, first, last, norm);
        if (tcf) *tcf = k;
    });
}

int hmd_dynamics_sample(hmd_dynamics* x)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] { x->d->sample(); });
}

int hmd_dynamics_finalise(hmd_dynamics* x)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] { x->d->finalise(); });
}

int hmd_dynamics_result(hmd_dynamics* x, int32_t tcf, double* mean, double* error, uint64_t* count)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] { x->d->result(tcf, mean, error, count); });
}

int hmd_dynamics_shells(hmd_dynamics* x, int32_t tcf, uint32_t* nshell, double* wavenumber)
{
    DYN_OR_FAIL(x);
    return guard(x->owner, [&] { x->d->shells(tcf, nshell, wavenumber); });
}

int hmd_msd_pair_noalloc(const double* origin, const double* position, uint32_t count, double* out, void* stream)
{
    return guard(nullptr, [&] {
        hmd::msd_pair_noalloc(origin, position, count, out, static_cast<cudaStream_t>(stream));
    });
}

} // extern "C"
