/*
 * Every entry point of include/halmd_gb300.h called from C (not through a
 * binding): the host-language side of the drop-in boundary as a Lua C
 * module or any other C caller would use it.  Builds with a C compiler
 * against the header and the library alone (plus the CUDA runtime for the
 * device buffers of the allocation-free MSD entry point).  Exits 0 and
 * prints "harness ok" when every call returned HMD_OK (or the documented
 * error) and the results pass plain sanity checks.
 *
 * test infrastructure: run by tests/test_gpu_c_abi.py on a GPU, compiled
 * and linked (not run) by tests/test_abi.py on any machine
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "halmd_gb300.h"

static hmd_engine* g_eng = NULL;
static int g_failed = 0;

#define CHECK(call)                                                                    \
    do {                                                                               \
        int rc_ = (call);                                                              \
        if (rc_ != HMD_OK) {                                                           \
            char msg_[512] = "";                                                       \
            hmd_last_error(g_eng, msg_, sizeof msg_);                                  \
            fprintf(stderr, "%s:%d: %s -> %d (%s)\n", __FILE__, __LINE__, #call, rc_, msg_); \
            exit(1);                                                                   \
        }                                                                              \
    } while (0)

#define EXPECT(cond)                                                          \
    do {                                                                      \
        if (!(cond)) {                                                        \
            fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #cond); \
            g_failed = 1;                                                     \
        }                                                                     \
    } while (0)

/* fcc lattice of 4 m^3 particles at density rho, jittered deterministically */
static double fcc(uint32_t m, double rho, double* r)
{
    const double L = m * cbrt(4.0 / rho), a = L / m;
    const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    uint32_t k = 0;
    for (uint32_t x = 0; x < m; ++x)
        for (uint32_t y = 0; y < m; ++y)
            for (uint32_t z = 0; z < m; ++z)
                for (int b = 0; b < 4; ++b, ++k) {
                    const double j = 0.02 * sin(1.7 * k);
                    r[3 * k + 0] = (x + basis[b][0] + 0.25) * a - 0.5 * L + j;
                    r[3 * k + 1] = (y + basis[b][1] + 0.25) * a - 0.5 * L - j;
                    r[3 * k + 2] = (z + basis[b][2] + 0.25) * a - 0.5 * L + 0.5 * j;
                }
    return L;
}

int main(void)
{
    const uint32_t m = 6, n = 4 * m * m * m;
    double* r = malloc(sizeof(double) * 3 * n);
    double* v = malloc(sizeof(double) * 3 * n);
    double* f = malloc(sizeof(double) * 3 * n);
    const double L = fcc(m, 0.8442, r);
    for (uint32_t k = 0; k < 3 * n; ++k) v[k] = 0.5 * sin(0.37 * k + 0.1);

    /* ---- engine of one LJ system ---- */
    hmd_system_desc d;
    hmd_system_desc_init(&d);
    d.nparticle = n;
    d.box[0] = d.box[1] = d.box[2] = L;
    d.r_cut[0] = 2.5;
    d.truncation = HMD_TRUNC_SHIFTED;
    d.skin = 0.3;
    d.timestep = 0.005;
    CHECK(hmd_engine_create(HMD_PRECISION_DSFLOAT, 0, &g_eng));
    uint32_t sys = 99;
    CHECK(hmd_engine_add_system(g_eng, &d, &sys));
    EXPECT(sys == 0);
    CHECK(hmd_engine_set_option(g_eng, "force_lanes", 4));
    CHECK(hmd_engine_commit(g_eng));
    int64_t opt = -1;
    CHECK(hmd_engine_get_option(g_eng, "force_lanes", &opt));
    EXPECT(opt == 4);
    void* stream = NULL;
    CHECK(hmd_engine_stream(g_eng, &stream));
    CHECK(hmd_set(g_eng, 0, "position", r, 3 * (size_t)n));
    CHECK(hmd_set(g_eng, 0, "velocity", v, 3 * (size_t)n));

    /* ---- module calls and the captured step ---- */
    CHECK(hmd_profile_enable(g_eng, 1));
    CHECK(hmd_force(g_eng, 1));
    CHECK(hmd_integrate(g_eng));
    CHECK(hmd_force(g_eng, 0));
    CHECK(hmd_finalize(g_eng));
    double ms = 0;
    uint64_t calls = 0;
    CHECK(hmd_profile_get(g_eng, "force", &ms, &calls));
    EXPECT(calls >= 1 && ms > 0);
    CHECK(hmd_profile_enable(g_eng, 0));
    CHECK(hmd_step(g_eng, 20, 1));
    CHECK(hmd_request_rebuild(g_eng, 0));
    CHECK(hmd_step(g_eng, 5, 1));
    double th[HMD_NTHERMO];
    CHECK(hmd_thermo(g_eng, 0, th));
    EXPECT(th[13] == n && isfinite(th[0]) && th[5] < 0);
    hmd_system_info info;
    CHECK(hmd_info(g_eng, 0, &info));
    EXPECT(info.nparticle == n && info.step == 26 && info.rebuilds >= 2);   /* 1 module step + 25 */
    CHECK(hmd_get(g_eng, 0, "force", f, 3 * (size_t)n));
    double fsum[3] = {0, 0, 0};
    for (uint32_t k = 0; k < n; ++k)
        for (int q = 0; q < 3; ++q) fsum[q] += f[3 * k + q];
    EXPECT(fabs(fsum[0]) + fabs(fsum[1]) + fabs(fsum[2]) < 1e-3);   /* Newton's third law */
    float* raw = malloc(16 * (size_t)info.slots);
    CHECK(hmd_get_raw(g_eng, 0, "position_hi", raw, 16 * (size_t)info.slots));
    double disp = -1;
    CHECK(hmd_max_displacement(g_eng, 0, &disp));
    EXPECT(disp >= 0 && disp <= 0.5 * d.skin);
    uint32_t* counts = malloc(sizeof(uint32_t) * n);
    uint32_t* lists = malloc(sizeof(uint32_t) * (size_t)n * info.neighbour_capacity);
    CHECK(hmd_neighbour_lists(g_eng, 0, counts, lists, info.neighbour_capacity));
    EXPECT(counts[0] > 20 && counts[0] < 150);
    uint32_t* keys = malloc(sizeof(uint32_t) * n);
    CHECK(hmd_hilbert_keys(g_eng, 0, keys));
    double ist[8];
    CHECK(hmd_integrator_state(g_eng, 0, ist));
    EXPECT(ist[0] == 0.0);

    /* ---- dynamics: MSD, MQD, VACF, ISF on the blocking scheme ---- */
    hmd_dynamics* dyn = NULL;
    CHECK(hmd_dynamics_create(g_eng, 0, 0.5, 0.05, 10, 3, 10, &dyn));
    int32_t t_msd = -1, t_mqd = -1, t_vacf = -1, t_isf = -1;
    CHECK(hmd_dynamics_add_msd(dyn, 0, n, &t_msd));
    CHECK(hmd_dynamics_add_mqd(dyn, 0, n, &t_mqd));
    CHECK(hmd_dynamics_add_vacf(dyn, 0, n, &t_vacf));
    const double kq = 7.25;
    CHECK(hmd_dynamics_add_isf(dyn, &kq, 1, 0.05, 7, 0, n, n, &t_isf));
    for (int s = 0; s <= 100; ++s) {
        CHECK(hmd_dynamics_sample(dyn));
        CHECK(hmd_step(g_eng, 1, 0));
    }
    CHECK(hmd_dynamics_finalise(dyn));
    uint32_t levels = 0, bs = 0;
    CHECK(hmd_dynamics_levels(dyn, &levels, &bs));
    EXPECT(levels >= 1 && bs == 10);
    double* tgrid = malloc(sizeof(double) * levels * bs);
    CHECK(hmd_dynamics_time(dyn, tgrid));
    uint32_t nshell = 0;
    double kshell[4];
    CHECK(hmd_dynamics_shells(dyn, t_isf, &nshell, kshell));
    EXPECT(nshell == 1);
    double* mean = malloc(sizeof(double) * levels * bs * 4);
    double* err = malloc(sizeof(double) * levels * bs * 4);
    uint64_t* cnt = malloc(sizeof(uint64_t) * levels * bs * 4);
    CHECK(hmd_dynamics_result(dyn, t_msd, mean, err, cnt));
    EXPECT(cnt[1] > 0 && mean[1] > 0);
    CHECK(hmd_dynamics_result(dyn, t_isf, mean, err, cnt));
    CHECK(hmd_dynamics_destroy(dyn));

    /* ---- the allocation-free MSD on device copies of two samples ---- */
    double *da = NULL, *db = NULL, *dout = NULL, out[3];
    if (cudaMalloc((void**)&da, 24 * (size_t)n) != cudaSuccess || cudaMalloc((void**)&db, 24 * (size_t)n) != cudaSuccess ||
        cudaMalloc((void**)&dout, 24) != cudaSuccess) {
        fprintf(stderr, "cudaMalloc failed\n");
        return 1;
    }
    CHECK(hmd_get(g_eng, 0, "unwrapped_position", r, 3 * (size_t)n));
    cudaMemcpy(da, r, 24 * (size_t)n, cudaMemcpyHostToDevice);
    CHECK(hmd_step(g_eng, 10, 0));
    CHECK(hmd_get(g_eng, 0, "unwrapped_position", r, 3 * (size_t)n));
    cudaMemcpy(db, r, 24 * (size_t)n, cudaMemcpyHostToDevice);
    CHECK(hmd_msd_pair_noalloc(da, db, n, dout, stream));
    cudaStreamSynchronize((cudaStream_t)stream);
    cudaMemcpy(out, dout, 24, cudaMemcpyDeviceToHost);
    EXPECT(out[0] == n && out[1] > 0);
    EXPECT(hmd_msd_pair_noalloc(da, db, HMD_MSD_NOALLOC_MAX_PARTICLES + 1u, dout, stream) == HMD_ERR_INVALID);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dout);

    /* ---- set-up modules and descent on a second engine (KA mixture) ---- */
    hmd_engine* ka = NULL;
    CHECK(hmd_engine_create(HMD_PRECISION_DSFLOAT, 0, &ka));
    hmd_system_desc k;
    hmd_system_desc_init(&k);
    k.nparticle = n;
    k.nspecies = 2;
    k.box[0] = k.box[1] = k.box[2] = cbrt(n / 1.2);
    const double eps[4] = {1.0, 1.5, 1.5, 0.5}, sig[4] = {1.0, 0.8, 0.8, 0.88};
    for (int q = 0; q < 4; ++q) {
        k.epsilon[q] = eps[q];
        k.sigma[q] = sig[q];
        k.r_cut[q] = 2.5;
    }
    k.truncation = HMD_TRUNC_SMOOTH_R4;
    k.smoothing = 0.005;
    k.skin = 0.3;
    k.timestep = 0.002;
    k.integrator = HMD_INTEGRATOR_ANDERSEN;
    k.temperature = 0.7;
    k.collision_rate = 1.0;
    k.seed = 5;
    CHECK(hmd_engine_add_system(ka, &k, &sys));
    CHECK(hmd_engine_commit(ka));
    uint32_t* sp = malloc(sizeof(uint32_t) * n);
    for (uint32_t q = 0; q < n; ++q) sp[q] = (q % 5 == 0) ? 1u : 0u;
    CHECK(hmd_set(ka, 0, "species", sp, n));
    CHECK(hmd_positions_lattice(ka, 0, NULL));
    CHECK(hmd_velocities_boltzmann(ka, 0, 0.7, 11));
    CHECK(hmd_minimize(ka, 0, 50, 1e-3, 0.05));
    CHECK(hmd_step(ka, 50, 1));
    CHECK(hmd_thermo(ka, 0, th));
    EXPECT(th[13] == n && isfinite(th[5]));
    CHECK(hmd_engine_destroy(ka));

    /* ---- capacity mode: systems join and leave a running engine ---- */
    hmd_engine* cap = NULL;
    CHECK(hmd_engine_create(HMD_PRECISION_DSFLOAT, 0, &cap));
    CHECK(hmd_engine_reserve(cap, 1u << 15, 4, 288));
    CHECK(hmd_engine_commit(cap));
    uint32_t s0 = 0, s1 = 0;
    d.nparticle = n;
    CHECK(hmd_engine_add_system(cap, &d, &s0));
    CHECK(hmd_set(cap, s0, "position", r, 3 * (size_t)n));
    CHECK(hmd_get(g_eng, 0, "position", r, 3 * (size_t)n));
    CHECK(hmd_engine_add_system(cap, &d, &s1));
    CHECK(hmd_set(cap, s1, "position", r, 3 * (size_t)n));
    CHECK(hmd_set_steps_left(cap, s0, 7));
    CHECK(hmd_set_steps_left(cap, s1, 3));
    CHECK(hmd_step(cap, 10, 0));
    uint64_t stp[4];
    uint32_t left[4];
    CHECK(hmd_engine_progress(cap, stp, left, 2));
    EXPECT(stp[s0] == 7 && stp[s1] == 3 && left[s0] == 0 && left[s1] == 0);
    uint64_t capacity[8];
    CHECK(hmd_engine_capacity(cap, capacity));
    CHECK(hmd_engine_remove_system(cap, s1));
    CHECK(hmd_engine_destroy(cap));

    /* ---- errors come back as codes with a message ---- */
    EXPECT(hmd_set(g_eng, 7, "position", r, 3 * (size_t)n) == HMD_ERR_INVALID);
    char msg[256] = "";
    EXPECT(hmd_last_error(g_eng, msg, sizeof msg) >= 0 && strlen(msg) > 0);
    EXPECT(hmd_engine_add_system(g_eng, &d, &sys) == HMD_ERR_STATE);
    CHECK(hmd_engine_destroy(g_eng));

    free(r); free(v); free(f); free(raw); free(counts); free(lists); free(keys); free(tgrid);
    free(mean); free(err); free(cnt); free(sp);
    if (g_failed) return 1;
    printf("harness ok\n");
    return 0;
}
