/*
 * halmd_gb300.h — C ABI of the GB300-native molecular-dynamics step.
 *
 * Drop-in boundary for HALMD's mdsim/gpu backend.  The reference exposes its
 * modules to Lua through luaponte bindings (luaopen_libhalmd_mdsim_gpu_*, e.g.
 * halmd/mdsim/gpu/particle.cpp:304-357); this library exports plain C entry
 * points with opaque handles, host pointers and sizes, and integer status
 * codes (0 = ok, negative = error, message via hmd_last_error).  One handle
 * (an "engine") holds one or more independent systems that advance together
 * on one GPU; a single reference simulation is an engine with one system.
 *
 * Threading: an engine is thread-compatible (one thread at a time per
 * handle), like the reference's single-threaded module graph.  All array
 * accessors take and return data in particle-tag order (the reference's
 * particle id), independent of the device's internal Hilbert order.
 */
#ifndef HALMD_GB300_H
#define HALMD_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define HMD_API __attribute__((visibility("default")))
#else
#define HMD_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define HMD_OK 0
#define HMD_ERR_INVALID (-1)   /* bad argument (std::invalid_argument in the reference) */
#define HMD_ERR_CUDA (-2)      /* CUDA runtime error */
#define HMD_ERR_STATE (-3)     /* call not valid in the current state (std::logic_error) */
#define HMD_ERR_NOMEM (-4)     /* device allocation failed */
#define HMD_ERR_OVERFLOW (-5)  /* capacity overflow that retries could not resolve */

#define HMD_PRECISION_FLOAT 0     /* particle_3_float   (particle.lua.in:46-57) */
#define HMD_PRECISION_DSFLOAT 1   /* particle_3_dsfloat (default precision) */
/* FP64 arithmetic in force, integrate and finalize (no counterpart among the
 * reference's GPU particle types; the precision of its host backend, kept
 * here as the drift and force reference run from the same start): storage
 * as dsfloat (hi + lo words, 48 significant bits), forces in double;
 * Lennard-Jones potentials with any truncation and velocity Verlet only */
#define HMD_PRECISION_DOUBLE 2

#define HMD_TRUNC_SHARP 0          /* truncations/sharp.hpp */
#define HMD_TRUNC_SHIFTED 1        /* truncations/shifted.hpp (truncate.lua.in:289 default) */
#define HMD_TRUNC_SMOOTH_R4 2      /* truncations/smooth_r4.hpp */
#define HMD_TRUNC_FORCE_SHIFTED 3  /* truncations/force_shifted.hpp */
/* no truncation: the untruncated potential over all pairs, no neighbour list
 * (forces/pair_full.hpp; lua/halmd/mdsim/forces/pair.lua.in:78-83 picks it
 * when the potential has no r_cut); r_cut and skin are ignored */
#define HMD_TRUNC_NONE 4

/* pair potentials (mdsim/gpu/potentials/pair/{lennard_jones,mie,morse,power_law}.cpp; every truncation applies to each) */
#define HMD_POTENTIAL_LENNARD_JONES 0  /* lennard_jones.cpp (default) */
#define HMD_POTENTIAL_MIE 1            /* mie.cpp: epsilon, sigma, index_repulsion m, index_attraction n */
#define HMD_POTENTIAL_MORSE 2          /* morse.cpp: epsilon, sigma, r_min, distortion B */
#define HMD_POTENTIAL_POWER_LAW 3      /* power_law.cpp: epsilon, sigma, index n */

#define HMD_INTEGRATOR_VERLET 0    /* integrators/verlet.cpp */
#define HMD_INTEGRATOR_ANDERSEN 1  /* integrators/verlet_nvt_andersen.cpp */
#define HMD_INTEGRATOR_HOOVER 2    /* integrators/verlet_nvt_hoover.cpp (Nose-Hoover chain of two) */
#define HMD_INTEGRATOR_BOLTZMANN 3 /* lua/halmd/mdsim/integrators/verlet_nvt_boltzmann.lua.in */
#define HMD_INTEGRATOR_EULER 4     /* integrators/euler.cpp */

#define HMD_MAX_SPECIES 4
#define HMD_NTHERMO 14

typedef struct hmd_engine hmd_engine;
typedef struct hmd_dynamics hmd_dynamics;

/*
 * Parameters of one system.  Replaces the constructor arguments of
 * particle(nparticle, nspecies)            lua/halmd/mdsim/particle.lua.in:229-290
 * box(edges)                               mdsim/box.cpp:40-60
 * lennard_jones(epsilon, sigma)            mdsim/gpu/potentials/pair/lennard_jones.cpp:45-71
 * mie(epsilon, sigma, index_repulsion, index_attraction)
 *                                          mdsim/gpu/potentials/pair/mie.cpp, lua/.../pair/mie.lua.in:66-72
 * morse(epsilon, sigma, r_min, distortion) mdsim/gpu/potentials/pair/morse.cpp, lua/.../pair/morse.lua.in:75-81
 * power_law(epsilon, sigma, index)         mdsim/gpu/potentials/pair/power_law.cpp, lua/.../pair/power_law.lua.in:56-61
 *   :truncate{kind, cutoff, h}             lua/halmd/mdsim/potentials/pair/adapters/truncate.lua.in:287-305
 * neighbour{skin, occupancy, sort}         lua/halmd/mdsim/neighbour.lua.in:151-306, from_binning.cpp:96-119
 * binning{occupancy}                       mdsim/gpu/binning.cpp:47-116
 * verlet(dt) / verlet_nvt_andersen(dt, T, rate) / verlet_nvt_hoover(dt, T, resonance_frequency)
 *   / verlet_nvt_boltzmann(dt, T, rate) / euler(dt)
 *                                          lua/halmd/mdsim/integrators/{verlet,verlet_nvt_andersen,
 *                                          verlet_nvt_hoover,verlet_nvt_boltzmann,euler}.lua.in
 * Matrices are nspecies x nspecies, row-major; r_cut in units of sigma.
 */
typedef struct hmd_system_desc {
    uint32_t nparticle;
    uint32_t nspecies;
    double box[3];
    double epsilon[HMD_MAX_SPECIES * HMD_MAX_SPECIES];
    double sigma[HMD_MAX_SPECIES * HMD_MAX_SPECIES];
    double r_cut[HMD_MAX_SPECIES * HMD_MAX_SPECIES];
    int32_t truncation;
    double smoothing;            /* h of smooth_r4 */
    double skin;                 /* neighbour list skin (default 0.5) */
    double cell_occupancy;       /* binning occupancy (default 0.5) */
    double neighbour_occupancy;  /* list occupancy (default 0.4, from_binning.cpp:285-287) */
    double timestep;
    int32_t integrator;
    double temperature;          /* Andersen heat bath */
    double collision_rate;       /* Andersen collision rate nu */
    uint64_t seed;               /* Andersen random stream */
    int32_t sort;                /* 1: Hilbert reorder at every list rebuild (default) */
    int32_t potential;           /* HMD_POTENTIAL_* (default lennard_jones) */
    uint32_t index_repulsion[HMD_MAX_SPECIES * HMD_MAX_SPECIES];   /* mie m: even, > n (default 12) */
    uint32_t index_attraction[HMD_MAX_SPECIES * HMD_MAX_SPECIES];  /* mie n: even, >= 2 (default 6) */
    uint32_t index[HMD_MAX_SPECIES * HMD_MAX_SPECIES];             /* power_law n >= 1 (default 12) */
    double r_min[HMD_MAX_SPECIES * HMD_MAX_SPECIES];      /* morse: position of the minimum (required) */
    double distortion[HMD_MAX_SPECIES * HMD_MAX_SPECIES]; /* morse: B > 0 (default 1) */
    double resonance_frequency;  /* verlet_nvt_hoover: heat-bath resonance frequency (required, > 0) */
} hmd_system_desc;

/* per-system state readable after any call (hmd_info) */
typedef struct hmd_system_info {
    uint32_t nparticle, nspecies;
    uint32_t slot_offset, slots;     /* device slot range */
    int32_t ncell[3];
    uint32_t cell_size;
    uint32_t neighbour_capacity;
    uint32_t hilbert_depth;
    uint32_t max_neighbours;         /* largest list of the last build */
    uint32_t max_cell_occupancy;     /* largest cell of the last build */
    uint64_t step;                   /* completed integration steps */
    uint64_t rebuilds;               /* neighbour-list builds so far */
    uint32_t sort_key_bits;          /* bits of the engine's sort key (radix passes = ceil(bits/8)) */
    uint32_t rebuild_kernels;        /* kernels one conditional rebuild launches */
    float box_f32[3];                /* box edges as the device stores them */
    float rr_cut_skin[HMD_MAX_SPECIES * HMD_MAX_SPECIES];  /* float (r_c + skin)^2 table */
    float rr_cut[HMD_MAX_SPECIES * HMD_MAX_SPECIES];       /* float r_c^2 table */
} hmd_system_info;

/* fill with the reference's defaults (Lua module defaults) */
HMD_API void hmd_system_desc_init(hmd_system_desc* desc);

/* last error of an engine (engine == NULL: last error of this thread) */
HMD_API int hmd_last_error(const hmd_engine* engine, char* buf, size_t size);

/* ---- engine lifecycle --------------------------------------------------- */

/* precision HMD_PRECISION_*; device = CUDA ordinal (main.cpp:56-63 --device) */
HMD_API int hmd_engine_create(int precision, int device, hmd_engine** out);
HMD_API int hmd_engine_destroy(hmd_engine* engine);
/* add a system before hmd_engine_commit; *index receives its number */
HMD_API int hmd_engine_add_system(hmd_engine* engine, const hmd_system_desc* desc, uint32_t* index);
/* lay out and allocate all device arrays (particle.cpp:56-160 ctor) */
HMD_API int hmd_engine_commit(hmd_engine* engine);
/*
 * Reserve device capacity before commit so that systems can join and leave
 * the committed engine between steps (continuous batching; no counterpart in
 * the reference, whose modules are sized once per simulation): `slots`
 * particle slots, `systems` table entries, `neighbour_capacity` list slots
 * per particle (0: from the systems present at commit).  After commit,
 * hmd_engine_add_system places a new system in free capacity
 * (HMD_ERR_NOMEM when it does not fit) and hmd_engine_remove_system frees one.
 */
HMD_API int hmd_engine_reserve(hmd_engine* engine, uint32_t slots, uint32_t systems, uint32_t neighbour_capacity);
HMD_API int hmd_engine_remove_system(hmd_engine* engine, uint32_t sys);
/* out[8]: slots total, slots in use, cells total, cells in use, list slots per
 * particle, systems in use, system table size, device bytes per slot */
HMD_API int hmd_engine_capacity(hmd_engine* engine, uint64_t* out);
/* completed steps and steps still to do of the first n table entries (one read) */
HMD_API int hmd_engine_progress(hmd_engine* engine, uint64_t* step, uint32_t* steps_left, uint32_t n);
/*
 * Tuning options (autotuned or set by the caller):
 *   "force_lanes"   threads per particle in the force kernel: 0 (auto), 1, 2, 4, 8
 *                   (the reference's unroll_force_loop, neighbour.lua.in:98-101, is 32)
 *   "neighbour_scan" list build: 0 (auto: 2 for systems of at least 2^18 particles, else 1),
 *                   1 (each thread scans the 27 cells around its particle), 2 (each warp scans the
 *                   cells around its 32 particles once); both give the same pair sets
 *   "neighbour_capacity" (get only) list slots per particle
 *   "rebuild_chains"     (get only) steps in which the rebuild chain ran (any system rebuilt)
 *   "list_block"    0 (auto), 4 or 8: entries per block of the list layout; each force thread
 *                   reads list_block / force_lanes entries with one load (2 or 4 lanes: 4 or 8)
 *   "fuse_steps"    1 (default): captured chunks run the finalize of step k and the integrate of
 *                   step k+1 as one kernel; 0: separate kernels (same results)
 *   "float_cutoff"  HMD_PRECISION_DOUBLE engines: 1 takes the pair set of the float list
 *                   criterion on the hi words (the other engines' cut-off test), 0 (default)
 *                   r^2 < r_c^2 in double
 *   "step_kernels"       (get only) kernels of the captured step graphs launched so far
 *                        (rebuild chains not included: rebuild_chains x hmd_system_info.rebuild_kernels)
 */
HMD_API int hmd_engine_set_option(hmd_engine* engine, const char* name, int64_t value);
HMD_API int hmd_engine_get_option(hmd_engine* engine, const char* name, int64_t* value);
/* CUDA stream all work of the engine is issued on (cudaStream_t) */
HMD_API int hmd_engine_stream(hmd_engine* engine, void** stream);
HMD_API int hmd_info(hmd_engine* engine, uint32_t sys, hmd_system_info* info);

/*
 * Phase-space access in tag order (particle.cpp get/set_{position,velocity,
 * species,mass,image,force,potential_energy,stress_pot,id,reverse_id}):
 *   "position"  double[3n] (wrapped into the box on set; the image absorbs the shift)
 *   "velocity"  double[3n]     "mass" double[n]     "species" uint32[n]
 *   "image"     double[3n]     "force" double[3n] (get)
 *   "potential_energy" double[n] (get)   "stress_pot" double[6n] (get)
 *   "unwrapped_position" double[3n] (get; position + image * box)
 *   "reverse_id" uint32[n] (get; slot of each tag, relative to the system)
 *   "id"        uint32[slots] (get; tag of each slot, 0xFFFFFFFF for ghosts)
 * count is the number of elements of the host array.
 */
HMD_API int hmd_set(hmd_engine* engine, uint32_t sys, const char* name, const void* host, size_t count);
HMD_API int hmd_get(hmd_engine* engine, uint32_t sys, const char* name, void* host, size_t count);

/*
 * Raw device arrays in slot order (float words as stored), for checking:
 *   "position_hi" / "position_lo" / "velocity_hi" / "velocity_lo" / "image" /
 *   "force" / "r0": float[4*slots];  "cells": uint32[ncells*cell_size]
 *   (slot numbers relative to the system).
 */
HMD_API int hmd_get_raw(hmd_engine* engine, uint32_t sys, const char* name, void* host, size_t bytes);

/* ---- the MD step -------------------------------------------------------- */

/*
 * Advance every system by nsteps velocity-Verlet steps (sampler.cpp:49-83 ->
 * core.cpp:30-63 mdstep: integrate, lazy neighbour rebuild, force, finalize),
 * as replays of a captured CUDA graph; rebuilds are decided on the device.
 * aux_last != 0: the last step also computes potential energy and stress
 * (particle::aux_enable, particle.cpp:221-253).
 */
HMD_API int hmd_step(hmd_engine* engine, uint64_t nsteps, int aux_last);
/* module-level calls (integrators/verlet.cpp integrate()/finalize(),
 * forces/pair_trunc.hpp apply()), launched one at a time */
HMD_API int hmd_integrate(hmd_engine* engine);
HMD_API int hmd_force(hmd_engine* engine, int aux);
HMD_API int hmd_finalize(hmd_engine* engine);
/* request a neighbour-list rebuild (with sort) before the next force */
HMD_API int hmd_request_rebuild(hmd_engine* engine, uint32_t sys);
/* steps a system still has to do (serving); ~0u = unbounded */
HMD_API int hmd_set_steps_left(hmd_engine* engine, uint32_t sys, uint32_t steps);
/*
 * Steepest-descent minimisation of one system's potential energy, used to
 * relax random start positions (no counterpart in the reference, which has
 * no minimiser).  Each step moves every particle by step_size * F_i, cut to
 * max_move in length, then recomputes forces (lists rebuilt by the usual
 * skin rule).  Other systems of the engine do not advance meanwhile;
 * velocities and the step counter are left as they were.
 */
HMD_API int hmd_minimize(hmd_engine* engine, uint32_t sys, uint32_t steps, double step_size, double max_move);

/*
 * Per-phase runtime accumulators (utility/profiler.hpp:56-99, the modules'
 * scoped_timer runtime structs, e.g. forces/pair_trunc.hpp:141-148):
 * while enabled, hmd_integrate / hmd_force / hmd_finalize bracket their
 * kernels with CUDA events on the engine stream.  Phases: "integrate",
 * "force", "force_aux", "finalize", "rebuild".
 */
HMD_API int hmd_profile_enable(hmd_engine* engine, int enable);
HMD_API int hmd_profile_get(hmd_engine* engine, const char* phase, double* total_ms, uint64_t* count);

/* maximum displacement since the last build (max_displacement.cpp:77-106) */
HMD_API int hmd_max_displacement(hmd_engine* engine, uint32_t sys, double* displacement);

/*
 * FP64 sums (observables/gpu/thermodynamics.cpp:68-190), valid after a step
 * or force call with aux: out[HMD_NTHERMO] =
 *   Σ m v², Σ m v (3), Σ m, Σ E_pot, Σ tr(stress), stress (6), N
 */
HMD_API int hmd_thermo(hmd_engine* engine, uint32_t sys, double* out);

/*
 * positions.lattice (mdsim/host/positions/lattice.cpp:63-175,
 * gpu/positions/lattice_kernel.cu): place the particles of a committed
 * system on an fcc lattice filling the slab (slab[3]: fraction of each box
 * edge at the centre of the box; NULL = the whole box) with the smallest
 * lattice constant that gives enough sites, vacancies spread evenly, image
 * counters zeroed.  HMD_ERR_STATE for slab extents outside (0, 1].
 */
HMD_API int hmd_positions_lattice(hmd_engine* engine, uint32_t sys, const double* slab);
/*
 * velocities.boltzmann set() (mdsim/gpu/velocities/boltzmann.cpp,
 * boltzmann_kernel.cu:47-140): each velocity component N(0, sqrt(T)) divided
 * by sqrt(m), then the centre-of-mass velocity removed.  The random stream is
 * Philox4x32-10 keyed by (seed, tag) (the reference draws from rand48).
 */
HMD_API int hmd_velocities_boltzmann(hmd_engine* engine, uint32_t sys, double temperature, uint64_t seed);

/*
 * Thermostat state of a system (verlet_nvt_hoover.cpp:252-283 properties
 * `position`, `velocity`, `internal_energy`): out[0..1] chain positions xi,
 * out[2..3] chain velocities v_xi, out[4] the chain's energy per particle
 * (en_nhc, verlet_nvt_hoover.cpp:134-140), out[5..7] the centre-of-mass
 * velocity removed by the last Maxwell-Boltzmann draw (verlet_nvt_boltzmann).
 * Zero for the other integrators.
 */
HMD_API int hmd_integrator_state(hmd_engine* engine, uint32_t sys, double* out);

/*
 * Neighbour lists of the last build (neighbours/from_binning.cpp g_neighbour()):
 * counts[n] and lists[n*maxn] in tag numbering, each list ascending, padded
 * with 0xFFFFFFFF.  Returns HMD_ERR_INVALID if maxn is too small.
 */
HMD_API int hmd_neighbour_lists(hmd_engine* engine, uint32_t sys, uint32_t* counts, uint32_t* lists, uint32_t maxn);

/* Hilbert keys of the current positions, tag order (hilbert_kernel.cu:39-66) */
HMD_API int hmd_hilbert_keys(hmd_engine* engine, uint32_t sys, uint32_t* keys);

/* ---- dynamic correlations (observables/dynamics) ------------------------ */

/*
 * Blocking scheme (observables/dynamics/blocking_scheme.cpp:35-200) over one
 * system: max_lag_time and resolution in time units, block_size, shift,
 * separation as the reference.
 */
HMD_API int hmd_dynamics_create(hmd_engine* engine, uint32_t sys, double max_lag_time, double resolution,
                        uint32_t block_size, uint32_t shift, uint32_t separation, hmd_dynamics** out);
HMD_API int hmd_dynamics_destroy(hmd_dynamics* dyn);
/* number of levels and the time grid [levels*block_size] */
HMD_API int hmd_dynamics_levels(hmd_dynamics* dyn, uint32_t* levels, uint32_t* block_size);
HMD_API int hmd_dynamics_time(hmd_dynamics* dyn, double* time);
/* MSD of the particles with tag in [first, last) (id_range particle group) */
HMD_API int hmd_dynamics_add_msd(hmd_dynamics* dyn, uint32_t first, uint32_t last, int32_t* tcf);
/* mean quartic displacement (mean_quartic_displacement.hpp:34-41) and velocity
 * autocorrelation (velocity_autocorrelation.hpp:34-38) of the same groups */
HMD_API int hmd_dynamics_add_mqd(hmd_dynamics* dyn, uint32_t first, uint32_t last, int32_t* tcf);
HMD_API int hmd_dynamics_add_vacf(hmd_dynamics* dyn, uint32_t first, uint32_t last, int32_t* tcf);
/*
 * ISF of a particle group at the given wavenumbers (wavevector.cpp:40-160:
 * shells of reciprocal-lattice vectors within tolerance, <= max_count each),
 * normalised by `norm` (intermediate_scattering_function.hpp:89-113)
 */
HMD_API int hmd_dynamics_add_isf(hmd_dynamics* dyn, const double* wavenumber, uint32_t nk, double tolerance,
                         uint32_t max_count, uint32_t first, uint32_t last, double norm, int32_t* tcf);
/* sample at the current step (blocking_scheme::sample) / drain (finalise) */
HMD_API int hmd_dynamics_sample(hmd_dynamics* dyn);
HMD_API int hmd_dynamics_finalise(hmd_dynamics* dyn);
/* result of a correlation: mean, error of mean and count per (level, lag,
 * shell); arrays of levels*block_size*nshell (nshell = 1 for MSD) */
HMD_API int hmd_dynamics_result(hmd_dynamics* dyn, int32_t tcf, double* mean, double* error, uint64_t* count);
HMD_API int hmd_dynamics_shells(hmd_dynamics* dyn, int32_t tcf, uint32_t* nshell, double* wavenumber);

/* ---- allocation-free MSD of one sample pair ----------------------------- */

/*
 * No counterpart in the reference.  This entry point is for callers that
 * must not allocate device memory when they sample: cudaMalloc/cudaFree
 * synchronise the whole device (stalling a simulation whose steps are in
 * flight), and a server that reserved nearly all of HBM for its engine may
 * have no room left.  It allocates nothing; its scratch is a fixed array of
 * the library in device memory (96 KiB on every device that loads the
 * library, held until the process exits).
 *
 * origin, position: device arrays of count x 3 doubles (unwrapped positions
 * in the same particle order).  out: device array of 3 doubles, written with
 * (count, mean, variance) of |position - origin|^2, the triple the dynamics
 * path accumulates.  stream: a cudaStream_t (NULL for the legacy default
 * stream); the call enqueues two kernels and returns without synchronising.
 *
 * - count above HMD_MSD_NOALLOC_MAX_PARTICLES (2^25) is rejected with
 *   HMD_ERR_INVALID, as are null, misaligned or non-device pointers and
 *   buffers whose allocation ends before the bytes the call reads or writes.
 * - The first call in each CUDA context (on a device: its primary context,
 *   and again after cudaDeviceReset, which makes a new one) looks up the
 *   scratch array's address, which can load this library's device code
 *   into that context.
 * - Nothing needs to be zeroed first.
 * - All calls on one device share the one scratch array: calls that can
 *   overlap (different streams, or host threads without ordering) race and
 *   return wrong results.  Serialise them on one stream.
 */
#define HMD_MSD_NOALLOC_MAX_PARTICLES (1u << 25)
HMD_API int hmd_msd_pair_noalloc(const double* origin, const double* position, uint32_t count, double* out,
                                 void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HALMD_GB300_H */
