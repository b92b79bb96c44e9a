/*
 * rrsph_cuda.h — C ABI of the GB300 (sm_103a) WCSPH step.
 *
 * This library is a drop-in for the time loop of RRSPH_OMP:
 *   void time_integration(vheap_darray_floatn& r, vheap_darray_floatn& v,
 *                         heap_darray<rr_float>& rho, heap_darray<rr_float>& p,
 *                         heap_darray<rr_int>& itype)
 *   (sources/RRSPH_OMP/include/TimeIntegration.h:4-9, loop body in
 *    sources/RRSPH_OMP/src/TimeIntegration.cpp:21-102)
 * and for the pieces of that loop the reference's own tests call one at a time
 * (grid_find, density_sum/density_con, the per-pair force terms).
 *
 * Conventions
 *  - Every function returns an int status (RRSPH_OK == 0); nothing throws across
 *    the ABI. rrsph_last_error() gives a human-readable message for the calling
 *    thread's last failure.
 *  - Host vectors (positions, velocities) are particle-major with a caller-given
 *    stride in doubles: component d of particle i is ptr[i*stride + d]. The
 *    reference's rr_float2 arrays have stride 2, its padded rr_float3 arrays
 *    stride 4 (RRSPH_PARAMS/include/RRFloat3.h:5).
 *  - Particle ids are the row order of the dump CSV, as in the reference.
 *  - A solver handle owns one CUDA stream and all device buffers. Handles are not
 *    thread-safe; use one handle per host thread.
 */
#ifndef RRSPH_CUDA_H
#define RRSPH_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RRSPH_ABI_VERSION 1

/* ---- status codes -------------------------------------------------------- */
enum {
    RRSPH_OK = 0,
    RRSPH_ERR_INVALID_ARGUMENT = 1,
    RRSPH_ERR_CUDA = 2,
    RRSPH_ERR_OUT_OF_MEMORY = 3,
    /* "making neighbours grid: error occured" (GridFind.cpp:157-171,184-186) */
    RRSPH_ERR_NEIGHBOUR_OVERFLOW = 4,
    /* "cell_idx was >= params.max_cells" (GridFind.cpp:61-72) */
    RRSPH_ERR_OUT_OF_DOMAIN = 5,
    /* non-finite r/v/rho/p (ConsistencyCheck.cpp:78-145) */
    RRSPH_ERR_NON_FINITE = 6,
    /* particle outside the geometry box (ConsistencyCheck.cpp:162-218) */
    RRSPH_ERR_OUTSIDE_GEOMETRY = 7,
    RRSPH_ERR_UNSUPPORTED = 8,
    RRSPH_ERR_IO = 9,
    RRSPH_ERR_PARSE = 10,
    /* "never ending simulation" (UpdateAcceleration.cpp:26-28) */
    RRSPH_ERR_NEVER_ENDING = 11,
    RRSPH_ERR_NO_DEVICE = 12
};

/* Sticky device-side status flags, read with rrsph_status(). */
#define RRSPH_FLAG_NEIGHBOUR_OVERFLOW 0x1u
#define RRSPH_FLAG_OUT_OF_DOMAIN      0x2u
#define RRSPH_FLAG_NON_FINITE         0x4u
#define RRSPH_FLAG_OUTSIDE_GEOMETRY   0x8u
#define RRSPH_FLAG_NEVER_ENDING       0x10u

/* Arithmetic of the pair loops.
 * FP64:  every operation in double, like RRSPH_OMP.
 * MIXED: pair arithmetic in float32 on cell-relative coordinates with
 *        Kahan-compensated density and force sums; positions, velocities,
 *        densities, the integration update and the piston stay in double.
 *        Cell keys and neighbour sets are identical to FP64 (pairs near the
 *        cutoff are re-tested in double). */
enum { RRSPH_PRECISION_FP64 = 0, RRSPH_PRECISION_MIXED = 1 };

/* Force terms for rrsph_forces() (UpdateAcceleration.cpp:66-97). */
#define RRSPH_TERM_GRAVITY   0x1u  /* a.y = -g start value                       */
#define RRSPH_TERM_EXTERNAL  0x2u  /* external_force_part  (ExtForce.h:15-60)    */
#define RRSPH_TERM_INTERNAL  0x4u  /* find_internal_changes_part (InternalForce.h:121-141) */
#define RRSPH_TERM_ART_VISC  0x8u  /* artificial_viscosity_part (ArtificialViscosity.h:29-65) */
#define RRSPH_TERM_AVERAGE_VELOCITY 0x10u /* average_velocity_part (AverageVelocity.h:20-37) */
#define RRSPH_TERM_ALL       0x1Fu /* what update_acceleration sums, per params  */

/* Value of rrsph_params.dt_dynamic_reduce: how DT_CORRECTION_DYNAMIC picks dt.
 * 0: as the OpenMP build of RRSPH_OMP does — its max reduction is compiled out
 *    (UpdateAcceleration.cpp:107-121), so update_dt(0, 0) gives dt = CFL*h/c.
 * 1: the true max of |a| and mu over particles (the serial OMP / CL behaviour). */

/*
 * Every field of ExperimentParams (sources/RRSPH_PARAMS/include/Params.h:8-196)
 * that the step reads, plus the derived values fileInput() computes
 * (sources/RRSPH_COMMON/src/Input.cpp:93-138). Plain old data; all integers are
 * fixed width. Fill with rrsph_params_defaults(), then from JSON with
 * rrsph_experiment_load_params(), then rrsph_params_derive().
 */
typedef struct rrsph_params {
    uint32_t struct_size;          /* = sizeof(rrsph_params), set by rrsph_params_defaults */
    uint32_t dim;                  /* 2 or 3 */

    /* ParticleParams.json */
    uint64_t ntotal, nfluid, nvirt;
    double x_mingeom, x_maxgeom, y_mingeom, y_maxgeom, z_mingeom, z_maxgeom;
    double delta;
    double rho0;
    double depth;                  /* 0 => find_depth() from the fluid rows */
    uint64_t nwm_particles_start, nwm_particles_end;

    /* ModelParams.json */
    uint32_t density_treatment;    /* 0 summation, 1 continuity, 2 continuity + delta-SPH */
    uint32_t density_skf;
    double density_delta_sph_coef;
    uint32_t eos_sound_vel_method; /* 0 dam break, 1 specific */
    uint32_t intf_sph_approximation;
    double eos_sound_vel, eos_sound_vel_coef;
    double intf_hsml_coef;
    uint32_t intf_skf;
    uint32_t artificial_pressure;
    uint32_t artificial_pressure_skf;
    uint32_t artificial_viscosity;
    double artificial_pressure_index, artificial_pressure_coef;
    double artificial_shear_visc, artificial_bulk_visc;
    uint32_t artificial_viscosity_skf;
    uint32_t average_velocity;
    double average_velocity_coef;
    uint32_t average_velocity_skf;
    uint32_t consistency_check;
    uint32_t consistency_treatment; /* 0 print, 1 stop, 2 fix */
    uint32_t boundary_treatment;    /* 0 dynamic, 1 repulsive (Lennard-Jones) */
    uint32_t nwm;                   /* 0 none, 2/3 piston 1st/2nd order, 4 wall disappear, 5 solitary */
    uint32_t nwm_direction;
    double nwm_time_start, nwm_wave_length, nwm_wave_magnitude, nwm_phase;
    double simulation_time;
    uint32_t dt_correction_method;  /* 0 const value, 1 const CFL, 2 dynamic */
    uint32_t dt_dynamic_reduce;     /* see above; default 0 */
    double dt, CFL_coef;
    uint32_t max_neighbours;
    uint32_t local_threads;
    double save_time, dump_time;
    uint32_t use_dump, save_every_step;
    uint32_t save_velocity, save_pressure;
    uint32_t save_density, use_crash_dump;
    double start_simulation_time;

    /* derived by rrsph_params_derive (Input.cpp:93-138) */
    double hsml, mass, cell_scale_k;
    uint64_t maxn, max_cells;
    double nwm_wave_number, nwm_freq, nwm_piston_magnitude;

    /* constants of ExperimentParams (Params.h:176-193) */
    double pi, g;
    int32_t type_boundary, type_non_existent, type_water;
    uint32_t reserved0;
} rrsph_params;

typedef struct rrsph_solver rrsph_solver;

/* ---- ABI introspection ---------------------------------------------------- */
int rrsph_abi_version(void);
size_t rrsph_params_sizeof(void);
/* Byte offset of a named rrsph_params field; RRSPH_ERR_INVALID_ARGUMENT if unknown. */
int rrsph_params_offsetof(const char* field, size_t* offset);
/* Message for the calling thread's last non-zero status. Never NULL. */
const char* rrsph_last_error(void);

/* ---- parameters (host only, no GPU needed) -------------------------------- */
/* Defaults of ExperimentParams + ModelParams + ParticleParams
 * (Params.h:8-196, ModelParams.h:11-78, ParticleParams.cpp:109-147). */
int rrsph_params_defaults(rrsph_params* p);
/* load_particle_params + load_model_params + apply_*_params
 * (ParticleParams.cpp:51-149, ModelParams.cpp:185-311) from
 * <dir>/ParticleParams.json and <dir>/ModelParams.json. Mandatory keys and the
 * reference's "Need optional param"/"Not implemented" checks are enforced. */
int rrsph_experiment_load_params(const char* experiment_dir, rrsph_params* p);
/* fillInComputingParams + find_depth + postFillInModelParams
 * (Input.cpp:17-138, 238-331). r holds the ntotal loaded positions. */
int rrsph_params_derive(rrsph_params* p, const double* r, uint32_t stride);
/* Start time taken from a dump file name stem, as Input.cpp:258 (std::stod). */
int rrsph_layer_time_from_path(const char* path, double* t);

/* ---- particle layers (CSV; host only) ------------------------------------- */
/* loadArrays (Input.cpp:203-236): columns x,y[,z],itype,vx,vy[,vz],rho by name;
 * p is read if present. Row count must equal p->ntotal. */
int rrsph_layer_read(const char* csv_path, const rrsph_params* p,
                     double* r, uint32_t stride, double* v, double* rho,
                     double* pres, int32_t* itype);
/* print_dump / print (Output.cpp:118-221): std::to_string formatting (6
 * decimals). dump != 0 writes every column; otherwise the save_* switches
 * choose v, rho, p. */
int rrsph_layer_write(const char* csv_path, const rrsph_params* p,
                      const double* r, uint32_t stride, const double* v,
                      const double* rho, const double* pres,
                      const int32_t* itype, int dump);

/* ---- solver --------------------------------------------------------------- */
/* Allocates device buffers for p->ntotal particles on the current CUDA device.
 * p must be derived. precision: RRSPH_PRECISION_FP64 or RRSPH_PRECISION_MIXED. */
int rrsph_create(const rrsph_params* p, int precision, rrsph_solver** out);
void rrsph_destroy(rrsph_solver* s);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
 * work after the solver's. */
int rrsph_get_stream(rrsph_solver* s, void** stream);

/* Host -> device copy of the whole state (ntotal rows). Resets the step
 * counter, the accelerations and drho to zero, as time_integration() starts
 * with fresh work arrays (TimeIntegration.cpp:35-50). pres may be NULL. */
int rrsph_upload(rrsph_solver* s, const double* r, uint32_t stride,
                 const double* v, const double* rho, const double* pres,
                 const int32_t* itype);
/* Device -> host copy of the state; any pointer may be NULL to skip it. */
int rrsph_download(rrsph_solver* s, double* r, uint32_t stride, double* v,
                   double* rho, double* pres, int32_t* itype);

/* nsteps iterations of the time loop body (TimeIntegration.cpp:60-100):
 * predict_half_step, grid_find, density, update_acceleration, piston
 * (when nwm is a piston and time >= nwm_time_start), whole_step, time += dt.
 * *time_io is the simulation time before the first step and is advanced.
 * The first step after rrsph_upload uses dt/2 for velocities (WholeStep.cpp:33). */
int rrsph_step(rrsph_solver* s, uint64_t nsteps, double* time_io);
/* The drop-in call on host arrays, as the reference's time_integration runs
 * on its arrays: rrsph_upload(r, stride, v, rho, NULL, itype), rrsph_step(
 * nsteps, time_io), rrsph_download(r, stride, v, rho, pres, itype), with one
 * wait at the end (rho is not read with summation density, whose first step
 * recomputes it; a page-locked itype, read at the upload, is rewritten only if
 * a step changed a type). r, v, rho and itype are read, then overwritten with the
 * state after the steps; pres (may be NULL) receives p. With graph replay, p
 * (and rho with summation density, which the whole step does not change)
 * come back while the last step's force gather runs. Page-locked arrays are
 * read and written over the host link by kernels, as in rrsph_upload and
 * rrsph_download. */
int rrsph_step_host(rrsph_solver* s, uint64_t nsteps, double* time_io, double* r, uint32_t stride, double* v,
                    double* rho, double* pres, int32_t* itype);
/* rrsph_step(nsteps, time_io) then rrsph_download(r, stride, v, rho, pres,
 * itype) with one wait, the state staying on the device (any array may be
 * NULL), and p / rho brought back during the last force gather as in
 * rrsph_step_host: the per-step call of a loop that hands the host arrays to
 * its output after every step. */
int rrsph_step_download(rrsph_solver* s, uint64_t nsteps, double* time_io, double* r, uint32_t stride, double* v,
                        double* rho, double* pres, int32_t* itype);
/* Asynchronous form of rrsph_step: enqueues nsteps steps on the handle's
 * stream and returns without waiting. The simulation time continues on the
 * device from the previous step (or from rrsph_set_time). Errors raised by the
 * device checks are reported by the next rrsph_sync. */
int rrsph_step_async(rrsph_solver* s, uint64_t nsteps);
/* Sets the simulation time of the next step (stream-ordered). */
int rrsph_set_time(rrsph_solver* s, double time);
/* Waits for the enqueued steps; *time_out (may be NULL) receives the time
 * after the last step. Returns the status the device flags imply. The flags
 * stay set (rrsph_status reads and clears them; rrsph_step clears them when
 * it starts). */
int rrsph_sync(rrsph_solver* s, double* time_out);
/* The time loop with the layer output of RRSPHOutput (TimeIntegration.cpp:53-100,
 * Output.cpp:28-79, 223-446), from the uploaded state at *time_io until time
 * exceeds simulation_time or max_steps steps ran: writes
 * <dir>/data/<t>.csv at the start and whenever time - last_save > save_time
 * (every step with save_every_step), <dir>/dump/<t>.csv when use_dump and
 * time - last_dump > dump_time, and <dir>/crash_dump_<t>.csv when a
 * CONSISTENCY_STOP bounds check fails (use_crash_dump), then returns its
 * error. Names use the reference's time formatting (TimeFormat.cpp:36-53).
 * Layers are formatted on writer threads while the GPU keeps stepping; the
 * call returns after every file is written. *steps_done (may be NULL)
 * receives the number of steps run. */
int rrsph_run(rrsph_solver* s, const char* experiment_dir, double* time_io,
              uint64_t max_steps, uint64_t* steps_done);
/* Sticky RRSPH_FLAG_* bits raised by device checks since the last clear. */
int rrsph_status(rrsph_solver* s, uint32_t* flags, int clear);

/* Global checks of the current state, summed in double on the device in a
 * fixed order (the same bits every call on the same state). No counterpart in
 * the reference: the mass and energy checks that stay in double beside the
 * FP32-mixed step. Fluid particles (itype > 0): mass, kinetic energy
 * m|v|^2/2, potential energy m g y, the Tait EOS's internal energy m e(rho)
 * (e = the integral of p/rho^2 from rho0) and momentum; boundary particles
 * (itype < 0): mass. Non-existent particles count nowhere. */
typedef struct rrsph_diagnostics {
    double mass;           /* fluid */
    double kinetic;        /* fluid */
    double potential;      /* fluid, g along -y */
    double internal;       /* fluid */
    double momentum[3];    /* fluid; [2] = 0 in 2D */
    double mass_boundary;  /* boundary particles */
    uint64_t fluid;        /* fluid particles */
    uint64_t boundary;     /* boundary particles */
} rrsph_diagnostics;
int rrsph_diagnostics_get(rrsph_solver* s, rrsph_diagnostics* out);
/* The rates of the last completed step: the accelerations a (the a_var that
 * update_acceleration wrote, UpdateAcceleration.cpp:33-125, stride `stride`)
 * and, with continuity density, drho (density_con, Density.h:63-114). Either
 * may be NULL. Zero after an upload, as the loop's fresh work arrays. */
int rrsph_download_rates(rrsph_solver* s, double* a, uint32_t stride, double* drho);
/* Directed neighbour pairs (the entries find_neighbours would list) of the
 * last completed step, and summed over the steps since rrsph_upload. */
int rrsph_pair_count(rrsph_solver* s, uint64_t* last_step, uint64_t* total);
/* What the last rrsph_step / rrsph_sync read back, without touching the
 * device: the time after its last step, the device flags, and the pairs of
 * rrsph_pair_count as of that call (any pointer may be NULL). All zero before
 * the first rrsph_step / rrsph_sync. */
int rrsph_last_report(rrsph_solver* s, double* time, uint32_t* flags, uint64_t* pairs_last,
                      uint64_t* pairs_total);
/* Current time step (changes under DT_CORRECTION_DYNAMIC with dt_dynamic_reduce). */
int rrsph_get_dt(rrsph_solver* s, double* dt);

/* ---- loop pieces, on the uploaded state (the reference's unit-test path) ---- */
/* make_grid (GridFind.cpp:47-88): keys[i] = Morton cell index of particle i
 * (get_cell_idx2/3, GridUtils.h:135-150); grid = particle ids sorted by
 * (cell, id); cells_start (max_cells+1 entries, may be NULL) = index of the
 * first grid entry of each cell, as after the reference's reverse scatter. */
int rrsph_grid_find(rrsph_solver* s, uint32_t* keys, uint32_t* grid,
                    uint32_t* cells_start);
/* find_neighbours (GridFind.cpp:112-189): counts[j] = number of neighbours of
 * particle j, list[j*max_per + n] = n-th neighbour in the reference's order
 * (3^dim cells x-major, ids ascending within a cell). Needs
 * counts[j] <= max_per; otherwise RRSPH_ERR_NEIGHBOUR_OVERFLOW. */
int rrsph_neighbours(rrsph_solver* s, uint32_t* counts, uint32_t* list,
                     uint32_t max_per, uint64_t* total_pairs);
/* The neighbour pairs the last completed step of the FP32-mixed solver with
 * neighbour reuse used: the list its density pass wrote (the candidates that
 * passed the reference's cutoff test of find_neighbours, GridFind.cpp:124,
 * 150-156, in float with a double re-test near the cutoff, or the stencil
 * search of a particle whose candidate list overflowed), as particle ids:
 * counts[j], list[j*max_per + n]. The order within a row is the candidate
 * order of the last list build, not the reference's; the sets are the
 * reference's. RRSPH_ERR_UNSUPPORTED for other solvers; RRSPH_ERR_INVALID_ARGUMENT
 * when no step has run since the last upload, loop-piece call or reuse
 * setting; RRSPH_ERR_NEIGHBOUR_OVERFLOW when a row does not fit max_per. */
int rrsph_step_neighbours(rrsph_solver* s, uint32_t* counts, uint32_t* list,
                          uint32_t max_per, uint64_t* total_pairs);
/* density_sum (Density.h:25-61) or density_con (Density.h:63-114) by
 * density_treatment, on r, v, rho of the uploaded state. Writes rho (summation)
 * or drho (continuity) into out_rho_or_drho and p into out_p, and stores rho/p
 * in the device state as the loop does. */
int rrsph_density(rrsph_solver* s, double* out_rho_or_drho, double* out_p);
/* Sum over neighbours of the selected terms (RRSPH_TERM_*), on r, v, rho, p of
 * the device state: a[j] (stride `stride`), av[j] (XSPH, may be NULL), mu[j] =
 * max |mu_ij| of the artificial viscosity (may be NULL). Terms also need their
 * params switch on (artificial_viscosity, average_velocity, boundary_treatment). */
int rrsph_forces(rrsph_solver* s, uint32_t terms, double* a, uint32_t stride,
                 double* av, double* mu);

/* ---- grid sort without allocation ----------------------------------------- */
/* Largest n rrsph_sort_pairs_noalloc accepts. */
#define RRSPH_SORT_NOALLOC_MAX_PAIRS (1u << 20)
/* Stable sort of n (cell key, particle id) pairs by the low key_bits bits of
 * the key: the grid sort rrsph_grid_find runs, for callers that cannot
 * allocate device memory (code whose device memory belongs to another
 * framework's pool, or a step loop that must not allocate because cudaMalloc
 * can block or fail mid-run). No counterpart in the reference.
 * Every pointer is a device pointer owned by the caller; the two outputs must
 * not overlap the inputs or each other (any overlap of the n-word ranges is
 * refused with RRSPH_ERR_INVALID_ARGUMENT), and the inputs are left unchanged.
 * A CUDA error already pending from the caller's earlier work is returned as
 * RRSPH_ERR_CUDA and left pending. The working memory is a
 * fixed array inside the library (about 9.4 MB; every GPU that loads the
 * library holds it until the process exits), so n is limited to
 * RRSPH_SORT_NOALLOC_MAX_PAIRS and a larger n returns
 * RRSPH_ERR_INVALID_ARGUMENT. The call allocates nothing and is asynchronous
 * on `stream` (a cudaStream_t; NULL = the default stream). Its first call on a
 * device looks up the array's device address and keeps it for the process;
 * make that first call before any stream capture, and do not call it on a
 * device after a cudaDeviceReset of that device. All calls on a device share the array, so calls that may
 * overlap on the GPU race: order them (one stream, or events). */
int rrsph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* ids_in,
                             uint32_t* keys_out, uint32_t* ids_out, uint32_t n,
                             uint32_t key_bits, void* stream);

/* ---- piston optimisation: Fourier piston and the adjoint of the loop -------- */
/* Maximum number of Fourier coefficients of rrsph_set_piston_fourier. */
#define RRSPH_PISTON_FOURIER_MAX 16
/* Replaces the velocity law of the piston (nwm == 2, dynamic_boundaries,
 * WaveMaker.cpp:34-82) by the displacement X(t) = sum_k coef[k-1] sin(k omega t),
 * k = 1..ncoef: every step the particles [nwm_particles_start,
 * nwm_particles_end) get v.x = X'(t) and r.x += X'(t) dt, as the reference's
 * piston does with its own law. ncoef = 0 restores the reference's law.
 * RRSPH_ERR_UNSUPPORTED unless nwm == 2. */
int rrsph_set_piston_fourier(rrsph_solver* s, uint32_t ncoef, double omega, const double* coef);

/* A forward run recorded for rrsph_adjoint_reverse. The gauge is the
 * reference's maxInLayer (tools/WaterProfile/include/HeightTesting.h:25-54):
 * the largest y > 0 over particles of itype == gauge_type (0: any) with
 * |x - gauge_x| < gauge_search_n * hsml, sampled on the states after
 * sample_from, sample_from + sample_every, ... <= nsteps steps. */
typedef struct rrsph_adjoint_config {
    uint32_t struct_size;        /* sizeof(rrsph_adjoint_config) */
    uint32_t checkpoint_every;   /* K >= 1: the state is stored every K steps, the steps in between are recomputed */
    uint64_t nsteps;
    double gauge_x;
    double gauge_search_n;
    int32_t gauge_type;
    uint32_t sample_every;       /* >= 1 */
    uint64_t sample_from;
} rrsph_adjoint_config;

/* Runs cfg->nsteps steps of the FP64 loop from the uploaded state at *time_io,
 * storing checkpoints, and returns the gauge series (gauges[s], s <
 * *nsamples <= max_samples). Method set: FP64 solver, 2D, summation density,
 * cubic kernel, no artificial pressure / XSPH, constant dt, no wall-disappear
 * wave maker; otherwise RRSPH_ERR_UNSUPPORTED. */
int rrsph_adjoint_forward(rrsph_solver* s, const rrsph_adjoint_config* cfg, double* time_io, double* gauges,
                          uint64_t max_samples, uint64_t* nsamples);
/* Reverse sweep of the last rrsph_adjoint_forward: given dL/dgauge[s], returns
 * dL/dcoef[k] of the Fourier piston (dcoef may be NULL; ncoef entries) and
 * dL/d(piston velocity of step n) (dpiston_vx may be NULL; nsteps entries).
 * Each step's adjoint is a gather over the step's neighbour pairs (recomputed
 * from the checkpoints; no atomics). The solver's state afterwards is the
 * state at the end of the forward run. */
int rrsph_adjoint_reverse(rrsph_solver* s, const double* dgauges, double* dcoef, double* dpiston_vx);

/* ---- ensembles of tanks and tuning ---------------------------------------- */
/* One piston of an ensemble: the particles [particles_start, particles_end)
 * move with dynamic_boundaries' law (WaveMaker.cpp:34-82) built from these
 * parameters, as the params' nwm_* fields build it for a single experiment
 * (wave number 2 pi / wave_length, frequency sqrt(g k tanh(k depth)),
 * Input.cpp:125-137). */
typedef struct rrsph_wave_maker {
    uint64_t particles_start, particles_end;
    uint32_t nwm;            /* 2: first order, 3: second order */
    uint32_t reserved;
    double time_start, phase, wave_length, wave_magnitude, depth;
} rrsph_wave_maker;
/* Replaces the params' wave maker by a table of pistons, one per tank of an
 * ensemble packed into one particle set (count = 0 restores the params' wave
 * maker). Ranges must not overlap. */
int rrsph_set_wave_makers(rrsph_solver* s, uint32_t count, const rrsph_wave_maker* makers);
/* Block sizes of the density and force gathers (multiples of 32, <= 256). */
int rrsph_set_gather_threads(rrsph_solver* s, uint32_t density_threads, uint32_t force_threads);
/* Autotuner: times `steps` steps on the uploaded state for every pair of
 * candidate gather block sizes (64, 128, 256), keeps the fastest and puts the
 * state back. threads_out[2] (may be NULL) receives {density, forces}. */
int rrsph_autotune(rrsph_solver* s, uint32_t steps, uint32_t* threads_out);
/* Autotuner of the candidate lists' skin (the FP32-mixed step with neighbour
 * reuse): for skins of 0.2, 0.3, 0.4, 0.5, 0.6 and 0.8 hsml in turn, rebuilds
 * the grid and lists of the uploaded state, runs two untimed steps, times
 * `steps` steps (with the rebuilds that skin asks for) and puts the state
 * back; keeps the fastest skin, and the next step rebuilds. A trial of a few
 * tens of steps weighs the rebuild frequency. skin_out (may be NULL)
 * receives the skin in hsml. RRSPH_ERR_UNSUPPORTED for other solvers. */
int rrsph_autotune_skin(rrsph_solver* s, uint32_t steps, double* skin_out);

/* Neighbour reuse of the FP32-mixed step, 2D or 3D, summation or continuity
 * density (on by default there): each particle's candidate list holds the particles within
 * (cell_scale_k + skin_over_h) * hsml of it at the last grid build, and the
 * grid and lists are rebuilt only when a particle has moved more than half the
 * skin since then, so every pair within the cutoff stays in the lists. Each
 * step still applies the reference's cutoff test to the list: the pairs are
 * the reference's. The skin defaults to 0.5 hsml in 2D and 0.3 hsml in 3D;
 * skin_over_h = 0 keeps the current one. Every call makes the next step
 * rebuild the grid and the lists. RRSPH_ERR_UNSUPPORTED for other solvers. */
int rrsph_set_neighbour_reuse(rrsph_solver* s, int enable, double skin_over_h);
/* Grid + list rebuilds since the solver was created (0 without reuse). */
int rrsph_neighbour_rebuilds(rrsph_solver* s, uint64_t* rebuilds);

/* ---- timing hooks for benchmarks ------------------------------------------ */
/* Number of kernel phases one step launches and their names. */
int rrsph_phase_count(rrsph_solver* s, int* count);
const char* rrsph_phase_name(rrsph_solver* s, int phase);
/* When enabled, rrsph_step records CUDA events around every phase; the
 * accumulated milliseconds per phase (since the last reset) and the number of
 * steps are returned by rrsph_phase_times. Enabling it disables graph replay. */
int rrsph_set_phase_timing(rrsph_solver* s, int enable);
int rrsph_phase_times(rrsph_solver* s, double* ms_per_phase, int count,
                      uint64_t* steps, int reset);
/* Launches of the library's own kernels since creation (all phases). */
int rrsph_kernel_launches(rrsph_solver* s, uint64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* RRSPH_CUDA_H */
