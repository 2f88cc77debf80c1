/*
 * hgpu.h -- C ABI of the GB300-native finite-volume Euler update.
 *
 * This is the drop-in boundary for HydroGPU's OpenCL solver path
 * (KennethYeah/HydrodynamicsGPU).  The reference has no C ABI: its host app
 * drives C++ classes (HydroGPUApp -> ISolver/Solver -> Integrator -> OpenCL
 * kernels).  Each entry point below replaces one reference interface; the
 * replaced interface is cited beside it as file:line of the reference project.
 *
 * Conventions
 *  - Plain C types only; no exceptions cross this boundary.  Every function
 *    returns an hgpu_status (0 = HGPU_OK).
 *  - State arrays use the reference layout: array-of-structures, ghost cells
 *    included, element (state j, cell x,y,z) at
 *        j + N * (x + SIZE_X * (y + SIZE_Y * z))
 *    (res/include/HydroGPU/Shared/Common.h:59-60, res/Roe.cl:106-108), with
 *    N = dim + 2 conserved states: density, momentum x..(dim), total energy
 *    (src/Equation/Euler.cpp:36-40).
 *  - Element type is double for HGPU_FP64 solvers and float for HGPU_FP32.
 *  - The library owns all device memory.  A handle is used by one host thread
 *    at a time; different handles are independent.
 */
#ifndef HGPU_HGPU_H
#define HGPU_HGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HGPU_ABI_VERSION 1

/* ---- status codes (replace the reference's C++ exceptions:
 *      src/Solver/Solver.cpp:150,201; src/HydroGPUApp.cpp:347,509) ---- */
typedef enum hgpu_status {
    HGPU_OK = 0,
    HGPU_ERR_CONFIG = 1,      /* invalid configuration value                  */
    HGPU_ERR_CUDA = 2,        /* a CUDA runtime/driver call failed            */
    HGPU_ERR_NONFINITE = 3,   /* NaN/Inf in the CFL reduction or the state    */
    HGPU_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up           */
    HGPU_ERR_OOB = 5,         /* a size/offset argument is out of range       */
    HGPU_ERR_ARG = 6,         /* NULL handle/pointer or wrong element count   */
    HGPU_ERR_UNSUPPORTED = 7, /* combination not provided by this build       */
    HGPU_ERR_NOMEM = 8,       /* device allocation failed                     */
    HGPU_ERR_UNPHYSICAL = 9   /* density or pressure <= 0 in the state (strict health mode) */
} hgpu_status;

/* ---- solver family (src/HydroGPUApp.cpp:90-118 solver registry) ---- */
enum {
    HGPU_SOLVER_ROE = 0,   /* "EulerRoe"  (src/Solver/EulerRoe.cpp)  */
    HGPU_SOLVER_HLLC = 1,  /* "EulerHLLC" (src/Solver/EulerHLLC.cpp) */
    HGPU_SOLVER_HLL = 2    /* "EulerHLL"  (src/Solver/EulerHLL.cpp, res/EulerHLL.cl) */
};

/* ---- boundary methods (include/HydroGPU/Boundary/Boundary.h:8-14; the
 *      "MIRROR" method reflects the normal momentum, src/Equation/Euler.cpp:63-75) ---- */
enum {
    HGPU_BOUNDARY_NONE = -1,
    HGPU_BOUNDARY_PERIODIC = 0,
    HGPU_BOUNDARY_MIRROR = 1,
    HGPU_BOUNDARY_FREEFLOW = 2
};

/* ---- slope limiters, in the order of res/SlopeLimiter.cl:5-68 ---- */
enum {
    HGPU_LIMITER_DONORCELL = 0,
    HGPU_LIMITER_LAXWENDROFF,
    HGPU_LIMITER_BEAMWARMING,
    HGPU_LIMITER_FROMM,
    HGPU_LIMITER_CHARM,
    HGPU_LIMITER_HCUS,
    HGPU_LIMITER_HQUICK,
    HGPU_LIMITER_KOREN,
    HGPU_LIMITER_MINMOD,
    HGPU_LIMITER_OSHKER,
    HGPU_LIMITER_OSPRE,
    HGPU_LIMITER_SMART,
    HGPU_LIMITER_SWEBY,
    HGPU_LIMITER_UMIST,
    HGPU_LIMITER_VANALBADA1,
    HGPU_LIMITER_VANALBADA2,
    HGPU_LIMITER_VANLEER,
    HGPU_LIMITER_MONOTIZEDCENTRAL,
    HGPU_LIMITER_SUPERBEE,
    HGPU_LIMITER_BARTHJESPERSEN,
    HGPU_NUM_LIMITERS
};

/* ---- integrators (src/Solver/Solver.cpp:178-204 registry;
 *      tableaus include/HydroGPU/Integrator/RungeKutta.h:129-294).
 *      BackwardEulerConjugateGradient is not provided: the reference's
 *      version throws unconditionally (src/Integrator/BackwardEulerConjugateGradient.cpp:80). ---- */
enum {
    HGPU_INTEGRATOR_FORWARD_EULER = 0,
    HGPU_INTEGRATOR_RK2,            /* RungeKutta2 (midpoint)   */
    HGPU_INTEGRATOR_RK2_HEUN,
    HGPU_INTEGRATOR_RK2_RALSTON,
    HGPU_INTEGRATOR_RK3,
    HGPU_INTEGRATOR_RK4,
    HGPU_INTEGRATOR_RK4_38,         /* RungeKutta4_3_8thsRule   */
    HGPU_INTEGRATOR_RK2_TVD,
    HGPU_INTEGRATOR_RK2_NONTVD,
    HGPU_INTEGRATOR_RK3_TVD,
    HGPU_INTEGRATOR_RK4_TVD,
    HGPU_INTEGRATOR_RK4_NONTVD,
    HGPU_NUM_INTEGRATORS
};

enum { HGPU_FP64 = 0, HGPU_FP32 = 1 };

/* Numerical compatibility.
 *  HGPU_COMPAT_REF : reproduce the reference step exactly, including its
 *                    6-significant-digit DX literals, frozen per-step eigenbasis,
 *                    never-written (zero) Delta-q-tilde at faces 1 and SIZE-1 and
 *                    stale stage ghost cells.
 *  HGPU_COMPAT_SEAM: same scheme, but eigenbasis/Delta-q-tilde also on faces 1 and
 *                    SIZE-1 and a ghost refresh of every stage state, so periodic
 *                    domains conserve totals to round-off. */
enum { HGPU_COMPAT_REF = 0, HGPU_COMPAT_SEAM = 1 };

/* Headless equivalent of the HydroGPUApp config fields the solver path reads
 * (include/HydroGPU/HydroGPUApp.h:72-94; src/HydroGPUApp.cpp:164-208;
 *  src/Solver/Solver.cpp:285-307). */
typedef struct hgpu_config {
    int solver;            /* HGPU_SOLVER_*                                              */
    int dim;               /* 1..3, or 0 = last axis with size > 1 (HydroGPUApp.cpp:214-221) */
    int size[3];           /* cells per axis INCLUDING 2 ghost layers per side; 1 = unused */
    double xmin[3];        /* domain spans all SIZE cells; dx = (xmax-xmin)/size          */
    double xmax[3];
    double gamma;          /* defs.idealGas_heatCapacityRatio (Lua number)               */
    float cfl;             /* a C float, as in HydroGPUApp.h:84                           */
    int use_fixed_dt;
    double fixed_dt;
    int boundary[3][2];    /* [axis][min,max] of HGPU_BOUNDARY_*                          */
    int limiter;           /* HGPU_LIMITER_* ("slopeLimiter" key, Solver.cpp:285-287)     */
    int integrator;        /* HGPU_INTEGRATOR_* ("integratorName" key)                    */
    int precision;         /* HGPU_FP64 / HGPU_FP32                                       */
    int compat;            /* HGPU_COMPAT_*                                               */
    /* self-gravity (src/Solver/SelfGravitation.cpp:35-124, res/SelfGravitation.cl) */
    int use_gravity;       /* "useGravity" (config.lua:65; HydroGPUApp.cpp:77, 207)      */
    int gauss_seidel_max_iter;   /* "gaussSeidelMaxIter" (config.lua:68; HydroGPUApp.cpp:78, 208) */
    double gravitational_constant; /* defs.selfGrav_gravitationalConstant (config.lua:74) */
    int reserved[4];       /* zero                                                        */
} hgpu_config;

typedef struct hgpu_solver hgpu_solver;  /* opaque handle */

/* Fill *cfg with the reference's defaults (HydroGPUApp.cpp:60-126 constructor:
 * cfl .5, fixedDT .001, xmin -.5, xmax .5; Solver.cpp:285 Superbee;
 * Solver.cpp:196 ForwardEuler) for a 2D 256x256 EulerRoe run. */
int hgpu_config_default(hgpu_config* cfg);

/* Fill *cfg from a config.lua-style settings file: replaces the Lua configuration
 * the reference host reads through LuaCxx (src/HydroGPUApp.cpp:157-208, :330;
 * src/Solver/Solver.cpp:196-197, 285-307; res/config.lua:26-94).  The file holds
 * assignments of literal values (numbers with arithmetic, strings, booleans,
 * tables, reads of names assigned earlier); keys read: solverName, integratorName,
 * slopeLimiter (not slopeLimiterName, which the reference never reads), size,
 * xmin, xmax, boundaryMethods, cfl, useFixedDT, fixedDT, useGravity,
 * gaussSeidelMaxIter, defs.idealGas_heatCapacityRatio and
 * defs.selfGrav_gravitationalConstant; absent keys keep hgpu_config_default's
 * values.  Statements that need a Lua interpreter (require, function calls, if,
 * function definitions) are refused with HGPU_ERR_CONFIG and their line number
 * (hgpu_last_error); a missing solverName (the reference default EulerBurgers) or
 * BackwardEulerConjugateGradient with HGPU_ERR_UNSUPPORTED.  *cfg is written only
 * on success. */
int hgpu_config_from_file(const char* path, hgpu_config* cfg);
/* The same from the text of such a file. */
int hgpu_config_from_string(const char* text, hgpu_config* cfg);

/* Human-readable name of a status code. */
const char* hgpu_status_string(int status);

/* Message of the last failure on the calling thread ("" if none). */
const char* hgpu_last_error(void);

/* Validate cfg and create a solver: replaces Solver::init (src/Solver/Solver.cpp:48-205),
 * i.e. NDRange setup, program build, initBuffers/initKernels and integrator selection.
 * Allocates every device buffer the step needs; later calls allocate nothing. */
int hgpu_create(const hgpu_config* cfg, hgpu_solver** out);

/* Free the handle and all device memory it owns. */
int hgpu_destroy(hgpu_solver* s);

/* Number of cells V = size[0]*size[1]*size[2] and states N of a solver. */
int hgpu_get_shape(const hgpu_solver* s, int* dim, int* num_states, size_t* volume);

/* Upload a full state (ghosts included, AoS): replaces Solver::resetState's
 * Converter::toGPU (src/Solver/Solver.cpp:333-337) and SelfGravitation::resetState
 * (SelfGravitation.cpp:35-98) with a zero potential channel.  count = V*N elements
 * of the solver's precision.  With use_gravity the potential starts as -density,
 * is relaxed 100 x gauss_seidel_max_iter times (ghost fill, then one relaxation
 * sweep) and the starting guess is added to the total energy, as the reference does. */
int hgpu_set_state(hgpu_solver* s, const void* host_state, size_t count);

/* The same with the initial conditions' potential channel (V elements, or NULL for
 * zero; SelfGravitationBehavior's Converter, include/HydroGPU/Solver/
 * SelfGravitationBehavior.h:54-96): without use_gravity it is uploaded as the
 * potential (a static field the step's flux and gravity source then see) and added
 * to the total energy; with use_gravity it is replaced by -density as above. */
int hgpu_set_state_potential(hgpu_solver* s, const void* host_state, size_t count, const void* host_potential,
                             size_t potential_count);

/* Download the gravitational potential (V elements, ghosts included): the potential
 * half of the Converter's fromGPU (SelfGravitationBehavior.h:84-90). */
int hgpu_get_potential(hgpu_solver* s, void* host_potential, size_t count);

/* Download the full state: replaces Converter::fromGPU (Solver.cpp:339-342). */
int hgpu_get_state(hgpu_solver* s, void* host_state, size_t count);

/* Advance nsteps time steps: each is Solver::update (src/Solver/Solver.cpp:521-546)
 * = boundary(); initStep(); dt = useFixedDT ? fixedDT : calcTimestep(); step(dt)
 * with EulerRoe::step / EulerHLL::step including SelfGravitation::applyPotential
 * (src/Solver/EulerRoe.cpp:31-34, EulerHLL.cpp:25-28).  dt stays on the device;
 * the call returns after the last step's work is queued and, if last_dt is
 * non-NULL, after it finished, with that step's dt.  */
int hgpu_update(hgpu_solver* s, int nsteps, double* last_dt);

/* The same call under the name a step-oriented binding uses. */
int hgpu_step(hgpu_solver* s, int nsteps, double* last_dt);

/* Upload, advance, download in one call: host_in -> Converter::toGPU + resetState
 * (Solver.cpp:333-337, as hgpu_set_state), nsteps x Solver::update (as hgpu_update),
 * then Converter::fromGPU (Solver.cpp:339-342) into host_out, with the same bits as
 * those three calls.  In 2D and 3D without a fixed dt, gravity or a static
 * potential, the copies are cut into bands along the slowest axis and overlapped
 * with the first step's ghost fill and eigenbasis (EulerRoe) or wave speeds
 * (EulerHLLC, EulerHLL) and with the last step's final combine; page-locked host
 * buffers let them run asynchronously.  host_in and host_out (in_count = out_count
 * = the state's element count) may be the same buffer.  Returns after the download,
 * with the last step's dt in last_dt. */
int hgpu_update_host(hgpu_solver* s, const void* host_in, size_t in_count, int nsteps, void* host_out,
                     size_t out_count, double* last_dt);

/* dt of the most recent step (blocks on the solver's stream). */
int hgpu_last_dt(hgpu_solver* s, double* dt);

/* Wait for queued work; returns HGPU_ERR_NONFINITE if a step saw NaN in the
 * CFL reduction (health word), HGPU_ERR_CUDA on a CUDA error. */
int hgpu_synchronize(hgpu_solver* s);

/* ---- failure detection.  The reference has none (it only throws at set-up:
 *      src/Solver/Solver.cpp:150-153, 201); here every step ends, and every upload
 *      is followed, by a check of the state's interior cells on the device. ---- */
#define HGPU_HEALTH_NONFINITE_DT    1u   /* a NaN in the CFL reduction                            */
#define HGPU_HEALTH_HLLC_NOBRANCH   2u   /* an HLLC interface where no flux branch was taken       */
#define HGPU_HEALTH_STATE_NONFINITE 4u   /* a NaN or infinity in a checked state                   */
#define HGPU_HEALTH_STATE_DENSITY   8u   /* density <= 0 in a checked state                        */
#define HGPU_HEALTH_STATE_PRESSURE 16u   /* pressure <= 0: 2 rho (E - rho phi) <= |m|^2, rounded   */
#define HGPU_HEALTH_COPY_TIMEOUT   32u   /* a bounded wait for a bulk copy gave up (work skipped)  */

/* Read and clear the device-side health word (HGPU_HEALTH_* bits, ORed since the
 * last read). */
int hgpu_health(hgpu_solver* s, uint32_t* flags);

/* What the state check does: HGPU_HEALTH_OFF skips it; HGPU_HEALTH_RECORD (the
 * default) sets the health bits; HGPU_HEALTH_STRICT also makes hgpu_set_state,
 * hgpu_set_state_potential, hgpu_update and hgpu_update_host wait for the stream and
 * return HGPU_ERR_NONFINITE (non-finite state or dt) or HGPU_ERR_UNPHYSICAL
 * (density or pressure <= 0) while such bits are set; the state is still written
 * and the bits stay set until hgpu_health reads them.  The check reads the state
 * once per step (one kernel). */
enum { HGPU_HEALTH_OFF = 0, HGPU_HEALTH_RECORD = 1, HGPU_HEALTH_STRICT = 2 };
int hgpu_set_health_mode(hgpu_solver* s, int mode);

/* Device pointer of the current state buffer (for device-resident pipelines;
 * the buffer is owned by the solver). */
int hgpu_state_device_ptr(hgpu_solver* s, void** dptr);

/* CUDA stream the solver launches on (a cudaStream_t). */
int hgpu_stream(hgpu_solver* s, void** stream);

/* Use CUDA-graph replay for hgpu_update (default on; off runs the same kernels
 * as plain launches). */
int hgpu_set_graphs(hgpu_solver* s, int enabled);

/* Run each Runge-Kutta stage as two fused per-direction kernels instead of four
 * (EulerRoe, FP64, 2D, a Runge-Kutta integrator; HGPU_ERR_UNSUPPORTED otherwise):
 * the reference's calcDeltaQTilde, calcFlux, calcFluxDeriv and multAdd of a stage
 * (src/Solver/Roe.cpp:101-112, res/Roe.cl:152-320, res/CalcFluxDeriv.cl:7-44,
 * res/Common.cl:201-210) become an x pass (stage rows staged by bulk copies; the
 * Delta-q-tilde and limited flux of x faces in shared memory; the x part of each
 * cell's divergence) and a y pass (stage rows staged by 2D tensor copies while it
 * marches down 32-column strips; y faces, divergence and the integrator's combine).
 * Same operations, same bits as the default four kernels.  Off by default. */
int hgpu_set_fused_stages(hgpu_solver* s, int enabled);

/* Number of kernels one step launches (for launch accounting). */
int hgpu_kernels_per_step(const hgpu_solver* s, int* count);

/* Make `device` current for this thread's later hgpu_create calls (the library
 * carries its own CUDA runtime state).  Replica runs use one device per process. */
int hgpu_select_device(int device);

/* Advance nsteps like hgpu_update and return their device time in milliseconds,
 * measured with CUDA events recorded on the solver's stream around the steps. */
int hgpu_timed_update(hgpu_solver* s, int nsteps, float* ms);

/* Per-kernel device time of nsteps updates run as plain launches, each launch
 * bracketed by CUDA events on the solver's stream.  Fills up to cap entries. */
typedef struct hgpu_kernel_time {
    char name[32];
    int launches;
    double total_ms;
} hgpu_kernel_time;
int hgpu_profile_update(hgpu_solver* s, int nsteps, hgpu_kernel_time* out, int cap, int* count);

/* Page-locked host buffers for state transfers (cudaHostAlloc / cudaFreeHost). */
int hgpu_host_alloc(size_t bytes, void** ptr);
int hgpu_host_free(void* ptr);

/* ---- output ----
 * The display scalar of every cell (ghosts included), as the reference's
 * convertToTex (res/EulerMHDCommon.cl:4-116) computes it for its texture, into a
 * headless buffer: one float per cell.  `method` is the reference's DISPLAY_* index,
 * numbered per dimension (src/Equation/Euler.cpp:18-27): DENSITY, VELOCITY,
 * VELOCITY_X, [VELOCITY_Y], [VELOCITY_Z], PRESSURE, ENERGY_INTERNAL, ENERGY_KINETIC,
 * ENERGY_TOTAL, POTENTIAL (7 + dim methods). */
int hgpu_display(hgpu_solver* s, int method, float* host_out, size_t count);
/* Same into a caller-owned DEVICE array of volume floats, queued on the solver's stream. */
int hgpu_display_device(hgpu_solver* s, int method, void* d_out);
/* Solver::save (src/Solver/Solver.cpp:549-589): one FITS file per channel
 * (DENSITY, MOMENTUM_X.., ENERGY_TOTAL, potential) named <channel><index>.fits in
 * `directory`, index = the first one whose DENSITY file does not exist; 32-bit
 * float images of size[0] x size[1] x size[2]. */
int hgpu_save_fits(hgpu_solver* s, const char* directory, int* save_index);

/* ---- batches of independent problems ----
 * No reference counterpart: the reference runs one problem per process
 * (src/HydroGPUApp.cpp:330-349).  A batch holds problems of the same solver, dim,
 * integrator, limiter, precision and use_fixed_dt, each with its own size, domain,
 * gamma, cfl, boundary methods and dt; every step of all of them is one CUDA graph of
 * persistent launches that pull work tiles from an atomic queue.  Each problem's
 * result is bit-identical to running it alone with hgpu_update. */
typedef struct hgpu_batch hgpu_batch;

typedef struct hgpu_batch_tuning {
    int tile_x, tile_y, tile_z;   /* cells per work tile (product <= 256 x cells_per_thread) */
    int staged;                   /* Roe eigenbasis: per-cell values via shared memory
                                     (tiles of at most 256 cells)                        */
    int blocks_per_sm;            /* persistent blocks per SM pulling tiles from the queue,
                                     0 = occupancy limit; -1 = one block per tile, no queue */
    int split_flux;               /* FP64 EulerRoe: the flux in two passes (corrections,
                                     then transforms) instead of one                     */
    int cells_per_thread;         /* 1..8: threads per cell = 1 / cells_per_thread       */
} hgpu_batch_tuning;

int hgpu_batch_create(const hgpu_config* cfgs, int nproblems, hgpu_batch** out);
int hgpu_batch_destroy(hgpu_batch* b);
int hgpu_batch_info(const hgpu_batch* b, int* nproblems, long long* total_cells, int* kernels_per_step);
/* Upload / download problem p's full state (AoS, ghosts included). */
int hgpu_batch_set_state(hgpu_batch* b, int problem, const void* host_state, size_t count);
int hgpu_batch_get_state(hgpu_batch* b, int problem, void* host_state, size_t count);
/* Advance every problem nsteps Solver::update steps (graph replays; returns when queued). */
int hgpu_batch_update(hgpu_batch* b, int nsteps);
/* The same call under the name a step-oriented binding uses. */
int hgpu_batch_step(hgpu_batch* b, int nsteps);
/* Same, returning the device time of the nsteps in milliseconds (CUDA events). */
int hgpu_batch_timed_update(hgpu_batch* b, int nsteps, float* ms);
/* dt of the most recent step of every problem (n = number of problems). */
int hgpu_batch_dts(hgpu_batch* b, double* dts, int n);
int hgpu_batch_health(hgpu_batch* b, uint32_t* flags);
/* Read and clear every problem's own health word (HGPU_HEALTH_STATE_* bits of the
 * state check that ends each batched step; n = number of problems).  No reference
 * counterpart (the reference has no run-time checks, src/Solver/Solver.cpp:150-153). */
int hgpu_batch_problem_health(hgpu_batch* b, uint32_t* flags, int n);
int hgpu_batch_get_tuning(const hgpu_batch* b, hgpu_batch_tuning* t);
int hgpu_batch_set_tuning(hgpu_batch* b, const hgpu_batch_tuning* t);
/* Time candidate tunings for `steps` steps each on this batch (its state is restored
 * afterwards) and keep the fastest; with a cache file the result is looked up first
 * and appended after tuning, keyed by the batch's shape. */
int hgpu_batch_autotune(hgpu_batch* b, const char* cache_path, int steps);

/* ---- differentiation (EulerRoe, FP64, REF scheme) ----
 * No reference counterpart: the reference runs the forward scheme only
 * (src/Solver/Roe.cpp:82-112).  The differentiated step is Solver::update with dt
 * held at a given value ("frozen"): ghost fill, eigenbasis of u^n, the integrator's
 * stages.  With the dt the CFL condition chose, the frozen step is bit-identical to
 * hgpu_update's step. */

/* Advance nsteps steps with the given dt per step (host array of nsteps values). */
int hgpu_update_frozen_dt(hgpu_solver* h, int nsteps, const double* dts);

/* One vector-Jacobian product: lambda_n = (d u^{n+1} / d u^n)^T lambda_next for the
 * step from u_n with dt.  All three are DEVICE arrays of the full state (AoS, ghosts
 * included); lambda_n must not alias lambda_next.  Runs on the solver's stream and
 * returns when queued; the solver's own state is not touched. */
int hgpu_adjoint_step(hgpu_solver* h, const void* d_u_n, const void* d_lambda_next, void* d_lambda_n, double dt);

/* Checkpointed trajectory of nsteps steps from the solver's current state: the
 * forward keeps the state every `every` steps (and each step's dt), the backward
 * recomputes one segment at a time and runs its reverse steps. */
typedef struct hgpu_checkpoint hgpu_checkpoint;
int hgpu_checkpoint_create(hgpu_solver* h, int nsteps, int every, hgpu_checkpoint** out);
/* The same trajectory with every step's tape recorded during the forward (the
 * adjoint's recording step: the same kernels and dt as hgpu_update), so the backward
 * runs the reverse steps only.  Memory: nsteps tapes (about 40 doubles per cell and
 * stage for 2D RK); HGPU_ERR_NOMEM when they do not fit.  The forward leaves the
 * final state in the solver like the checkpointed one (it runs no state check). */
int hgpu_checkpoint_create_taped(hgpu_solver* h, int nsteps, hgpu_checkpoint** out);
/* dts: nsteps frozen values, or NULL for the CFL dt of each step (recorded). */
int hgpu_checkpoint_forward(hgpu_checkpoint* c, const double* dts);
int hgpu_checkpoint_dts(hgpu_checkpoint* c, double* dts, int n);
/* lambda_0 = (d u^T / d u^0)^T lambda_T; DEVICE arrays of the full state. */
int hgpu_checkpoint_backward(hgpu_checkpoint* c, const void* d_lambda_T, void* d_lambda_0);
/* device time of the last forward and backward (CUDA events on the solver stream) */
int hgpu_checkpoint_times(hgpu_checkpoint* c, float* forward_ms, float* backward_ms);
int hgpu_checkpoint_destroy(hgpu_checkpoint* c);

/* CFL timestep of a ghost-filled device state without allocating device memory.
 * No counterpart in the reference: it is for callers that cannot call cudaMalloc
 * (hosts that own the whole device-memory budget through their own pool, code that
 * runs where allocation is forbidden, plug-in hosts that only lend their buffers).
 * Returns in *dt_out what Solver::calcTimestep would return for d_state (AoS, ghosts
 * included, the precision of cfg) with a zero gravitational potential, i.e. cfl * min
 * over interior cells and axes of the cell timestep, and blocks until it is on the
 * host; for a state a solver steps with a nonzero static potential it is not that
 * solver's dt.  Scratch is one fixed array inside the library (about 512 KiB, kept
 * until exit), so grids above 16,777,216 cells are rejected with HGPU_ERR_OOB.  The
 * library's module is loaded lazily: the first call on a device loads it, which
 * reserves the array on that device, and looks up the array's device address
 * (cudaGetSymbolAddress); make that first call at set-up, before the host's device
 * memory is handed to a pool and before any stream capture.  All calls share the
 * array: calls that overlap on the GPU (different streams or threads at once) race
 * and must be serialised by the caller.  `stream` is a cudaStream_t or NULL. */
int hgpu_cfl_timestep_noalloc(const hgpu_config* cfg, const void* d_state, double* dt_out, void* stream);

/* Checked build (the library compiled with HGPU_CHECKED, libhgpu_checked.so): every
 * cell index a kernel computes is tested against its grid and a violation is recorded
 * and skipped instead of trapping, and every device allocation carries guard bands of
 * a fixed byte pattern.  Waits for the device, then returns in *flags bit 0 (an index
 * outside a grid) and bit 1 (a guard band overwritten) since the last call, clears
 * them, and names the first finding in hgpu_last_error.  The reference has no checks
 * of its own (its 1D ghost kernels write out of bounds: res/Common.cl:97-194).  In
 * the normal build: HGPU_ERR_UNSUPPORTED. */
int hgpu_checked_status(uint32_t* flags);

/* Diagnostic: measured FP64 fused multiply-add issue rate of the current device
 * (fma instructions per second, all SMs), the denominator of the FP64 roofline. */
int hgpu_fp64_peak(double* fma_per_second);
/* Self-test of the kernels' integer-pipe binary64 product and quotient: compares
 * them bit for bit with the FP64 unit on `cases` seeded operand pairs (all exponent
 * ranges, short significands, zeros, subnormals, Inf, NaN) and returns the counts
 * of differing results (NaN == NaN). */
int hgpu_fp64_selftest(unsigned long long seed, long long cases, long long* mul_mismatches,
                       long long* div_mismatches);
/* Self-test of the kernels' bit-pattern MinMod and Superbee (FP64): compares them with
 * the res/SlopeLimiter.cl expressions under C-library fmin/fmax semantics, bit for bit
 * (signs of zero included), on `cases` seeded ratios; returns the mismatch count. */
int hgpu_limiter_selftest(unsigned long long seed, long long cases, long long* mismatches);

#ifdef __cplusplus
}
#endif

#endif /* HGPU_HGPU_H */
