/*
 * pd_gb300.h -- C ABI of the GB300 (sm_103a) implicit bond-based peridynamics
 * step: a drop-in for the PD path of SCI-Solver_Peridynamic's PeriCUDAEngine.
 *
 * The reference has no plugin or FFI layer; its boundary is the C++ classes
 * SystemParameter (src/core/parameters.h:146-162) and Simulator
 * (src/core/simulator.h:32-57).  Each entry point below names the reference
 * call it replaces.  All calls return a pd_status instead of calling exit()
 * (the reference's checkCudaErrors / TRUE_OR_DIE, src/core/helper_cuda.h:906-930,
 * src/core/utilities.h:27-36).  Pointers are host pointers; caller buffers are
 * copied; the handle owns every device allocation.  One handle per host
 * thread; calls on one handle are not re-entrant (as Simulator, which keeps
 * static CG objects, src/core/simulator.cu:745-757).
 *
 * Units: positions and lengths are in the simulation's internal units, as the
 * reference keeps them on the device (src/core/parameters.cu:409-429); the
 * PD_VAR_POSITION_SCALED export multiplies by scaleFactor as DataIO does
 * (src/core/memory_manager.cu:274-298).
 */
#ifndef PD_GB300_H
#define PD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PD_GB300_ABI_VERSION 5

typedef enum pd_status {
    PD_OK = 0,
    PD_ERR_INVALID_ARGUMENT = 1,
    PD_ERR_CUDA = 2,               /* a CUDA runtime call failed; see pd_last_error_message */
    PD_ERR_NOT_READY = 3,          /* pd_make_ready has not run */
    PD_ERR_BOND_OVERFLOW = 4,      /* a particle has more bonds than max_bonds_per_particle */
    PD_ERR_NO_DEVICE = 5,
    PD_ERR_FILE = 6,               /* parameter file could not be opened */
    PD_ERR_OUT_OF_MEMORY = 7,
    PD_ERR_STATE = 8               /* call out of order (e.g. set_particles after make_ready) */
} pd_status;

/* src/core/definitions.h:154-158 */
typedef enum pd_integrator { PD_IMPLICIT_EULER = 0, PD_NEWMARK_BETA = 1 } pd_integrator;

/* 0..3 are the reference's Activity enum (src/core/parameters.h:137-144).
 * PD_CLAMPED and PD_PRESCRIBED have no reference counterpart: a clamped
 * particle keeps velocity 0, a prescribed one keeps the velocity it was given;
 * both are Dirichlet rows of the implicit solve. */
typedef enum pd_activity {
    PD_ACTIVE = 0, PD_SEMI_ACTIVE = 1, PD_INACTIVE = 2, PD_INVISIBLE = 3,
    PD_CLAMPED = 4, PD_PRESCRIBED = 5
} pd_activity;

typedef enum pd_precision {
    PD_PRECISION_MIXED = 0,  /* FP32 forces/SpMV/CG vectors; FP64 stretch test, master state; ~FP64 dots */
    PD_PRECISION_FP64 = 1    /* every step quantity in FP64 */
} pd_precision;

/* The PD-path fields of SimulationParameters (src/core/parameters.h:16-88).
 * pd_params_derive fills the derived ones exactly as
 * SystemParameter::calculateDependentParameters (src/core/parameters.cu:351-453). */
typedef struct pd_sim_params {
    int num_pd_particle;
    int num_cell_x, num_cell_y, num_cell_z, num_cells;
    double cell_size;
    double sph_kernel_coeff;
    double pd_kernel_coeff;
    double sph_particle_mass;
    double pd_particle_mass;
    double boundary_min_x, boundary_min_y, boundary_min_z;
    double boundary_max_x, boundary_max_y, boundary_max_z;
    int pd_max_num_bonds;          /* output of make_ready */
    int pd_time_step;              /* ticks of the time-step base */
    double sph_particle_radius;
    double pd_particle_radius;     /* input: radius_pd_over_sph; after derive: radius (internal units) */
    double pd_horizon;
    double pd_C_times_V;
    double clockScale;
    double scaleFactor;
} pd_sim_params;

/* RunningParameters (src/core/parameters.h:90-135). */
typedef struct pd_run_params {
    int adaptive_integration;
    int gpu_device;
    int step_per_frame;
    int step_per_state;
    int start_step;
    int final_step;
    int wall_thickness;
    int tube_radius;
    float sph_initial_velocity;
    float mesh_translation_x, mesh_translation_y, mesh_translation_z;
    float pd_stretch_limit_s0;
    float pd_initial_velocity;
    int dump_activity, dump_density, dump_velocity, dump_pd_bond_list_top;
    int integrator;                /* pd_integrator */
    char obj_file[512];
    char saving_path[512];
} pd_run_params;

/* What the reference hard-codes in src/core/definitions.h, plus the knobs of
 * this implementation.  pd_solver_options_default gives the reference values. */
typedef struct pd_solver_options {
    int precision;                 /* pd_precision; default PD_PRECISION_MIXED */
    double cg_relative_tolerance;  /* CG_RELATIVE_TOLERANCE (1e-20), definitions.h:135 */
    int cg_max_iterations;         /* MAX_CG_ITERATION (100000), definitions.h:134 */
    double time_step_base;         /* SYSTEM_TIMESTEP_BASE (2^-23 s), definitions.h:65 */
    int time_step_min;             /* TIMESTEP_PD_MIN (100), definitions.h:69 */
    int max_substep;               /* MAX_SUBSTEP (10), definitions.h:71 */
    int phase_in_steps;            /* PHASEIN (30), definitions.h:103 */
    double pd_k;                   /* PD_K (5 * 2.94315e9), definitions.h:87 */
    double bond_stiffness;         /* > 0 overrides pd_C_times_V * PD_K (no reference counterpart) */
    double gravity[3];             /* acceleration; reference (0, -9.8, 0), cg_solver.cuh:330 */
    double restitution;            /* RESTITUTION (0.001), definitions.h:74 */
    int box_enabled;               /* 1: reflect at boundary_min/max +- radius (reference); 0: no walls */
    double stretch_a, stretch_b;   /* 10, 9 in (a - b*clockScale)*s0, cg_solver.cuh:326 */
    double alpha;                  /* alpha_pr (0.25), definitions.h:109 */
    int max_bonds_per_particle;    /* MAX_PD_BOND_COUNT (528), definitions.h:101 */
    /* rigid-sphere penalty contact (no reference counterpart) */
    int sphere_enabled;
    double sphere_center[3];       /* at simulated time 0 */
    double sphere_velocity[3];
    double sphere_radius;
    double sphere_stiffness;
    /* performance knobs: 0 = automatic */
    int lanes_per_particle;        /* 4, 8, 16 or 32 lanes cooperate on one bond row of the SpMV */
    int cg_check_interval;         /* CG iterations between convergence tests of the loop: the
                                      graph's while-node body (even, default 4) with cg_loop 0,
                                      a host batch (default 8) with cg_loop 1 */
    int spmv_unroll;               /* 1, 2 or 4 bonds loaded per lane before computing */
    /* CG initial guess (no reference counterpart for 1, 2 and 3): 0 = the
     * previous solution, as the reference (simulator.cu:745-770); 1 = previous
     * solution plus the learned correction of pd_ws_set_params' network (mixed
     * precision only); 2 = previous solution plus its Galerkin correction in
     * the span of the last history_size solutions (history projection, either
     * precision); 3 = as 2 with the network's predicted correction as one more
     * column of the projection (mixed precision; history_size <= 7): the
     * Galerkin solve weights it only as far as it lowers the A-norm error, so
     * the guess is never worse than 2's.  The CG still runs to the same
     * tolerance. */
    int warm_start;
    /* mixed-precision SpMV path: 2 = per-bond gathers from global memory;
     * 1 = shared-memory tiles of 256 consecutive rows and their halos
     * (measured slower than the gathers at 1M particles; kept as an option);
     * 3 = lattice stencil: for bodies whose particles each lie within 0.3
     * spacings (2 r) of a distinct site of a simple-cubic lattice -- as the
     * reference's Scene fills them -- the slots are renumbered brick by
     * brick and the product walks each row's stencil of lattice offsets over
     * the brick's halo staged in shared memory (other bodies fall back to
     * 2); 0 = automatic: from 20000 particles, 3 when the body is a lattice
     * fill, timed against the lanes x unroll shapes of 2 at make_ready (from
     * 250000 particles a lattice body takes 3 without timing the others).
     * pd_get_options reports the path in use (1, 2 or 3). */
    int spmv_path;
    /* PD-PD contact (collectPDParticles / collidePDParticles,
     * src/core/simulator.cuh:606-768, compiled out in the reference): every
     * two particles closer than contact_distance repel with
     * contact_stiffness * (r - d)^2 / contact_volume along their separation,
     * added to the force each step.  Defaults: off, FCELL *
     * PERIDYNAMICS_MIN_DISTANCE = 0.75 * 0.0005, Kc = 1e7, PD_V = 0.0005^3
     * (definitions.h:86-98). */
    int contact_enabled;
    double contact_distance;
    double contact_stiffness;
    double contact_volume;
    /* warm_start = 2: solutions kept for the projection, 1..8; 0 = 8 */
    int history_size;
    /* how the CG iterations of a step are driven (no reference counterpart:
     * the reference's CUSP cg loop tests on the host, simulator.cu:735-799):
     * 0 = a CUDA graph launched once per solve, whose while node repeats
     * cg_check_interval iterations until the device-side convergence test
     * stops it -- no host read-back inside the solve; 1 = batches of
     * iterations launched from the host, each followed by a read-back of the
     * test.  Both run the same kernels in the same order, so the results are
     * identical.  Default 0; a device where the graph cannot be built falls
     * back to 1 (pd_step_stats.cg_graph_solves stays 0). */
    int cg_loop;
    /* CG preconditioner (the reference's cusp::precond::diagonal is
     * commented out, simulator.cu:767-769, so it runs plain CG): 0 = none, as
     * the reference; 1 = the inverse diagonal of A (Jacobi); 2 = the inverse
     * 3x3 diagonal blocks of A (block Jacobi; a block that is not positive
     * definite takes 1's rule).  The stopping test stays ||r|| <= tol ||b||,
     * so the tolerance means the same.  Single handles only (a batch scene
     * with a preconditioner is rejected). */
    int preconditioner;
} pd_solver_options;

/* Export selectors for pd_get. */
typedef enum pd_variable {
    PD_VAR_POSITION = 0,           /* double[4n], internal units (w = 0) */
    PD_VAR_VELOCITY = 1,           /* double[4n] */
    PD_VAR_ACTIVITY = 2,           /* int32[n] */
    PD_VAR_BOND_COUNT = 3,         /* int32[n]: live bonds = pd_bond_list_top + 1 */
    PD_VAR_STRETCH = 4,            /* double[n]: pd_stretch */
    PD_VAR_ORIGINAL_STRETCH = 5,   /* double[n]: pd_original_stretch (s0_i) */
    PD_VAR_NEW_STRETCH = 6,        /* double[n]: pd_new_stretch of the last force pass */
    PD_VAR_FORCE = 7,              /* double[4n]: pd_force of the last force pass */
    PD_VAR_SOLUTION = 8,           /* double[4n]: pd_system_solution of the last solve */
    PD_VAR_BOND_ROW_PTR = 9,       /* int64[n+1]: row starts of the bond list below */
    PD_VAR_BOND_LIST = 10,         /* int32[total]: per particle, live neighbours ascending then broken ones ascending */
    PD_VAR_POSITION_SCALED = 11,   /* double[4n]: positions * scaleFactor (DataIO convention) */
    PD_VAR_ORIGINAL_POSITION = 12, /* double[4n]: pd_original_pos */
    PD_VAR_SLOT_PERMUTATION = 13,  /* int32[n]: caller index of each device slot (operator view order) */
    PD_VAR_BROKEN_MASK = 14        /* uint8[total]: 1 where the PD_VAR_BOND_LIST entry is a broken bond */
} pd_variable;

typedef struct pd_step_stats {
    int current_step;              /* Simulator::get_current_step */
    int cg_converged;              /* Simulator::CGConvergence */
    int last_cg_iterations;
    double last_cg_residual;       /* ||r|| at exit */
    double last_cg_tolerance;      /* rel_tol * ||b|| */
    long long total_cg_iterations;
    int time_step_ticks;           /* current pd_time_step */
    int substep;                   /* current_substep_ of the adaptive scheme */
    int retries_last_step;         /* integrate() calls that rolled back in the last advance */
    long long bonds_initial;
    long long bonds_alive;
    int max_bonds_per_particle;    /* pd_max_num_bonds */
    double clock_scale;
    double sim_time;               /* simulated seconds */
    long long ws_guesses_kept;     /* steps whose learned guess beat the previous solution, or
                                      (warm_start 2) whose history projection was applied */
    double last_ws_residual_ratio; /* ||r(guess)|| / ||r(previous solution)|| of the last step */
    long long ws_learned_used;     /* warm_start 3: projections that gave the network's column a nonzero weight */
    long long host_syncs;          /* host waits on the GPU inside pd_advance since pd_make_ready: the
                                      adaptive time step's test (Newmark-beta or adaptive_integration)
                                      and the read-back of each solve's result, plus one per host
                                      batch with cg_loop 1 */
    long long cg_graph_solves;     /* solves whose iterations ran in the CG graph (cg_loop 0) */
    long long ws_guesses_skipped;  /* batch learned warm start: steps whose learned pass was paused
                                      (3 guesses rejected in a row; retried every 16 steps) */
} pd_step_stats;

/* Device time per kernel class, accumulated with CUDA events on the handle's
 * stream while profiling is on (pd_set_profiling).  Force and update launches
 * are each timed; the CG loop's SpMV and vector launches are timed on every
 * 8th iteration and total_ms is their mean duration times the exact count of
 * live launches. */
typedef enum pd_kernel_class {
    PD_KC_FORCE = 0, PD_KC_SPMV = 1, PD_KC_CG_VECTOR = 2, PD_KC_UPDATE = 3,
    PD_KC_GUESS = 4,               /* initial-guess work of warm_start 2 (its products, Gram passes, update) */
    PD_KC_COUNT = 5
} pd_kernel_class;

typedef struct pd_kernel_times {
    long long launches[PD_KC_COUNT];
    double total_ms[PD_KC_COUNT];
} pd_kernel_times;

/* Device-side view of a handle's current linear system A = M + beta h^2 K
 * (beta = 1 implicit Euler, 1/4 Newmark), for applying the matrix-free
 * operator outside pd_advance: the role of the reference's
 * PeridynamicsMatrix linear operator (src/core/cg_solver.cuh:386-428).
 * Pointers are device pointers into the handle's state, valid until the next
 * pd_make_ready or pd_destroy.  Vectors are in slot order (perm[slot] = caller
 * index), 4 components per particle (float in mixed precision, double in
 * FP64 mode; w ignored).  Dirichlet rows (clamped, prescribed, invisible)
 * map to 0. */
typedef struct pd_operator_view {
    int n;                         /* particles */
    int precision;                 /* pd_precision of the vectors */
    int lanes_per_particle;        /* 4, 8, 16 or 32 */
    int blocks;                    /* thread blocks of a launch; 0 = automatic */
    const uint8_t* activity;       /* n: low 3 bits pd_activity, bit 3 = in sphere contact */
    const int32_t* row_ptr;        /* n + 1 */
    const int32_t* bond_count;     /* n: live bonds per row */
    const int32_t* bond_slot;      /* neighbour slots of each row */
    const int32_t* perm;           /* n: slot -> caller index */
    const void* ref_pos;           /* mixed: float4 original positions minus origin */
    const void* disp;              /* mixed: float4 displacement x - X */
    const void* pos_cell;          /* mixed: float4 position offset in its supercell, w = packed supercell coords */
    const float* inv_d0;           /* mixed: 1 / d0 per bond slot */
    double supercell_size;         /* mixed: supercell edge (a power of two) */
    const double* jac;             /* FP64: 6 entries per bond slot (xx yy zz xy xz yz) */
    const double* jac_diag;        /* FP64: 6 entries per particle */
    double mass;
    double t2;                     /* beta h^2 */
    double bond_coeff;
    double sphere_center_local[3]; /* sphere centre minus origin (mixed contact rows) */
    double sphere_stiffness;
} pd_operator_view;

typedef struct pd_handle pd_handle;

/* ---- parameters (SystemParameter, src/core/parameters.cu) ---------------- */

/* SystemParameter::initParameters (parameters.cu:40-86) + RunningParameters() (parameters.h:92-104) */
pd_status pd_params_default(pd_sim_params* sim, pd_run_params* run);
/* SystemParameter(const char*) (parameters.cu:21-25, 89-347): key/value file, then derive */
pd_status pd_params_load(const char* path, pd_sim_params* sim, pd_run_params* run);
/* SystemParameter::calculateDependentParameters (parameters.cu:351-453) */
pd_status pd_params_derive(pd_sim_params* sim, pd_run_params* run);
/* definitions.h constants; no reference call (they are compile-time there) */
pd_status pd_solver_options_default(pd_solver_options* opt);

/* ---- simulator (Simulator, src/core/simulator.h:32-57) -------------------- */

/* Simulator(int deviceID, SimulationParameters&, RunningParameters&) (simulator.cu:34-53).
 * opt may be NULL (reference defaults).  The device is run->gpu_device. */
pd_status pd_create(const pd_sim_params* sim, const pd_run_params* run,
                    const pd_solver_options* opt, pd_handle** out);
/* ~Simulator */
pd_status pd_destroy(pd_handle* h);
/* Replaces filling get_pd_position/get_pd_velocity/get_pd_activity host arrays
 * before makeReady (examples/main.cpp:64-66, examples/scene.cpp:360-395).
 * pos4, vel4: n*4 doubles (x, y, z, w; w is ignored).  activity may be NULL
 * (all PD_ACTIVE), vel4 may be NULL (zero).  n must equal num_pd_particle. */
pd_status pd_set_particles(pd_handle* h, const double* pos4, const double* vel4,
                           const int32_t* activity, int n);
/* Optional: per-particle stretch limits s0_i instead of getstretch() after
 * srand(1973) (simulator.cu:802-822, 852-857). */
pd_status pd_set_stretch_limits(pd_handle* h, const double* s0, int n);
/* Simulator::makeReady (simulator.cu:56-89): bonds on the GPU (uniform grid +
 * radix sort + CSR) instead of the host kd-tree (simulator.cu:825-943). */
pd_status pd_make_ready(pd_handle* h);
/* nsteps x Simulator::advance (simulator.cu:1159-1217).  Stops early when the
 * solver has not converged (finished() becomes true). */
pd_status pd_advance(pd_handle* h, int nsteps);
/* Simulator::finished (simulator.cu:141-144) */
pd_status pd_finished(pd_handle* h, int* finished);
/* Simulator::CGConvergence (simulator.cu:147-150) */
pd_status pd_cg_converged(pd_handle* h, int* converged);
/* Simulator::get_current_step (simulator.cu:153-156) */
pd_status pd_get_current_step(pd_handle* h, int* step);
/* Replaces get_pd_position/velocity/activity + MemoryManager::downloadFromDevice
 * (memory_manager.cu:274-298).  bytes must be at least the size of the export. */
pd_status pd_get(pd_handle* h, pd_variable var, void* dst, size_t bytes);
/* Size in bytes of an export (the bond list size is known after make_ready). */
pd_status pd_get_size(pd_handle* h, pd_variable var, size_t* bytes);
/* CG iterations / residual (simulator.cu:773-790 prints them) and step state */
pd_status pd_get_stats(pd_handle* h, pd_step_stats* stats);
/* Resolved solver options and simulation parameters in use (after derive). */
pd_status pd_get_params(pd_handle* h, pd_sim_params* sim, pd_run_params* run, pd_solver_options* opt);

/* ---- the system operator (PeridynamicsMatrix, src/core/cg_solver.cuh:386-428) */

/* Fills a view of the operator of the current step (after pd_make_ready; the
 * time step and contact state of the latest pd_advance). */
pd_status pd_get_operator_view(pd_handle* h, pd_operator_view* view);
/* y = A x on device vectors (PeridynamicsMatrix::operator(), which launches
 * computeAx, cg_solver.cuh:343-383, 414-427); *d_dot (device double, may be
 * NULL) receives <x, A x>.  Runs on the handle's stream with the handle's
 * scratch; returns after enqueueing. */
pd_status pd_apply_operator(pd_handle* h, const void* d_x, void* d_y, double* d_dot);

/* No counterpart in the reference.  pd_apply_operator without any device
 * allocation, for callers that cannot call cudaMalloc: a host application
 * that owns every device allocation and hands this library only pointers
 * into its own pool, or code that must not allocate inside a time-critical
 * loop.  The caller passes the view (e.g. from pd_get_operator_view), the
 * input and output vectors and the stream (NULL: the legacy default stream).
 * The reduction scratch is a static device array of this library (one FP64
 * partial per block for at most 4096 blocks plus a counter, ~33 KB on every
 * GPU that loads the library, kept until exit); a view asking for more than
 * 4096 blocks is rejected with PD_ERR_INVALID_ARGUMENT.  pd_get_operator_view
 * fills `blocks` with the handle's own grid, which exceeds 4096 on large
 * scenes: set view.blocks = 0 (automatic, at most 4096 blocks; every row is
 * still covered) before passing such a view.  The first call on a device
 * resolves the array's device address (one-time set-up), so make that first
 * call before any stream capture.  Call with the device that holds the
 * view's arrays current (a view on another device is rejected), in the
 * runtime's primary context; the resolved address is kept for the life of
 * the process and is not refreshed after cudaDeviceReset.  Every call shares
 * the array: calls whose launches overlap on the GPU race.  Calls no
 * cudaMalloc or cudaFree.  Returns after enqueueing; errors are read with
 * pd_last_error_message(NULL). */
pd_status pd_apply_operator_noalloc(const pd_operator_view* view, const void* d_x, void* d_y, double* d_dot,
                                    void* stream);

/* ---- learned CG warm start (no reference counterpart) ----------------------
 * A per-particle MLP (64 features -> 128 -> 128 -> 3, GELU; BF16 tensor-core
 * GEMMs with FP32 accumulation) predicts the change of the CG solution over
 * the previous solution.  Parameters are one FP32 blob of
 * pd_mlp_param_count() values: W1[64x128], b1[128], W2[128x128], b2[128],
 * W3[128x3], b3[3] (row-major, input x output). */
size_t pd_mlp_param_count(void);
/* Glorot-uniform initial parameters (output layer scaled by 0.1). */
pd_status pd_mlp_init(unsigned seed, float* params);
/* Y[rows x 3] = MLP(X[rows x 64]) on `device` (inputs rounded to BF16).
 * Inference runs as one tcgen05 kernel per 128-row tile (TMEM accumulators,
 * the three layers and their bias/GELU fused), as the warm start does each
 * step; training (loss_grad, train) runs each layer's products as separate
 * tcgen05 GEMMs. */
pd_status pd_mlp_predict(int device, const float* X, long long rows, const float* params, float* Y);
/* Mean squared error over rows (sum over the 3 outputs) and its gradient. */
pd_status pd_mlp_loss_grad(int device, const float* X, const float* T, int rows, const float* params, float* grad,
                           double* loss);
/* Adam training on the GPU (batches drawn without replacement per epoch);
 * params are read and overwritten; *final_loss = loss over all rows. */
pd_status pd_mlp_train(int device, const float* X, const float* T, long long rows, int iterations, int batch,
                       float lr, unsigned seed, float* params, double* final_loss);
/* Network used by warm_start = 1 on this handle. */
pd_status pd_ws_set_params(pd_handle* h, const float* params, size_t count);
pd_status pd_ws_get_params(pd_handle* h, float* params, size_t count);
/* Record up to samples_per_step (features, target) rows per step into a ring
 * buffer of `capacity` rows (0 disables); targets are (x_new - x_prev) / sigma. */
pd_status pd_ws_collect(pd_handle* h, int samples_per_step, long long capacity);
/* Copies the recorded rows (at most max_rows) to X[rows x 64], T[rows x 3]. */
pd_status pd_ws_dataset(pd_handle* h, float* X, float* T, long long max_rows, long long* rows);

/* ---- profiling (Monitor, src/core/monitor.cu:53-95) ----------------------- */
pd_status pd_set_profiling(pd_handle* h, int enabled);
pd_status pd_get_kernel_times(pd_handle* h, pd_kernel_times* t);
pd_status pd_reset_kernel_times(pd_handle* h);
/* Number of kernels this library launched on the handle's stream so far. */
pd_status pd_get_launch_count(pd_handle* h, long long* launches);
/* The cudaStream_t (as void*) every call of this handle runs on, e.g. to
 * record CUDA events around pd_advance. */
pd_status pd_get_stream(pd_handle* h, void** stream);
/* Waits until all work of the handle has finished on the device. */
pd_status pd_synchronize(pd_handle* h);

/* ---- DataIO (src/core/dataIO.h:20-44) -------------------------------------
 * Output under run->saving_path, as the reference's DataIO: frames
 * DATA/<VAR>/frame.<savedFrame> (raw arrays in caller order: PD_POSITION
 * double4 scaled by scaleFactor; with the run's dump_velocity /
 * dump_activity / dump_pd_bond_list_top also PD_VELOCITY double4,
 * PD_ACTIVITY int32, PD_ORIGINAL_BOND_COUNT and PD_BOND_LIST_TOP int32 as
 * counts - 1), DATA/sim_info.dat (the reference's SimulationParameters,
 * raw) and DATA/viz_info.dat.  Checkpoints go to DATA/STATE/state.<step>
 * (the folder the reference creates; its saveState writes STATE/, which it
 * never creates): the reference's leading savedFrame, then this library's
 * own state layout. */
/* DataIO::getDataAndWrite (dataIO.cu:82-124), creating the folders of
 * createOutputFolders (dataIO.cu:207-249) and sim_info on first use */
pd_status pd_dataio_get_data_and_write(pd_handle* h);
/* DataIO::newFrame (dataIO.cu:200-204) */
pd_status pd_dataio_new_frame(pd_handle* h);
/* DataIO::savedFrame */
pd_status pd_dataio_saved_frame(pd_handle* h, size_t* frame);
/* DataIO::saveState (dataIO.cu:150-175) */
pd_status pd_dataio_save_state(pd_handle* h, size_t timestep);
/* DataIO::loadState (dataIO.cu:178-203): into a handle made ready on the same
 * scene (same particles and bonds); the run then continues bit for bit.
 * Without DATA/STATE/state.<step> it reads the reference's own
 * STATE/state.<step> (pd_dataio_load_state_reference). */
pd_status pd_dataio_load_state(pd_handle* h, size_t timestep);
/* DataIO::saveState (dataIO.cu:123-150) in the reference's own layout, to
 * STATE/state.<step> under saving_path: savedFrame, then every MemoryManager
 * array (memory_manager.h:29-90) in enum order with the sizes of
 * memory_manager.cu:16-178 for the counts of DATA/sim_info.dat (written
 * first): positions times scaleFactor, bond lists bond-major
 * (list[j * num_pd_particle + p], live bonds first) with their tops and backup
 * tops; arrays this library does not keep (SPH, cells) are zeros, and the
 * system matrix is a hole of its length (the reference rebuilds it every
 * step). */
pd_status pd_dataio_save_state_reference(pd_handle* h, size_t timestep);
/* DataIO::loadState (dataIO.cu:152-198) of a file in the reference's layout,
 * sized by DATA/sim_info.dat of the same run, into a handle made ready on the
 * same scene (original positions and activity are checked): positions,
 * velocities and their backups, stretch limits, bond lists and tops, the CG
 * solution and savedFrame; pd_time_step and clockScale from sim_info.dat; the
 * step counter becomes `timestep` and the adaptive scheme's sub-step count 0
 * (the reference keeps both out of the file, in Simulator members): a state
 * saved while the halved time step was still in its sub-steps continues with
 * a fresh count. */
pd_status pd_dataio_load_state_reference(pd_handle* h, size_t timestep);

/* SPH <-> PD collision: the reference's collideDifferentParticles
 * (src/core/simulator.cuh:1590-1733, called after the PD step at
 * simulator.cu:1188-1206), for SPH particles the caller simulates itself
 * (this library has no SPH model).  sph_pos4 / sph_vel4: double[4 * n_sph]
 * host arrays in internal units, updated in place.  Every SPH particle whose
 * cell of the grid of sim (cell_size from boundary_min, num_cell_x/y/z) is
 * inside the grid and that has a PD particle closer than sph_particle_radius +
 * pd_particle_radius in the 27 cells around it is moved to that distance from
 * the nearest one, and the two exchange velocity: normal parts to the
 * mass-weighted mean, tangential parts mixed by (1 - slip) (slip = the
 * reference's sph_pd_slip, 1.0 by default).  The PD particle's velocity is
 * set on the handle (several SPH particles on one PD particle: the one of
 * the smallest index).  The PD positions and velocities are the handle's at
 * the call; the reference uses copies sorted at the start of its step and
 * reads the PD velocity from a wrong index.  collided (may be NULL): SPH
 * particles corrected. */
pd_status pd_sph_collide(pd_handle* h, double* sph_pos4, double* sph_vel4, int n_sph, double slip, int* collided);

/* ---- example scene: an OBJ mesh filled with particles (src/examples/scene.cpp) */
typedef struct pd_scene pd_scene;
/* Scene(simParams, runningParams, arrangement) (scene.cpp:18-135): reads
 * run->obj_file (cyTriMesh OBJ reading: v / f lines, polygons as fans), scales
 * the mesh to half of 0.9 x the smallest box extent with its minimum corner at
 * boundary_min, and keeps the points of a lattice of spacing 2 r inside the
 * mesh -- the inside test runs on the GPU (run->gpu_device) with exact
 * predicates.  jittered = 0: REGULAR_GRID; 1: JITTERED_GRID, offsets
 * (frand() * 2 - 1) * 0.01 r from the C library's rand() stream after
 * srand(jitter_seed) (1: the stream of a process that never called srand).
 * Sets sim->num_pd_particle. */
pd_status pd_scene_create(pd_sim_params* sim, const pd_run_params* run, int jittered, unsigned jitter_seed,
                          pd_scene** out);
pd_status pd_scene_particle_count(pd_scene* s, int* count);
/* Scene::initPeridynamicsParticles (scene.cpp:360-395): positions translated
 * by mesh_translation / scaleFactor, activity PD_ACTIVE, every velocity
 * component pd_initial_velocity.  Arrays of num_pd_particle entries
 * (pos4 / vel4: 4 doubles each). */
pd_status pd_scene_init_pd_particles(pd_scene* s, int32_t* activity, double* pos4, double* vel4);
pd_status pd_scene_destroy(pd_scene* s);
const char* pd_scene_last_error_message(void);

/* ---- batched scenes (no reference counterpart) -----------------------------
 * Many independent scenes (each with the parameter surface of one Simulator)
 * stepped together: per step, two cooperative persistent launches cover every
 * scene -- force passes and adaptive decisions, then the CG iterations of all
 * scenes until each has converged, then the update -- replayed from one CUDA
 * graph.  Each scene keeps its own step state, time step, CG scalars and
 * statistics, and gives the same results as a pd_handle of its own (within the
 * CG tolerance: per-scene sums are reduced in a different, fixed order).  All
 * scenes of a batch use the same precision.  Scenes are numbered in the order
 * of pd_batch_add_scene; "offsets" are the scenes' first particles in the
 * concatenation of all scenes in that order. */
typedef struct pd_batch pd_batch;

typedef struct pd_batch_options {
    int lanes_per_particle;   /* SpMV lanes per particle row: 4 or 8, 0 = autotune */
    int spmv_unroll;          /* 2 or 4, 0 = autotune */
    int item_rows;            /* rows per work item: 64..4096, 0 = autotune */
    int use_graph;            /* 1 (default): replay each step from a CUDA graph */
    /* CG initial guess of every scene (mixed precision only; the scenes'
     * own warm_start option is not used in a batch): 0 (default) = the
     * previous solution, as the reference; 1 = the previous solution plus the
     * learned correction of the network set by pd_batch_ws_set_params (one
     * network for all scenes, run once per step over the rows of every
     * scene), kept only where its residual is not larger -- the CG still
     * runs to each scene's tolerance.  No reference counterpart. */
    int warm_start;
} pd_batch_options;

/* The launch shape in use after pd_batch_make_ready. */
typedef struct pd_batch_config {
    int lanes_per_particle;
    int spmv_unroll;
    int item_rows;
    int work_items;
    int grid_pre;             /* blocks of the force/decision launch */
    int grid_cg;              /* blocks of the CG launch */
    int autotuned;            /* 1 when the shape was measured, 0 when fixed/default */
    double tuned_spmv_ms;     /* SpMV phase time of the chosen shape (autotuned only) */
    int warm_start;           /* the batch option in use */
} pd_batch_config;

pd_status pd_batch_options_default(pd_batch_options* opt);
/* device: CUDA device ordinal; opt may be NULL. */
pd_status pd_batch_create(int device, const pd_batch_options* opt, pd_batch** out);
pd_status pd_batch_destroy(pd_batch* b);
/* Adds a scene (as pd_create; opt may be NULL); its index is returned in *scene. */
pd_status pd_batch_add_scene(pd_batch* b, const pd_sim_params* sim, const pd_run_params* run,
                             const pd_solver_options* opt, int* scene);
/* As pd_set_particles / pd_set_stretch_limits for one scene. */
pd_status pd_batch_set_particles(pd_batch* b, int scene, const double* pos4, const double* vel4,
                                 const int32_t* activity, int n);
pd_status pd_batch_set_stretch_limits(pd_batch* b, int scene, const double* s0, int n);
/* Parameters of the warm-start network (pd_mlp_param_count() floats, as
 * pd_ws_set_params), before or after pd_batch_make_ready; without a call the
 * network starts from pd_mlp_init's seed-1 parameters.  No reference
 * counterpart. */
pd_status pd_batch_ws_set_params(pd_batch* b, const float* params, size_t count);
/* pd_make_ready of every scene, then work items, launch shape and graph. */
pd_status pd_batch_make_ready(pd_batch* b);
/* nsteps steps of every scene (a scene whose CG failed stops, as pd_advance). */
pd_status pd_batch_advance(pd_batch* b, int nsteps);
pd_status pd_batch_scene_count(pd_batch* b, int* count);
/* offsets[0..count]: first particle of each scene in the concatenation; offsets[count] = total. */
pd_status pd_batch_scene_offsets(pd_batch* b, int64_t* offsets, int count_plus_one);
/* Per-scene queries (as the pd_handle calls). */
pd_status pd_batch_get(pd_batch* b, int scene, pd_variable var, void* dst, size_t bytes);
pd_status pd_batch_get_size(pd_batch* b, int scene, pd_variable var, size_t* bytes);
pd_status pd_batch_get_stats(pd_batch* b, int scene, pd_step_stats* stats);
pd_status pd_batch_finished(pd_batch* b, int scene, int* finished);
pd_status pd_batch_get_config(pd_batch* b, pd_batch_config* config);
pd_status pd_batch_get_launch_count(pd_batch* b, long long* launches);
pd_status pd_batch_get_stream(pd_batch* b, void** stream);
pd_status pd_batch_synchronize(pd_batch* b);
/* Last error text of a batch. */
const char* pd_batch_last_error_message(pd_batch* b);

/* ---- errors --------------------------------------------------------------- */
const char* pd_status_string(pd_status s);
/* Last error text of a handle (or of the last failed pd_create when h is NULL). */
const char* pd_last_error_message(pd_handle* h);
/* ABI version of the loaded library. */
int pd_abi_version(void);

/* ---- host logic exposed for testing without a GPU ------------------------ */

/* glibc-compatible rand() stream: s0_i = getstretch(s0) after srand(1973)
 * (simulator.cu:802-822, 852-857), for i = 0..n-1. */
pd_status pd_sample_stretch_limits(float s0, int n, double* out);

/* One decision of the adaptive time-step scheme of integratePeridynamics*
 * (simulator.cu:332-401): given has_broken, updates *ticks and *substep and
 * returns through *rollback whether the step must be rolled back. */
pd_status pd_adaptive_decide(int has_broken, int ticks_base, int ticks_min, int max_substep,
                             int* ticks, int* substep, int* rollback);

#ifdef __cplusplus
}
#endif
#endif /* PD_GB300_H */
