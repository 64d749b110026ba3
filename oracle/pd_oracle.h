/*
 * pd_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (FP64, no FMA contraction) of SCI-Solver_Peridynamic's
 * implicit bond-based peridynamics step.  It is the checker that the CUDA
 * path is compared against; it is never linked into, loaded by or called from
 * the product library.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may use it.
 *
 * Parity is pinned against the reference's own kernel source compiled on the
 * host (see oracle/build_ref.sh, outputs in oracle/_ref/) and against golden
 * vectors generated from that build (tests/golden/).
 *
 * Reference files restated (paths inside the reference project):
 *   src/core/simulator.cu:802-943    s0 sampling + bond construction
 *   src/core/kdtree.h:66-79,304-353  bond predicate  sqrt(sum (a-b)^2) < horizon
 *   src/core/cg_solver.cuh:200-339   force / breakage / Jacobian
 *   src/core/cg_solver.cuh:343-383   block SpMV (computeAx)
 *   src/core/implicit_euler.cuh      IE assembly + update
 *   src/core/newmark_beta.cuh        Newmark-beta assembly + update
 *   src/core/simulator.cu:297-652    step orchestration + adaptive rollback
 *   src/core/simulator.cu:735-799    CG call (CUSP krylov::cg, identity precond.)
 *   src/core/simulator.cu:1159-1178  advance(): phase-in of clockScale
 */
#ifndef PD_ORACLE_H
#define PD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Activity codes.  0..3 follow the reference's Activity enum
 * (src/core/parameters.h:137-144).  4 and 5 are extensions with no reference
 * counterpart: a clamped particle (velocity 0) and a particle whose velocity
 * is prescribed to its initial value. */
enum { PDO_ACTIVE = 0, PDO_SEMI_ACTIVE = 1, PDO_INACTIVE = 2, PDO_INVISIBLE = 3,
       PDO_CLAMPED = 4, PDO_PRESCRIBED = 5 };

typedef struct pdo_params {
    int    n;                /* number of PD particles */
    int    integrator;       /* 0 implicit Euler, 1 Newmark-beta */
    int    adaptive;         /* adaptive_integration (implicit Euler only; Newmark always adapts) */
    double horizon;          /* pd_horizon */
    double radius;           /* pd_particle_radius */
    double bond_coeff;       /* force coefficient; reference: pd_C_times_V * PD_K */
    double mass;             /* pd_particle_mass */
    double dt_base;          /* SYSTEM_TIMESTEP_BASE (2^-23 in the reference) */
    int    dt_ticks;         /* pd_time_step, in units of dt_base (128) */
    int    dt_ticks_min;     /* TIMESTEP_PD_MIN (100) */
    int    max_substep;      /* MAX_SUBSTEP (10) */
    int    phase_in;         /* PHASEIN (30) */
    double stretch_a;        /* 10.0 in (a - b*clockScale)*s0 - alpha*smin */
    double stretch_b;        /* 9.0 */
    double alpha;            /* alpha_pr (0.25) */
    double gravity[3];       /* acceleration; reference (0, -9.8, 0) */
    double box_min[3];       /* boundary_min_* */
    double box_max[3];       /* boundary_max_* */
    double restitution;      /* RESTITUTION (0.001) */
    double cg_rel_tol;       /* CG_RELATIVE_TOLERANCE (1e-20) */
    int    cg_max_iter;      /* MAX_CG_ITERATION (100000) */
    int    max_bonds;        /* MAX_PD_BOND_COUNT (528) */
    double s0;               /* pd_stretch_limit_s0 (a float in the reference, promoted) */
    int    sphere_on;        /* rigid-sphere penalty contact (extension) */
    double sphere_c0[3];
    double sphere_v[3];
    double sphere_radius;
    double sphere_k;
    /* PD-PD contact (collidePDParticles, simulator.cuh:675-768; off in the reference) */
    int    contact_on;
    double contact_dist;     /* FCELL * PERIDYNAMICS_MIN_DISTANCE */
    double contact_k;        /* Kc */
    double contact_vol;      /* PD_V */
    /* CG preconditioner (extension; the reference's cusp::precond::diagonal
     * is commented out at simulator.cu:767-769): 0 none, 1 inverse diagonal,
     * 2 inverse 3x3 diagonal blocks of the assembled matrix */
    int    precond;
} pdo_params;

typedef struct pdo_state pdo_state;

/* Fills the reference defaults (definitions.h constants); n and the
 * geometric quantities must then be set by the caller. */
void pdo_default_params(pdo_params* p);

pdo_state* pdo_create(const pdo_params* p);
void pdo_destroy(pdo_state* s);

/* pos4/vel4: n*4 doubles (x,y,z,w).  act: n ints (may be NULL = all ACTIVE). */
int pdo_set_particles(pdo_state* s, const double* pos4, const double* vel4, const int* act);
/* Optional caller-supplied per-particle stretch limits (else srand(1973) procedure). */
/* test hook: current positions only (reference positions unchanged) */
int pdo_set_position(pdo_state* s, const double* pos4);
int pdo_set_stretch(pdo_state* s, const double* s0);
/* Bond construction + s0 sampling.  Returns 0, or -1 if a row exceeds max_bonds. */
int pdo_make_ready(pdo_state* s);
/* One Simulator::advance(). */
int pdo_advance(pdo_state* s);

/* Diagnostics. */
int    pdo_current_step(const pdo_state* s);
int    pdo_cg_converged(const pdo_state* s);
int    pdo_last_cg_iters(const pdo_state* s);
double pdo_last_cg_residual(const pdo_state* s);
int    pdo_dt_ticks(const pdo_state* s);
int    pdo_substep(const pdo_state* s);
int    pdo_retries_last_step(const pdo_state* s);
long   pdo_num_bonds_total(const pdo_state* s);       /* sum of initial row lengths */
double pdo_clock_scale(const pdo_state* s);
double pdo_sim_time(const pdo_state* s);

/* Array exports, original particle order.  Sizes: 4n doubles for vectors,
 * n for scalars, n+1 for row_ptr, total bonds for col. */
void pdo_get_position(const pdo_state* s, double* out4);
void pdo_get_velocity(const pdo_state* s, double* out4);
void pdo_get_force(const pdo_state* s, double* out4);
void pdo_get_solution(const pdo_state* s, double* out4);
void pdo_get_rhs(const pdo_state* s, double* out4);
void pdo_get_stretch(const pdo_state* s, double* out);
void pdo_get_new_stretch(const pdo_state* s, double* out);
void pdo_get_original_stretch(const pdo_state* s, double* out);
void pdo_get_bond_count(const pdo_state* s, int* out);     /* alive bonds (top+1) */
void pdo_get_row_ptr(const pdo_state* s, long* out);       /* initial CSR row starts */
void pdo_get_bond_list(const pdo_state* s, int* out);      /* rows in current (swapped) order */

/* Building blocks for unit tests. */
int  pdo_force_pass(pdo_state* s, int* has_broken);      /* force/break/Jacobian at current state */
void pdo_apply_A(pdo_state* s, const double* x4, double* y4);  /* y = A x, current assembled A */
void pdo_get_diag_blocks(const pdo_state* s, double* out9);     /* diagonal blocks of A, 9 per particle */
void pdo_get_position_backup(const pdo_state* s, double* out4);  /* adaptive scheme's backups */
void pdo_get_velocity_backup(const pdo_state* s, double* out4);
void pdo_get_top_backup(const pdo_state* s, int* out);
void pdo_get_top(const pdo_state* s, int* out);                   /* pd_bond_list_top: live bonds - 1 */
void pdo_assemble(pdo_state* s);                           /* fill A and b after a force pass */
/* SPH <-> PD collision (collideDifferentParticles, simulator.cuh:1590-1733)
 * of n_sph caller SPH particles (pos4 / vel4 updated) against the current PD
 * state, on the grid (lo, cell, n) with the distance r_sph + P.radius; the
 * PD velocity of a particle hit is set from the SPH particle of the smallest
 * index.  Returns the SPH particles corrected. */
int pdo_sph_collide(pdo_state* s, const double lo[3], double cell, const int n[3], double r_sph, double m_sph,
                    double slip, double* pos4, double* vel4, int n_sph);

/* glibc-compatible rand() stream used for s0 (exposed to pin the product's copy). */
void pdo_sample_stretch(int n, double s0, double* out);

#ifdef __cplusplus
}
#endif
#endif
