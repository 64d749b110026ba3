/*
 * pd_oracle.c -- TEST INFRASTRUCTURE ONLY (see pd_oracle.h).
 *
 * FP64 CPU restatement of the reference's implicit bond-based PD step.  Every
 * floating-point expression keeps the reference's operation order so that,
 * compiled with -ffp-contract=off, it reproduces the reference kernels run on
 * the host bit for bit (checked against oracle/_ref and tests/golden/).
 *
 * Layout: bonds are a CSR whose row p has capacity equal to its initial bond
 * count; the first top[p]+1 entries are the live bonds, exactly as the
 * reference's bond-major list with pd_bond_list_top (src/core/kdtree.h:338-353,
 * src/core/cg_solver.cuh:264-275).  Jacobian blocks are stored per bond slot
 * like pd_system_matrix (src/core/cg_solver.cuh:307,322).
 */
#include "pd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define SMALL_D 1.0e-10          /* src/core/definitions.h:62 */
#define DOT_CHUNK 4096           /* fixed reduction chunking: deterministic for any thread count */

struct pdo_state {
    pdo_params P;
    int n;
    double *pos, *vel, *opos, *force, *sol, *rhs;   /* 4n each */
    double *pos_bk, *vel_bk;
    double *st, *ost, *nst;                          /* n each */
    int *act;
    int *top, *top_bk;
    long *row_ptr;                                   /* n+1 */
    int *col;                                        /* bonds */
    double *diag;                                    /* 9n */
    double *off;                                     /* 9 * bonds */
    double *ctc;                                     /* 4n: contact normal (xyz) + stiffness (w) */
    double *cg_r, *cg_p, *cg_y, *partial;
    int stretch_set;
    int ready;
    int step, substep, ticks, retries;
    int cg_converged, cg_iters;
    double cg_res;
    double clock_scale, sim_time;
    long total_bonds;
};

/* host fmaxf of the reference (src/core/helper_math.h:43): float arguments */
static inline float ref_fmaxf(float a, float b) { return a > b ? a : b; }

void pdo_default_params(pdo_params* p)
{
    memset(p, 0, sizeof(*p));
    p->integrator = 0;
    p->adaptive = 0;
    p->dt_base = 1.0 / 8388608.0;     /* definitions.h:65 */
    p->dt_ticks = 128;                /* definitions.h:68 */
    p->dt_ticks_min = 100;            /* definitions.h:69 */
    p->max_substep = 10;              /* definitions.h:71 */
    p->phase_in = 30;                 /* definitions.h:103 */
    p->stretch_a = 10.0;              /* cg_solver.cuh:326 */
    p->stretch_b = 9.0;
    p->alpha = 0.25;                  /* definitions.h:109 */
    p->gravity[0] = 0.0; p->gravity[1] = -9.8; p->gravity[2] = 0.0;   /* cg_solver.cuh:330 */
    p->restitution = 0.001;           /* definitions.h:74 */
    p->cg_rel_tol = 1e-20;            /* definitions.h:135 */
    p->cg_max_iter = 100000;          /* definitions.h:134 */
    p->max_bonds = 528;               /* definitions.h:101 */
    p->box_min[0] = p->box_min[1] = p->box_min[2] = -1e300;
    p->box_max[0] = p->box_max[1] = p->box_max[2] = 1e300;
    p->contact_on = 0;
    p->contact_dist = 0.75 * 0.0005;   /* FCELL * PERIDYNAMICS_MIN_DISTANCE, definitions.h:86,98 */
    p->contact_k = 1.0e7;              /* Kc, definitions.h:90 */
    p->contact_vol = 0.0005 * 0.0005 * 0.0005;   /* PD_V, definitions.h:87 */
}

static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

pdo_state* pdo_create(const pdo_params* p)
{
    if (!p || p->n < 0) return NULL;
    pdo_state* s = (pdo_state*)xcalloc(1, sizeof(pdo_state));
    s->P = *p;
    s->n = p->n;
    size_t n = (size_t)p->n;
    s->pos = xcalloc(4 * n, sizeof(double));
    s->vel = xcalloc(4 * n, sizeof(double));
    s->opos = xcalloc(4 * n, sizeof(double));
    s->force = xcalloc(4 * n, sizeof(double));
    s->sol = xcalloc(4 * n, sizeof(double));
    s->rhs = xcalloc(4 * n, sizeof(double));
    s->pos_bk = xcalloc(4 * n, sizeof(double));
    s->vel_bk = xcalloc(4 * n, sizeof(double));
    s->ctc = xcalloc(4 * n, sizeof(double));
    s->cg_r = xcalloc(4 * n, sizeof(double));
    s->cg_p = xcalloc(4 * n, sizeof(double));
    s->cg_y = xcalloc(4 * n, sizeof(double));
    s->partial = xcalloc(4 * n / DOT_CHUNK + 2, sizeof(double));
    s->st = xcalloc(n, sizeof(double));
    s->ost = xcalloc(n, sizeof(double));
    s->nst = xcalloc(n, sizeof(double));
    s->act = xcalloc(n, sizeof(int));
    s->top = xcalloc(n, sizeof(int));
    s->top_bk = xcalloc(n, sizeof(int));
    s->row_ptr = xcalloc(n + 1, sizeof(long));
    s->diag = xcalloc(9 * n, sizeof(double));
    s->ticks = p->dt_ticks;
    s->cg_converged = 1;
    s->clock_scale = p->phase_in > 0 ? 0.0 : 1.0;
    return s;
}

void pdo_destroy(pdo_state* s)
{
    if (!s) return;
    free(s->pos); free(s->vel); free(s->opos); free(s->force); free(s->sol); free(s->rhs);
    free(s->pos_bk); free(s->vel_bk); free(s->ctc); free(s->cg_r); free(s->cg_p); free(s->cg_y);
    free(s->partial); free(s->st); free(s->ost); free(s->nst); free(s->act); free(s->top);
    free(s->top_bk); free(s->row_ptr); free(s->col); free(s->diag); free(s->off);
    free(s);
}

int pdo_set_particles(pdo_state* s, const double* pos4, const double* vel4, const int* act)
{
    size_t n = (size_t)s->n;
    memcpy(s->pos, pos4, 4 * n * sizeof(double));
    if (vel4) memcpy(s->vel, vel4, 4 * n * sizeof(double));
    else memset(s->vel, 0, 4 * n * sizeof(double));
    for (size_t i = 0; i < n; ++i) s->act[i] = act ? act[i] : PDO_ACTIVE;
    s->ready = 0;
    return 0;
}

/* Test hook with no reference counterpart: overwrite the current positions
 * (pd_position) after make_ready, keeping the reference positions, so that a
 * force pass can be evaluated at a chosen deformed state. */
int pdo_set_position(pdo_state* s, const double* pos4)
{
    memcpy(s->pos, pos4, 4 * (size_t)s->n * sizeof(double));
    return 0;
}

int pdo_set_stretch(pdo_state* s, const double* s0)
{
    memcpy(s->ost, s0, (size_t)s->n * sizeof(double));
    memcpy(s->st, s0, (size_t)s->n * sizeof(double));
    s->stretch_set = 1;
    return 0;
}

/* ---------------------------------------------------------------------------
 * s0 sampling: src/core/simulator.cu:802-822 (frand, getstretch) and :852-857
 * (srand(1973) then one getstretch per particle in index order).  Uses the C
 * library's rand(), i.e. glibc's generator on Linux as the reference did. */
static double ref_frand(void) { return rand() / (double)RAND_MAX; }

static double ref_getstretch(double s0)
{
    double sum = 0.0;
    for (int i = 0; i < 12; ++i) sum += ref_frand();
    sum -= 6.0;
    return ((sum * 0.01 + 1.0) * s0);
}

void pdo_sample_stretch(int n, double s0, double* out)
{
    srand(1973);
    for (int i = 0; i < n; ++i) out[i] = ref_getstretch(s0);
}

/* ---------------------------------------------------------------------------
 * Bond predicate of src/core/kdtree.h:66-79 (dist) used at :319-320:
 * howfar = 0; howfar += (a[j]-b[j])^2 for j=0..2; bond iff sqrt(howfar) < horizon,
 * a = the query particle, b = the candidate.  The kd-tree's box pruning never
 * removes a candidate that passes this test (rounding is monotone), so the
 * bond set is the exact radius query, built here with a uniform grid. */
static inline double ref_dist(const double* a, const double* b)
{
    double howfar = 0.0;
    for (int j = 0; j < 3; ++j) howfar += (a[j] - b[j]) * (a[j] - b[j]);
    return sqrt(howfar);
}

static int cmp_int(const void* a, const void* b)
{
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

static int build_bonds(pdo_state* s)
{
    const int n = s->n;
    const double h = s->P.horizon;
    free(s->col); s->col = NULL;
    free(s->off); s->off = NULL;
    if (n == 0) { s->row_ptr[0] = 0; s->total_bonds = 0; s->col = xcalloc(1, sizeof(int)); s->off = xcalloc(9, sizeof(double)); return 0; }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            double v = s->opos[4 * i + k];
            if (v < lo[k]) lo[k] = v;
            if (v > hi[k]) hi[k] = v;
        }
    double cs = h > 0 ? h : 1.0;
    long dim[3];
    for (int k = 0; k < 3; ++k) {
        dim[k] = (long)floor((hi[k] - lo[k]) / cs) + 1;
        if (dim[k] < 1) dim[k] = 1;
    }
    while (dim[0] * dim[1] * dim[2] > 64L * n + 1024) {  /* keep the grid O(n) */
        cs *= 2.0;
        for (int k = 0; k < 3; ++k) { dim[k] = (long)floor((hi[k] - lo[k]) / cs) + 1; if (dim[k] < 1) dim[k] = 1; }
    }
    long ncell = dim[0] * dim[1] * dim[2];
    long* cell_start = xcalloc((size_t)ncell + 1, sizeof(long));
    int* cell_of = xcalloc((size_t)n, sizeof(int));
    int* sorted = xcalloc((size_t)n, sizeof(int));
    for (int i = 0; i < n; ++i) {
        long c[3];
        for (int k = 0; k < 3; ++k) {
            c[k] = (long)floor((s->opos[4 * i + k] - lo[k]) / cs);
            if (c[k] < 0) c[k] = 0;
            if (c[k] >= dim[k]) c[k] = dim[k] - 1;
        }
        cell_of[i] = (int)((c[2] * dim[1] + c[1]) * dim[0] + c[0]);
        cell_start[cell_of[i] + 1]++;
    }
    for (long c = 0; c < ncell; ++c) cell_start[c + 1] += cell_start[c];
    long* fill = xcalloc((size_t)ncell, sizeof(long));
    for (int i = 0; i < n; ++i) sorted[cell_start[cell_of[i]] + fill[cell_of[i]]++] = i;
    free(fill);

    int* count = xcalloc((size_t)n, sizeof(int));
    int overflow = 0;
    const int maxb = s->P.max_bonds;
    /* pass 1: counts; pass 2: fill + sort ascending (src/core/simulator.cu:886-930) */
    for (int pass = 0; pass < 2; ++pass) {
        #pragma omp parallel for schedule(dynamic, 256) reduction(|:overflow)
        for (int i = 0; i < n; ++i) {
            const double* a = s->opos + 4 * i;
            long ci = cell_of[i];
            long cx = ci % dim[0], cy = (ci / dim[0]) % dim[1], cz = ci / (dim[0] * dim[1]);
            int cnt = 0;
            long out = pass ? s->row_ptr[i] : 0;
            for (long dz = -1; dz <= 1; ++dz) for (long dy = -1; dy <= 1; ++dy) for (long dx = -1; dx <= 1; ++dx) {
                long x = cx + dx, y = cy + dy, z = cz + dz;
                if (x < 0 || y < 0 || z < 0 || x >= dim[0] || y >= dim[1] || z >= dim[2]) continue;
                long c = (z * dim[1] + y) * dim[0] + x;
                for (long k = cell_start[c]; k < cell_start[c + 1]; ++k) {
                    int q = sorted[k];
                    if (q == i) continue;
                    if (ref_dist(a, s->opos + 4 * q) < h) {
                        if (pass) s->col[out + cnt] = q;
                        ++cnt;
                    }
                }
            }
            if (!pass) { count[i] = cnt; if (cnt > maxb) overflow = 1; }
            else qsort(s->col + out, (size_t)cnt, sizeof(int), cmp_int);
        }
        if (pass == 0) {
            if (overflow) break;
            s->row_ptr[0] = 0;
            for (int i = 0; i < n; ++i) s->row_ptr[i + 1] = s->row_ptr[i] + count[i];
            s->total_bonds = s->row_ptr[n];
            s->col = xcalloc((size_t)s->total_bonds, sizeof(int));
            s->off = xcalloc(9 * (size_t)s->total_bonds, sizeof(double));
        }
    }
    for (int i = 0; i < n; ++i) s->top[i] = count[i] - 1;
    free(count); free(cell_start); free(cell_of); free(sorted);
    return overflow ? -1 : 0;
}

/* src/core/simulator.cu:825-943 (initPeridynamicsBonds) + :56-76 (makeReady) */
int pdo_make_ready(pdo_state* s)
{
    size_t n = (size_t)s->n;
    memcpy(s->opos, s->pos, 4 * n * sizeof(double));
    if (!s->stretch_set) {
        pdo_sample_stretch(s->n, s->P.s0, s->ost);
        memcpy(s->st, s->ost, n * sizeof(double));
    }
    memcpy(s->nst, s->ost, n * sizeof(double));
    if (build_bonds(s) != 0) return -1;
    memcpy(s->top_bk, s->top, n * sizeof(int));
    memcpy(s->pos_bk, s->pos, 4 * n * sizeof(double));
    memcpy(s->vel_bk, s->vel, 4 * n * sizeof(double));
    memset(s->sol, 0, 4 * n * sizeof(double));         /* initPDSolutions, cg_solver.cuh:184-194 */
    memset(s->rhs, 0, 4 * n * sizeof(double));
    s->step = 0; s->substep = 0; s->ticks = s->P.dt_ticks;
    s->clock_scale = s->P.phase_in > 0 ? 0.0 : 1.0;
    s->sim_time = 0.0;
    s->cg_converged = 1;
    s->ready = 1;
    return 0;
}

/* ---------------------------------------------------------------------------
 * calculatePDForceDerivative, src/core/cg_solver.cuh:200-339, for one particle. */
static void force_particle(pdo_state* s, int p, double cs, int* broke)
{
    const pdo_params* P = &s->P;
    if (s->act[p] == PDO_INVISIBLE) return;
    const double* X = s->pos + 4 * p;
    const double* O = s->opos + 4 * p;
    double f[4] = {0.0, 0.0, 0.0, 0.0};
    double sum[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long base = s->row_ptr[p];
    int top = s->top[p];
    const int otop = top;
    const double stretch = s->st[p];
    double smin = 0.0;
    int bond = 0;
    while (bond <= top) {
        const long idx = base + bond;
        const int q = s->col[idx];
        const double* Q = s->pos + 4 * q;
        double e[4] = {Q[0] - X[0], Q[1] - X[1], Q[2] - X[2], Q[3] - X[3]};
        const double dij = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        const double D = (double)ref_fmaxf((float)dij, (float)SMALL_D);
        e[0] /= D; e[1] /= D; e[2] /= D; e[3] /= D;
        const double* OQ = s->opos + 4 * q;
        const double dv[4] = {O[0] - OQ[0], O[1] - OQ[1], O[2] - OQ[2], O[3] - OQ[3]};
        const double d0 = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2] + dv[3] * dv[3]);
        const double drdivd = dij / d0 - 1.0;
        if (drdivd > (double)ref_fmaxf((float)stretch, (float)s->st[q])) {
            const long last = base + top;
            s->col[idx] = s->col[last];
            s->col[last] = q;
            --top;
            continue;
        }
        double vscale = 1.0;
        if (d0 > (P->horizon - P->radius)) vscale = 0.5 + (P->horizon - d0) / 2.0 / P->radius;
        if (drdivd < smin) smin = drdivd;
        const double kk = drdivd * vscale;
        f[0] += kk * e[0]; f[1] += kk * e[1]; f[2] += kk * e[2]; f[3] += kk * e[3];
        double m[9];
        const double r = d0 / dij;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) m[3 * i + j] = e[i] * e[j];
        for (int k = 0; k < 9; ++k) m[k] *= r;
        double fd[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double dg = 1.0 - d0 / dij;
        fd[0] = dg; fd[4] = dg; fd[8] = dg;
        for (int k = 0; k < 9; ++k) fd[k] += m[k];
        const double c = P->bond_coeff / d0;
        for (int k = 0; k < 9; ++k) fd[k] *= c;
        for (int k = 0; k < 9; ++k) sum[k] += fd[k];
        for (int k = 0; k < 9; ++k) fd[k] *= -1.0;
        memcpy(s->off + 9 * idx, fd, sizeof(fd));
        ++bond;
    }
    memcpy(s->diag + 9 * (size_t)p, sum, sizeof(sum));
    for (int k = 0; k < 4; ++k) f[k] *= P->bond_coeff;
    const double ss0 = (P->stretch_a - P->stretch_b * cs) * s->ost[p];
    s->nst[p] = ss0 - P->alpha * smin;
    for (int k = 0; k < 3; ++k)
        if (P->gravity[k] != 0.0) f[k] -= (cs * (-P->gravity[k]) * P->mass);
    /* extension: rigid-sphere penalty contact at the start-of-step position */
    double* C = s->ctc + 4 * p;
    C[0] = C[1] = C[2] = C[3] = 0.0;
    if (P->sphere_on) {
        double c[3], dx[3];
        for (int k = 0; k < 3; ++k) { c[k] = P->sphere_c0[k] + P->sphere_v[k] * s->sim_time; dx[k] = X[k] - c[k]; }
        const double d = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        const double pen = (P->sphere_radius + P->radius) - d;
        if (pen > 0.0 && d > 0.0) {
            for (int k = 0; k < 3; ++k) { C[k] = dx[k] / d; f[k] += P->sphere_k * pen * C[k]; }
            C[3] = P->sphere_k;
        }
    }
    f[3] = 0.0;
    memcpy(s->force + 4 * p, f, sizeof(f));
    if (otop != top) {
        s->top[p] = top;
        *broke = 1;
    }
}

/* collidePDParticles (simulator.cuh:675-768): every pair closer than the
 * contact distance repels with Kc (r - d)^2 / V along x_p - x_q; all pairs
 * by brute force, in q order (test scenes are small). */
static void contact_particle(pdo_state* s, int p)
{
    const pdo_params* P = &s->P;
    if (s->act[p] == PDO_INVISIBLE) return;
    const double* X = s->pos + 4 * p;
    double f[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < s->n; ++q) {
        if (q == p || s->act[q] == PDO_INVISIBLE) continue;
        const double* Q = s->pos + 4 * q;
        const double pq[3] = {X[0] - Q[0], X[1] - Q[1], X[2] - Q[2]};
        const double r = sqrt(pq[0] * pq[0] + pq[1] * pq[1] + pq[2] * pq[2]);
        if (r >= P->contact_dist || r == 0.0) continue;
        const double howfar = r - P->contact_dist;
        const double mag = P->contact_k * (howfar * howfar) / P->contact_vol;
        for (int k = 0; k < 3; ++k) f[k] += mag * (pq[k] / r);
    }
    if (sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) > 1e-10)
        for (int k = 0; k < 3; ++k) s->force[4 * p + k] += f[k];
}

int pdo_force_pass(pdo_state* s, int* has_broken)
{
    int broke = 0;
    const double cs = s->clock_scale;
    #pragma omp parallel for schedule(dynamic, 64) reduction(|:broke)
    for (int p = 0; p < s->n; ++p) {
        int b = 0;
        force_particle(s, p, cs, &b);
        broke |= b;
    }
    if (s->P.contact_on) {
        #pragma omp parallel for schedule(dynamic, 64)
        for (int p = 0; p < s->n; ++p) contact_particle(s, p);
    }
    if (has_broken) *has_broken = broke;
    return 0;
}

static double timestep(const pdo_state* s) { return s->ticks * s->P.dt_base; }

/* fillMatrix* + fillVectorB* (implicit_euler.cuh:19-86, newmark_beta.cuh:19-86) */
void pdo_assemble(pdo_state* s)
{
    const pdo_params* P = &s->P;
    double t2 = timestep(s);
    if (P->integrator == 0) t2 = t2 * t2;
    else t2 = (t2 * t2) / 4.0;
    const double ts = timestep(s);
    #pragma omp parallel for schedule(static)
    for (int p = 0; p < s->n; ++p) {
        if (s->act[p] == PDO_INVISIBLE) continue;
        double* d = s->diag + 9 * (size_t)p;
        const double* C = s->ctc + 4 * p;
        if (C[3] != 0.0)   /* extension: contact stiffness k n n^T on the diagonal block */
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) d[3 * i + j] += C[3] * C[i] * C[j];
        for (int k = 0; k < 9; ++k) d[k] *= t2;
        for (int k = 0; k < 9; ++k) d[k] += (k % 4 == 0) ? P->mass : 0.0;
        const long base = s->row_ptr[p];
        for (int b = 0; b <= s->top[p]; ++b) {
            double* o = s->off + 9 * (base + b);
            for (int k = 0; k < 9; ++k) o[k] *= t2;
        }
        const double* v = s->vel + 4 * p;
        const double* f = s->force + 4 * p;
        double* bb = s->rhs + 4 * p;
        if (P->integrator == 0) {
            for (int k = 0; k < 4; ++k) bb[k] = P->mass * v[k] + ts * f[k];
        } else {
            const double hh = 0.5 * ts;
            for (int k = 0; k < 4; ++k) bb[k] = ts * (P->mass * v[k] + hh * f[k]);
        }
    }
}

/* computeAx, src/core/cg_solver.cuh:343-383 */
void pdo_apply_A(pdo_state* s, const double* x, double* y)
{
    #pragma omp parallel for schedule(static)
    for (int p = 0; p < s->n; ++p) {
        const double* A = s->diag + 9 * (size_t)p;
        const double* xp = x + 4 * p;
        double a0 = A[0] * xp[0] + A[1] * xp[1] + A[2] * xp[2];
        double a1 = A[3] * xp[0] + A[4] * xp[1] + A[5] * xp[2];
        double a2 = A[6] * xp[0] + A[7] * xp[1] + A[8] * xp[2];
        const long base = s->row_ptr[p];
        for (int b = 0; b <= s->top[p]; ++b) {
            const int q = s->col[base + b];
            const double* xq = x + 4 * q;
            const double* B = s->off + 9 * (base + b);
            a0 += B[0] * xq[0] + B[1] * xq[1] + B[2] * xq[2];
            a1 += B[3] * xq[0] + B[4] * xq[1] + B[5] * xq[2];
            a2 += B[6] * xq[0] + B[7] * xq[1] + B[8] * xq[2];
        }
        y[4 * p + 0] = a0; y[4 * p + 1] = a1; y[4 * p + 2] = a2; y[4 * p + 3] = 0.0;
    }
}

/* Fixed-order dot product over 4n doubles. */
static double dot4n(pdo_state* s, const double* a, const double* b)
{
    const long len = 4L * s->n;
    const long nch = (len + DOT_CHUNK - 1) / DOT_CHUNK;
    #pragma omp parallel for schedule(static)
    for (long c = 0; c < nch; ++c) {
        double acc = 0.0;
        const long e = (c + 1) * DOT_CHUNK < len ? (c + 1) * DOT_CHUNK : len;
        for (long i = c * DOT_CHUNK; i < e; ++i) acc += a[i] * b[i];
        s->partial[c] = acc;
    }
    double t = 0.0;
    for (long c = 0; c < nch; ++c) t += s->partial[c];
    return t;
}

static int is_dirichlet(int a) { return a == PDO_INVISIBLE || a == PDO_CLAMPED || a == PDO_PRESCRIBED; }

/* Inverse of a symmetric 3x3 diagonal block D (xx yy zz xy xz yz): the
 * block's inverse by adjugate over determinant where it is positive definite
 * (mode 2), else -- and for mode 1 -- the inverse of its diagonal, 1 / mass
 * for a non-positive entry.  The preconditioner option of the GPU path
 * (an extension: the reference's diagonal preconditioner is commented out,
 * simulator.cu:767-769). */
static void pc_invert(int mode, double mass, const double D[6], double M[6])
{
    const double a = D[0], b = D[1], c = D[2], d = D[3], e = D[4], f = D[5];
    if (mode == 2) {
        const double c00 = b * c - f * f, c11 = a * c - e * e, c22 = a * b - d * d;
        const double c01 = e * f - d * c, c02 = d * f - b * e, c12 = d * e - a * f;
        const double det = a * c00 + d * c01 + e * c02;
        if (a > 0.0 && c22 > 0.0 && det > 0.0) {
            const double id = 1.0 / det;
            M[0] = c00 * id; M[1] = c11 * id; M[2] = c22 * id;
            M[3] = c01 * id; M[4] = c02 * id; M[5] = c12 * id;
            return;
        }
    }
    const double im = 1.0 / mass;
    M[0] = a > 0.0 ? 1.0 / a : im;
    M[1] = b > 0.0 ? 1.0 / b : im;
    M[2] = c > 0.0 ? 1.0 / c : im;
    M[3] = M[4] = M[5] = 0.0;
}

/* z = M r per particle (Dirichlet rows: r is 0 there) */
static void pc_apply(const pdo_state* s, const double* M, const double* r, double* z)
{
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; ++i) {
        const double* m = M + 6 * (size_t)i;
        const double* ri = r + 4 * i;
        z[4 * i + 0] = m[0] * ri[0] + m[3] * ri[1] + m[4] * ri[2];
        z[4 * i + 1] = m[3] * ri[0] + m[1] * ri[1] + m[5] * ri[2];
        z[4 * i + 2] = m[4] * ri[0] + m[5] * ri[1] + m[2] * ri[2];
        z[4 * i + 3] = 0.0;
    }
}

/* CUSP krylov::cg with identity preconditioner and default_monitor(b, maxit, reltol)
 * (called at src/core/simulator.cu:760-770), restated; Dirichlet rows
 * (extension) are handled by projection.  With P.precond (extension) the
 * same loop preconditioned: rho = <r, z>, z = M r, p = z + beta p, the test
 * still on ||r||.  Returns 1 if converged. */
static int solve_cg(pdo_state* s)
{
    const pdo_params* P = &s->P;
    const int n = s->n;
    double *x = s->sol, *b = s->rhs, *r = s->cg_r, *p = s->cg_p, *y = s->cg_y;
    const double ts = timestep(s);
    int has_d = 0;
    for (int i = 0; i < n; ++i) {
        if (!is_dirichlet(s->act[i])) continue;
        has_d = 1;
        double u[3] = {0.0, 0.0, 0.0};
        if (s->act[i] == PDO_PRESCRIBED)
            for (int k = 0; k < 3; ++k) u[k] = P->integrator == 0 ? s->vel[4 * i + k] : ts * s->vel[4 * i + k];
        for (int k = 0; k < 3; ++k) x[4 * i + k] = u[k];
        x[4 * i + 3] = 0.0;
    }
    /* tolerance: relative to ||b|| over the free rows */
    if (has_d) {
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 4; ++k) y[4 * i + k] = is_dirichlet(s->act[i]) ? 0.0 : b[4 * i + k];
    } else {
        memcpy(y, b, 4 * (size_t)n * sizeof(double));
    }
    const double bnorm = sqrt(dot4n(s, y, y));
    const double tol = 0.0 + P->cg_rel_tol * bnorm;
    pdo_apply_A(s, x, y);
    for (long i = 0; i < 4L * n; ++i) r[i] = 1.0 * b[i] + -1.0 * y[i];
    if (has_d)
        for (int i = 0; i < n; ++i)
            if (is_dirichlet(s->act[i])) r[4 * i] = r[4 * i + 1] = r[4 * i + 2] = r[4 * i + 3] = 0.0;
    /* preconditioner: inverse diagonal blocks of the assembled matrix */
    double *M = NULL, *z = r;
    if (P->precond) {
        M = (double*)xcalloc(6 * (size_t)n, sizeof(double));
        z = (double*)xcalloc(4 * (size_t)n, sizeof(double));
        for (int i = 0; i < n; ++i) {
            if (is_dirichlet(s->act[i])) continue;
            const double* A = s->diag + 9 * (size_t)i;
            const double D[6] = {A[0], A[4], A[8], A[1], A[2], A[5]};
            pc_invert(P->precond, P->mass, D, M + 6 * (size_t)i);
        }
        pc_apply(s, M, r, z);
    }
    memcpy(p, z, 4 * (size_t)n * sizeof(double));
    double rr = dot4n(s, r, r);
    double rz = P->precond ? dot4n(s, r, z) : rr;
    int it = 0;
    int conv = 0;
    double rnorm = 0.0;
    for (;;) {
        rnorm = sqrt(rr);   /* nrm2(r); without a preconditioner z = r, so <r,z> is the same fixed-order sum */
        if (rnorm <= tol) { conv = 1; break; }
        if (it >= P->cg_max_iter) break;
        pdo_apply_A(s, p, y);
        if (has_d)
            for (int i = 0; i < n; ++i)
                if (is_dirichlet(s->act[i])) y[4 * i] = y[4 * i + 1] = y[4 * i + 2] = y[4 * i + 3] = 0.0;
        const double alpha = rz / dot4n(s, y, p);
        for (long i = 0; i < 4L * n; ++i) x[i] = alpha * p[i] + x[i];
        for (long i = 0; i < 4L * n; ++i) r[i] = -alpha * y[i] + r[i];
        const double rz_old = rz;
        rr = dot4n(s, r, r);
        if (P->precond) {
            pc_apply(s, M, r, z);
            rz = dot4n(s, r, z);
        } else {
            rz = rr;
        }
        const double beta = rz / rz_old;
        for (long i = 0; i < 4L * n; ++i) p[i] = 1.0 * z[i] + beta * p[i];
        ++it;
    }
    if (P->precond) {
        free(M);
        free(z);
    }
    s->cg_iters = it;
    s->cg_res = rnorm;
    return conv;
}

/* box reflection of updatePDPosition* (implicit_euler.cuh:116-168) */
static void reflect(const pdo_params* P, double* np, double* nv)
{
    for (int k = 0; k < 3; ++k) {
        const double mn = P->box_min[k] + P->radius;
        const double mx = P->box_max[k] - P->radius;
        if (np[k] > mx) { nv[k] *= -P->restitution; np[k] = mx - P->restitution * (np[k] - mx); }
        if (np[k] < mn) { nv[k] *= -P->restitution; np[k] = mn + P->restitution * (mn - np[k]); }
    }
}

static void update(pdo_state* s)
{
    const pdo_params* P = &s->P;
    const double ts = timestep(s);
    if (P->integrator == 0) {
        /* transferData(PD_VELOCITY <- PD_SYSTEM_SOLUTION), simulator.cu:449 */
        memcpy(s->vel, s->sol, 4 * (size_t)s->n * sizeof(double));
        #pragma omp parallel for schedule(static)
        for (int p = 0; p < s->n; ++p) {
            if (s->act[p] == PDO_INVISIBLE) continue;
            double nv[4], np[4];
            const double* op = s->pos + 4 * p;
            memcpy(nv, s->vel + 4 * p, sizeof(nv));
            for (int k = 0; k < 4; ++k) np[k] = op[k] + nv[k] * P->dt_base * s->ticks;
            reflect(P, np, nv);
            memcpy(s->pos + 4 * p, np, sizeof(np));
            memcpy(s->vel + 4 * p, nv, sizeof(nv));
        }
    } else {
        #pragma omp parallel for schedule(static)
        for (int p = 0; p < s->n; ++p) {
            if (s->act[p] == PDO_INVISIBLE) continue;
            double* v = s->vel + 4 * p;
            const double* dx = s->sol + 4 * p;
            for (int k = 0; k < 4; ++k) v[k] = 2.0 / ts * dx[k] - v[k];
            double nv[4], np[4];
            memcpy(nv, v, sizeof(nv));
            const double* op = s->pos + 4 * p;
            for (int k = 0; k < 4; ++k) np[k] = op[k] + dx[k];
            reflect(P, np, nv);
            memcpy(s->pos + 4 * p, np, sizeof(np));
            memcpy(v, nv, sizeof(nv));
        }
    }
}

/* integratePeridynamicsImplicitEuler / NewmarkBeta, simulator.cu:297-652 */
static int integrate(pdo_state* s)
{
    const pdo_params* P = &s->P;
    const size_t n = (size_t)s->n;
    memset(s->diag, 0, 9 * n * sizeof(double));
    if (s->total_bonds) memset(s->off, 0, 9 * (size_t)s->total_bonds * sizeof(double));
    int broke = 0;
    pdo_force_pass(s, &broke);
    const int adaptive = (P->integrator == 1) ? 1 : P->adaptive;
    if (adaptive) {
        if (broke) {
            if (s->ticks > P->dt_ticks_min) {
                s->ticks /= 2;
                memcpy(s->top, s->top_bk, n * sizeof(int));
                memcpy(s->pos, s->pos_bk, 4 * n * sizeof(double));
                memcpy(s->vel, s->vel_bk, 4 * n * sizeof(double));
                return 0;
            }
            s->substep = 1;
        } else {
            if (s->substep > 0) ++s->substep;
            if (s->substep >= P->max_substep) {
                s->ticks *= 2;
                s->substep = (s->ticks >= P->dt_ticks) ? 0 : 1;
            }
        }
        memcpy(s->top_bk, s->top, n * sizeof(int));
        memcpy(s->pos_bk, s->pos, 4 * n * sizeof(double));
        memcpy(s->vel_bk, s->vel, 4 * n * sizeof(double));
    }
    memcpy(s->st, s->nst, n * sizeof(double));   /* updatePDStretchNeighborList */
    pdo_assemble(s);
    if (!solve_cg(s)) s->cg_converged = 0;
    update(s);
    s->sim_time += timestep(s);
    return 1;
}

int pdo_advance(pdo_state* s)
{
    if (!s->ready) return -1;
    ++s->step;
    if (s->step <= s->P.phase_in) s->clock_scale = (double)s->step / (double)s->P.phase_in;
    s->retries = 0;
    while (!integrate(s)) ++s->retries;
    return 0;
}

int pdo_current_step(const pdo_state* s) { return s->step; }
int pdo_cg_converged(const pdo_state* s) { return s->cg_converged; }
int pdo_last_cg_iters(const pdo_state* s) { return s->cg_iters; }
double pdo_last_cg_residual(const pdo_state* s) { return s->cg_res; }
int pdo_dt_ticks(const pdo_state* s) { return s->ticks; }
int pdo_substep(const pdo_state* s) { return s->substep; }
int pdo_retries_last_step(const pdo_state* s) { return s->retries; }
long pdo_num_bonds_total(const pdo_state* s) { return s->total_bonds; }
double pdo_clock_scale(const pdo_state* s) { return s->clock_scale; }
double pdo_sim_time(const pdo_state* s) { return s->sim_time; }

void pdo_get_position(const pdo_state* s, double* o) { memcpy(o, s->pos, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_velocity(const pdo_state* s, double* o) { memcpy(o, s->vel, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_force(const pdo_state* s, double* o) { memcpy(o, s->force, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_solution(const pdo_state* s, double* o) { memcpy(o, s->sol, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_rhs(const pdo_state* s, double* o) { memcpy(o, s->rhs, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_stretch(const pdo_state* s, double* o) { memcpy(o, s->st, (size_t)s->n * sizeof(double)); }
void pdo_get_new_stretch(const pdo_state* s, double* o) { memcpy(o, s->nst, (size_t)s->n * sizeof(double)); }
void pdo_get_original_stretch(const pdo_state* s, double* o) { memcpy(o, s->ost, (size_t)s->n * sizeof(double)); }
void pdo_get_bond_count(const pdo_state* s, int* o) { for (int i = 0; i < s->n; ++i) o[i] = s->top[i] + 1; }
void pdo_get_row_ptr(const pdo_state* s, long* o) { memcpy(o, s->row_ptr, ((size_t)s->n + 1) * sizeof(long)); }
void pdo_get_bond_list(const pdo_state* s, int* o) { if (s->total_bonds) memcpy(o, s->col, (size_t)s->total_bonds * sizeof(int)); }

/* Diagonal 3x3 blocks of the assembled system matrix (row-major, 9 per particle). */
/* the adaptive scheme's backups (the reference's PD_POSITION_BACKUP,
 * PD_VELOCITY_BACKUP, PD_BOND_LIST_TOP_BACKUP), the step counters */
void pdo_get_position_backup(const pdo_state* s, double* o) { memcpy(o, s->pos_bk, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_velocity_backup(const pdo_state* s, double* o) { memcpy(o, s->vel_bk, 4 * (size_t)s->n * sizeof(double)); }
void pdo_get_top_backup(const pdo_state* s, int* o) { memcpy(o, s->top_bk, (size_t)s->n * sizeof(int)); }
void pdo_get_top(const pdo_state* s, int* o) { memcpy(o, s->top, (size_t)s->n * sizeof(int)); }
void pdo_get_diag_blocks(const pdo_state* s, double* out) { memcpy(out, s->diag, 9 * (size_t)s->n * sizeof(double)); }

/* ---- SPH <-> PD collision ------------------------------------------------------------
 * collideDifferentParticles (src/core/simulator.cuh:1590-1733) restated with
 * the GPU path's semantics: calcGridPos / calcGridHash (simulator.cuh:61-87)
 * for both particle kinds, the nearest PD particle of the 27 cells around the
 * SPH particle's cell closer than r_sph + r_pd (ties: the smallest PD index),
 * the reference's position correction and velocity exchange in its operation
 * order (the distance divisor rounded to float as its fmaxf), the PD velocity
 * read from the nearest particle (the reference reads a wrong index) and
 * written by the SPH particle of the smallest index. */
static int sph_cell(const double lo[3], double cell, const int n[3], const double* p, int c[3])
{
    for (int k = 0; k < 3; ++k) c[k] = (int)floor((p[k] - lo[k]) / cell);
    if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= n[0] || c[1] >= n[1] || c[2] >= n[2]) return -1;
    return (c[2] * n[1] + c[1]) * n[0] + c[0];
}

int pdo_sph_collide(pdo_state* s, const double lo[3], double cell, const int n[3], double r_sph, double m_sph,
                    double slip, double* pos4, double* vel4, int n_sph)
{
    const int np = s->n;
    const double min_dist = r_sph + s->P.radius, mi = m_sph, mj = s->P.mass;
    int* pcell = (int*)xcalloc(3 * (size_t)np + 1, sizeof(int));
    int* pin = (int*)xcalloc((size_t)np + 1, sizeof(int));
    int* winner = (int*)xcalloc((size_t)np + 1, sizeof(int));
    int* hit = (int*)xcalloc((size_t)n_sph + 1, sizeof(int));
    double* vnew = (double*)xcalloc(3 * (size_t)n_sph + 1, sizeof(double));
    for (int j = 0; j < np; ++j) {
        pin[j] = sph_cell(lo, cell, n, s->pos + 4 * (size_t)j, pcell + 3 * (size_t)j) >= 0;
        winner[j] = -1;
    }
    int count = 0;
    for (int i = 0; i < n_sph; ++i) {
        hit[i] = -1;
        double* pi = pos4 + 4 * (size_t)i;
        int c[3];
        if (sph_cell(lo, cell, n, pi, c) < 0) continue;
        double best = min_dist;
        int bj = -1;
        for (int j = 0; j < np; ++j) {
            if (!pin[j]) continue;
            const int* cj = pcell + 3 * (size_t)j;
            if (abs(cj[0] - c[0]) > 1 || abs(cj[1] - c[1]) > 1 || abs(cj[2] - c[2]) > 1) continue;
            const double* pj = s->pos + 4 * (size_t)j;
            const double ex = pj[0] - pi[0], ey = pj[1] - pi[1], ez = pj[2] - pi[2];
            const double d = sqrt(ex * ex + ey * ey + ez * ez);
            if (d < best || (d == best && bj >= 0 && j < bj)) {
                best = d;
                bj = j;
            }
        }
        if (bj < 0) continue;
        const double* pj = s->pos + 4 * (size_t)bj;
        const double* vj = s->vel + 4 * (size_t)bj;
        double* vi = vel4 + 4 * (size_t)i;
        const double D = (double)ref_fmaxf((float)best, (float)SMALL_D);
        const double e[3] = {(pj[0] - pi[0]) / D, (pj[1] - pi[1]) / D, (pj[2] - pi[2]) / D};
        const double di = e[0] * vi[0] + e[1] * vi[1] + e[2] * vi[2];
        const double dj = e[0] * vj[0] + e[1] * vj[1] + e[2] * vj[2];
        const double mm = mi + mj;
        const double ci = mi + mj * slip, cj = mj + mi * slip;
        const double ti = mj * (1.0 - slip), tj = mi * (1.0 - slip);
        double xo[3], vo[3];
        for (int k = 0; k < 3; ++k) {
            xo[k] = pj[k] - min_dist * e[k];
            const double vin = e[k] * di, vit = vi[k] - vin;
            const double vjn = e[k] * dj, vjt = vj[k] - vjn;
            const double vn2 = (mi * vin + mj * vjn) / mm;
            const double vit2 = (ci * vit + ti * vjt) / mm;
            const double vjt2 = (cj * vjt + tj * vit) / mm;
            vo[k] = vn2 + vit2;
            vnew[3 * (size_t)i + k] = vn2 + vjt2;
        }
        for (int k = 0; k < 3; ++k) {
            pi[k] = xo[k];
            vi[k] = vo[k];
        }
        hit[i] = bj;
        if (winner[bj] < 0) winner[bj] = i;
        ++count;
    }
    for (int i = 0; i < n_sph; ++i) {
        const int j = hit[i];
        if (j < 0 || winner[j] != i) continue;
        for (int k = 0; k < 3; ++k) s->vel[4 * (size_t)j + k] = vnew[3 * (size_t)i + k];
        s->vel[4 * (size_t)j + 3] = 0.0;
    }
    free(pcell); free(pin); free(winner); free(hit); free(vnew);
    return count;
}
