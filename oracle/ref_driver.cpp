/*
 * ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's own PD kernels (compiled on the host through
 * ref_shim.h; the kernel text is streamed from the reference tree by
 * build_ref.sh and precedes this file in the same translation unit) the way
 * Simulator does:
 *   makeReady / initPeridynamicsBonds   src/core/simulator.cu:56-89, 825-943
 *   integratePeridynamicsImplicitEuler   src/core/simulator.cu:297-467
 *   integratePeridynamicsNewmarkBeta     src/core/simulator.cu:470-652
 *   advance                              src/core/simulator.cu:1159-1182
 * Bonds come from the reference's KDtree (src/core/kdtree.h) and s0 from its
 * getstretch() after srand(1973).  CUSP is not available, so the CG is a
 * restatement of CUSP's krylov::cg with identity preconditioner and
 * default_monitor (same fixed-order dot products as oracle/pd_oracle.c);
 * its matrix-vector product is the reference's computeAx kernel.
 *
 * Reference mode only (gravity -y, C*V*PD_K stiffness, 2^-23 time base).
 */
#include <vector>

namespace {

struct RefSim {
    int n = 0;
    int integrator = 0, adaptive = 0;
    double horizon = 0, radius = 0, cv = 0, mass = 0;
    double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    float s0 = 0.f;
    double cg_tol = 1e-20;
    int cg_max = 100000;
    int ticks = TIMESTEP_PD;
    int step = 0, substep = 0;
    double clock_scale = 0.0;
    bool cg_ok = true;
    int cg_iters = 0;
    double cg_res = 0.0;
    int max_bonds = 0;
    std::vector<double4> pos, vel, opos, force, sol, rhs, pos_bk, vel_bk, r, p, y;
    std::vector<double> st, ost, nst;
    std::vector<int> act, bond_list, top, top_bk;
    std::vector<Mat3x3> matrix;
    std::vector<double> partial;
    int has_broken = 0;
};

template <typename F>
void for_each_particle(int n, F&& f)
{
    #pragma omp parallel for schedule(dynamic, 64)
    for (int p = 0; p < n; ++p) {
        blockIdx.x = (unsigned)p; blockIdx.y = blockIdx.z = 0;
        blockDim.x = 1; blockDim.y = blockDim.z = 1;
        threadIdx.x = threadIdx.y = threadIdx.z = 0;
        f();
    }
}

const long kChunk = 4096;   /* must match oracle/pd_oracle.c DOT_CHUNK */

double dot4n(RefSim& s, const std::vector<double4>& a, const std::vector<double4>& b)
{
    const double* x = (const double*)a.data();
    const double* y = (const double*)b.data();
    const long len = 4L * s.n;
    const long nch = (len + kChunk - 1) / kChunk;
    s.partial.assign((size_t)nch + 1, 0.0);
    #pragma omp parallel for schedule(static)
    for (long c = 0; c < nch; ++c) {
        double acc = 0.0;
        const long e = std::min(len, (c + 1) * kChunk);
        for (long i = c * kChunk; i < e; ++i) acc += x[i] * y[i];
        s.partial[c] = acc;
    }
    double t = 0.0;
    for (long c = 0; c < nch; ++c) t += s.partial[c];
    return t;
}

void computeA(RefSim& s, std::vector<double4>& x, std::vector<double4>& y)
{
    for_each_particle(s.n, [&] {
        computeAx(s.bond_list.data(), s.top.data(), s.matrix.data(), x.data(), y.data(), s.n);
    });
}

bool solve(RefSim& s)
{
    const int n = s.n;
    double* x = (double*)s.sol.data();
    double* b = (double*)s.rhs.data();
    double* r = (double*)s.r.data();
    double* p = (double*)s.p.data();
    double* y = (double*)s.y.data();
    const double bnorm = std::sqrt(dot4n(s, s.rhs, s.rhs));
    const double tol = 0.0 + s.cg_tol * bnorm;
    computeA(s, s.sol, s.y);
    for (long i = 0; i < 4L * n; ++i) r[i] = 1.0 * b[i] + -1.0 * y[i];
    std::memcpy(p, r, sizeof(double) * 4 * (size_t)n);
    double rz = dot4n(s, s.r, s.r);
    int it = 0;
    bool conv = false;
    double rnorm = 0.0;
    for (;;) {
        rnorm = std::sqrt(rz);
        if (rnorm <= tol) { conv = true; break; }
        if (it >= s.cg_max) break;
        computeA(s, s.p, s.y);
        const double alpha = rz / dot4n(s, s.y, s.p);
        for (long i = 0; i < 4L * n; ++i) x[i] = alpha * p[i] + x[i];
        for (long i = 0; i < 4L * n; ++i) r[i] = -alpha * y[i] + r[i];
        const double rz_old = rz;
        rz = dot4n(s, s.r, s.r);
        const double beta = rz / rz_old;
        for (long i = 0; i < 4L * n; ++i) p[i] = 1.0 * r[i] + beta * p[i];
        ++it;
    }
    s.cg_iters = it;
    s.cg_res = rnorm;
    return conv;
}

bool integrate(RefSim& s)
{
    const int n = s.n;
    std::fill(s.matrix.begin(), s.matrix.end(), Mat3x3{});
    s.has_broken = 0;
    std::vector<int> broken_flag((size_t)n, 0);
    for_each_particle(n, [&] {
        int p = (int)blockIdx.x;
        calculatePDForceDerivative(s.act.data(), s.pos.data(), s.force.data(), s.opos.data(),
                                   s.ost.data(), s.st.data(), s.nst.data(), s.bond_list.data(),
                                   s.top.data(), s.matrix.data(), &broken_flag[(size_t)p], n,
                                   s.horizon, s.radius, s.cv, s.clock_scale, s.mass);
    });
    for (int p = 0; p < n; ++p) s.has_broken |= broken_flag[(size_t)p];
    const bool adaptive = (s.integrator == NEWMARK_BETA) ? true : (s.adaptive != 0);
    if (adaptive) {
        if (s.has_broken) {
            if (s.ticks > TIMESTEP_PD_MIN) {
                s.ticks /= 2;
                s.top = s.top_bk;
                s.pos = s.pos_bk;
                s.vel = s.vel_bk;
                return false;
            }
            s.substep = 1;
        } else {
            if (s.substep > 0) ++s.substep;
            if (s.substep >= MAX_SUBSTEP) {
                s.ticks *= 2;
                s.substep = (s.ticks >= TIMESTEP_PD) ? 0 : 1;
            }
        }
        s.top_bk = s.top;
        s.pos_bk = s.pos;
        s.vel_bk = s.vel;
    }
    s.st = s.nst;   /* updatePDStretchNeighborList (simulator.cuh:2601-2620), stretch part */
    if (s.integrator == IMPLICIT_EULER) {
        for_each_particle(n, [&] {
            fillMatrixImplicitEuler(s.act.data(), s.top.data(), s.matrix.data(), n, s.ticks, s.mass);
        });
        for_each_particle(n, [&] {
            fillVectorBImplicitEuler(s.act.data(), s.force.data(), s.vel.data(), s.rhs.data(), n,
                                     s.ticks, s.mass);
        });
        if (!solve(s)) s.cg_ok = false;
        s.vel = s.sol;
        for_each_particle(n, [&] {
            updatePDPositionImplicitEuler(s.act.data(), s.pos.data(), s.vel.data(), n, s.ticks,
                                          s.radius, s.bmin[0], s.bmin[1], s.bmin[2], s.bmax[0],
                                          s.bmax[1], s.bmax[2]);
        });
    } else {
        for_each_particle(n, [&] {
            fillMatrixNewmarkBeta(s.act.data(), s.top.data(), s.matrix.data(), n, s.ticks, s.mass);
        });
        for_each_particle(n, [&] {
            fillVectorBNewmarkBeta(s.act.data(), s.force.data(), s.vel.data(), s.rhs.data(), n,
                                   s.ticks, s.mass);
        });
        if (!solve(s)) s.cg_ok = false;
        for_each_particle(n, [&] {
            updatePDVelocityNewmarkBeta(s.act.data(), s.vel.data(), s.sol.data(), n, s.ticks);
        });
        for_each_particle(n, [&] {
            updatePDPositionNewmarkBeta(s.act.data(), s.pos.data(), s.vel.data(), s.sol.data(), n,
                                        s.ticks, s.radius, s.bmin[0], s.bmin[1], s.bmin[2],
                                        s.bmax[0], s.bmax[1], s.bmax[2]);
        });
    }
    return true;
}

}  // namespace

extern "C" {

void* ref_create(int n, int integrator, int adaptive, double horizon, double radius,
                 double c_times_v, double mass, const double* bmin, const double* bmax,
                 float s0, double cg_tol, int cg_max)
{
    RefSim* s = new RefSim();
    s->n = n; s->integrator = integrator; s->adaptive = adaptive;
    s->horizon = horizon; s->radius = radius; s->cv = c_times_v; s->mass = mass;
    for (int k = 0; k < 3; ++k) { s->bmin[k] = bmin[k]; s->bmax[k] = bmax[k]; }
    s->s0 = s0; s->cg_tol = cg_tol; s->cg_max = cg_max;
    const size_t N = (size_t)n;
    for (auto* v : {&s->pos, &s->vel, &s->opos, &s->force, &s->sol, &s->rhs, &s->pos_bk, &s->vel_bk,
                    &s->r, &s->p, &s->y})
        v->assign(N, make_double4(0.0, 0.0, 0.0, 0.0));
    s->st.assign(N, 0.0); s->ost.assign(N, 0.0); s->nst.assign(N, 0.0);
    s->act.assign(N, ACTIVE);
    s->bond_list.assign(N * MAX_PD_BOND_COUNT, 0);
    s->top.assign(N, -1); s->top_bk.assign(N, -1);
    /* one block more than the reference allocates, so a full 528-bond row stays in bounds */
    s->matrix.assign(N * (MAX_PD_BOND_COUNT + 1), Mat3x3{});
    return s;
}

void ref_destroy(void* h) { delete (RefSim*)h; }

void ref_set_particles(void* h, const double* pos4, const double* vel4, const int* act)
{
    RefSim& s = *(RefSim*)h;
    for (int i = 0; i < s.n; ++i) {
        s.pos[i] = make_double4(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], pos4[4 * i + 3]);
        s.vel[i] = make_double4(vel4[4 * i], vel4[4 * i + 1], vel4[4 * i + 2], vel4[4 * i + 3]);
        s.act[i] = act ? act[i] : ACTIVE;
    }
}

/* Simulator::initPeridynamicsBonds (simulator.cu:825-943), then makeReady's
 * initPDSolutions.  Returns the maximum bond count. */
int ref_make_ready(void* h)
{
    RefSim& s = *(RefSim*)h;
    const int n = s.n;
    Point* point = new Point[n > 0 ? n : 1];
    srand(1973);
    for (int i = 0; i < n; ++i) {
        s.opos[i] = s.pos[i];
        s.ost[i] = s.st[i] = getstretch(s.s0);
        s.top[i] = -1;
        point[i] = Point(s.pos[i].x, s.pos[i].y, s.pos[i].z, i);
    }
    int maxbonds = 0;
    if (n > 0) {
        Point tiny(-1000000.0, -1000000.0, -1000000.0, -1);
        Point huge(1000000.0, 1000000.0, 1000000.0, -1);
        KDNode* root = new KDNode(&point[0], n, tiny, huge);
        KDtree kd(n, root, 100, s.bond_list.data(), s.top.data(), s.horizon);
        kd.buildtree(root);
        for (int i = 0; i < n; ++i) kd.find_neighbors(point[i], root);
        std::vector<int> tmp(MAX_PD_BOND_COUNT);
        for (int i = 0; i < n; ++i) {
            const int cnt = s.top[i] + 1;
            maxbonds = std::max(maxbonds, cnt);
            for (int j = 0; j < cnt; ++j) tmp[j] = s.bond_list[(size_t)j * n + i];
            std::sort(tmp.begin(), tmp.begin() + cnt);
            for (int j = 0; j < cnt; ++j) s.bond_list[(size_t)j * n + i] = tmp[j];
        }
    }
    delete[] point;
    s.nst = s.ost;
    s.top_bk = s.top; s.pos_bk = s.pos; s.vel_bk = s.vel;
    for_each_particle(n, [&] { initPDSolutions(s.sol.data(), n); });
    s.step = 0; s.substep = 0; s.ticks = TIMESTEP_PD; s.clock_scale = 0.0; s.cg_ok = true;
    s.max_bonds = maxbonds;
    return maxbonds;
}

/* Simulator::advance (simulator.cu:1159-1182); returns the number of retries */
int ref_advance(void* h)
{
    RefSim& s = *(RefSim*)h;
    ++s.step;
    if (s.step <= PHASEIN) s.clock_scale = (real_t)s.step / (real_t)PHASEIN;
    int retries = 0;
    while (!integrate(s)) ++retries;
    return retries;
}

int ref_cg_iters(void* h) { return ((RefSim*)h)->cg_iters; }
double ref_cg_residual(void* h) { return ((RefSim*)h)->cg_res; }
int ref_cg_converged(void* h) { return ((RefSim*)h)->cg_ok ? 1 : 0; }
int ref_ticks(void* h) { return ((RefSim*)h)->ticks; }
int ref_has_broken(void* h) { return ((RefSim*)h)->has_broken; }

static void copy4(const std::vector<double4>& v, double* out)
{
    std::memcpy(out, v.data(), sizeof(double4) * v.size());
}
void ref_get_position(void* h, double* o) { copy4(((RefSim*)h)->pos, o); }
void ref_get_velocity(void* h, double* o) { copy4(((RefSim*)h)->vel, o); }
void ref_get_force(void* h, double* o) { copy4(((RefSim*)h)->force, o); }
void ref_get_solution(void* h, double* o) { copy4(((RefSim*)h)->sol, o); }
void ref_get_stretch(void* h, double* o) { std::memcpy(o, ((RefSim*)h)->st.data(), sizeof(double) * ((RefSim*)h)->n); }
void ref_get_new_stretch(void* h, double* o) { std::memcpy(o, ((RefSim*)h)->nst.data(), sizeof(double) * ((RefSim*)h)->n); }
void ref_get_original_stretch(void* h, double* o) { std::memcpy(o, ((RefSim*)h)->ost.data(), sizeof(double) * ((RefSim*)h)->n); }
void ref_get_bond_count(void* h, int* o)
{
    RefSim& s = *(RefSim*)h;
    for (int i = 0; i < s.n; ++i) o[i] = s.top[i] + 1;
}
/* bond j of particle i in the reference's bond-major layout: out[j*n + i], j < 528 */
void ref_get_bond_list(void* h, int* o)
{
    RefSim& s = *(RefSim*)h;
    std::memcpy(o, s.bond_list.data(), sizeof(int) * s.bond_list.size());
}

}  // extern "C"
