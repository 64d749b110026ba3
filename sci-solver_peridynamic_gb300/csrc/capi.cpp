// capi.cpp -- extern "C" entry points of libpd_gb300.so (declared in include/pd_gb300.h).
#include <cstring>
#include <new>
#include <string>

#include "engine.h"
#include "pd_gb300.h"

struct pd_handle {
    pdgb::Engine* eng;
};

namespace {
thread_local std::string g_create_error;
}

namespace pdgb {
// Error text of calls that have no handle (read with pd_last_error_message(NULL)).
void set_handleless_error(const std::string& msg) { g_create_error = msg; }
}  // namespace pdgb

extern "C" {

int pd_abi_version(void) { return PD_GB300_ABI_VERSION; }

const char* pd_status_string(pd_status s)
{
    switch (s) {
    case PD_OK: return "ok";
    case PD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PD_ERR_CUDA: return "CUDA error";
    case PD_ERR_NOT_READY: return "not ready (make_ready has not run)";
    case PD_ERR_BOND_OVERFLOW: return "bond count exceeds the per-particle maximum";
    case PD_ERR_NO_DEVICE: return "no usable CUDA device";
    case PD_ERR_FILE: return "could not open parameter file";
    case PD_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PD_ERR_STATE: return "call out of order";
    }
    return "unknown status";
}

const char* pd_last_error_message(pd_handle* h)
{
    if (!h || !h->eng) return g_create_error.c_str();
    return h->eng->error().c_str();
}

pd_status pd_create(const pd_sim_params* sim, const pd_run_params* run, const pd_solver_options* opt,
                    pd_handle** out)
{
    if (!sim || !run || !out) return PD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (sim->num_pd_particle < 0) {
        g_create_error = "num_pd_particle < 0";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (run->integrator != PD_IMPLICIT_EULER && run->integrator != PD_NEWMARK_BETA) {
        g_create_error = "unknown integrator";
        return PD_ERR_INVALID_ARGUMENT;
    }
    pd_solver_options o;
    if (opt) o = *opt;
    else pd_solver_options_default(&o);
    if (o.precision != PD_PRECISION_MIXED && o.precision != PD_PRECISION_FP64) {
        g_create_error = "unknown precision mode";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (!(o.time_step_base > 0) || sim->pd_time_step <= 0) {
        g_create_error = "time step must be positive";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (o.warm_start < 0 || o.warm_start > 3 || o.history_size < 0 || o.history_size > pdgb::kHistMax ||
        (o.warm_start == 3 && o.history_size > pdgb::kHistMax - 1)) {
        g_create_error = "warm_start 0..3, history_size 0..8 (0..7 with warm_start 3)";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (o.cg_loop < 0 || o.cg_loop > 1 || o.cg_check_interval < 0) {
        g_create_error = "cg_loop 0 (graph) or 1 (host batches), cg_check_interval >= 0";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (o.preconditioner < 0 || o.preconditioner > 2) {
        g_create_error = "preconditioner 0 (none), 1 (diagonal) or 2 (3x3 blocks)";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (o.contact_enabled && !(o.contact_distance > 0 && o.contact_volume > 0)) {
        g_create_error = "contact distance and volume must be positive";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (o.spmv_path < 0 || o.spmv_path > 3 ||
        (o.lanes_per_particle != 0 && o.lanes_per_particle != 4 && o.lanes_per_particle != 8 &&
         o.lanes_per_particle != 16 && o.lanes_per_particle != 32) ||
        (o.spmv_unroll != 0 && o.spmv_unroll != 1 && o.spmv_unroll != 2 && o.spmv_unroll != 4)) {
        g_create_error = "SpMV options: spmv_path 0..3, lanes 0/4/8/16/32, unroll 0/1/2/4";
        return PD_ERR_INVALID_ARGUMENT;
    }
    pd_handle* h = new (std::nothrow) pd_handle{nullptr};
    if (!h) return PD_ERR_OUT_OF_MEMORY;
    h->eng = new (std::nothrow) pdgb::Engine(*sim, *run, o);
    if (!h->eng) {
        delete h;
        return PD_ERR_OUT_OF_MEMORY;
    }
    pd_status s = h->eng->init_device();
    if (s != PD_OK) {
        g_create_error = h->eng->error();
        delete h->eng;
        delete h;
        return s;
    }
    *out = h;
    return PD_OK;
}

pd_status pd_destroy(pd_handle* h)
{
    if (!h) return PD_ERR_INVALID_ARGUMENT;
    delete h->eng;
    delete h;
    return PD_OK;
}

#define ENG(h)                                              \
    do {                                                    \
        if (!(h) || !(h)->eng) return PD_ERR_INVALID_ARGUMENT; \
    } while (0)

pd_status pd_set_particles(pd_handle* h, const double* pos4, const double* vel4, const int32_t* activity, int n)
{
    ENG(h);
    return h->eng->set_particles(pos4, vel4, activity, n);
}

pd_status pd_set_stretch_limits(pd_handle* h, const double* s0, int n)
{
    ENG(h);
    return h->eng->set_stretch(s0, n);
}

pd_status pd_make_ready(pd_handle* h)
{
    ENG(h);
    return h->eng->make_ready();
}

pd_status pd_advance(pd_handle* h, int nsteps)
{
    ENG(h);
    return h->eng->advance(nsteps);
}

pd_status pd_finished(pd_handle* h, int* finished)
{
    ENG(h);
    if (!finished) return PD_ERR_INVALID_ARGUMENT;
    *finished = h->eng->finished() ? 1 : 0;
    return PD_OK;
}

pd_status pd_cg_converged(pd_handle* h, int* converged)
{
    ENG(h);
    if (!converged) return PD_ERR_INVALID_ARGUMENT;
    *converged = h->eng->cg_converged() ? 1 : 0;
    return PD_OK;
}

pd_status pd_get_current_step(pd_handle* h, int* step)
{
    ENG(h);
    if (!step) return PD_ERR_INVALID_ARGUMENT;
    *step = h->eng->current_step();
    return PD_OK;
}

pd_status pd_get(pd_handle* h, pd_variable var, void* dst, size_t bytes)
{
    ENG(h);
    return h->eng->get(var, dst, bytes);
}

pd_status pd_get_size(pd_handle* h, pd_variable var, size_t* bytes)
{
    ENG(h);
    if (!bytes) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->get_size(var, bytes);
}

pd_status pd_get_stats(pd_handle* h, pd_step_stats* stats)
{
    ENG(h);
    if (!stats) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->stats(stats);
}

pd_status pd_get_params(pd_handle* h, pd_sim_params* sim, pd_run_params* run, pd_solver_options* opt)
{
    ENG(h);
    h->eng->params(sim, run, opt);
    return PD_OK;
}

pd_status pd_set_profiling(pd_handle* h, int enabled)
{
    ENG(h);
    h->eng->set_profiling(enabled != 0);
    return PD_OK;
}

pd_status pd_get_kernel_times(pd_handle* h, pd_kernel_times* t)
{
    ENG(h);
    if (!t) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->kernel_times(t);
}

pd_status pd_reset_kernel_times(pd_handle* h)
{
    ENG(h);
    h->eng->reset_kernel_times();
    return PD_OK;
}

pd_status pd_get_launch_count(pd_handle* h, long long* launches)
{
    ENG(h);
    if (!launches) return PD_ERR_INVALID_ARGUMENT;
    *launches = h->eng->launches();
    return PD_OK;
}

pd_status pd_get_operator_view(pd_handle* h, pd_operator_view* view)
{
    ENG(h);
    if (!view) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->operator_view(view);
}

pd_status pd_apply_operator(pd_handle* h, const void* d_x, void* d_y, double* d_dot)
{
    ENG(h);
    return h->eng->apply_operator(d_x, d_y, d_dot);
}

pd_status pd_ws_set_params(pd_handle* h, const float* params, size_t count)
{
    ENG(h);
    return h->eng->ws_set_params(params, count);
}

pd_status pd_ws_get_params(pd_handle* h, float* params, size_t count)
{
    ENG(h);
    return h->eng->ws_get_params(params, count);
}

pd_status pd_ws_collect(pd_handle* h, int samples_per_step, long long capacity)
{
    ENG(h);
    return h->eng->ws_collect(samples_per_step, capacity);
}

pd_status pd_ws_dataset(pd_handle* h, float* X, float* T, long long max_rows, long long* rows)
{
    ENG(h);
    return h->eng->ws_dataset(X, T, max_rows, rows);
}

pd_status pd_get_stream(pd_handle* h, void** stream)
{
    ENG(h);
    if (!stream) return PD_ERR_INVALID_ARGUMENT;
    *stream = (void*)h->eng->stream();
    return PD_OK;
}

pd_status pd_synchronize(pd_handle* h)
{
    ENG(h);
    return h->eng->synchronize();
}

pd_status pd_sph_collide(pd_handle* h, double* sph_pos4, double* sph_vel4, int n_sph, double slip, int* collided)
{
    ENG(h);
    return h->eng->sph_collide(sph_pos4, sph_vel4, n_sph, slip, collided);
}

}  // extern "C"
