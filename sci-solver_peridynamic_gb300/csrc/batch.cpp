// batch.cpp -- many independent scenes stepped together (pd_batch_*).
//
// Each scene is an Engine (its own parameters, device state, step state);
// the batch adds the work-item list over all scenes, the per-scene step-loop
// records that the persistent kernels advance on the device (batch.cu), an
// autotuner for the SpMV launch shape and item size, and the CUDA graph that
// replays one step (two cooperative launches).  After pd_batch_advance the
// device records are copied back into the scenes' Engine objects, so every
// per-scene query (pd_batch_get, pd_batch_get_stats) answers as a pd_handle.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "batch.h"
#include "engine.h"
#include "pd_gb300.h"

namespace pdgb {

#define BCK(call, what)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return fail(e_, what);    \
    } while (0)

class Batch {
public:
    Batch(int device, const pd_batch_options& o) : device_(device), opt_(o) {}
    ~Batch();
    pd_status init();
    pd_status add_scene(const pd_sim_params& sim, const pd_run_params& run, const pd_solver_options& opt, int* idx);
    Engine* scene(int s) { return (s >= 0 && s < (int)eng_.size()) ? eng_[(size_t)s].get() : nullptr; }
    int count() const { return (int)eng_.size(); }
    pd_status make_ready();
    pd_status relayout(int lanes, int unroll);
    pd_status advance(int nsteps);
    pd_status config(pd_batch_config* c) const;
    pd_status ws_set_params(const float* params, size_t count);
    long long launches() const { return launches_; }
    cudaStream_t stream() const { return stream_; }
    pd_status synchronize();
    bool ready() const { return ready_; }
    const std::string& error() const { return err_; }
    void set_error(const std::string& e) { err_ = e; }

private:
    pd_status fail(cudaError_t e, const char* what);
    void free_device();
    pd_status build_items(int item_rows);
    BatchArgs args(int tune_reps) const;
    pd_status enqueue_step();
    pd_status tune();
    pd_status build_graph();
    pd_status pull_state();
    pd_status ws_setup();

    int device_;
    pd_batch_options opt_;
    cudaStream_t stream_ = nullptr;
    int sm_count_ = 0;
    std::vector<std::unique_ptr<Engine>> eng_;
    bool fp64_ = false;
    bool ready_ = false;
    std::vector<WorkItem> items_;
    std::vector<SceneDesc> h_desc_;
    std::vector<SceneRun> h_run_;
    SceneDesc* d_desc_ = nullptr;
    SceneRun* d_run_ = nullptr;
    WorkItem* d_items_ = nullptr;
    double* d_partials_ = nullptr;
    size_t items_cap_ = 0;
    unsigned* d_counters_ = nullptr;
    BatchSync* d_sync_ = nullptr;
    int max_cg_iters_ = 1;
    int lanes_ = 8, unroll_ = 2, item_rows_ = 128;
    int grid_pre_ = 0, grid_cg_ = 0;
    bool autotuned_ = false;
    double tuned_ms_ = 0.0;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    // learned warm start: one network for all scenes, run once per step over
    // the concatenated feature rows of every scene
    std::vector<float> ws_params_;
    MlpDev mlp_{};
    MlpWork mlp_work_{};
    __nv_bfloat16* d_feat_ = nullptr;
    float* d_ws_y_ = nullptr;
    long long total_rows_ = 0;
    long long launches_ = 0;
    std::string err_;
};

Batch::~Batch()
{
    if (device_ >= 0) cudaSetDevice(device_);
    free_device();
    eng_.clear();
    if (stream_) cudaStreamDestroy(stream_);
}

void Batch::free_device()
{
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    cudaFree(d_desc_);
    cudaFree(d_run_);
    cudaFree(d_items_);
    cudaFree(d_partials_);
    cudaFree(d_counters_);
    cudaFree(d_sync_);
    cudaFree(d_feat_);
    cudaFree(d_ws_y_);
    d_feat_ = nullptr;
    d_ws_y_ = nullptr;
    mlp_work_free(&mlp_work_);
    mlp_free(&mlp_);
    d_desc_ = nullptr;
    d_run_ = nullptr;
    d_items_ = nullptr;
    d_partials_ = nullptr;
    d_counters_ = nullptr;
    d_sync_ = nullptr;
    items_cap_ = 0;
}

pd_status Batch::fail(cudaError_t e, const char* what)
{
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? PD_ERR_OUT_OF_MEMORY : PD_ERR_CUDA;
}

pd_status Batch::init()
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device_ < 0 || device_ >= count) {
        cudaGetLastError();
        err_ = "no usable CUDA device";
        return PD_ERR_NO_DEVICE;
    }
    BCK(cudaSetDevice(device_), "cudaSetDevice");
    BCK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    BCK(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "device attribute");
    int coop = 0;
    BCK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device_), "device attribute");
    if (!coop) {
        err_ = "the device does not support cooperative launches";
        return PD_ERR_NO_DEVICE;
    }
    return PD_OK;
}

pd_status Batch::add_scene(const pd_sim_params& sim, const pd_run_params& run, const pd_solver_options& opt, int* idx)
{
    if (ready_) {
        err_ = "add_scene after make_ready";
        return PD_ERR_STATE;
    }
    if (opt.contact_enabled) {
        err_ = "PD-PD contact is not available in batches";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (opt.warm_start == 2 || opt.warm_start == 3) {
        err_ = "the history-projection guess (warm_start 2 and 3) is not available in batches";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (opt.preconditioner != 0) {
        err_ = "the preconditioned CG is not available in batches";
        return PD_ERR_INVALID_ARGUMENT;
    }
    pd_run_params r = run;
    r.gpu_device = device_;
    std::unique_ptr<Engine> e(new (std::nothrow) Engine(sim, r, opt));
    if (!e) return PD_ERR_OUT_OF_MEMORY;
    pd_status s = e->init_device();
    if (s != PD_OK) {
        err_ = e->error();
        return s;
    }
    if (!eng_.empty() && e->fp64_ != eng_[0]->fp64_) {
        err_ = "all scenes of a batch must use the same precision";
        return PD_ERR_INVALID_ARGUMENT;
    }
    eng_.push_back(std::move(e));
    if (idx) *idx = (int)eng_.size() - 1;
    return PD_OK;
}

pd_status Batch::build_items(int item_rows)
{
    items_.clear();
    for (size_t s = 0; s < eng_.size(); ++s) {
        SceneConst& C = h_desc_[s].C;
        C.item_begin = (int)items_.size();
        for (int lo = 0; lo < C.n; lo += item_rows) items_.push_back(WorkItem{(int)s, lo, std::min(C.n, lo + item_rows)});
        C.item_end = (int)items_.size();
    }
    const size_t n = std::max<size_t>(items_.size(), 1);
    if (n > items_cap_) {
        cudaFree(d_items_);
        cudaFree(d_partials_);
        d_items_ = nullptr;
        d_partials_ = nullptr;
        items_cap_ = 0;
        BCK(cudaMalloc((void**)&d_items_, sizeof(WorkItem) * n), "alloc items");
        BCK(cudaMalloc((void**)&d_partials_, sizeof(double) * 3 * n), "alloc partials");
        items_cap_ = n;
    }
    if (!items_.empty())
        BCK(cudaMemcpyAsync(d_items_, items_.data(), sizeof(WorkItem) * items_.size(), cudaMemcpyHostToDevice, stream_),
            "upload items");
    BCK(cudaMemcpyAsync(d_desc_, h_desc_.data(), sizeof(SceneDesc) * h_desc_.size(), cudaMemcpyHostToDevice, stream_),
        "upload scenes");
    BCK(cudaStreamSynchronize(stream_), "batch sync");
    item_rows_ = item_rows;
    return PD_OK;
}

BatchArgs Batch::args(int tune_reps) const
{
    BatchArgs A{};
    A.scenes = d_desc_;
    A.run = d_run_;
    A.items = d_items_;
    A.n_items = (int)items_.size();
    A.n_scenes = (int)eng_.size();
    A.partials = d_partials_;
    A.counters = d_counters_;
    A.sync = d_sync_;
    A.max_rounds = 66;
    A.max_cg_iters = max_cg_iters_;
    A.tune_reps = tune_reps;
    A.warm_start = opt_.warm_start;
    return A;
}

pd_status Batch::enqueue_step()
{
    const BatchArgs A = args(0);
    BCK(cudaMemsetAsync(d_sync_, 0, sizeof(BatchSync), stream_), "reset barrier");
    BCK(cudaMemsetAsync(d_counters_, 0, sizeof(unsigned) * eng_.size(), stream_), "reset counters");
    BCK(launch_batch_pre(fp64_, A, grid_pre_, stream_), "k_batch_pre launch");
    if (opt_.warm_start && total_rows_ > 0) {
        BCK(mlp_infer_tc(mlp_, d_feat_, (int)total_rows_, d_ws_y_, stream_), "network launch");
        const int grid_ws = std::max(1, batch_ws_blocks_per_sm(lanes_, unroll_)) * sm_count_;
        BCK(launch_batch_ws_guess(lanes_, unroll_, A, grid_ws, stream_), "k_batch_ws_guess launch");
    }
    BCK(launch_batch_cg(fp64_, lanes_, unroll_, A, grid_cg_, stream_), "k_batch_cg launch");
    return PD_OK;
}

// Learned warm start: every scene's warm-start state (without a network of
// its own), the batch's feature and output rows, and the network.
pd_status Batch::ws_setup()
{
    total_rows_ = 0;
    for (auto& e : eng_) total_rows_ += e->n_;
    if (total_rows_ >= (1LL << 31)) {
        err_ = "learned warm start: more than 2^31 particles in the batch";
        return PD_ERR_INVALID_ARGUMENT;
    }
    for (size_t s = 0; s < eng_.size(); ++s) {
        Engine& e = *eng_[s];
        pd_status st = e.ws_prepare(false);
        if (st != PD_OK) {
            err_ = "scene " + std::to_string(s) + ": " + e.error();
            return st;
        }
    }
    const size_t rows = (size_t)std::max<long long>(total_rows_, 1);
    BCK(cudaMalloc((void**)&d_feat_, sizeof(__nv_bfloat16) * kMlpIn * rows), "alloc features");
    BCK(cudaMalloc((void**)&d_ws_y_, sizeof(float) * kMlpOutPad * rows), "alloc network output");
    BCK(cudaMemsetAsync(d_feat_, 0, sizeof(__nv_bfloat16) * kMlpIn * rows, stream_), "memset features");
    BCK(mlp_alloc(&mlp_, false), "alloc network");
    BCK(mlp_work_alloc(&mlp_work_, (long long)rows, false), "alloc network rows");
    if (ws_params_.size() != mlp_param_count()) {
        ws_params_.assign(mlp_param_count(), 0.f);
        mlp_init_params(ws_params_.data(), 1u);
    }
    BCK(cudaMemcpyAsync(mlp_.params, ws_params_.data(), sizeof(float) * ws_params_.size(), cudaMemcpyHostToDevice,
                        stream_), "upload network");
    mlp_refresh_bf16(mlp_, stream_);
    BCK(cudaGetLastError(), "network set-up");
    long long off = 0;
    for (size_t s = 0; s < eng_.size(); ++s) {
        Engine& e = *eng_[s];
        SceneDesc& D = h_desc_[s];
        D.W = e.W_;
        D.W.features = d_feat_ + (size_t)off * kMlpIn;
        D.rsave = e.ws_rsave_;
        D.ws_y = d_ws_y_ + (size_t)off * kMlpOutPad;
        off += e.n_;
    }
    return PD_OK;
}

pd_status Batch::ws_set_params(const float* params, size_t count)
{
    if (!params || count != mlp_param_count()) {
        err_ = "ws_set_params: expected pd_mlp_param_count() values";
        return PD_ERR_INVALID_ARGUMENT;
    }
    ws_params_.assign(params, params + count);
    if (mlp_.params) {
        BCK(cudaSetDevice(device_), "cudaSetDevice");
        BCK(cudaMemcpyAsync(mlp_.params, ws_params_.data(), sizeof(float) * count, cudaMemcpyHostToDevice, stream_),
            "upload network");
        mlp_refresh_bf16(mlp_, stream_);
        BCK(cudaStreamSynchronize(stream_), "batch sync");
    }
    return PD_OK;
}

// Orders every scene's bond slots for the (lanes, unroll) SpMV shape (on the
// scenes' own streams, waited for before the batch's next launch).
pd_status Batch::relayout(int lanes, int unroll)
{
    for (auto& e : eng_) e->relayout_bonds(lanes, fp64_ ? 1 : unroll);
    for (auto& e : eng_) BCK(cudaStreamSynchronize(e->stream_), "relayout sync");
    return PD_OK;
}

// Launch shape: SpMV lanes x unroll and rows per work item, timed on the
// batch's own SpMV phase (y = A x over all scenes, which changes no state).
pd_status Batch::tune()
{
    std::vector<int> lanes_c = {4, 8}, unroll_c = {2, 4}, rows_c = {64, 128, 256, 512};
    if (opt_.lanes_per_particle) lanes_c = {opt_.lanes_per_particle};
    if (opt_.spmv_unroll || fp64_) unroll_c = {fp64_ ? 2 : opt_.spmv_unroll};
    if (opt_.item_rows) rows_c = {opt_.item_rows};
    long long total = 0;
    for (auto& e : eng_) total += e->n_;
    const bool measure = total >= 20000 && lanes_c.size() * unroll_c.size() * rows_c.size() > 1;
    autotuned_ = false;
    if (!measure) {
        lanes_ = lanes_c.size() == 1 ? lanes_c[0] : 8;
        unroll_ = unroll_c.size() == 1 ? unroll_c[0] : 2;
        const int rows = rows_c.size() == 1 ? rows_c[0] : 128;
        grid_cg_ = std::max(1, batch_cg_blocks_per_sm(fp64_, lanes_, unroll_)) * sm_count_;
        pd_status s = relayout(lanes_, unroll_);
        if (s != PD_OK) return s;
        return build_items(rows);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BCK(cudaEventCreate(&e0), "event");
    BCK(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    int bl = lanes_c[0], bu = unroll_c[0], br = rows_c[0];
    constexpr int reps = 4;
    for (int rows : rows_c) {
        pd_status s = build_items(rows);
        if (s != PD_OK) return s;
        for (int l : lanes_c) {
            for (int u : unroll_c) {
                const int grid = std::max(1, batch_cg_blocks_per_sm(fp64_, l, u)) * sm_count_;
                s = relayout(l, u);
                if (s != PD_OK) return s;
                BCK(cudaMemsetAsync(d_sync_, 0, sizeof(BatchSync), stream_), "reset barrier");
                BCK(launch_batch_cg(fp64_, l, u, args(1), grid, stream_), "tune launch");
                BCK(cudaEventRecord(e0, stream_), "event");
                BCK(launch_batch_cg(fp64_, l, u, args(reps), grid, stream_), "tune launch");
                BCK(cudaEventRecord(e1, stream_), "event");
                BCK(cudaEventSynchronize(e1), "tune sync");
                launches_ += 2;
                float ms = 0.f;
                BCK(cudaEventElapsedTime(&ms, e0, e1), "event");
                if (ms < best) {
                    best = ms;
                    bl = l;
                    bu = u;
                    br = rows;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    BatchSync sync{};
    BCK(cudaMemcpy(&sync, d_sync_, sizeof(sync), cudaMemcpyDeviceToHost), "read barrier");
    if (sync.error) {
        err_ = "batch autotune: a grid barrier wait timed out";
        return PD_ERR_CUDA;
    }
    lanes_ = bl;
    unroll_ = bu;
    grid_cg_ = std::max(1, batch_cg_blocks_per_sm(fp64_, lanes_, unroll_)) * sm_count_;
    tuned_ms_ = best / reps;
    autotuned_ = true;
    pd_status s = relayout(lanes_, unroll_);
    if (s != PD_OK) return s;
    return build_items(br);
}

pd_status Batch::build_graph()
{
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    BCK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
    pd_status s = enqueue_step();
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (s != PD_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess) return fail(e, "end capture");
    graph_ = g;
    BCK(cudaGraphInstantiate(&exec_, graph_, 0), "graph instantiate");
    return PD_OK;
}

pd_status Batch::make_ready()
{
    if (eng_.empty()) {
        err_ = "make_ready: the batch has no scenes";
        return PD_ERR_STATE;
    }
    BCK(cudaSetDevice(device_), "cudaSetDevice");
    ready_ = false;
    free_device();
    for (size_t s = 0; s < eng_.size(); ++s) {
        Engine& e = *eng_[s];
        e.batch_member_ = true;   // the batch kernels walk the builder's CSR rows
        pd_status st = e.make_ready();
        if (st == PD_OK) st = e.synchronize();
        if (st != PD_OK) {
            err_ = "scene " + std::to_string(s) + ": " + e.error();
            return st;
        }
    }
    fp64_ = eng_[0]->fp64_;
    if (opt_.warm_start && fp64_) {
        err_ = "the learned warm start needs mixed precision";
        return PD_ERR_INVALID_ARGUMENT;
    }
    const size_t ns = eng_.size();
    h_desc_.assign(ns, SceneDesc{});
    h_run_.assign(ns, SceneRun{});
    max_cg_iters_ = 1;
    for (size_t s = 0; s < ns; ++s) {
        Engine& e = *eng_[s];
        SceneDesc& D = h_desc_[s];
        D.P = e.step_params();
        D.S = e.S_;
        SceneConst& C = D.C;
        C.n = e.n_;
        C.integrator = e.run_.integrator;
        C.adaptive = (e.run_.integrator == PD_NEWMARK_BETA || e.run_.adaptive_integration != 0) ? 1 : 0;
        C.ticks_base = e.sim_.pd_time_step;
        C.ticks_min = e.opt_.time_step_min;
        C.max_substep = e.opt_.max_substep;
        C.phase_in_steps = e.opt_.phase_in_steps;
        C.dt_base = e.opt_.time_step_base;
        for (int k = 0; k < 3; ++k) {
            C.sphere_center0[k] = e.opt_.sphere_center[k];
            C.sphere_velocity[k] = e.opt_.sphere_velocity[k];
            C.origin[k] = e.origin_[k];
        }
        SceneRun& R = h_run_[s];
        R.step = e.step_;
        R.substep = e.substep_;
        R.ticks = e.ticks_;
        R.cg_converged = e.cg_converged_ ? 1 : 0;
        R.cs = e.clock_scale_;
        R.sim_time = e.sim_time_;
        max_cg_iters_ = std::max(max_cg_iters_, e.opt_.cg_max_iterations + 1);
    }
    if (opt_.warm_start) {
        pd_status st = ws_setup();
        if (st != PD_OK) return st;
    }
    BCK(cudaMalloc((void**)&d_desc_, sizeof(SceneDesc) * ns), "alloc scenes");
    BCK(cudaMalloc((void**)&d_run_, sizeof(SceneRun) * ns), "alloc run");
    BCK(cudaMalloc((void**)&d_counters_, sizeof(unsigned) * ns), "alloc counters");
    BCK(cudaMalloc((void**)&d_sync_, sizeof(BatchSync)), "alloc barrier");
    BCK(cudaMemsetAsync(d_counters_, 0, sizeof(unsigned) * ns, stream_), "reset counters");
    BCK(cudaMemsetAsync(d_sync_, 0, sizeof(BatchSync), stream_), "reset barrier");
    BCK(cudaMemcpyAsync(d_run_, h_run_.data(), sizeof(SceneRun) * ns, cudaMemcpyHostToDevice, stream_), "upload run");
    grid_pre_ = std::max(1, batch_pre_blocks_per_sm(fp64_)) * sm_count_;
    pd_status st = tune();
    if (st != PD_OK) return st;
    if (opt_.use_graph) {
        st = build_graph();
        if (st != PD_OK) return st;
    }
    BCK(cudaStreamSynchronize(stream_), "batch sync");
    ready_ = true;
    return PD_OK;
}

// Device step records -> the scenes' Engine mirrors.
pd_status Batch::pull_state()
{
    const size_t ns = eng_.size();
    BCK(cudaMemcpyAsync(h_run_.data(), d_run_, sizeof(SceneRun) * ns, cudaMemcpyDeviceToHost, stream_), "read run");
    BCK(cudaMemcpyAsync(h_desc_.data(), d_desc_, sizeof(SceneDesc) * ns, cudaMemcpyDeviceToHost, stream_), "read scenes");
    BatchSync sync{};
    BCK(cudaMemcpyAsync(&sync, d_sync_, sizeof(sync), cudaMemcpyDeviceToHost, stream_), "read barrier");
    BCK(cudaStreamSynchronize(stream_), "batch sync");
    for (size_t s = 0; s < ns; ++s) {
        Engine& e = *eng_[s];
        const SceneRun& R = h_run_[s];
        e.step_ = R.step;
        e.substep_ = R.substep;
        e.ticks_ = R.ticks;
        e.clock_scale_ = R.cs;
        e.sim_time_ = R.sim_time;
        e.cg_converged_ = R.cg_converged != 0;
        e.last_iters_ = R.last_iters;
        e.total_iters_ = R.total_iters;
        e.last_res_ = R.last_res;
        e.last_tol_ = R.last_tol;
        e.retries_ = R.retries;
        e.last_params_ = h_desc_[s].P;
    }
    if (opt_.warm_start) {
        std::vector<CgScalars> sc(ns);
        for (size_t s = 0; s < ns; ++s)
            BCK(cudaMemcpyAsync(&sc[s], eng_[s]->S_.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, stream_),
                "read CG scalars");
        BCK(cudaStreamSynchronize(stream_), "batch sync");
        for (size_t s = 0; s < ns; ++s) {
            Engine& e = *eng_[s];
            e.ws_kept_ = sc[s].ws_kept;
            e.ws_skipped_ = sc[s].ws_skipped;
            e.last_ws_ratio_ = (sc[s].rz_plain > 0 && !sc[s].ws_skip) ? std::sqrt(sc[s].rz_learned / sc[s].rz_plain)
                                                                      : 0.0;
        }
    }
    if (sync.error) {
        ready_ = false;
        err_ = "batch step: a grid barrier wait timed out";
        return PD_ERR_CUDA;
    }
    if (opt_.warm_start && mlp_tc_take_error()) {
        err_ = "batch step: a wait of the warm-start network's tensor-core kernel ran out of time";
        return PD_ERR_CUDA;
    }
    for (size_t s = 0; s < ns; ++s) {
        if (h_run_[s].error) {
            err_ = "scene " + std::to_string(s) + ": adaptive time step: too many rollbacks";
            return PD_ERR_STATE;
        }
    }
    return PD_OK;
}

pd_status Batch::advance(int nsteps)
{
    if (!ready_) {
        err_ = "advance: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    if (nsteps < 0) return PD_ERR_INVALID_ARGUMENT;
    BCK(cudaSetDevice(device_), "cudaSetDevice");
    for (int k = 0; k < nsteps; ++k) {
        if (exec_) {
            BCK(cudaGraphLaunch(exec_, stream_), "graph launch");
        } else {
            pd_status s = enqueue_step();
            if (s != PD_OK) return s;
        }
        launches_ += 2 + (opt_.warm_start ? 2 : 0);   // + the network's tensor-core kernel and the guess
    }
    return pull_state();
}

pd_status Batch::config(pd_batch_config* c) const
{
    std::memset(c, 0, sizeof(*c));
    c->lanes_per_particle = lanes_;
    c->spmv_unroll = fp64_ ? 1 : unroll_;
    c->item_rows = item_rows_;
    c->work_items = (int)items_.size();
    c->grid_pre = grid_pre_;
    c->grid_cg = grid_cg_;
    c->autotuned = autotuned_ ? 1 : 0;
    c->tuned_spmv_ms = tuned_ms_;
    c->warm_start = opt_.warm_start;
    return PD_OK;
}

pd_status Batch::synchronize()
{
    BCK(cudaSetDevice(device_), "cudaSetDevice");
    BCK(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return PD_OK;
}

}  // namespace pdgb

struct pd_batch {
    pdgb::Batch* b;
};

namespace {
thread_local std::string g_batch_error;

pd_status scene_checked(pd_batch* b, int scene, pdgb::Engine** e)
{
    if (!b || !b->b) return PD_ERR_INVALID_ARGUMENT;
    *e = b->b->scene(scene);
    if (!*e) {
        b->b->set_error("scene index out of range");
        return PD_ERR_INVALID_ARGUMENT;
    }
    return PD_OK;
}
}  // namespace

extern "C" {

pd_status pd_batch_options_default(pd_batch_options* opt)
{
    if (!opt) return PD_ERR_INVALID_ARGUMENT;
    std::memset(opt, 0, sizeof(*opt));
    opt->use_graph = 1;
    return PD_OK;
}

pd_status pd_batch_create(int device, const pd_batch_options* opt, pd_batch** out)
{
    if (!out) return PD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    pd_batch_options o;
    if (opt) o = *opt;
    else pd_batch_options_default(&o);
    if ((o.lanes_per_particle != 0 && o.lanes_per_particle != 4 && o.lanes_per_particle != 8) ||
        (o.spmv_unroll != 0 && o.spmv_unroll != 2 && o.spmv_unroll != 4) ||
        (o.item_rows != 0 && (o.item_rows < 64 || o.item_rows > 4096)) || (o.warm_start != 0 && o.warm_start != 1)) {
        g_batch_error = "batch options: lanes 0/4/8, unroll 0/2/4, item_rows 0 or 64..4096, warm_start 0/1";
        return PD_ERR_INVALID_ARGUMENT;
    }
    pd_batch* h = new (std::nothrow) pd_batch{nullptr};
    if (!h) return PD_ERR_OUT_OF_MEMORY;
    h->b = new (std::nothrow) pdgb::Batch(device, o);
    if (!h->b) {
        delete h;
        return PD_ERR_OUT_OF_MEMORY;
    }
    pd_status s = h->b->init();
    if (s != PD_OK) {
        g_batch_error = h->b->error();
        delete h->b;
        delete h;
        return s;
    }
    *out = h;
    return PD_OK;
}

pd_status pd_batch_destroy(pd_batch* b)
{
    if (!b) return PD_ERR_INVALID_ARGUMENT;
    delete b->b;
    delete b;
    return PD_OK;
}

pd_status pd_batch_add_scene(pd_batch* b, const pd_sim_params* sim, const pd_run_params* run,
                             const pd_solver_options* opt, int* scene)
{
    if (!b || !b->b || !sim || !run) return PD_ERR_INVALID_ARGUMENT;
    if (sim->num_pd_particle < 0 || (run->integrator != PD_IMPLICIT_EULER && run->integrator != PD_NEWMARK_BETA)) {
        b->b->set_error("num_pd_particle < 0 or unknown integrator");
        return PD_ERR_INVALID_ARGUMENT;
    }
    pd_solver_options o;
    if (opt) o = *opt;
    else pd_solver_options_default(&o);
    if ((o.precision != PD_PRECISION_MIXED && o.precision != PD_PRECISION_FP64) || !(o.time_step_base > 0) ||
        sim->pd_time_step <= 0) {
        b->b->set_error("unknown precision mode or non-positive time step");
        return PD_ERR_INVALID_ARGUMENT;
    }
    return b->b->add_scene(*sim, *run, o, scene);
}

pd_status pd_batch_set_particles(pd_batch* b, int scene, const double* pos4, const double* vel4,
                                 const int32_t* activity, int n)
{
    pdgb::Engine* e = nullptr;
    pd_status s = scene_checked(b, scene, &e);
    if (s != PD_OK) return s;
    if (!pos4 && n > 0) return PD_ERR_INVALID_ARGUMENT;
    s = e->set_particles(pos4, vel4, activity, n);
    if (s != PD_OK) b->b->set_error(e->error());
    return s;
}

pd_status pd_batch_set_stretch_limits(pd_batch* b, int scene, const double* s0, int n)
{
    pdgb::Engine* e = nullptr;
    pd_status s = scene_checked(b, scene, &e);
    if (s != PD_OK) return s;
    if (!s0 && n > 0) return PD_ERR_INVALID_ARGUMENT;
    s = e->set_stretch(s0, n);
    if (s != PD_OK) b->b->set_error(e->error());
    return s;
}

pd_status pd_batch_ws_set_params(pd_batch* b, const float* params, size_t count)
{
    if (!b || !b->b) return PD_ERR_INVALID_ARGUMENT;
    return b->b->ws_set_params(params, count);
}

pd_status pd_batch_make_ready(pd_batch* b)
{
    if (!b || !b->b) return PD_ERR_INVALID_ARGUMENT;
    return b->b->make_ready();
}

pd_status pd_batch_advance(pd_batch* b, int nsteps)
{
    if (!b || !b->b) return PD_ERR_INVALID_ARGUMENT;
    return b->b->advance(nsteps);
}

pd_status pd_batch_scene_count(pd_batch* b, int* count)
{
    if (!b || !b->b || !count) return PD_ERR_INVALID_ARGUMENT;
    *count = b->b->count();
    return PD_OK;
}

pd_status pd_batch_scene_offsets(pd_batch* b, int64_t* offsets, int count_plus_one)
{
    if (!b || !b->b || !offsets || count_plus_one != b->b->count() + 1) return PD_ERR_INVALID_ARGUMENT;
    int64_t acc = 0;
    for (int s = 0; s < b->b->count(); ++s) {
        offsets[s] = acc;
        pd_sim_params sim;
        b->b->scene(s)->params(&sim, nullptr, nullptr);
        acc += sim.num_pd_particle;
    }
    offsets[b->b->count()] = acc;
    return PD_OK;
}

pd_status pd_batch_get(pd_batch* b, int scene, pd_variable var, void* dst, size_t bytes)
{
    pdgb::Engine* e = nullptr;
    pd_status s = scene_checked(b, scene, &e);
    if (s != PD_OK) return s;
    s = e->get(var, dst, bytes);
    if (s != PD_OK) b->b->set_error(e->error());
    return s;
}

pd_status pd_batch_get_size(pd_batch* b, int scene, pd_variable var, size_t* bytes)
{
    pdgb::Engine* e = nullptr;
    pd_status s = scene_checked(b, scene, &e);
    if (s != PD_OK) return s;
    if (!bytes) return PD_ERR_INVALID_ARGUMENT;
    return e->get_size(var, bytes);
}

pd_status pd_batch_get_stats(pd_batch* b, int scene, pd_step_stats* stats)
{
    pdgb::Engine* e = nullptr;
    pd_status s = scene_checked(b, scene, &e);
    if (s != PD_OK) return s;
    if (!stats) return PD_ERR_INVALID_ARGUMENT;
    return e->stats(stats);
}

pd_status pd_batch_finished(pd_batch* b, int scene, int* finished)
{
    pdgb::Engine* e = nullptr;
    pd_status s = scene_checked(b, scene, &e);
    if (s != PD_OK) return s;
    if (!finished) return PD_ERR_INVALID_ARGUMENT;
    *finished = e->finished() ? 1 : 0;
    return PD_OK;
}

pd_status pd_batch_get_config(pd_batch* b, pd_batch_config* config)
{
    if (!b || !b->b || !config) return PD_ERR_INVALID_ARGUMENT;
    if (!b->b->ready()) return PD_ERR_NOT_READY;
    return b->b->config(config);
}

pd_status pd_batch_get_launch_count(pd_batch* b, long long* launches)
{
    if (!b || !b->b || !launches) return PD_ERR_INVALID_ARGUMENT;
    long long n = b->b->launches();
    for (int s = 0; s < b->b->count(); ++s) n += b->b->scene(s)->launches();
    *launches = n;
    return PD_OK;
}

pd_status pd_batch_get_stream(pd_batch* b, void** stream)
{
    if (!b || !b->b || !stream) return PD_ERR_INVALID_ARGUMENT;
    *stream = (void*)b->b->stream();
    return PD_OK;
}

pd_status pd_batch_synchronize(pd_batch* b)
{
    if (!b || !b->b) return PD_ERR_INVALID_ARGUMENT;
    return b->b->synchronize();
}

const char* pd_batch_last_error_message(pd_batch* b)
{
    if (!b || !b->b) return g_batch_error.c_str();
    return b->b->error().c_str();
}

}  // extern "C"
