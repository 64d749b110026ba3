// engine.h -- host driver of the GB300 PD step (the Simulator of the reference).
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pd_gb300.h"
#include "pd_kernels.h"

namespace pdgb {

class Batch;

// profiling: CG-loop kernels are timed on every kMarkStride-th iteration
constexpr int kMarkStride = 8;

class Engine {
    friend class Batch;   // the multi-scene step drives the scenes' device state

public:
    Engine(const pd_sim_params& sim, const pd_run_params& run, const pd_solver_options& opt);
    ~Engine();

    pd_status init_device();
    pd_status set_particles(const double* pos4, const double* vel4, const int32_t* act, int n);
    pd_status set_stretch(const double* s0, int n);
    pd_status make_ready();
    pd_status advance(int nsteps);
    bool finished() const;
    bool cg_converged() const { return cg_converged_; }
    int current_step() const { return step_; }
    pd_status get(pd_variable var, void* dst, size_t bytes);
    pd_status get_size(pd_variable var, size_t* bytes) const;
    pd_status stats(pd_step_stats* s) const;
    void params(pd_sim_params* s, pd_run_params* r, pd_solver_options* o) const;
    void set_profiling(bool on) { profiling_ = on; }
    pd_status kernel_times(pd_kernel_times* t);
    void reset_kernel_times();
    long long launches() const { return launches_; }
    cudaStream_t stream() const { return stream_; }
    pd_status synchronize();
    pd_status operator_view(pd_operator_view* v) const;
    pd_status apply_operator(const void* d_x, void* d_y, double* d_dot);
    pd_status ws_set_params(const float* params, size_t count);
    pd_status ws_get_params(float* params, size_t count);
    pd_status ws_collect(int samples_per_step, long long capacity);
    pd_status ws_dataset(float* X, float* T, long long max_rows, long long* rows);
    const std::string& error() const { return err_; }
    // DataIO (dataio.cpp): frames, simulation info and checkpoints under run.saving_path
    pd_status dataio_write_frame();
    void dataio_new_frame() { ++saved_frame_; }
    size_t dataio_saved_frame() const { return saved_frame_; }
    pd_status dataio_save_state(size_t timestep);
    pd_status dataio_load_state(size_t timestep);
    // the reference's own checkpoint layout (STATE/state.<step>, dataIO.cu:123-198)
    pd_status dataio_save_state_reference(size_t timestep);
    pd_status dataio_load_state_reference(size_t timestep);
    std::string ref_state_path(size_t timestep) const;
    // SPH <-> PD collision (collideDifferentParticles) with the caller's SPH particles
    pd_status sph_collide(double* pos4, double* vel4, int n_sph, double slip, int* collided);

private:
    pd_status dataio_write_sim_info();
    pd_status cuda_fail(cudaError_t e, const char* what);
    pd_status allocate();
    void free_all();
    StepParams step_params() const;
    int grid_for_rows(int lanes, int blocks_per_sm) const;
    pd_status tune_spmv();
    // y = A in with this handle's product (lattice stencil or CSR rows)
    void apply_op(const StepParams& P, const void* in, void* out, ReduceSlot slot, double* dot_out);
    void lattice_resync(bool force);   // the lattice product's 1/d0 table from the live CSR bonds
    // mixed mode: reorders every row's live bonds for the (g, u) SpMV shape
    void relayout_bonds(int g, int u);
    // allocates the warm-start state on first use; without the network
    // (a batch scene: the batch owns the features, the network and its rows)
    pd_status ws_prepare(bool with_network = true);
    void ws_free();
    bool ws_features_needed() const;
    pd_status ws_before_cg(const StepParams& P);
    pd_status ws_after_cg(const StepParams& P);
    // history projection (warm_start = 2): buffers, the guess, the push of an
    // accepted solution, and forgetting the history (new state)
    pd_status hist_prepare();
    void hist_free();
    pd_status hist_project(const StepParams& P);
    pd_status hist_push();
    void hist_reset() { hist_m_ = 0, hist_next_ = 0; }
    void* hist_vec(int j) const;
    pd_status integrate(bool* advanced);
    pd_status solve(const StepParams& P);
    // one CG iteration's launches (iteration k of the solve: on lattice bodies
    // its parity picks the direction buffers); cond: the CG graph's while
    // condition when captured into it, else 0
    void cg_iteration(const StepParams& P, int k, cudaGraphConditionalHandle cond, bool sample);
    int cg_kernels_per_iteration() const { return (L_.lattice && d_p2_) ? 2 : 3; }
    int cg_graph_body() const;
    // iterations 1.. of a solve as one graph launch: a while node repeating
    // cg_graph_body() iterations until the device-side test stops it
    cudaError_t cg_graph_launch(const StepParams& P);
    pd_status cg_host_loop(const StepParams& P);   // the same iterations in host-checked batches
    void hist_collect();   // the projection's statistics, after the solve's read-back
    template <typename T>
    pd_status download_scatter(const T* dev, T* host_out, size_t count_per, size_t elem_count);
    pd_status ensure_stage(size_t bytes);   // device staging buffer of the exports
    pd_status export_vec4(const void* dev, bool real_is_float, double* dst);
    pd_status export_bonds(int64_t* row_ptr_out, int32_t* list_out);
    // profiling
    struct Mark {
        int kc;
        int iter;   // CG iteration index for SpMV marks, -1 otherwise
        cudaEvent_t a, b;
    };
    void mark_begin(int kc, int iter);
    void mark_end();
    // synced: every mark was recorded before the latest stream synchronisation
    void flush_marks(int live_iters, bool synced = false);
    cudaEvent_t take_event();

    pd_sim_params sim_;
    pd_run_params run_;
    pd_solver_options opt_;
    bool fp64_ = false;
    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    int sm_count_ = 0;
    int n_ = 0;
    bool particles_set_ = false;
    bool stretch_set_ = false;
    bool ready_ = false;
    std::vector<double> h_pos_, h_vel_, h_s0_;
    std::vector<int32_t> h_act_;
    std::vector<int> perm_, inv_, cnt_init_;
    double origin_[3] = {0, 0, 0};
    double sup_ = 0;              // supercell edge of the FP32 positions
    double sup_lo_[3] = {0, 0, 0};
    double bond_coeff_ = 0;
    long long total_slots_ = 0;
    long long bonds_initial_ = 0;
    DeviceState S_{};
    int* d_perm_ = nullptr;
    void* d_stage_ = nullptr;     // exports in caller order before the copy to the host
    size_t stage_cap_ = 0;
    CgScalars* h_sc_ = nullptr;   // pinned
    int* h_flags_ = nullptr;      // pinned
    LaunchCfg L_{};
    StepParams last_params_{};   // constants of the latest step (the operator's time step)
    float tuned_ms_ = 0.f;       // SpMV time of the autotuned variant
    int lay_g_ = 1, lay_u_ = 1;  // SpMV shape the bond slots are ordered for (u = 1: build order)
    // learned warm start
    WsState W_{};
    MlpDev mlp_{};
    MlpWork mlp_work_{};
    float4* ws_rsave_ = nullptr;
    bool ws_ready_ = false;
    bool ws_params_loaded_ = false;
    std::vector<float> ws_params_;
    int ws_samples_ = 0;
    long long ws_cap_ = 0, ws_pos_ = 0, ws_count_ = 0;
    unsigned long long ws_rng_ = 88172645463325252ull;
    double last_ws_ratio_ = 0.0;
    long long ws_kept_ = 0;
    long long ws_skipped_ = 0;    // batch scenes: steps whose learned pass was paused
    // history projection
    int hist_cap_ = 0, hist_m_ = 0, hist_next_ = 0, hist_blocks_ = 0;
    void* d_hist_ = nullptr;      // hist_cap_ vectors of n entries: accepted solutions, Dirichlet rows 0
    void* d_ahist_ = nullptr;     // their products with this step's operator
    void* d_hnet_ = nullptr;      // warm_start 3: the network's correction (the projection's last column)
    long long ws_net_used_ = 0;   // warm_start 3: projections that gave the network's column a weight
    double* d_hpart_ = nullptr;   // per-block partial sums of a Gram pass
    CgScalars* h_sc_hist_ = nullptr;   // pinned: scalars after the projected residual
    HistSolve* d_hsol_ = nullptr;      // the m x m solve's result (device)
    HistSolve* h_hsol_ = nullptr;      // pinned: written by the host callback, copied to d_hsol_
    double* h_hpart_ = nullptr;        // pinned: block partials of both Gram passes
    CgScalars* h_sc_pre_ = nullptr;    // pinned: scalars of the previous solution's residual
    HistHostSolve hist_cb_{};          // arguments of the callback (alive until it ran)
    bool hist_pending_ = false;        // a projection ran in this solve
    // step state (Simulator members)
    int step_ = 0;
    int substep_ = 0;
    int ticks_ = 0;
    double clock_scale_ = 0;
    double sim_time_ = 0;
    bool cg_converged_ = true;
    int last_iters_ = 0;
    double last_res_ = 0;
    double last_tol_ = 0;
    long long total_iters_ = 0;
    int retries_ = 0;
    int predicted_iters_ = 0;
    long long host_syncs_ = 0;         // stream synchronisations of the step loop
    long long cg_graph_solves_ = 0;    // solves whose iterations ran in the CG graph
    bool cg_graph_failed_ = false;     // the graph could not be built: host-checked batches
    // profiling
    bool profiling_ = false;
    std::vector<cudaEvent_t> event_pool_;
    std::vector<Mark> marks_;
    int open_mark_ = -1;
    long long kc_launches_[PD_KC_COUNT] = {};
    double kc_ms_[PD_KC_COUNT] = {};
    long long kc_samples_[PD_KC_COUNT] = {};   // sampled CG iterations
    double kc_sample_ms_[PD_KC_COUNT] = {};
    long long launches_ = 0;
    // lattice-stencil product (mixed mode, lattice-filled bodies)
    LatticeParams lat_{};
    LatticeBuffers latb_{};
    bool lat_ok_ = false;
    bool lat_fixed_built_ = false;     // the stencil is the 80-entry one (compile-time kernel available)
    void* d_p2_ = nullptr;             // second CG direction buffer of the lattice product's fused update
    bool batch_member_ = false;        // set by Batch: its scenes keep the builder's slot order
    ContactBuffers contact_{};         // PD-PD contact hash (when enabled)
    SphBuffers sph_{};                 // SPH <-> PD collision scratch
    size_t saved_frame_ = 0;           // DataIO::savedFrame
    bool wrote_sim_info_ = false;      // DataIO::writtenSimulationParameter
    std::string err_;
};

}  // namespace pdgb
