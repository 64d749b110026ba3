// engine.cpp -- host driver of the GB300 PD step.
//
// Mirrors Simulator (src/core/simulator.cu): makeReady (:56-89), advance
// (:1159-1182), integratePeridynamicsImplicitEuler/NewmarkBeta (:297-652)
// including the adaptive time-step rollback (:332-401, :506-572), and
// solveLinearSystem (:735-799).  Differences by design:
//  * bonds are built on the GPU (bonds.cu) instead of the host kd-tree;
//  * particles live in cell-sorted slots; exports map back to caller order;
//  * the CG runs on the device: its scalars never leave the GPU inside an
//    iteration; the host reads one small record every few iterations;
//  * errors are returned as pd_status instead of exit().
#include "engine.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

namespace pdgb {

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

template <typename T>
static cudaError_t dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, sizeof(T) * count);
}

Engine::Engine(const pd_sim_params& sim, const pd_run_params& run, const pd_solver_options& opt)
    : sim_(sim), run_(run), opt_(opt)
{
    fp64_ = opt_.precision == PD_PRECISION_FP64;
    device_ = run_.gpu_device;
    n_ = sim_.num_pd_particle;
    ticks_ = sim_.pd_time_step;
    clock_scale_ = opt_.phase_in_steps > 0 ? sim_.clockScale : 1.0;
    // the reference evaluates pd_C_times_V * PD_K inside the kernel (cg_solver.cuh:299,325)
    bond_coeff_ = opt_.bond_stiffness > 0 ? opt_.bond_stiffness : sim_.pd_C_times_V * opt_.pd_k;
}

Engine::~Engine()
{
    if (device_ >= 0) cudaSetDevice(device_);
    free_all();
    for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
    for (Mark& m : marks_) {
        cudaEventDestroy(m.a);
        cudaEventDestroy(m.b);
    }
    if (h_sc_) cudaFreeHost(h_sc_);
    if (h_flags_) cudaFreeHost(h_flags_);
    if (stream_) cudaStreamDestroy(stream_);
}

pd_status Engine::cuda_fail(cudaError_t e, const char* what)
{
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return PD_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice || e == cudaErrorInsufficientDriver)
        return PD_ERR_NO_DEVICE;
    return PD_ERR_CUDA;
}

pd_status Engine::init_device()
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        err_ = "no CUDA device";
        cudaGetLastError();
        return PD_ERR_NO_DEVICE;
    }
    if (device_ < 0 || device_ >= count) {
        err_ = "gpu_device out of range";
        return PD_ERR_NO_DEVICE;
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    CK(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "device attribute");
    CK(cudaMallocHost((void**)&h_sc_, sizeof(CgScalars)), "cudaMallocHost");
    CK(cudaMallocHost((void**)&h_flags_, sizeof(int) * 4), "cudaMallocHost");
    std::memset(h_sc_, 0, sizeof(CgScalars));
    return PD_OK;
}

pd_status Engine::set_particles(const double* pos4, const double* vel4, const int32_t* act, int n)
{
    if (n != n_ || n < 0 || (n > 0 && !pos4)) {
        err_ = "set_particles: n must equal num_pd_particle";
        return PD_ERR_INVALID_ARGUMENT;
    }
    h_pos_.assign(pos4, pos4 + 4 * (size_t)n);
    if (vel4) h_vel_.assign(vel4, vel4 + 4 * (size_t)n);
    else h_vel_.assign(4 * (size_t)n, 0.0);
    if (act) {
        h_act_.assign(act, act + n);
        for (int i = 0; i < n; ++i)
            if (h_act_[i] < 0 || h_act_[i] > PD_PRESCRIBED) {
                err_ = "set_particles: activity code out of range";
                return PD_ERR_INVALID_ARGUMENT;
            }
    } else {
        h_act_.assign(n, PD_ACTIVE);
    }
    for (int i = 0; i < 4 * n; ++i)
        if (!std::isfinite(h_pos_[i]) || !std::isfinite(h_vel_[i])) {
            err_ = "set_particles: non-finite position or velocity";
            return PD_ERR_INVALID_ARGUMENT;
        }
    particles_set_ = true;
    ready_ = false;
    return PD_OK;
}

pd_status Engine::set_stretch(const double* s0, int n)
{
    if (n != n_ || (n > 0 && !s0)) return PD_ERR_INVALID_ARGUMENT;
    h_s0_.assign(s0, s0 + n);
    stretch_set_ = true;
    ready_ = false;
    return PD_OK;
}

void Engine::free_all()
{
    ws_free();
    hist_free();
    void* ptrs[] = {S_.act, S_.x64, S_.v64, S_.X64, S_.x64_bk, S_.v64_bk, S_.st, S_.ost, S_.nst, S_.row_ptr,
                    S_.cnt, S_.cnt_bk, S_.col, S_.X32, S_.u32, S_.xs4, S_.inv_d0, S_.jac, S_.jdiag, S_.force, S_.rhs, S_.sol,
                    S_.r, S_.p, S_.y, S_.z, S_.pc, S_.sc, S_.partials, S_.counters, S_.flags, S_.lidx, S_.d0sq, S_.lim,
                    S_.xlo4, d_perm_, d_stage_};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    free_tiles(S_);
    lattice_free(&latb_);
    sph_buffers_free(&sph_);
    lat_ = LatticeParams{};
    lat_ok_ = false;
    lat_fixed_built_ = false;
    if (d_p2_) cudaFree(d_p2_);
    d_p2_ = nullptr;
    L_.lattice = 0;
    L_.lat = nullptr;
    cudaFree(contact_.counts);
    cudaFree(contact_.start);
    cudaFree(contact_.cursor);
    cudaFree(contact_.bucket);
    cudaFree(contact_.list);
    contact_ = ContactBuffers{};
    S_ = DeviceState{};
    d_perm_ = nullptr;
    d_stage_ = nullptr;
    stage_cap_ = 0;
}

pd_status Engine::allocate()
{
    const size_t n = (size_t)n_;
    const size_t r4 = fp64_ ? sizeof(dbl4) : sizeof(float4);
    S_.n = n_;
    CK(dalloc(&S_.act, n), "alloc act");
    CK(dalloc(&S_.x64, n), "alloc x");
    CK(dalloc(&S_.v64, n), "alloc v");
    CK(dalloc(&S_.X64, n), "alloc X");
    CK(dalloc(&S_.x64_bk, n), "alloc x backup");
    CK(dalloc(&S_.v64_bk, n), "alloc v backup");
    CK(dalloc(&S_.st, n), "alloc stretch");
    CK(dalloc(&S_.ost, n), "alloc original stretch");
    CK(dalloc(&S_.nst, n), "alloc new stretch");
    CK(dalloc(&S_.lim, n), "alloc stretch limits");
    CK(dalloc(&S_.row_ptr, n + 1), "alloc row_ptr");
    CK(dalloc(&S_.cnt, n), "alloc cnt");
    CK(dalloc(&S_.cnt_bk, n), "alloc cnt backup");
    CK(dalloc(&S_.X32, n), "alloc X32");
    CK(dalloc(&S_.u32, n), "alloc u32");
    if (!fp64_) CK(dalloc(&S_.xs4, n), "alloc xs4");
    if (!fp64_) CK(dalloc(&S_.xlo4, n), "alloc xlo4");
    void** vecs[] = {&S_.force, &S_.rhs, &S_.sol, &S_.r, &S_.p, &S_.y};
    for (void** v : vecs) {
        CK(cudaMalloc(v, r4 * (n ? n : 1)), "alloc vector");
        CK(cudaMemsetAsync(*v, 0, r4 * (n ? n : 1), stream_), "memset vector");
    }
    if (fp64_) CK(dalloc(&S_.jdiag, 6 * n), "alloc jdiag");
    if (opt_.preconditioner) {   // z and the inverse diagonal blocks (two Real4 per particle)
        CK(cudaMalloc(&S_.z, r4 * (n ? n : 1)), "alloc z");
        CK(cudaMemsetAsync(S_.z, 0, r4 * (n ? n : 1), stream_), "memset z");
        CK(cudaMalloc(&S_.pc, 2 * r4 * (n ? n : 1)), "alloc preconditioner");
    }
    CK(dalloc(&S_.sc, 1), "alloc scalars");
    CK(dalloc(&S_.partials, 4 * (size_t)kMaxPartials), "alloc partials");
    CK(dalloc(&S_.counters, 8), "alloc counters");
    CK(dalloc(&S_.flags, 4), "alloc flags");
    CK(cudaMemsetAsync(S_.counters, 0, sizeof(unsigned) * 8, stream_), "memset counters");
    CK(cudaMemsetAsync(S_.flags, 0, sizeof(int) * 4, stream_), "memset flags");
    CK(cudaMemsetAsync(S_.u32, 0, sizeof(float4) * (n ? n : 1), stream_), "memset u32");
    return PD_OK;
}

pd_status Engine::make_ready()
{
    if (!particles_set_) {
        err_ = "make_ready: particles not set";
        return PD_ERR_NOT_READY;
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    ready_ = false;
    free_all();
    pd_status s = allocate();
    if (s != PD_OK) return s;
    const int n = n_;
    const size_t N = (size_t)n;

    struct Tmp {   // staging buffers in caller order, freed on every return path
        dbl4* pos = nullptr;
        double* s0 = nullptr;
        int* act = nullptr;
        ~Tmp() { cudaFree(pos); cudaFree(s0); cudaFree(act); }
    } tmp;
    CK(dalloc(&tmp.pos, N), "alloc tmp");
    CK(dalloc(&tmp.s0, N), "alloc tmp");
    CK(dalloc(&tmp.act, N), "alloc tmp");
    dbl4* d_tmp4 = tmp.pos;
    double* d_tmp1 = tmp.s0;
    int* d_tmpi = tmp.act;

    // bonds (replaces initPeridynamicsBonds' kd-tree, simulator.cu:825-943)
    if (n > 0) CK(cudaMemcpyAsync(d_tmp4, h_pos_.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice, stream_), "upload pos");
    BondBuildOut out{};
    out.row_ptr = S_.row_ptr;
    out.cnt = S_.cnt;
    CK(build_bonds(d_tmp4, n, sim_.pd_horizon, opt_.max_bonds_per_particle, S_.x64, S_.X32, origin_, &out, stream_),
       "build_bonds");
    d_perm_ = out.perm;
    S_.col = out.col;
    if (out.overflow) {
        err_ = out.overflow == 2 ? "bond list exceeds 2^31 slots"
                                 : "a particle has more bonds than max_bonds_per_particle";
        sim_.pd_max_num_bonds = out.max_bonds;
        return PD_ERR_BOND_OVERFLOW;
    }
    if (n == 0) {
        CK(dalloc(&d_perm_, 1), "alloc perm");
        CK(dalloc(&S_.col, 8), "alloc col");
    }
    total_slots_ = out.total;
    bonds_initial_ = out.bonds;
    sim_.pd_max_num_bonds = out.max_bonds;
    // lattice-filled bodies: slots renumbered brick by brick for the stencil
    // product (mixed mode; automatic above kLatticeMinRows particles, or asked
    // for with spmv_path 3).  Bodies that are not a lattice fill keep the
    // builder's order and the gather product.
    if (!fp64_ && n > 0 && !batch_member_ &&
        (opt_.spmv_path == 3 || (opt_.spmv_path == 0 && n >= kLatticeMinRows))) {
        int ok = 0;
        CK(lattice_build(n, 2.0 * sim_.pd_particle_radius, S_.x64, S_.X32, d_perm_, S_.row_ptr, S_.cnt, &S_.col,
                         total_slots_, &lat_, &latb_, &ok, stream_),
           "lattice build");
        lat_ok_ = ok != 0;
        lat_fixed_built_ = lat_ok_ && lat_.fixed != 0;
        if (lat_ok_) CK(cudaMalloc(&d_p2_, sizeof(float4) * N), "alloc second direction buffer");
    }
    if (n > 0) {
        CK(cudaMemcpyAsync(S_.X64, S_.x64, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "copy X");
        CK(cudaMemcpyAsync(d_tmp4, h_vel_.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice, stream_), "upload v");
        gather_double4(d_tmp4, d_perm_, S_.v64, n, stream_);
        CK(cudaMemcpyAsync(d_tmpi, h_act_.data(), sizeof(int) * N, cudaMemcpyHostToDevice, stream_), "upload act");
        gather_int_to_u8(d_tmpi, d_perm_, S_.act, n, stream_);
        // s0_i = getstretch(s0) after srand(1973), in caller order (simulator.cu:852-857)
        std::vector<double> s0 = h_s0_;
        if (!stretch_set_) {
            s0.assign(N, 0.0);
            pd_sample_stretch_limits(run_.pd_stretch_limit_s0, n, s0.data());
        }
        CK(cudaMemcpyAsync(d_tmp1, s0.data(), sizeof(double) * N, cudaMemcpyHostToDevice, stream_), "upload s0");
        gather_double(d_tmp1, d_perm_, S_.ost, n, stream_);
        CK(cudaMemcpyAsync(S_.st, S_.ost, sizeof(double) * N, cudaMemcpyDeviceToDevice, stream_), "copy st");
        CK(cudaMemcpyAsync(S_.nst, S_.ost, sizeof(double) * N, cudaMemcpyDeviceToDevice, stream_), "copy nst");
        if (!fp64_) {
            launch_stretch_limits(S_, (int)std::min<long long>(((long long)n + kBlock - 1) / kBlock, 4096), stream_);
            ++launches_;
        }
        CK(cudaMemcpyAsync(S_.cnt_bk, S_.cnt, sizeof(int) * N, cudaMemcpyDeviceToDevice, stream_), "backup cnt");
        CK(cudaMemcpyAsync(S_.x64_bk, S_.x64, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "backup x");
        CK(cudaMemcpyAsync(S_.v64_bk, S_.v64, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "backup v");
        launches_ += 3;
    }
    if (fp64_) {
        CK(dalloc(&S_.jac, 6 * (size_t)std::max<long long>(total_slots_, 1)), "alloc jac");
    } else {
        // 1/d0 per bond slot, and the supercell frame of the FP32 positions:
        // edge = the smallest power of two >= horizon, +-512 cells around the box centre
        const size_t slots = (size_t)std::max<long long>(total_slots_, 1);
        CK(dalloc(&S_.inv_d0, slots), "alloc inv_d0");
        CK(cudaMemsetAsync(S_.inv_d0, 0, sizeof(float) * slots, stream_), "memset inv_d0");
        CK(dalloc(&S_.d0sq, slots), "alloc d0sq");
        CK(cudaMemsetAsync(S_.d0sq, 0, sizeof(float2) * slots, stream_), "memset d0sq");
        if (n > 0) {
            const int g = (int)std::min<long long>(std::max<long long>(((long long)n + kBlock - 1) / kBlock, 1), kMaxPartials);
            launch_bond_geometry(S_, g, stream_);
            ++launches_;
            if (lat_ok_) {
                launch_lattice_ell(S_, lat_, 1, g, stream_);
                ++launches_;
            }
        }
        const double h = sim_.pd_horizon > 0 ? sim_.pd_horizon : 1.0;
        sup_ = std::ldexp(1.0, (int)std::ceil(std::log2(h)));
        for (int k = 0; k < 3; ++k) sup_lo_[k] = origin_[k] - 512.0 * sup_;
        // tiles of consecutive rows and their halos (shared-memory SpMV),
        // built when that path is asked for: measured at 1M particles it is
        // slower than the per-bond gathers (307 vs 283 us per product)
        if (n > 0 && opt_.spmv_path == 1) {
            CK(dalloc(&S_.lidx, slots), "alloc local indices");
            S_.tile_rows = kTileRows;
            int max_halo = 0;
            CK(build_tiles(S_, n, &max_halo, stream_), "build tiles");
            launches_ += 2;
            S_.halo_cap = std::min(max_halo, kMaxHaloCap);
        }
    }
    // PD-PD contact hash: a power-of-two bucket count >= 2 n
    if (opt_.contact_enabled && n > 0) {
        unsigned nb = 1;
        while (nb < 2u * (unsigned)n) nb <<= 1;
        contact_.buckets = nb;
        CK(dalloc(&contact_.counts, (size_t)nb + 1), "alloc contact");
        CK(dalloc(&contact_.start, (size_t)nb + 1), "alloc contact");
        CK(dalloc(&contact_.cursor, (size_t)nb), "alloc contact");
        CK(dalloc(&contact_.bucket, N), "alloc contact");
        CK(dalloc(&contact_.list, N), "alloc contact");
    }
    // CG scalars (initPDSolutions zeroed the solution, cg_solver.cuh:184-194)
    std::memset(h_sc_, 0, sizeof(CgScalars));
    h_sc_->rel_tol = opt_.cg_relative_tolerance;
    h_sc_->max_iter = opt_.cg_max_iterations;
    CK(cudaMemcpyAsync(S_.sc, h_sc_, sizeof(CgScalars), cudaMemcpyHostToDevice, stream_), "upload scalars");
    // host copies of the slot permutation and the initial row lengths
    perm_.assign(N, 0);
    inv_.assign(N, 0);
    cnt_init_.assign(N, 0);
    if (n > 0) {
        CK(cudaMemcpyAsync(perm_.data(), d_perm_, sizeof(int) * N, cudaMemcpyDeviceToHost, stream_), "download perm");
        CK(cudaMemcpyAsync(cnt_init_.data(), S_.cnt, sizeof(int) * N, cudaMemcpyDeviceToHost, stream_), "download cnt");
    }
    CK(cudaStreamSynchronize(stream_), "make_ready sync");
    for (int i = 0; i < n; ++i) inv_[perm_[i]] = i;
    // launch geometry
    const long long need_vec = ((long long)n + kBlock - 1) / kBlock;
    // 4 blocks per SM: the CG vector kernels measured 0.090 of the 1M step
    // against 0.099 at 8, 0.097 at 2 and 0.125 at 16
    L_.grid_vec = (int)std::max<long long>(1, std::min<long long>({need_vec, (long long)sm_count_ * 4, (long long)kMaxPartials}));
    // 4 lanes per row: at 1M particles 1.25 ms per force pass against 1.74 (8) and 2.9 (16)
    L_.force_lanes = 4;
    L_.grid_force = grid_for_rows(L_.force_lanes, force_kernel_blocks_per_sm(fp64_, L_.force_lanes));
    if (!fp64_ && n > 0) {   // supercell positions of the initial state (read by the SpMV)
        launch_refresh(fp64_, step_params(), S_, L_, stream_);
        ++launches_;
        if (lat_ok_) {   // and the lattice product's deviations (its candidates are timed next)
            launch_lattice_delta(S_, lat_, sup_, stream_);
            ++launches_;
        }
    }
    s = tune_spmv();
    if (s != PD_OK) return s;
    if (opt_.warm_start == 2 || opt_.warm_start == 3) {
        s = hist_prepare();
        if (s != PD_OK) return s;
    }
    // step state
    step_ = 0;
    substep_ = 0;
    ticks_ = sim_.pd_time_step;
    clock_scale_ = opt_.phase_in_steps > 0 ? 0.0 : 1.0;
    sim_time_ = 0.0;
    cg_converged_ = true;
    last_iters_ = 0;
    total_iters_ = 0;
    predicted_iters_ = 0;
    last_params_ = step_params();
    ready_ = true;
    return PD_OK;
}

int Engine::grid_for_rows(int lanes, int blocks_per_sm) const
{
    const long long rows_per_block = kBlock / lanes;
    const long long need = ((long long)n_ + rows_per_block - 1) / rows_per_block;
    return (int)std::max<long long>(1, std::min<long long>({need, (long long)sm_count_ * blocks_per_sm,
                                                             (long long)kMaxPartials}));
}

// Project autotuner: times each (lanes, unroll) variant of the SpMV on this
// problem with CUDA events (one warm-up and three timed launches each) and
// keeps the fastest.  Fixed choices in the options are respected.
pd_status Engine::tune_spmv()
{
    struct Cand {
        int tiled, g, u, lattice = 0;
    };
    std::vector<Cand> cand;
    const int fixed_lanes = opt_.lanes_per_particle;
    const int fixed_unroll = opt_.spmv_unroll;
    const bool can_tile = !fp64_ && S_.n_tiles > 0 && S_.halo_cap > 0 && opt_.spmv_path != 2;
    const bool can_rows = fp64_ || opt_.spmv_path != 1 || !can_tile;
    if (can_tile) {
        for (int g : {4, 8}) {
            if (fixed_lanes && g != fixed_lanes) continue;
            for (int u : {1, 2, 4}) {
                if (fixed_unroll && u != fixed_unroll) continue;
                cand.push_back({1, g, u});
            }
        }
    }
    if (can_rows) {
        for (int g : {4, 8, 16}) {
            if (fixed_lanes && g != fixed_lanes) continue;
            for (int u : {1, 2, 4}) {
                if (fp64_ && u != 1) continue;
                if (fixed_unroll && u != fixed_unroll) continue;
                cand.push_back({0, g, u});
            }
        }
    }
    if (lat_ok_) {
        // asked for, or a large lattice body (from 250k particles the stencil
        // product measured well ahead of every gather shape: 186 against
        // 253 us per product at 1M), where timing the gather shapes and their
        // bond reorderings would cost make_ready ~45 ms: the stencil only
        if (opt_.spmv_path == 3 || n_ >= kLatticeOnlyRows) cand.clear();
        cand.push_back({0, 1, 1, 1});
        // the 80-entry stencil also runs on the general kernel (offsets from
        // the launch parameters instead of compile-time constants)
        if (lat_fixed_built_ && n_ >= 20000) cand.push_back({0, 1, 1, 2});
    }
    if (cand.empty()) cand.push_back({0, fixed_lanes ? fixed_lanes : 8, fixed_unroll ? fixed_unroll : 1});
    auto apply = [&](const Cand& c) {
        L_.lattice = c.lattice ? 1 : 0;
        L_.lat = c.lattice ? &lat_ : nullptr;
        if (c.lattice) {
            lat_.fixed = (c.lattice == 1 && lat_fixed_built_) ? 1 : 0;
            L_.tiled = 0;
            L_.lanes = 1;
            L_.unroll = 1;
            L_.grid_bonds = lat_.grid;
            return;
        }
        if (c.tiled) relayout_bonds(1, 1);
        else relayout_bonds(c.g, c.u);
        L_.tiled = c.tiled;
        L_.lanes = c.g;
        L_.unroll = c.u;
        if (c.tiled) {
            const int bps = std::max(1, tile_spmv_blocks_per_sm(c.g, c.u, S_.halo_cap));
            L_.grid_tiles = std::max(1, std::min(S_.n_tiles, bps * sm_count_));
        } else {
            L_.grid_bonds = grid_for_rows(c.g, row_kernel_blocks_per_sm(fp64_, c.g, c.u));
        }
    };
    if (cand.size() == 1 || n_ < 20000) {
        // small problems: launch overhead dominates, keep the default (the
        // tiled path when it was asked for)
        Cand c = cand.size() == 1 ? cand[0] : Cand{0, 8, fp64_ ? 1 : 2};
        if (lat_ok_ && opt_.spmv_path == 3) c = Cand{0, 1, 1, 1};
        if (opt_.spmv_path == 1 && can_tile && cand.size() > 1) c = Cand{1, fixed_lanes ? fixed_lanes : 8, fixed_unroll ? fixed_unroll : 2};
        apply(c);
        return PD_OK;
    }
    const StepParams P = step_params();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    Cand best_c = cand[0];
    // each candidate: one warm-up launch, then the best of three timed pairs
    // of the CG iteration's product as the CG loop launches it (y = A p with
    // <p, y>; the lattice product with the direction update fused in; the
    // scalars and the second direction buffer it writes are reset by the
    // first solve)
    const auto cg_product = [&]() {
        if (L_.lattice && d_p2_)
            launch_spmv_lattice(true, P, S_, lat_, S_.p, S_.y, ReduceSlot{S_.partials, S_.counters + 1}, S_.sc,
                                nullptr, S_.r, d_p2_, stream_);
        else
            launch_spmv(fp64_, true, P, S_, L_, stream_);
    };
    for (const auto& c : cand) {
        apply(c);
        cg_product();
        ++launches_;
        if (cudaGetLastError() != cudaSuccess) continue;   // a shape that cannot launch is not a candidate
        float ms_c = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            CK(cudaEventRecord(e0, stream_), "event");
            for (int k = 0; k < 2; ++k) cg_product();
            CK(cudaGetLastError(), "tune launch");
            CK(cudaEventRecord(e1, stream_), "event");
            CK(cudaEventSynchronize(e1), "tune sync");
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1), "event");
            ms_c = std::min(ms_c, ms / 2.0f);
            launches_ += 2;
        }
        if (ms_c < best) {
            best = ms_c;
            best_c = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply(best_c);
    tuned_ms_ = best;
    return PD_OK;
}

void Engine::apply_op(const StepParams& P, const void* in, void* out, ReduceSlot slot, double* dot_out)
{
    if (L_.lattice)
        launch_spmv_lattice(dot_out != nullptr, P, S_, lat_, in, out, slot, nullptr, dot_out, nullptr, nullptr, stream_);
    else launch_operator_u(fp64_, P, S_, L_.lanes, L_.unroll, L_.grid_bonds, in, out, slot, dot_out, stream_);
}

void Engine::lattice_resync(bool force)
{
    if (!lat_ok_ || n_ == 0) return;
    const int g = (int)std::min<long long>(((long long)n_ + kBlock - 1) / kBlock, (long long)sm_count_ * 8);
    launch_lattice_ell(S_, lat_, force ? 1 : 0, std::max(g, 1), stream_);
    ++launches_;
}

void Engine::relayout_bonds(int g, int u)
{
    if (fp64_ || n_ <= 0) return;
    if (u <= 1) g = 1, u = 1;
    if (g == lay_g_ && u == lay_u_) return;
    const int grid = (int)std::min<long long>(((long long)n_ + kBlock - 1) / kBlock, (long long)sm_count_ * 8);
    launch_bond_relayout(S_, std::max(grid, 1), lay_g_, lay_u_, g, u, stream_);
    ++launches_;
    lay_g_ = g;
    lay_u_ = u;
}

StepParams Engine::step_params() const
{
    StepParams P{};
    P.n = n_;
    P.integrator = run_.integrator;
    P.ticks = ticks_;
    P.box_enabled = opt_.box_enabled;
    P.sphere_on = opt_.sphere_enabled;
    P.cs = clock_scale_;
    P.bond_coeff = bond_coeff_;
    P.horizon = sim_.pd_horizon;
    P.radius = sim_.pd_particle_radius;
    P.vs_threshold = sim_.pd_horizon - sim_.pd_particle_radius;
    P.mass = sim_.pd_particle_mass;
    P.dt_base = opt_.time_step_base;
    P.h = ticks_ * opt_.time_step_base;
    P.t2 = run_.integrator == PD_IMPLICIT_EULER ? P.h * P.h : (P.h * P.h) / 4.0;
    for (int k = 0; k < 3; ++k) P.gravity[k] = opt_.gravity[k];
    P.stretch_a = opt_.stretch_a;
    P.stretch_b = opt_.stretch_b;
    P.alpha = opt_.alpha;
    P.bmin[0] = sim_.boundary_min_x; P.bmin[1] = sim_.boundary_min_y; P.bmin[2] = sim_.boundary_min_z;
    P.bmax[0] = sim_.boundary_max_x; P.bmax[1] = sim_.boundary_max_y; P.bmax[2] = sim_.boundary_max_z;
    P.restitution = opt_.restitution;
    for (int k = 0; k < 3; ++k) {
        P.sphere_c[k] = opt_.sphere_center[k] + opt_.sphere_velocity[k] * sim_time_;
        P.sphere_c_local[k] = P.sphere_c[k] - origin_[k];
    }
    P.sphere_r = opt_.sphere_radius;
    P.sphere_k = opt_.sphere_stiffness;
    for (int k = 0; k < 3; ++k) P.sup_lo[k] = sup_lo_[k];
    P.sup = sup_;
    P.inv_sup = sup_ > 0 ? 1.0 / sup_ : 0.0;
    return P;
}

// ---- learned warm start --------------------------------------------------------------
bool Engine::ws_features_needed() const
{
    return !fp64_ && ready_ && (opt_.warm_start == 1 || opt_.warm_start == 3 || ws_samples_ > 0);
}

void Engine::ws_free()
{
    void* p[] = {W_.diag, W_.dj, W_.features, W_.hist2, W_.hist3, W_.xsave, W_.ds_x, W_.ds_t, W_.sc, W_.free_list,
                 ws_rsave_};
    for (void* q : p)
        if (q) cudaFree(q);
    W_ = WsState{};
    ws_rsave_ = nullptr;
    mlp_work_free(&mlp_work_);
    mlp_free(&mlp_);
    ws_ready_ = false;
}

pd_status Engine::ws_prepare(bool with_network)
{
    if (ws_ready_) return PD_OK;
    const size_t N = (size_t)std::max(n_, 1);
    CK(dalloc(&W_.diag, N), "alloc ws");
    CK(dalloc(&W_.dj, N), "alloc ws");
    if (with_network) CK(dalloc(&W_.features, N * kMlpIn), "alloc ws");
    CK(dalloc(&W_.hist2, N), "alloc ws");
    CK(dalloc(&W_.hist3, N), "alloc ws");
    CK(dalloc(&W_.xsave, N), "alloc ws");
    CK(dalloc(&ws_rsave_, N), "alloc ws");
    CK(dalloc(&W_.sc, 1), "alloc ws");
    CK(cudaMemsetAsync(W_.hist2, 0, sizeof(float4) * N, stream_), "memset ws");
    CK(cudaMemsetAsync(W_.hist3, 0, sizeof(float4) * N, stream_), "memset ws");
    CK(cudaMemsetAsync(W_.xsave, 0, sizeof(float4) * N, stream_), "memset ws");
    // free slots (Dirichlet rows carry no prediction and no training sample)
    std::vector<int> free_slots;
    for (int i = 0; i < n_; ++i) {
        const int a = h_act_[perm_[i]];
        if (a != PD_INVISIBLE && a != PD_CLAMPED && a != PD_PRESCRIBED) free_slots.push_back(i);
    }
    W_.n_free_host = (int)free_slots.size();
    CK(dalloc(&W_.free_list, std::max<size_t>(free_slots.size(), 1)), "alloc ws");
    if (!free_slots.empty())
        CK(cudaMemcpyAsync(W_.free_list, free_slots.data(), sizeof(int) * free_slots.size(), cudaMemcpyHostToDevice,
                           stream_), "upload free list");
    WsScalars sc{};
    sc.n_free = W_.n_free_host;
    CK(cudaMemcpyAsync(W_.sc, &sc, sizeof(sc), cudaMemcpyHostToDevice, stream_), "upload ws scalars");
    W_.max_bonds = std::max(sim_.pd_max_num_bonds, 1);
    if (!with_network) {
        CK(cudaStreamSynchronize(stream_), "ws prepare");
        ws_ready_ = true;
        return PD_OK;
    }
    CK(mlp_alloc(&mlp_, false), "alloc mlp");
    CK(mlp_work_alloc(&mlp_work_, n_, false), "alloc mlp work");
    if (ws_params_.size() != mlp_param_count()) {
        ws_params_.assign(mlp_param_count(), 0.f);
        mlp_init_params(ws_params_.data(), 1u);
    }
    CK(cudaMemcpyAsync(mlp_.params, ws_params_.data(), sizeof(float) * ws_params_.size(), cudaMemcpyHostToDevice,
                       stream_), "upload mlp params");
    mlp_refresh_bf16(mlp_, stream_);
    if (ws_cap_ > 0) {
        CK(dalloc(&W_.ds_x, (size_t)ws_cap_ * kMlpIn), "alloc dataset");
        CK(dalloc(&W_.ds_t, (size_t)ws_cap_ * 3), "alloc dataset");
    }
    ws_pos_ = ws_count_ = 0;
    CK(cudaStreamSynchronize(stream_), "ws prepare");
    ws_ready_ = true;
    return PD_OK;
}

// After the CG set-up (x1 = previous solution with Dirichlet values, r = b - A x1):
// features, and with warm_start = 1 the learned guess x1 + sigma MLP(features),
// its residual, and the guard that keeps the better of the two guesses.
pd_status Engine::ws_before_cg(const StepParams& P)
{
    pd_status s = ws_prepare();
    if (s != PD_OK) return s;
    const size_t N = (size_t)n_;
    if (N == 0) return PD_OK;
    CK(cudaMemcpyAsync(W_.xsave, S_.sol, sizeof(float4) * N, cudaMemcpyDeviceToDevice, stream_), "save x1");
    ReduceSlot s0{S_.partials + kMaxPartials, S_.counters + 5};
    ReduceSlot s1{S_.partials + 2 * kMaxPartials, S_.counters + 6};
    ReduceSlot s2{S_.partials + 3 * kMaxPartials, S_.counters + 7};
    launch_ws_jacobi(P, S_, W_, 8, L_.grid_force, s0, s1, s2, stream_);
    launch_ws_features(P, S_, W_, L_.grid_force, stream_);
    launches_ += 2;
    if (opt_.warm_start == 3 && d_hnet_) {
        // the network's correction becomes the last column of the history
        // projection (hist_project runs next and decides its weight)
        CK(mlp_infer_tc(mlp_, W_.features, n_, mlp_work_.y, stream_), "network launch");
        launch_ws_column(P, S_, W_, mlp_work_.y, (float4*)d_hnet_, L_.grid_vec, stream_);
        launches_ += 2;
    }
    if (opt_.warm_start == 1) {
        CK(cudaMemcpyAsync(ws_rsave_, S_.r, sizeof(float4) * N, cudaMemcpyDeviceToDevice, stream_), "save r");
        launch_ws_save_plain(S_, stream_);
        CK(mlp_infer_tc(mlp_, W_.features, n_, mlp_work_.y, stream_), "network launch");
        launch_ws_apply(P, S_, W_, mlp_work_.y, L_.grid_vec, stream_);
        launch_spmv(fp64_, false, P, S_, L_, stream_);
        launch_cg_residual(fp64_, P, S_, L_, stream_);
        launch_ws_guard(P, S_, W_.xsave, ws_rsave_, L_.grid_vec, stream_);
        launches_ += 14;
    }
    CK(cudaGetLastError(), "warm start launch");
    return PD_OK;
}

pd_status Engine::ws_after_cg(const StepParams& P)
{
    if ((opt_.warm_start == 1 || opt_.warm_start == 3) && mlp_tc_take_error()) {
        err_ = "warm-start network: a tensor-core wait ran out of time";
        return PD_ERR_CUDA;
    }
    if (ws_samples_ > 0 && ws_cap_ > 0 && W_.n_free_host > 0) {
        const int count = std::min(ws_samples_, W_.n_free_host);
        const int stride = std::max(1, W_.n_free_host / count);
        ws_rng_ ^= ws_rng_ << 13;
        ws_rng_ ^= ws_rng_ >> 7;
        ws_rng_ ^= ws_rng_ << 17;
        const int offset = (int)(ws_rng_ % (unsigned long long)W_.n_free_host);
        launch_ws_collect(P, S_, W_, count, stride, offset, ws_pos_, ws_cap_, stream_);
        ++launches_;
        ws_pos_ = (ws_pos_ + count) % ws_cap_;
        ws_count_ = std::min(ws_count_ + count, ws_cap_);
    }
    float4* t = W_.hist3;   // x3 <- x2 <- x1
    W_.hist3 = W_.hist2;
    W_.hist2 = W_.xsave;
    W_.xsave = t;
    if (opt_.warm_start == 1) {
        last_ws_ratio_ = h_sc_->rz_plain > 0 ? std::sqrt(h_sc_->rz_learned / h_sc_->rz_plain) : 0.0;
        ws_kept_ = h_sc_->ws_kept;
    }
    CK(cudaGetLastError(), "warm start collect");
    return PD_OK;
}

pd_status Engine::ws_set_params(const float* params, size_t count)
{
    if (!params || count != mlp_param_count()) {
        err_ = "ws_set_params: expected pd_mlp_param_count() values";
        return PD_ERR_INVALID_ARGUMENT;
    }
    ws_params_.assign(params, params + count);
    if (ws_ready_) {
        CK(cudaSetDevice(device_), "cudaSetDevice");
        CK(cudaMemcpyAsync(mlp_.params, ws_params_.data(), sizeof(float) * count, cudaMemcpyHostToDevice, stream_),
           "upload mlp params");
        mlp_refresh_bf16(mlp_, stream_);
        CK(cudaStreamSynchronize(stream_), "upload mlp params");
    }
    return PD_OK;
}

pd_status Engine::ws_get_params(float* params, size_t count)
{
    if (!params || count != mlp_param_count()) return PD_ERR_INVALID_ARGUMENT;
    if (ws_params_.size() != count) {
        ws_params_.assign(count, 0.f);
        mlp_init_params(ws_params_.data(), 1u);
    }
    std::copy(ws_params_.begin(), ws_params_.end(), params);
    return PD_OK;
}

pd_status Engine::ws_collect(int samples_per_step, long long capacity)
{
    if (samples_per_step < 0 || capacity < 0) return PD_ERR_INVALID_ARGUMENT;
    if (fp64_ && samples_per_step > 0) {
        err_ = "ws_collect: the learned warm start works in mixed precision";
        return PD_ERR_INVALID_ARGUMENT;
    }
    const bool realloc = capacity != ws_cap_;
    ws_samples_ = samples_per_step;
    ws_cap_ = capacity;
    if (ws_ready_ && realloc) {
        if (W_.ds_x) cudaFree(W_.ds_x);
        if (W_.ds_t) cudaFree(W_.ds_t);
        W_.ds_x = nullptr;
        W_.ds_t = nullptr;
        if (ws_cap_ > 0) {
            CK(dalloc(&W_.ds_x, (size_t)ws_cap_ * kMlpIn), "alloc dataset");
            CK(dalloc(&W_.ds_t, (size_t)ws_cap_ * 3), "alloc dataset");
        }
        ws_pos_ = ws_count_ = 0;
    }
    return PD_OK;
}

pd_status Engine::ws_dataset(float* X, float* T, long long max_rows, long long* rows)
{
    if (!rows || max_rows < 0) return PD_ERR_INVALID_ARGUMENT;
    const long long r = std::min(ws_count_, max_rows);
    *rows = r;
    if (r == 0) return PD_OK;
    if (!X || !T) return PD_ERR_INVALID_ARGUMENT;
    std::vector<__nv_bfloat16> xb((size_t)r * kMlpIn);
    CK(cudaMemcpyAsync(xb.data(), W_.ds_x, sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyDeviceToHost, stream_),
       "download dataset");
    CK(cudaMemcpyAsync(T, W_.ds_t, sizeof(float) * (size_t)r * 3, cudaMemcpyDeviceToHost, stream_), "download dataset");
    CK(cudaStreamSynchronize(stream_), "download dataset");
    for (size_t i = 0; i < xb.size(); ++i) X[i] = __bfloat162float(xb[i]);
    return PD_OK;
}

pd_status Engine::synchronize()
{
    CK(cudaSetDevice(device_), "cudaSetDevice");
    CK(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return PD_OK;
}

pd_status Engine::operator_view(pd_operator_view* v) const
{
    if (!ready_) return PD_ERR_NOT_READY;
    std::memset(v, 0, sizeof(*v));
    const StepParams& P = last_params_;
    v->n = n_;
    v->precision = fp64_ ? PD_PRECISION_FP64 : PD_PRECISION_MIXED;
    // the view describes the CSR rows; with the lattice product in use it
    // carries a CSR launch shape of its own
    v->lanes_per_particle = L_.lattice ? 8 : L_.lanes;
    v->blocks = L_.lattice ? grid_for_rows(8, row_kernel_blocks_per_sm(fp64_, 8, 1)) : L_.grid_bonds;
    v->activity = S_.act;
    v->row_ptr = S_.row_ptr;
    v->bond_count = S_.cnt;
    v->bond_slot = S_.col;
    v->perm = d_perm_;
    v->ref_pos = S_.X32;
    v->disp = S_.u32;
    v->pos_cell = S_.xs4;
    v->inv_d0 = S_.inv_d0;
    v->supercell_size = sup_;
    v->jac = S_.jac;
    v->jac_diag = S_.jdiag;
    v->mass = P.mass;
    v->t2 = P.t2;
    v->bond_coeff = P.bond_coeff;
    for (int k = 0; k < 3; ++k) v->sphere_center_local[k] = P.sphere_c_local[k];
    v->sphere_stiffness = P.sphere_k;
    return PD_OK;
}

pd_status Engine::apply_operator(const void* d_x, void* d_y, double* d_dot)
{
    if (!ready_) {
        err_ = "apply_operator: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    if ((!d_x || !d_y) && n_ > 0) return PD_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(device_), "cudaSetDevice");
    // counter 4 of the handle's reduction scratch is reserved for this call
    ReduceSlot slot{S_.partials, S_.counters + 4};
    apply_op(last_params_, d_x, d_y, slot, d_dot);
    ++launches_;
    CK(cudaGetLastError(), "apply_operator launch");
    return PD_OK;
}

bool Engine::finished() const { return step_ > run_.final_step || !cg_converged_; }

pd_status Engine::advance(int nsteps)
{
    if (!ready_) {
        err_ = "advance: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    if (nsteps < 0) return PD_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(device_), "cudaSetDevice");
    for (int k = 0; k < nsteps; ++k) {
        if (!cg_converged_) break;
        ++step_;
        if (step_ <= opt_.phase_in_steps) clock_scale_ = (double)step_ / (double)opt_.phase_in_steps;
        retries_ = 0;
        for (;;) {
            bool advanced = false;
            pd_status s = integrate(&advanced);
            if (s != PD_OK) return s;
            if (advanced) break;
            if (++retries_ > 64) {
                err_ = "adaptive time step: too many rollbacks";
                return PD_ERR_STATE;
            }
        }
    }
    return PD_OK;
}

pd_status Engine::integrate(bool* advanced)
{
    *advanced = false;
    const StepParams Pf = step_params();   // force pass: does not depend on the time step
    const size_t N = (size_t)n_;
    CK(cudaMemsetAsync(S_.flags, 0, sizeof(int) * 2, stream_), "memset flags");
    mark_begin(PD_KC_FORCE, -1);
    launch_force(fp64_, Pf, S_, L_, stream_);
    mark_end();
    launches_ += fp64_ ? 1 : (L_.lattice ? 3 : 2);   // mixed: the supercell words (+ lattice deviations), the pass
    lattice_resync(false);        // only where the pass broke a bond (read on the device)
    const bool adaptive = run_.integrator == PD_NEWMARK_BETA || run_.adaptive_integration != 0;
    if (adaptive) {
        CK(cudaMemcpyAsync(h_flags_, S_.flags, sizeof(int) * 2, cudaMemcpyDeviceToHost, stream_), "read flag");
        CK(cudaStreamSynchronize(stream_), "step sync");
        ++host_syncs_;
        int rollback = 0;
        pd_adaptive_decide(h_flags_[0], sim_.pd_time_step, opt_.time_step_min, opt_.max_substep, &ticks_, &substep_,
                           &rollback);
        if (rollback) {
            // restoreBondListTopIndex / restorePDPosition / restorePDVelocity (memory_manager.cu:500-550)
            CK(cudaMemcpyAsync(S_.cnt, S_.cnt_bk, sizeof(int) * N, cudaMemcpyDeviceToDevice, stream_), "restore cnt");
            CK(cudaMemcpyAsync(S_.x64, S_.x64_bk, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "restore x");
            CK(cudaMemcpyAsync(S_.v64, S_.v64_bk, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "restore v");
            launch_refresh(fp64_, Pf, S_, L_, stream_);
            launches_ += L_.lattice ? 2 : 1;
            lattice_resync(true);   // the restored live sets
            return PD_OK;
        }
        CK(cudaMemcpyAsync(S_.cnt_bk, S_.cnt, sizeof(int) * N, cudaMemcpyDeviceToDevice, stream_), "backup cnt");
        CK(cudaMemcpyAsync(S_.x64_bk, S_.x64, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "backup x");
        CK(cudaMemcpyAsync(S_.v64_bk, S_.v64, sizeof(dbl4) * N, cudaMemcpyDeviceToDevice, stream_), "backup v");
    }
    // PD-PD contact forces (collidePDParticles, after the stretch-limit
    // update and before fillMatrix*, simulator.cu:410-426, 581-597)
    if (opt_.contact_enabled && n_ > 0) {
        const ContactParams C{opt_.contact_distance, opt_.contact_stiffness, opt_.contact_volume};
        mark_begin(PD_KC_FORCE, -1);
        CK(launch_contact(fp64_, S_, n_, C, contact_, stream_), "contact");
        mark_end();
        launches_ += 4;
    }
    // the assembly, solve and update of this step use the time step as the
    // adaptive decision left it (the reference doubles it in place)
    const StepParams P = step_params();
    last_params_ = P;
    pd_status s = solve(P);
    if (s != PD_OK) return s;
    mark_begin(PD_KC_UPDATE, -1);
    launch_update(fp64_, P, S_, L_, stream_);
    mark_end();
    ++launches_;
    CK(cudaGetLastError(), "step launch");
    sim_time_ += P.h;
    *advanced = true;
    return PD_OK;
}

pd_status Engine::solve(const StepParams& P)
{
    launch_cg_init(fp64_, P, S_, L_, stream_);
    launch_spmv(fp64_, false, P, S_, L_, stream_);
    launch_cg_residual(fp64_, P, S_, L_, stream_);
    launches_ += 3;
    if (opt_.warm_start == 3) {   // network column first, then the projection over history + column
        pd_status s = ws_before_cg(P);
        if (s == PD_OK) s = hist_project(P);
        if (s != PD_OK) return s;
    } else {
        if (opt_.warm_start == 2) {
            pd_status s = hist_project(P);
            if (s != PD_OK) return s;
        }
        if (ws_features_needed()) {
            pd_status s = ws_before_cg(P);
            if (s != PD_OK) return s;
        }
    }
    if (opt_.preconditioner) {
        // M from this step's operator, then z = M r and p = z for the final guess
        launch_pc_build(fp64_, opt_.preconditioner, P, S_, L_, stream_);
        launch_pcg_start(fp64_, P, S_, L_, stream_);
        launches_ += 2;
    }
    // iteration 0 from the host: the sample of the profiled kernel times (a
    // live launch unless the guess had already converged)
    cg_iteration(P, 0, 0, true);
    launches_ += cg_kernels_per_iteration();
    bool graph = false;
    if (opt_.cg_loop == 0 && !cg_graph_failed_) {
        const cudaError_t e = cg_graph_launch(P);
        if (e == cudaSuccess) {
            graph = true;
        } else {
            // the graph could not be built here: the solve goes on in host-checked batches
            cudaGetLastError();
            cg_graph_failed_ = true;
        }
    }
    if (graph) {
        CK(cudaMemcpyAsync(h_sc_, S_.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, stream_), "read cg scalars");
        CK(cudaStreamSynchronize(stream_), "cg sync");
        ++host_syncs_;
        ++cg_graph_solves_;
        // bodies run: at least one (the while node's first test is the default value 1)
        const int K = cg_graph_body();
        const int after0 = std::max(0, h_sc_->iter - 1);
        const long long bodies = std::max(1, (after0 + K - 1) / K);
        launches_ += bodies * K * cg_kernels_per_iteration();
    } else {
        pd_status s = cg_host_loop(P);
        if (s != PD_OK) return s;
    }
    last_iters_ = h_sc_->iter;
    last_res_ = h_sc_->rnorm;
    last_tol_ = h_sc_->tol;
    total_iters_ += last_iters_;
    predicted_iters_ = std::max(1, last_iters_);
    flush_marks(last_iters_, true);
    if (opt_.warm_start == 2 || opt_.warm_start == 3) {
        hist_collect();
        pd_status s = hist_push();
        if (s != PD_OK) return s;
    }
    if (profiling_) {
        kc_launches_[PD_KC_SPMV] += last_iters_;
        kc_launches_[PD_KC_CG_VECTOR] += (L_.lattice && d_p2_ ? 1LL : 2LL) * last_iters_;
    }
    if (!h_sc_->converged) cg_converged_ = false;
    if (ws_features_needed()) return ws_after_cg(P);
    return PD_OK;
}

void Engine::cg_iteration(const StepParams& P, int k, cudaGraphConditionalHandle cond, bool sample)
{
    // profiling times the host-launched iterations of every kMarkStride-th
    // index, so that the event records barely perturb the solve they measure;
    // the mean sampled duration is scaled to the exact launch count
    sample = sample && profiling_ && cond == 0 && (k % kMarkStride) == 0;
    if (L_.lattice && d_p2_) {
        // the direction update p = r + beta p is fused into the product, which
        // reads the previous direction from one buffer and writes the new one
        // to the other (buffer 0 = S_.p, set to r by the residual kernel)
        // (preconditioned: p = z + beta p, from the z buffer)
        void* p_prev = (k & 1) ? d_p2_ : S_.p;
        void* p_new = (k & 1) ? S_.p : d_p2_;
        if (sample) mark_begin(PD_KC_SPMV, k);
        launch_spmv_lattice(true, P, S_, lat_, p_prev, S_.y, ReduceSlot{S_.partials, S_.counters + 1}, S_.sc, nullptr,
                            opt_.preconditioner ? S_.z : S_.r, p_new, stream_);
        if (sample) mark_end();
        DeviceState Sj = S_;
        Sj.p = p_new;
        if (sample) mark_begin(PD_KC_CG_VECTOR, k);
        if (opt_.preconditioner) launch_cg_axpy_pc(fp64_, P, Sj, L_, stream_, cond);
        else launch_cg_axpy(fp64_, P, Sj, L_, stream_, cond);
        if (sample) mark_end();
    } else {
        if (sample) mark_begin(PD_KC_SPMV, k);
        launch_spmv(fp64_, true, P, S_, L_, stream_);
        if (sample) mark_end();
        if (sample) mark_begin(PD_KC_CG_VECTOR, k);
        if (opt_.preconditioner) {
            launch_cg_axpy_pc(fp64_, P, S_, L_, stream_, cond);
            DeviceState Sz = S_;   // p = z + beta p
            Sz.r = S_.z;
            launch_cg_xpby(fp64_, P, Sz, L_, stream_);
        } else {
            launch_cg_axpy(fp64_, P, S_, L_, stream_, cond);
            launch_cg_xpby(fp64_, P, S_, L_, stream_);
        }
        if (sample) mark_end();
    }
}

// Iterations per while-node body: an even count (the lattice product's
// direction buffers alternate), 4 unless cg_check_interval asks otherwise.
int Engine::cg_graph_body() const
{
    const int k = opt_.cg_check_interval > 0 ? opt_.cg_check_interval : 4;
    return std::min(64, (k + 1) & ~1);
}

// The graph holds one while node; its body is cg_graph_body() iterations
// captured from the launches of cg_iteration.  Every k_cg_axpy of the body
// sets the node's condition to "not converged and below the iteration limit"
// (cg_fin_axpy), or to 0 when the solve had finished before it ran, so the
// loop ends at most one body after the test that ends the solve: every body
// that runs holds a live iteration, and the iteration limit sets done.  The
// operator's constants (StepParams) change every step, so the graph is built
// and instantiated for each solve, while the GPU still runs the work queued
// before it.
cudaError_t Engine::cg_graph_launch(const StepParams& P)
{
    const int K = cg_graph_body();
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    cudaGraphConditionalHandle cond = 0;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, g, 1u, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
    if (e == cudaSuccess) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(stream_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int k = 1; k <= K; ++k) cg_iteration(P, k, cond, false);
            const cudaError_t le = cudaGetLastError();
            cudaGraph_t captured = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(stream_, &captured);
            e = le != cudaSuccess ? le : ce;
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(x, stream_);
    // an executable graph destroyed while in flight is freed when it completes
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
    return e;
}

pd_status Engine::cg_host_loop(const StepParams& P)
{
    const int check = opt_.cg_check_interval > 0 ? opt_.cg_check_interval : 8;
    int batch = std::max(1, predicted_iters_ - 1);
    int launched = 1;   // iteration 0 ran from solve()
    for (;;) {
        for (int k = 0; k < batch; ++k, ++launched) cg_iteration(P, launched, 0, true);
        launches_ += (long long)cg_kernels_per_iteration() * batch;
        CK(cudaGetLastError(), "cg launch");
        CK(cudaMemcpyAsync(h_sc_, S_.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, stream_), "read cg scalars");
        CK(cudaStreamSynchronize(stream_), "cg sync");
        ++host_syncs_;
        if (h_sc_->done) break;
        if (launched > opt_.cg_max_iterations + 2 * check) {
            err_ = "cg: iteration count not advancing";
            return PD_ERR_STATE;
        }
        batch = std::max(check, launched / 8);
    }
    return PD_OK;
}

// ---- history projection (warm_start = 2) ---------------------------------------------
// The guess x1 + H y of history.cu: H holds the last hist_cap_ accepted
// solutions, y is the Galerkin solution over the well-conditioned part of
// span H.  Per solve: m products A h_j, two Gram passes, one host sync for the
// m x m solve, x += H y and a fresh residual.
pd_status Engine::hist_prepare()
{
    hist_free();
    // warm_start 3 keeps one column of the Gram passes for the network's correction
    const bool net = opt_.warm_start == 3;
    const int cap_max = net ? kHistMax - 1 : kHistMax;
    hist_cap_ = opt_.history_size > 0 ? std::min(opt_.history_size, cap_max) : cap_max;
    const size_t vec = (size_t)std::max(n_, 1) * (fp64_ ? sizeof(dbl4) : sizeof(float4));
    hist_blocks_ = (int)std::max<long long>(1, std::min<long long>(((long long)n_ + kBlock - 1) / kBlock,
                                                                  2LL * sm_count_));
    CK(cudaMalloc(&d_hist_, vec * hist_cap_), "alloc history");
    CK(cudaMalloc(&d_ahist_, vec * (hist_cap_ + (net ? 1 : 0))), "alloc history products");
    if (net) {
        CK(cudaMalloc(&d_hnet_, vec), "alloc learned column");
        CK(cudaMemsetAsync(d_hnet_, 0, vec, stream_), "memset learned column");
    }
    const size_t npart = (size_t)hist_blocks_ * (hist_dots_count(0) + hist_dots_count(1));
    CK(cudaMalloc((void**)&d_hpart_, sizeof(double) * npart), "alloc history partials");
    CK(cudaMallocHost((void**)&h_hpart_, sizeof(double) * npart), "alloc history partials (host)");
    CK(cudaMallocHost((void**)&h_sc_pre_, sizeof(CgScalars)), "alloc history scalars (host)");
    CK(cudaMallocHost((void**)&h_sc_hist_, sizeof(CgScalars)), "alloc history scalars (host)");
    CK(cudaMalloc((void**)&d_hsol_, sizeof(HistSolve)), "alloc history solve");
    CK(cudaMallocHost((void**)&h_hsol_, sizeof(HistSolve)), "alloc history solve (host)");
    hist_reset();
    return PD_OK;
}

void Engine::hist_free()
{
    if (d_hist_) cudaFree(d_hist_);
    if (d_ahist_) cudaFree(d_ahist_);
    if (d_hnet_) cudaFree(d_hnet_);
    d_hnet_ = nullptr;
    if (d_hpart_) cudaFree(d_hpart_);
    if (h_sc_hist_) cudaFreeHost(h_sc_hist_);
    if (d_hsol_) cudaFree(d_hsol_);
    if (h_hsol_) cudaFreeHost(h_hsol_);
    if (h_hpart_) cudaFreeHost(h_hpart_);
    if (h_sc_pre_) cudaFreeHost(h_sc_pre_);
    h_hpart_ = nullptr;
    h_sc_pre_ = nullptr;
    d_hist_ = d_ahist_ = nullptr;
    d_hpart_ = nullptr;
    h_sc_hist_ = nullptr;
    d_hsol_ = nullptr;
    h_hsol_ = nullptr;
    hist_pending_ = false;
    hist_cap_ = 0;
    hist_reset();
}

void* Engine::hist_vec(int j) const
{
    const size_t vec = (size_t)std::max(n_, 1) * (fp64_ ? sizeof(dbl4) : sizeof(float4));
    return (char*)d_hist_ + vec * (size_t)j;
}

pd_status Engine::hist_project(const StepParams& P)
{
    // columns: the last hist_m_ accepted solutions, then (warm_start 3) the
    // network's correction of this step
    const bool net = opt_.warm_start == 3 && d_hnet_;
    const int m = hist_m_ + (net ? 1 : 0);
    if (m == 0 || n_ == 0 || !d_hist_) return PD_OK;
    const size_t vec = (size_t)n_ * (fp64_ ? sizeof(dbl4) : sizeof(float4));
    HistPtrs H{}, W{};
    for (int j = 0; j < m; ++j) {
        H.v[j] = (net && j == m - 1) ? d_hnet_ : hist_vec(j);
        W.v[j] = (const char*)d_ahist_ + vec * (size_t)j;
    }
    mark_begin(PD_KC_GUESS, -1);
    // products with this step's operator (counter 4 of the reduction scratch is unused without a dot)
    const ReduceSlot slot{S_.partials, S_.counters + 4};
    for (int j = 0; j < m; ++j) apply_op(P, H.v[j], (void*)W.v[j], slot, nullptr);
    // the block partials of both Gram passes
    const int na0 = hist_dots_count(0), na1 = hist_dots_count(1);
    launch_hist_dots(fp64_, 0, n_, m, H, W, S_.r, d_hpart_, hist_blocks_, stream_);
    launch_hist_dots(fp64_, 1, n_, m, H, W, nullptr, d_hpart_ + (size_t)hist_blocks_ * na0, hist_blocks_, stream_);
    // the m x m solve on the host, in stream order: partials and scalars to
    // pinned memory, the callback, its result back to the device (the GPU
    // waits for the round trip; the calling thread does not)
    CK(cudaMemcpyAsync(h_hpart_, d_hpart_, sizeof(double) * (size_t)hist_blocks_ * (na0 + na1),
                       cudaMemcpyDeviceToHost, stream_), "read history partials");
    CK(cudaMemcpyAsync(h_sc_pre_, S_.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, stream_), "read cg scalars");
    // columns whose part outside the others' span is below sqrt(rel) of the
    // largest norm are rounding noise of the stored precision
    // (measured on a 100k-particle impact: 1e-14 .. 1e-10 within 1 % of iterations; 1e-6 loses the gain)
    hist_cb_ = HistHostSolve{m, hist_blocks_, net ? m - 1 : -1, fp64_ ? 1e-26 : 1e-12, h_hpart_, h_sc_pre_, h_hsol_};
    CK(cudaLaunchHostFunc(stream_, [](void* a) { hist_host_solve(*(const HistHostSolve*)a); }, &hist_cb_),
       "history solve callback");
    CK(cudaMemcpyAsync(d_hsol_, h_hsol_, sizeof(HistSolve), cudaMemcpyHostToDevice, stream_), "upload history solve");
    // x1 + H y and its residual (the apply returns at once when no column was
    // used; the residual is then that of x1 again)
    launch_hist_apply(fp64_, n_, m, H, d_hsol_, S_.sol, L_.grid_vec, stream_);
    launch_spmv(fp64_, false, P, S_, L_, stream_);
    launch_cg_residual(fp64_, P, S_, L_, stream_);
    launches_ += m + 5;
    CK(cudaMemcpyAsync(h_sc_hist_, S_.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, stream_),
       "read projected residual");
    hist_pending_ = true;
    mark_end();
    CK(cudaGetLastError(), "history guess");
    return PD_OK;
}

// After the solve's read-back: whether the projection was applied, its
// residual relative to the previous solution's, and the network column's use.
void Engine::hist_collect()
{
    if (!hist_pending_) return;
    hist_pending_ = false;
    if (h_hsol_->used > 0) {
        ++ws_kept_;
        last_ws_ratio_ = h_hsol_->rz1 > 0.0 ? std::sqrt(h_sc_hist_->rz / h_hsol_->rz1) : 0.0;
    }
    if (h_hsol_->net_used) ++ws_net_used_;
}

pd_status Engine::hist_push()
{
    if (!d_hist_ || hist_cap_ == 0 || n_ == 0) return PD_OK;
    launch_hist_push(fp64_, n_, S_.act, S_.sol, hist_vec(hist_next_), L_.grid_vec, stream_);
    ++launches_;
    hist_next_ = (hist_next_ + 1) % hist_cap_;
    hist_m_ = std::min(hist_m_ + 1, hist_cap_);
    CK(cudaGetLastError(), "history push");
    return PD_OK;
}

// ---- profiling -------------------------------------------------------------------
cudaEvent_t Engine::take_event()
{
    if (!event_pool_.empty()) {
        cudaEvent_t e = event_pool_.back();
        event_pool_.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Engine::mark_begin(int kc, int iter)
{
    if (!profiling_) return;
    Mark m{kc, iter, take_event(), take_event()};
    cudaEventRecord(m.a, stream_);
    marks_.push_back(m);
    open_mark_ = (int)marks_.size() - 1;
}

void Engine::mark_end()
{
    if (!profiling_ || open_mark_ < 0) return;
    cudaEventRecord(marks_[open_mark_].b, stream_);
    open_mark_ = -1;
}

// Accumulates completed marks.  SpMV / CG-vector marks of iterations at or
// beyond `live_iters` were launches that returned immediately after
// convergence and are dropped.  live_iters < 0 keeps all.
void Engine::flush_marks(int live_iters, bool synced)
{
    if (marks_.empty()) return;
    if (!synced) cudaStreamSynchronize(stream_);
    for (Mark& m : marks_) {
        const bool dead = live_iters >= 0 && m.iter >= live_iters &&
                          (m.kc == PD_KC_SPMV || m.kc == PD_KC_CG_VECTOR);
        if (!dead) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) {
                if (m.kc == PD_KC_SPMV || m.kc == PD_KC_CG_VECTOR) {
                    // a sampled CG iteration; launches are counted per solve
                    kc_sample_ms_[m.kc] += ms;
                    kc_samples_[m.kc] += 1;
                } else {
                    kc_ms_[m.kc] += ms;
                    kc_launches_[m.kc] += 1;
                }
            }
        }
        event_pool_.push_back(m.a);
        event_pool_.push_back(m.b);
    }
    marks_.clear();
    open_mark_ = -1;
}

pd_status Engine::kernel_times(pd_kernel_times* t)
{
    // CG marks were filtered when their solve ended; what is left is complete work
    flush_marks(-1);
    for (int k = 0; k < PD_KC_COUNT; ++k) {
        t->launches[k] = kc_launches_[k];
        t->total_ms[k] = kc_ms_[k];
        if (k == PD_KC_SPMV || k == PD_KC_CG_VECTOR) {
            // mean duration of the sampled iterations x live iterations
            const long long iters = k == PD_KC_CG_VECTOR ? kc_launches_[k] / 2 : kc_launches_[k];
            t->total_ms[k] = kc_samples_[k] ? kc_sample_ms_[k] / (double)kc_samples_[k] * (double)iters : 0.0;
        }
    }
    return PD_OK;
}

void Engine::reset_kernel_times()
{
    flush_marks(-1);
    for (int k = 0; k < PD_KC_COUNT; ++k) {
        kc_launches_[k] = 0;
        kc_ms_[k] = 0.0;
        kc_samples_[k] = 0;
        kc_sample_ms_[k] = 0.0;
    }
}

// ---- exports -----------------------------------------------------------------------
pd_status Engine::ensure_stage(size_t bytes)
{
    if (bytes <= stage_cap_) return PD_OK;
    cudaFree(d_stage_);
    d_stage_ = nullptr;
    stage_cap_ = 0;
    CK(cudaMalloc(&d_stage_, bytes), "alloc export staging");
    stage_cap_ = bytes;
    return PD_OK;
}

// Slot-order device array -> caller order on the device, then one copy into
// the caller's buffer.
template <typename T>
pd_status Engine::download_scatter(const T* dev, T* host_out, size_t per, size_t count)
{
    if (count == 0) return PD_OK;
    const size_t bytes = sizeof(T) * per * count;
    pd_status s = ensure_stage(bytes);
    if (s != PD_OK) return s;
    scatter_words(dev, d_perm_, d_stage_, (int)(sizeof(T) * per / 4), (int)count, stream_);
    CK(cudaGetLastError(), "export scatter");
    CK(cudaMemcpyAsync(host_out, d_stage_, bytes, cudaMemcpyDeviceToHost, stream_), "download");
    CK(cudaStreamSynchronize(stream_), "download sync");
    return PD_OK;
}

pd_status Engine::export_vec4(const void* dev, bool is_float, double* dst)
{
    const size_t N = (size_t)n_;
    if (N == 0) return PD_OK;
    pd_status s = ensure_stage(sizeof(dbl4) * N);
    if (s != PD_OK) return s;
    scatter_to_d4_w0(dev, is_float, d_perm_, (dbl4*)d_stage_, (int)N, stream_);
    CK(cudaGetLastError(), "export scatter");
    CK(cudaMemcpyAsync(dst, d_stage_, sizeof(dbl4) * N, cudaMemcpyDeviceToHost, stream_), "download");
    CK(cudaStreamSynchronize(stream_), "download sync");
    return PD_OK;
}

pd_status Engine::export_bonds(int64_t* rp_out, int32_t* list_out)
{
    const size_t N = (size_t)n_;
    std::vector<int> rp(N + 1), cnt(N), col((size_t)std::max<long long>(total_slots_, 1));
    CK(cudaMemcpyAsync(rp.data(), S_.row_ptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, stream_), "download rp");
    if (N) CK(cudaMemcpyAsync(cnt.data(), S_.cnt, sizeof(int) * N, cudaMemcpyDeviceToHost, stream_), "download cnt");
    if (total_slots_ > 0)
        CK(cudaMemcpyAsync(col.data(), S_.col, sizeof(int) * (size_t)total_slots_, cudaMemcpyDeviceToHost, stream_),
           "download col");
    CK(cudaStreamSynchronize(stream_), "download sync");
    int64_t pos = 0;
    if (rp_out) rp_out[0] = 0;
    for (size_t o = 0; o < N; ++o) {
        const int s = inv_[o];
        const int base = rp[s], live = cnt[s], all = cnt_init_[s];
        if (list_out) {
            int32_t* row = list_out + pos;
            for (int j = 0; j < all; ++j) row[j] = perm_[col[base + j]];
            std::sort(row, row + live);
            std::sort(row + live, row + all);
        }
        pos += all;
        if (rp_out) rp_out[o + 1] = pos;
    }
    return PD_OK;
}

pd_status Engine::get_size(pd_variable var, size_t* bytes) const
{
    const size_t N = (size_t)n_;
    switch (var) {
    case PD_VAR_POSITION: case PD_VAR_VELOCITY: case PD_VAR_FORCE: case PD_VAR_SOLUTION:
    case PD_VAR_POSITION_SCALED: case PD_VAR_ORIGINAL_POSITION:
        *bytes = 4 * N * sizeof(double); return PD_OK;
    case PD_VAR_ACTIVITY: case PD_VAR_BOND_COUNT: case PD_VAR_SLOT_PERMUTATION:
        *bytes = N * sizeof(int32_t); return PD_OK;
    case PD_VAR_STRETCH: case PD_VAR_ORIGINAL_STRETCH: case PD_VAR_NEW_STRETCH: *bytes = N * sizeof(double); return PD_OK;
    case PD_VAR_BOND_ROW_PTR: *bytes = (N + 1) * sizeof(int64_t); return PD_OK;
    case PD_VAR_BOND_LIST: *bytes = (size_t)bonds_initial_ * sizeof(int32_t); return PD_OK;
    case PD_VAR_BROKEN_MASK: *bytes = (size_t)bonds_initial_; return PD_OK;
    }
    return PD_ERR_INVALID_ARGUMENT;
}

pd_status Engine::get(pd_variable var, void* dst, size_t bytes)
{
    size_t need = 0;
    if (get_size(var, &need) != PD_OK) return PD_ERR_INVALID_ARGUMENT;
    if (!dst && need > 0) return PD_ERR_INVALID_ARGUMENT;
    if (bytes < need) {
        err_ = "pd_get: destination too small";
        return PD_ERR_INVALID_ARGUMENT;
    }
    if (var == PD_VAR_ACTIVITY) {
        if (!particles_set_) return PD_ERR_NOT_READY;
        std::memcpy(dst, h_act_.data(), need);
        return PD_OK;
    }
    if (!ready_) {
        err_ = "pd_get: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    const size_t N = (size_t)n_;
    switch (var) {
    case PD_VAR_POSITION:
    case PD_VAR_POSITION_SCALED: {
        pd_status s = download_scatter((const double*)S_.x64, (double*)dst, 4, N);
        if (s != PD_OK) return s;
        if (var == PD_VAR_POSITION_SCALED)
            for (size_t i = 0; i < N; ++i)
                for (int k = 0; k < 3; ++k) ((double*)dst)[4 * i + k] *= sim_.scaleFactor;
        return PD_OK;
    }
    case PD_VAR_ORIGINAL_POSITION: return download_scatter((const double*)S_.X64, (double*)dst, 4, N);
    case PD_VAR_VELOCITY: return download_scatter((const double*)S_.v64, (double*)dst, 4, N);
    case PD_VAR_FORCE: return export_vec4(S_.force, !fp64_, (double*)dst);
    case PD_VAR_SOLUTION: return export_vec4(S_.sol, !fp64_, (double*)dst);
    case PD_VAR_BOND_COUNT: return download_scatter(S_.cnt, (int*)dst, 1, N);
    case PD_VAR_STRETCH: return download_scatter(S_.st, (double*)dst, 1, N);
    case PD_VAR_ORIGINAL_STRETCH: return download_scatter(S_.ost, (double*)dst, 1, N);
    case PD_VAR_NEW_STRETCH: return download_scatter(S_.nst, (double*)dst, 1, N);
    case PD_VAR_BOND_ROW_PTR: return export_bonds((int64_t*)dst, nullptr);
    case PD_VAR_BOND_LIST: return export_bonds(nullptr, (int32_t*)dst);
    case PD_VAR_SLOT_PERMUTATION:
        std::memcpy(dst, perm_.data(), N * sizeof(int32_t));
        return PD_OK;
    case PD_VAR_BROKEN_MASK: {
        // rows in caller order as PD_VAR_BOND_LIST: live bonds first, then broken
        std::vector<int> cnt(N);
        pd_status s = download_scatter(S_.cnt, cnt.data(), 1, N);
        if (s != PD_OK) return s;
        uint8_t* m = (uint8_t*)dst;
        size_t pos = 0;
        for (size_t o = 0; o < N; ++o) {
            const int live = cnt[o], all = cnt_init_[inv_[o]];
            for (int j = 0; j < all; ++j) m[pos + j] = j < live ? 0 : 1;
            pos += all;
        }
        return PD_OK;
    }
    default: return PD_ERR_INVALID_ARGUMENT;
    }
}

pd_status Engine::stats(pd_step_stats* s) const
{
    std::memset(s, 0, sizeof(*s));
    s->current_step = step_;
    s->cg_converged = cg_converged_ ? 1 : 0;
    s->last_cg_iterations = last_iters_;
    s->last_cg_residual = last_res_;
    s->last_cg_tolerance = last_tol_;
    s->total_cg_iterations = total_iters_;
    s->time_step_ticks = ticks_;
    s->substep = substep_;
    s->retries_last_step = retries_;
    s->bonds_initial = bonds_initial_;
    s->max_bonds_per_particle = sim_.pd_max_num_bonds;
    s->clock_scale = clock_scale_;
    s->sim_time = sim_time_;
    s->bonds_alive = bonds_initial_;
    s->ws_guesses_kept = ws_kept_;
    s->last_ws_residual_ratio = last_ws_ratio_;
    s->ws_learned_used = ws_net_used_;
    s->ws_guesses_skipped = ws_skipped_;
    s->host_syncs = host_syncs_;
    s->cg_graph_solves = cg_graph_solves_;
    if (ready_ && n_ > 0) {
        std::vector<int> c((size_t)n_);
        cudaSetDevice(device_);
        if (cudaMemcpyAsync(c.data(), S_.cnt, sizeof(int) * (size_t)n_, cudaMemcpyDeviceToHost, stream_) == cudaSuccess &&
            cudaStreamSynchronize(stream_) == cudaSuccess) {
            long long a = 0;
            for (int v : c) a += v;
            s->bonds_alive = a;
        }
    }
    return PD_OK;
}

// SPH <-> PD collision on the reference's grid (sim_.cell_size from
// boundary_min, num_cell_x/y/z) with the distance r_sph + r_pd
// (sph_pd_min_distance, parameters.cu:420-421); sph_coupling.cu.
pd_status Engine::sph_collide(double* pos4, double* vel4, int n_sph, double slip, int* collided)
{
    if (!ready_) {
        err_ = "sph_collide: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    if (n_sph < 0 || (n_sph > 0 && (!pos4 || !vel4)) || !std::isfinite(slip)) return PD_ERR_INVALID_ARGUMENT;
    if (sim_.num_cell_x <= 0 || sim_.num_cell_y <= 0 || sim_.num_cell_z <= 0 || !(sim_.cell_size > 0)) {
        err_ = "sph_collide: the simulation parameters define no grid";
        return PD_ERR_INVALID_ARGUMENT;
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    const SphGrid g{{sim_.boundary_min_x, sim_.boundary_min_y, sim_.boundary_min_z}, sim_.cell_size,
                    {sim_.num_cell_x, sim_.num_cell_y, sim_.num_cell_z}};
    const size_t bytes = sizeof(dbl4) * (size_t)std::max(n_sph, 1);
    for (auto pc : {std::make_pair(&sph_.pos, &sph_.pos_cap), std::make_pair(&sph_.vel, &sph_.vel_cap)}) {
        if (*pc.second < bytes) {
            if (*pc.first) cudaFree(*pc.first);
            *pc.first = nullptr;
            *pc.second = 0;
            CK(cudaMalloc((void**)pc.first, bytes), "alloc sph arrays");
            *pc.second = bytes;
        }
    }
    if (n_sph > 0) {
        CK(cudaMemcpyAsync(sph_.pos, pos4, sizeof(dbl4) * (size_t)n_sph, cudaMemcpyHostToDevice, stream_), "upload sph");
        CK(cudaMemcpyAsync(sph_.vel, vel4, sizeof(dbl4) * (size_t)n_sph, cudaMemcpyHostToDevice, stream_), "upload sph");
    }
    int c = 0;
    CK(sph_pd_collide(S_, d_perm_, g, sim_.sph_particle_radius + sim_.pd_particle_radius, sim_.sph_particle_mass,
                      sim_.pd_particle_mass, slip, n_sph, sph_.pos, sph_.vel, &sph_, &c, stream_), "sph collide");
    launches_ += 4 + (n_sph > 0 ? 2 : 0);
    if (n_sph > 0) {
        CK(cudaMemcpyAsync(pos4, sph_.pos, sizeof(dbl4) * (size_t)n_sph, cudaMemcpyDeviceToHost, stream_), "download sph");
        CK(cudaMemcpyAsync(vel4, sph_.vel, sizeof(dbl4) * (size_t)n_sph, cudaMemcpyDeviceToHost, stream_), "download sph");
        CK(cudaStreamSynchronize(stream_), "sph sync");
    }
    if (collided) *collided = c;
    return PD_OK;
}

void Engine::params(pd_sim_params* s, pd_run_params* r, pd_solver_options* o) const
{
    if (s) *s = sim_;
    if (r) *r = run_;
    if (o) {
        *o = opt_;
        if (ready_) {   // report the launch shape in use (autotuned when left at 0)
            o->lanes_per_particle = L_.lanes;
            o->spmv_unroll = L_.unroll;
            o->spmv_path = L_.lattice ? 3 : (L_.tiled ? 1 : 2);
        }
    }
}

}  // namespace pdgb
