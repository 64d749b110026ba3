// batch.cu -- persistent multi-scene step kernels (cooperative launches).
//
// Each phase of the reference step (Simulator::integratePeridynamics*,
// simulator.cu:297-652, and CUSP krylov::cg) runs over the work items of the
// scenes taking part, strided over all blocks so that a lone large scene still
// spreads over the whole GPU; phases are separated by a grid barrier.  Scalar
// work of a scene (adaptive time-step decision, CG alpha / beta / test) is done
// by the block that reduces the scene's last item (reductions) or by the
// scene's owner block (step-loop bookkeeping).
//
// Memory visibility: every barrier is a gpu-scope release/acquire; data that
// a phase writes and a later phase of the same launch gathers from other rows
// is read through the coherent load path, never the read-only one.
#include "batch.h"
#include "step_rows.cuh"
#include "warmstart_rows.cuh"

namespace pdgb {

namespace {

constexpr unsigned long long kBarrierTimeoutNs = 5000000000ull;   // 5 s
constexpr int kForceLanes = 4;   // as the single-scene force pass (fastest of 4 / 8 / 16 at 1M)

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Sense-counting grid barrier.  A wait is bounded: after kBarrierTimeoutNs
// the block records the error and every later barrier returns false at once,
// so the launch ends instead of hanging.  Returns false on error.
__device__ bool grid_barrier(BatchSync* sync)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned g = ld_acquire(&sync->gen);
        __threadfence();
        const unsigned prev = atomicAdd(&sync->count, 1u);
        if (prev == gridDim.x - 1) {
            atomicExch(&sync->count, 0u);
            __threadfence();
            atomicAdd(&sync->gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            unsigned spins = 0;
            while (ld_acquire(&sync->gen) == g) {
                if (*(volatile int*)&sync->error) break;
                __nanosleep(32);
                if ((++spins & 63u) == 0 && global_ns() - t0 > kBarrierTimeoutNs) {
                    atomicExch(&sync->error, 1);
                    break;
                }
            }
        }
        __threadfence();
        s_ok = *(volatile int*)&sync->error == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

// Block reduction of one item's partial; the block that completes a scene sums
// the scene's item partials in item order and runs fin(total) on thread 0.
template <typename Acc, typename Fin>
__device__ __forceinline__ void item_reduce(Acc acc, const BatchArgs& A, int item, const SceneConst& C, int s, Fin fin)
{
    __shared__ double warp_sums[kBlock / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    const double w = warp_total(acc);
    if (lane == 0) warp_sums[warp] = w;
    __syncthreads();
    const int count = C.item_end - C.item_begin;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += warp_sums[i];
        A.partials[item] = t;
        __threadfence();
        const unsigned prev = atomicAdd(A.counters + s, 1u);
        is_last = (prev == (unsigned)count - 1u);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) t += __ldcg(A.partials + C.item_begin + i);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    __syncthreads();
    if (lane == 0) warp_sums[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) total += warp_sums[i];
        A.counters[s] = 0u;
        fin(total);
        __threadfence();
    }
}

// item_reduce for three sums at once (the learned warm start's RMS scales):
// partial k of item i lives at partials[k * n_items + i]; one arrival count.
template <typename Fin>
__device__ __forceinline__ void item_reduce3(const DotAcc32 (&acc)[3], const BatchArgs& A, int item,
                                             const SceneConst& C, int s, Fin fin)
{
    __shared__ double warp_sums[3][kBlock / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double w = warp_total(acc[k]);
        if (lane == 0) warp_sums[k][warp] = w;
    }
    __syncthreads();
    const int count = C.item_end - C.item_begin;
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            double t = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += warp_sums[k][i];
            A.partials[(size_t)k * A.n_items + item] = t;
        }
        __threadfence();
        const unsigned prev = atomicAdd(A.counters + s, 1u);
        is_last = (prev == (unsigned)count - 1u);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t[3] = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < count; i += blockDim.x)
        for (int k = 0; k < 3; ++k) t[k] += __ldcg(A.partials + (size_t)k * A.n_items + C.item_begin + i);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t[k] += __shfl_xor_sync(0xffffffffu, t[k], off);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < 3; ++k) warp_sums[k][warp] = t[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        double total[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 3; ++k)
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) total[k] += warp_sums[k][i];
        A.counters[s] = 0u;
        fin(total[0], total[1], total[2]);
        __threadfence();
    }
}

// Time-dependent step constants of a scene (Engine::step_params).
__device__ __forceinline__ void set_time_fields(StepParams& P, const SceneConst& C, const SceneRun& R)
{
    P.ticks = R.ticks;
    P.cs = R.cs;
    P.h = R.ticks * C.dt_base;
    P.t2 = C.integrator == 0 ? P.h * P.h : (P.h * P.h) / 4.0;
    for (int k = 0; k < 3; ++k) {
        P.sphere_c[k] = C.sphere_center0[k] + C.sphere_velocity[k] * R.sim_time;
        P.sphere_c_local[k] = P.sphere_c[k] - C.origin[k];
    }
}

// The adaptive time-step decision of integratePeridynamics* (simulator.cu:540-572).
__device__ __forceinline__ int adaptive_decide(int has_broken, const SceneConst& C, SceneRun& R)
{
    if (has_broken) {
        if (R.ticks > C.ticks_min) {
            R.ticks /= 2;
            return 1;
        }
        R.substep = 1;
    } else {
        if (R.substep > 0) ++R.substep;
        if (R.substep >= C.max_substep) {
            R.ticks *= 2;
            R.substep = (R.ticks >= C.ticks_base) ? 0 : 1;
        }
    }
    return 0;
}

// ---- per-phase item lists ----------------------------------------------------------
// Block b owns items b, b + grid, b + 2 grid, ...: a scene's items spread over
// consecutive blocks, so a lone large scene still uses the whole GPU.  At the
// start of a phase each block tests up to kBlock of its items at once (one
// parallel round of flag loads) and compacts the ones taking part, in item
// order, into shared memory.
enum : int { kSelForce = 0, kSelRestore = 1, kSelSolving = 2, kSelRunning = 3, kSelAll = 4 };

struct ItemList {
    int idx[kBlock];
    int count;
};

__device__ __forceinline__ bool selected(const BatchArgs& A, int s, int sel)
{
    const SceneRun* R = A.run + s;
    switch (sel) {
    case kSelForce: return ld_volatile(&R->active) != 0;
    case kSelRestore: return ld_volatile(&R->restore) != 0;
    case kSelSolving: return ld_volatile(&R->solving) != 0;
    case kSelRunning: return ld_volatile(&R->solving) != 0 && ld_volatile(&A.scenes[s].S.sc->done) == 0;
    default: return true;
    }
}

__device__ __forceinline__ void build_chunk(const BatchArgs& A, int sel, int c0, ItemList& L)
{
    __shared__ int warp_cnt[kBlock / 32];
    __syncthreads();   // the previous chunk's items are done
    const int i = (int)blockIdx.x + (c0 + (int)threadIdx.x) * (int)gridDim.x;
    const bool f = i < A.n_items && selected(A, A.items[i].scene, sel);
    const unsigned b = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_cnt[warp] = __popc(b);
    __syncthreads();
    int off = 0;
    for (int w = 0; w < warp; ++w) off += warp_cnt[w];
    if (f) L.idx[off + __popc(b & ((1u << lane) - 1u))] = i;
    if (threadIdx.x == kBlock - 1) L.count = off + __popc(b);
    __syncthreads();
}

// fn(item index, item) for this block's items selected by `sel`; every
// thread of the block runs every call (fn may contain block barriers).
template <typename Fn>
__device__ __forceinline__ void for_each_item(const BatchArgs& A, int sel, ItemList& L, Fn fn)
{
    const int b = (int)blockIdx.x, g = (int)gridDim.x;
    const int mine = A.n_items > b ? (A.n_items - b + g - 1) / g : 0;
    for (int c0 = 0; c0 < mine; c0 += kBlock) {
        build_chunk(A, sel, c0, L);
        const int count = L.count;
        for (int k = 0; k < count; ++k) {
            const int i = L.idx[k];
            fn(i, A.items[i]);
        }
    }
}

// ---- phases ------------------------------------------------------------------------
template <int G, bool FP64>
__device__ void force_item(const SceneDesc& d, const WorkItem& it)
{
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    for (int p = it.lo + threadIdx.x / G; p < it.hi; p += gpb) force_row<G, FP64>(d.P, d.S, p, lane, gmask);
}

template <int G, bool FP64, bool DOT, int U, int LD, typename Acc>
__device__ void spmv_item(const SceneDesc& d, const WorkItem& it, const void* in_, void* out_, Acc& acc)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    // every group runs the same number of trips (the shuffles need whole groups)
    for (int p0 = it.lo; p0 < it.hi; p0 += gpb) {
        const int p = p0 + threadIdx.x / G;
        if (p < it.hi) spmv_row<G, FP64, DOT, U, LD>(d.P, d.S, (const V4*)in_, (V4*)out_, p, lane, gmask, acc);
    }
}

// ---- learned warm start (mixed precision) -------------------------------------------
// A scene whose guard rejected kWsRejectLimit guesses in a row pauses its
// learned pass (features, guess, guess residual): it starts from the previous
// solution as without the network, and tries the network again every
// kWsRetryPeriod steps; one kept guess ends the pause.
constexpr int kWsRejectLimit = 3;
constexpr int kWsRetryPeriod = 16;

__device__ __forceinline__ bool ws_paused(const SceneDesc& d) { return ld_volatile(&d.S.sc->ws_skip) != 0; }

// End of k_batch_pre: x1 saved, Jacobi step and the RMS scales, features of
// every solving scene whose learned pass is not paused (written into the
// batch's feature rows).
__device__ void ws_features_phases(const BatchArgs& A, ItemList& L)
{
    constexpr int G = 8;
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    // this step's pause decision, by the scene's owner thread (the fields are
    // not touched by the phase still running in other blocks)
    if (threadIdx.x == 0) {
        for (int s = blockIdx.x; s < A.n_scenes; s += gridDim.x) {
            if (!ld_volatile(&A.run[s].solving)) continue;
            CgScalars* sc = A.scenes[s].S.sc;
            const int rej = sc->ws_rejects;
            const int skip = rej >= kWsRejectLimit && (rej % kWsRetryPeriod) != kWsRetryPeriod - 1;
            sc->ws_skip = skip;
            if (skip) {
                sc->ws_rejects = rej + 1;
                sc->ws_skipped += 1;
            }
        }
    }
    if (!grid_barrier(A.sync)) return;
    for_each_item(A, kSelSolving, L, [&](int i, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        const float4* x = (const float4*)d.S.sol;
        // solution history of the features: x3 <- x2 <- the previous step's
        // x1, then x1 <- the current guess (kept current while paused)
        for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) {
            d.W.hist3[r] = d.W.hist2[r];
            d.W.hist2[r] = d.W.xsave[r];
            d.W.xsave[r] = x[r];
        }
        if (ws_paused(d)) return;   // every item of the scene returns: its reduction is not entered
        DotAcc32 acc[3];
        for (int p0 = it.lo; p0 < it.hi; p0 += gpb) {
            const int p = p0 + threadIdx.x / G;
            if (p < it.hi) ws_jacobi_row<G, kLdCoherent>(d.P, d.S, d.W, p, lane, gmask, acc[0], acc[1], acc[2]);
        }
        WsScalars* wsc = d.W.sc;
        item_reduce3(acc, A, i, d.C, it.scene, [wsc](double x2, double r2, double v2) {
            wsc->sum_x2 = x2;
            wsc->sum_r2 = r2;
            wsc->sum_v2 = v2;
        });
    });
    if (!grid_barrier(A.sync)) return;
    for_each_item(A, kSelSolving, L, [&](int, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        if (ws_paused(d)) return;
        const volatile WsScalars* wsc = d.W.sc;
        const float sx = safe_scale(wsc->sum_x2, wsc->n_free);
        const float sr = safe_scale(wsc->sum_r2, wsc->n_free);
        const float sv = safe_scale(wsc->sum_v2, wsc->n_free);
        for (int p0 = it.lo; p0 < it.hi; p0 += gpb) {
            const int p = p0 + threadIdx.x / G;
            if (p < it.hi) ws_features_row<G, kLdCoherent>(d.P, d.S, d.W, p, lane, gmask, sx, sr, sv);
        }
    });
}

// k_batch_ws_guess, after the network ran on the feature rows: the learned
// guess x0 = x1 + sigma MLP, its residual, and the guard that goes back to x1
// (and its residual) where the learned guess is worse.  The running-scene
// count follows the convergence flags the guard leaves.
template <int G, int U>
__device__ void ws_guess_phases(const BatchArgs& A, ItemList& L)
{
    using Acc = typename DotAccFor<float>::type;
    if (threadIdx.x == 0) {
        for (int s = blockIdx.x; s < A.n_scenes; s += gridDim.x)
            if (A.run[s].solving) A.scenes[s].S.sc->rz_plain = A.scenes[s].S.sc->rz;
    }
    for_each_item(A, kSelSolving, L, [&](int, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        if (ws_paused(d)) return;
        const WsScalars* wsc = d.W.sc;
        const float so = safe_scale(wsc->sum_x2, wsc->n_free) + safe_scale(wsc->sum_r2, wsc->n_free);
        const float4* r = (const float4*)d.S.r;
        for (int p = it.lo + threadIdx.x; p < it.hi; p += blockDim.x) {
            d.rsave[p] = r[p];
            ws_apply_elem(d.S, d.ws_y, p, so);
        }
    });
    if (!grid_barrier(A.sync)) return;
    for_each_item(A, kSelSolving, L, [&](int, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        if (ws_paused(d)) return;
        Acc acc;
        spmv_item<G, false, false, U, kLdCoherent>(d, it, d.S.sol, d.S.y, acc);
    });
    if (!grid_barrier(A.sync)) return;
    for_each_item(A, kSelSolving, L, [&](int i, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        if (ws_paused(d)) return;
        Acc acc;
        for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) residual_elem<false>(d.S, r, acc);
        CgScalars* sc = d.S.sc;
        BatchSync* sync = A.sync;
        item_reduce(acc, A, i, d.C, it.scene, [sc, sync](double rr) {
            const int was = sc->done ? 0 : 1;
            cg_fin_residual(sc, rr);
            ws_decide(sc);
            const int now = sc->done ? 0 : 1;
            if (now != was) atomicAdd(&sync->running, now - was);
        });
    });
    if (!grid_barrier(A.sync)) return;
    for_each_item(A, kSelSolving, L, [&](int, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        if (ws_paused(d) || !ld_volatile(&d.S.sc->ws_revert)) return;
        float4* x = (float4*)d.S.sol;
        float4* r = (float4*)d.S.r;
        float4* pv = (float4*)d.S.p;
        for (int p = it.lo + threadIdx.x; p < it.hi; p += blockDim.x) {
            x[p] = d.W.xsave[p];
            r[p] = d.rsave[p];
            pv[p] = d.rsave[p];
        }
    });
    grid_barrier(A.sync);
}

// The learned guess of every solving scene (a launch of its own between the
// network and k_batch_cg, so the CG kernel keeps its register budget).
template <int G, int U>
__global__ void __launch_bounds__(kBlock, 4) k_batch_ws_guess(BatchArgs A)
{
    __shared__ ItemList L;
    ws_guess_phases<G, U>(A, L);
}

// ---- k_batch_pre ---------------------------------------------------------------------
// The scenes' descriptors are read in place: their time-dependent fields are
// rewritten by owner blocks only in phases separated from the readers by a
// grid barrier.
// WS: with the learned warm start (a separate instantiation, so the plain
// kernels keep their register budget).
template <bool FP64, bool WS>
__global__ void __launch_bounds__(kBlock, FP64 ? 1 : 3) k_batch_pre(BatchArgs A)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using Acc = typename DotAccFor<Real>::type;
    __shared__ ItemList L;

    // step start (Simulator::advance: ++step, phase-in clockScale, retries = 0)
    if (threadIdx.x == 0) {
        for (int s = blockIdx.x; s < A.n_scenes; s += gridDim.x) {
            SceneRun& R = A.run[s];
            SceneDesc& D = A.scenes[s];
            R.solving = 0;
            R.restore = 0;
            R.active = 0;
            if (!R.cg_converged || R.error || D.C.n == 0) continue;
            R.step += 1;
            if (R.step <= D.C.phase_in_steps) R.cs = (double)R.step / (double)D.C.phase_in_steps;
            R.retries = 0;
            R.active = 1;
            set_time_fields(D.P, D.C, R);
            D.S.flags[0] = 0;
            D.S.flags[1] = 0;
        }
        if (blockIdx.x == 0) {
            A.sync->pending[0] = 0;
            A.sync->pending[1] = 0;
            A.sync->running = 0;
        }
    }
    if (!grid_barrier(A.sync)) return;

    for (int round = 0; round < A.max_rounds; ++round) {
        // force pass of the scenes still pending (mixed precision: their
        // supercell words first, which the rows read for their neighbours)
        if (!FP64) {
            for_each_item(A, kSelForce, L, [&](int, const WorkItem& it) {
                const SceneDesc& d = A.scenes[it.scene];
                for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) supercell_elem(d.P, d.S, r);
            });
            if (!grid_barrier(A.sync)) return;
        }
        for_each_item(A, kSelForce, L, [&](int, const WorkItem& it) {
            force_item<kForceLanes, FP64>(A.scenes[it.scene], it);
        });
        if (!grid_barrier(A.sync)) return;
        // decision (owner block of each scene).  Every block has read the
        // previous round's pending count by now, so its counter can be reset
        // for the next round.
        if (threadIdx.x == 0) {
            if (blockIdx.x == 0) A.sync->pending[(round + 1) & 1] = 0;
            for (int s = blockIdx.x; s < A.n_scenes; s += gridDim.x) {
                SceneRun& R = A.run[s];
                if (!R.active) {
                    R.restore = 0;
                    continue;
                }
                SceneDesc& D = A.scenes[s];
                volatile int* flags = D.S.flags;
                const int has_broken = flags[0];
                const int nbroken = flags[1];
                flags[0] = 0;
                flags[1] = 0;
                int rollback = 0;
                if (D.C.adaptive) rollback = adaptive_decide(has_broken, D.C, R);
                if (rollback) {
                    R.restore = 1;
                    R.rollbacks += 1;
                    if (++R.retries > 64) {
                        R.error = 1;
                        R.active = 0;
                        R.restore = 0;
                        continue;
                    }
                    atomicAdd(&A.sync->pending[round & 1], 1);
                } else {
                    R.restore = D.C.adaptive ? 2 : 0;
                    R.active = 0;
                    R.solving = 1;
                    R.broken += nbroken;
                }
                set_time_fields(D.P, D.C, R);
            }
        }
        if (!grid_barrier(A.sync)) return;
        // rollback restore (restoreBondListTopIndex / restorePDPosition /
        // restorePDVelocity, memory_manager.cu:500-550) or the step's backup
        for_each_item(A, kSelRestore, L, [&](int, const WorkItem& it) {
            const int mode = ld_volatile(&A.run[it.scene].restore);
            const DeviceState& S = A.scenes[it.scene].S;
            for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) {
                if (mode == 1) {
                    S.cnt[r] = S.cnt_bk[r];
                    S.x64[r] = S.x64_bk[r];
                    S.v64[r] = S.v64_bk[r];
                } else {
                    S.cnt_bk[r] = S.cnt[r];
                    S.x64_bk[r] = S.x64[r];
                    S.v64_bk[r] = S.v64[r];
                }
            }
        });
        if (!grid_barrier(A.sync)) return;
        if (ld_volatile(&A.sync->pending[round & 1]) == 0) break;
    }

    // CG set-up of the solving scenes: b, Dirichlet values, ||b||
    for_each_item(A, kSelSolving, L, [&](int i, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        Acc acc;
        for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) cg_init_elem<FP64>(d.P, d.S, r, acc);
        CgScalars* sc = d.S.sc;
        item_reduce(acc, A, i, d.C, it.scene, [sc](double bb) { cg_fin_init(sc, bb); });
    });
    if (!grid_barrier(A.sync)) return;
    // y = A x0 (warm start: the previous solution)
    for_each_item(A, kSelSolving, L, [&](int, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        Acc acc;
        spmv_item<8, FP64, false, 2, kLdCoherent>(d, it, d.S.sol, d.S.y, acc);
    });
    if (!grid_barrier(A.sync)) return;
    // r = b - A x0, p = r, convergence test
    for_each_item(A, kSelSolving, L, [&](int i, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        Acc acc;
        for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) residual_elem<FP64>(d.S, r, acc);
        CgScalars* sc = d.S.sc;
        BatchSync* sync = A.sync;
        item_reduce(acc, A, i, d.C, it.scene, [sc, sync](double rr) {
            cg_fin_residual(sc, rr);
            if (!sc->done) atomicAdd(&sync->running, 1);
        });
    });
    if constexpr (WS && !FP64) ws_features_phases(A, L);
}

// ---- k_batch_cg ----------------------------------------------------------------------
// 4 resident blocks per SM (64 registers): the CG phases are latency-bound
// gathers, and at 64 scenes / 1.39M particles this beats 79 registers and 3
// blocks by 16 % per step despite a few spilled registers.
template <int G, bool FP64, int U>
__global__ void __launch_bounds__(kBlock, 4) k_batch_cg(BatchArgs A)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using Acc = typename DotAccFor<Real>::type;
    __shared__ ItemList L;

    if (A.tune_reps > 0) {
        // autotuning: the SpMV phase alone (y = A x), no state changes
        for (int rep = 0; rep < A.tune_reps; ++rep) {
            for_each_item(A, kSelAll, L, [&](int, const WorkItem& it) {
                const SceneDesc& d = A.scenes[it.scene];
                Acc acc;
                spmv_item<G, FP64, false, U, kLdCoherentIn>(d, it, d.S.sol, d.S.y, acc);
            });
            if (!grid_barrier(A.sync)) return;
        }
        return;
    }

    for (int iter = 0; iter < A.max_cg_iters; ++iter) {
        if (ld_volatile(&A.sync->running) == 0) break;
        // y = A p, alpha = rz / <p, y>
        for_each_item(A, kSelRunning, L, [&](int i, const WorkItem& it) {
            const SceneDesc& d = A.scenes[it.scene];
            CgScalars* sc = d.S.sc;
            Acc acc;
            spmv_item<G, FP64, true, U, kLdCoherentIn>(d, it, d.S.p, d.S.y, acc);
            item_reduce(acc, A, i, d.C, it.scene, [sc](double pAp) { cg_fin_alpha(sc, pAp); });
        });
        if (!grid_barrier(A.sync)) return;
        // x += alpha p, r -= alpha y, beta, test (a scene is marked done only
        // after all its items have reported, so the selection stays valid)
        for_each_item(A, kSelRunning, L, [&](int i, const WorkItem& it) {
            const SceneDesc& d = A.scenes[it.scene];
            CgScalars* sc = d.S.sc;
            const Real alpha = (Real)__ldcg(&sc->alpha);
            Acc acc;
            for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) axpy_elem<FP64>(d.S, r, alpha, acc);
            BatchSync* sync = A.sync;
            item_reduce(acc, A, i, d.C, it.scene, [sc, sync](double rr) {
                cg_fin_axpy(sc, rr);
                if (sc->done) atomicSub(&sync->running, 1);
            });
        });
        if (!grid_barrier(A.sync)) return;
        if (ld_volatile(&A.sync->running) == 0) break;
        // p = r + beta p
        for_each_item(A, kSelRunning, L, [&](int, const WorkItem& it) {
            const SceneDesc& d = A.scenes[it.scene];
            const Real beta = (Real)__ldcg(&d.S.sc->beta);
            for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) xpby_elem<FP64>(d.S, r, beta);
        });
        if (!grid_barrier(A.sync)) return;
    }
    // update of the solved scenes
    for_each_item(A, kSelSolving, L, [&](int, const WorkItem& it) {
        const SceneDesc& d = A.scenes[it.scene];
        for (int r = it.lo + threadIdx.x; r < it.hi; r += blockDim.x) update_elem<FP64>(d.P, d.S, r);
    });
    // per-scene bookkeeping (owner block): solve statistics, simulated time.
    // `solving` stays set until the next step starts: other blocks may still
    // be reading it in the update phase above.
    if (threadIdx.x == 0) {
        for (int s = blockIdx.x; s < A.n_scenes; s += gridDim.x) {
            SceneRun& R = A.run[s];
            if (!R.solving) continue;
            const SceneDesc& D = A.scenes[s];
            const volatile CgScalars* sc = D.S.sc;
            R.last_iters = sc->iter;
            R.total_iters += sc->iter;
            R.last_res = sc->rnorm;
            R.last_tol = sc->tol;
            if (!sc->converged) R.cg_converged = 0;
            R.sim_time += D.P.h;
        }
    }
}

template <int G, int U>
cudaError_t cg_launch(bool fp64, const BatchArgs& A, int grid, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (fp64) return cudaLaunchKernelEx(&cfg, k_batch_cg<G, true, 1>, A);
    return cudaLaunchKernelEx(&cfg, k_batch_cg<G, false, U>, A);
}

template <int G, int U>
cudaError_t ws_launch(const BatchArgs& A, int grid, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch_ws_guess<G, U>, A);
}

template <int G, int U>
int cg_blocks(bool fp64)
{
    int b = 0;
    if (fp64) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_cg<G, true, 1>, kBlock, 0), b;
    // a small shared-memory carve-out (the rest stays L1): 4 blocks of ~1.3 KB
    // (+ 1 KB reserved each) do not fit the smallest one
    cudaFuncSetAttribute(k_batch_cg<G, false, U>, cudaFuncAttributePreferredSharedMemoryCarveout, 10);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_cg<G, false, U>, kBlock, 0);
    return b;
}

template <int G, int U>
int ws_blocks()
{
    int b = 0;
    cudaFuncSetAttribute(k_batch_ws_guess<G, U>, cudaFuncAttributePreferredSharedMemoryCarveout, 10);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_ws_guess<G, U>, kBlock, 0);
    return b;
}

}  // namespace

cudaError_t launch_batch_pre(bool fp64, const BatchArgs& A, int grid, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (fp64) return cudaLaunchKernelEx(&cfg, k_batch_pre<true, false>, A);
    if (A.warm_start) return cudaLaunchKernelEx(&cfg, k_batch_pre<false, true>, A);
    return cudaLaunchKernelEx(&cfg, k_batch_pre<false, false>, A);
}

cudaError_t launch_batch_cg(bool fp64, int lanes, int unroll, const BatchArgs& A, int grid, cudaStream_t st)
{
    if (lanes == 4) return unroll == 4 ? cg_launch<4, 4>(fp64, A, grid, st) : cg_launch<4, 2>(fp64, A, grid, st);
    return unroll == 4 ? cg_launch<8, 4>(fp64, A, grid, st) : cg_launch<8, 2>(fp64, A, grid, st);
}

int batch_pre_blocks_per_sm(bool fp64)
{
    int b = 0, c = 0;
    if (fp64) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_pre<true, false>, kBlock, 0), b;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_pre<false, false>, kBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_batch_pre<false, true>, kBlock, 0);
    return b < c ? b : c;
}

int batch_cg_blocks_per_sm(bool fp64, int lanes, int unroll)
{
    if (lanes == 4) return unroll == 4 ? cg_blocks<4, 4>(fp64) : cg_blocks<4, 2>(fp64);
    return unroll == 4 ? cg_blocks<8, 4>(fp64) : cg_blocks<8, 2>(fp64);
}

cudaError_t launch_batch_ws_guess(int lanes, int unroll, const BatchArgs& A, int grid, cudaStream_t st)
{
    if (lanes == 4) return unroll == 4 ? ws_launch<4, 4>(A, grid, st) : ws_launch<4, 2>(A, grid, st);
    return unroll == 4 ? ws_launch<8, 4>(A, grid, st) : ws_launch<8, 2>(A, grid, st);
}

int batch_ws_blocks_per_sm(int lanes, int unroll)
{
    if (lanes == 4) return unroll == 4 ? ws_blocks<4, 4>() : ws_blocks<4, 2>();
    return unroll == 4 ? ws_blocks<8, 4>() : ws_blocks<8, 2>();
}

}  // namespace pdgb
