// warmstart.cu -- per-particle features for the learned CG warm start, the
// application of the predicted guess, and training-sample collection.
//
// No reference counterpart.  Per step, with x1 = the previous solution (the
// reference's warm start), x2, x3 the two before it, r = b - A x1:
//   k_ws_jacobi    D_p = m + beta h^2 c sum_q (1/d0 - 2/(3d))  (trace/3 of the
//                  diagonal block), dj_p = r_p / D_p, and the RMS scales of
//                  x1, dj and v over free particles;
//   k_ws_features  64 features per particle (BF16): solution history,
//                  Jacobi step and its neighbour averages, bond-projected
//                  differences, velocity, stretch statistics, stiffness ratio,
//                  contact/boundary flags;
//   k_ws_apply     x0 = x1 + sigma_o * MLP(features) on free rows;
//   k_ws_column    h = sigma_o * MLP(features) (0 on Dirichlet rows), the
//                  learned column of the history projection;
//   k_ws_collect   (features, (x_new - x1) / sigma_o) rows into a dataset.
#include <cuda_bf16.h>

#include "pd_device.cuh"
#include "pd_kernels.h"
#include "warmstart_rows.cuh"

namespace pdgb {

namespace {

template <int G>
__global__ void __launch_bounds__(kBlock) k_ws_jacobi(StepParams P, DeviceState S, WsState W, ReduceSlot s0,
                                                      ReduceSlot s1, ReduceSlot s2)
{
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    const int stride = gridDim.x * gpb;
    DotAcc32 ax, ar, av;
    const int trips = (P.n + stride - 1) / stride;
    const int run_begin = blockIdx.x * trips * gpb;
    for (int t = 0; t < trips; ++t) {
        const int p = run_begin + t * gpb + threadIdx.x / G;
        if (p >= P.n) continue;
        ws_jacobi_row<G, kLdReadOnly>(P, S, W, p, lane, gmask, ax, ar, av);
    }
    WsScalars* sc = W.sc;
    block_reduce_finish(ax, s0, [sc](double v) { sc->sum_x2 = v; });
    block_reduce_finish(ar, s1, [sc](double v) { sc->sum_r2 = v; });
    block_reduce_finish(av, s2, [sc](double v) { sc->sum_v2 = v; });
}

template <int G>
__global__ void __launch_bounds__(kBlock) k_ws_features(StepParams P, DeviceState S, WsState W)
{
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    const int stride = gridDim.x * gpb;
    const WsScalars* sc = W.sc;
    const float sx = safe_scale(sc->sum_x2, sc->n_free);
    const float sr = safe_scale(sc->sum_r2, sc->n_free);
    const float sv = safe_scale(sc->sum_v2, sc->n_free);
    for (int p = blockIdx.x * gpb + threadIdx.x / G; p < P.n; p += stride)
        ws_features_row<G, kLdReadOnly>(P, S, W, p, lane, gmask, sx, sr, sv);
}

// x0 = x1 + sigma_o * y for free rows
__global__ void k_ws_apply(StepParams P, DeviceState S, WsState W, const float* __restrict__ Y)
{
    const WsScalars* sc = W.sc;
    const float so = safe_scale(sc->sum_x2, sc->n_free) + safe_scale(sc->sum_r2, sc->n_free);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x)
        ws_apply_elem(S, Y, p, so);
}

// the network's correction as a vector: h = sigma_o * y on free rows, 0 on
// Dirichlet rows (a column of the history projection, warm_start = 3)
__global__ void k_ws_column(StepParams P, DeviceState S, WsState W, const float* __restrict__ Y,
                            float4* __restrict__ h)
{
    const WsScalars* sc = W.sc;
    const float so = safe_scale(sc->sum_x2, sc->n_free) + safe_scale(sc->sum_r2, sc->n_free);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x) {
        const float* y = Y + (size_t)p * kMlpOutPad;
        h[p] = is_dirichlet(S.act[p] & kActMask) ? make_float4(0.f, 0.f, 0.f, 0.f)
                                                  : make_float4(so * y[0], so * y[1], so * y[2], 0.f);
    }
}

// dataset rows: features of particle p and (x_new - x1) / sigma_o
__global__ void k_ws_collect(StepParams P, DeviceState S, WsState W, int count, int stride, int offset,
                             long long pos, long long cap)
{
    const WsScalars* sc = W.sc;
    const float so = safe_scale(sc->sum_x2, sc->n_free) + safe_scale(sc->sum_r2, sc->n_free);
    const float4* xn = (const float4*)S.sol;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int p = W.free_list[((long long)offset + (long long)i * stride) % W.n_free_host];
        const long long row = (pos + i) % cap;
        const __nv_bfloat16* f = W.features + (size_t)p * kMlpIn;
        for (int k = 0; k < kMlpIn; ++k) W.ds_x[row * kMlpIn + k] = f[k];
        const float4 a = xn[p], b = W.xsave[p];
        W.ds_t[row * 3 + 0] = (a.x - b.x) / so;
        W.ds_t[row * 3 + 1] = (a.y - b.y) / so;
        W.ds_t[row * 3 + 2] = (a.z - b.z) / so;
    }
}

__global__ void k_count_free(const uint8_t* __restrict__ act, int n, int* __restrict__ out)
{
    int c = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += is_dirichlet(act[i] & kActMask) ? 0 : 1;
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, c);
}

}  // namespace

void launch_ws_jacobi(const StepParams& P, const DeviceState& S, const WsState& W, int lanes, int grid,
                      ReduceSlot s0, ReduceSlot s1, ReduceSlot s2, cudaStream_t st)
{
    (void)lanes;
    k_ws_jacobi<8><<<grid, kBlock, 0, st>>>(P, S, W, s0, s1, s2);
}

void launch_ws_features(const StepParams& P, const DeviceState& S, const WsState& W, int grid, cudaStream_t st)
{
    k_ws_features<8><<<grid, kBlock, 0, st>>>(P, S, W);
}

void launch_ws_apply(const StepParams& P, const DeviceState& S, const WsState& W, const float* Y, int grid,
                     cudaStream_t st)
{
    k_ws_apply<<<grid, kBlock, 0, st>>>(P, S, W, Y);
}

void launch_ws_column(const StepParams& P, const DeviceState& S, const WsState& W, const float* Y, float4* h,
                      int grid, cudaStream_t st)
{
    k_ws_column<<<grid, kBlock, 0, st>>>(P, S, W, Y, h);
}
void launch_ws_collect(const StepParams& P, const DeviceState& S, const WsState& W, int count, int stride, int offset,
                       long long pos, long long cap, cudaStream_t st)
{
    if (count <= 0) return;
    k_ws_collect<<<(count + kBlock - 1) / kBlock, kBlock, 0, st>>>(P, S, W, count, stride, offset, pos, cap);
}

void launch_count_free(const uint8_t* act, int n, int* out, cudaStream_t st)
{
    const int grid = n > 0 ? (n + kBlock - 1) / kBlock : 1;
    k_count_free<<<grid < 4096 ? grid : 4096, kBlock, 0, st>>>(act, n, out);
}

}  // namespace pdgb

namespace pdgb {
namespace {
__global__ void k_ws_save_plain(CgScalars* sc) { sc->rz_plain = sc->rz; }

// one thread: compare residuals, restore the plain scalars if the learned guess lost
__global__ void k_ws_decide(CgScalars* sc) { ws_decide(sc); }

__global__ void k_ws_revert(StepParams P, DeviceState S, const float4* __restrict__ xsave, const float4* __restrict__ rsave)
{
    if (!((volatile CgScalars*)S.sc)->ws_revert) return;
    float4* x = (float4*)S.sol;
    float4* r = (float4*)S.r;
    float4* p = (float4*)S.p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        x[i] = xsave[i];
        r[i] = rsave[i];
        p[i] = rsave[i];
    }
}
}  // namespace

void launch_ws_save_plain(const DeviceState& S, cudaStream_t st) { k_ws_save_plain<<<1, 1, 0, st>>>(S.sc); }

void launch_ws_guard(const StepParams& P, const DeviceState& S, const float4* xsave, const float4* rsave, int grid,
                     cudaStream_t st)
{
    k_ws_decide<<<1, 1, 0, st>>>(S.sc);
    k_ws_revert<<<grid, kBlock, 0, st>>>(P, S, xsave, rsave);
}
}  // namespace pdgb
