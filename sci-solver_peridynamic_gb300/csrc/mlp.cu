// mlp.cu -- the learned CG warm start: a per-particle MLP on BF16 tensor cores.
//
// No reference counterpart (the reference starts each CG from the previous
// solution, src/core/simulator.cu:745-770).  A small network
//   64 features -> 128 -> 128 -> 3,  GELU,  BF16 weights/activations,
//   FP32 accumulation on tcgen05 (mlp_tc.cu), FP32 master weights + Adam
// predicts the change of the solution over its previous value; the CG then
// runs to the same tolerance from the predicted guess, so the network only
// changes the iteration count, never the convergence test.
//
// Training runs each layer's forward and backward products as GEMMs on the
// 5th-generation tensor cores (gemm_tc: 128 x 128 tiles of C, K in slabs of
// 64, TMEM accumulators); inference runs the whole network in one kernel
// (mlp_infer_tc).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "pd_device.cuh"
#include "pd_gb300.h"
#include "pd_kernels.h"

namespace pdgb {
void set_handleless_error(const std::string& msg);   // capi.cpp

namespace {

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x)
{
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.3989422804014327f * expf(-0.5f * x * x);
}

// Z += bias (columns < nbias; the rest get none); H = GELU(Z) as BF16 (Z
// kept in FP32 for the backward pass)
__global__ void k_bias_gelu(float* __restrict__ Z, const float* __restrict__ bias, __nv_bfloat16* __restrict__ H, int M,
                            int N, int nbias, int act)
{
    const long long total = (long long)M * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % N);
        const float z = Z[i] + (c < nbias ? bias[c] : 0.f);
        Z[i] = z;
        if (H) H[i] = __float2bfloat16_rn(act ? gelu(z) : z);
    }
}

// dY = 2 (Y - T) / B over the first `nout` columns of Y (ldy), loss partials
__global__ void k_mse_grad(const float* __restrict__ Y, int ldy, const float* __restrict__ T, int nout, int B,
                           __nv_bfloat16* __restrict__ dY, int lddy, double* __restrict__ loss_acc)
{
    double local = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
        for (int c = 0; c < lddy; ++c) {
            float d = 0.f;
            if (c < nout) {
                const float e = Y[(size_t)i * ldy + c] - T[(size_t)i * nout + c];
                d = 2.f * e / (float)B;
                local += (double)e * (double)e;
            }
            dY[(size_t)i * lddy + c] = __float2bfloat16_rn(d);
        }
    }
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc, local / (double)B);
}

// dZ = dH * GELU'(Z) as BF16; dH (f32)
__global__ void k_gelu_back(const float* __restrict__ dH, const float* __restrict__ Z, __nv_bfloat16* __restrict__ dZ,
                            long long total)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
        dZ[i] = __float2bfloat16_rn(dH[i] * gelu_grad(Z[i]));
}

// column sums of a BF16 [M x N] matrix into f32 (bias gradients)
__global__ void k_colsum(const __nv_bfloat16* __restrict__ X, int M, int N, int ldx, float* __restrict__ out)
{
    const int c = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < M; r += blockDim.x) s += __bfloat162float(X[(size_t)r * ldx + c]);
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0 && c < N) out[c] = sh[0];
}

// Adam on the FP32 master parameters, refreshing the BF16 weight copies
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m1, float* __restrict__ m2,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = grad[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    }
}

// BF16 copy of a weight matrix, [rows x cols] row-major into [rows x ldo] (zero padded)
__global__ void k_to_bf16(const float* __restrict__ src, int rows, int cols, __nv_bfloat16* __restrict__ dst, int ldo)
{
    const int total = rows * ldo;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int r = i / ldo, c = i % ldo;
        dst[i] = __float2bfloat16_rn(c < cols ? src[r * cols + c] : 0.f);
    }
}

int blocks_for(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 8192) b = 8192;
    return (int)b;
}

// C = op(A) op(B) (+ C) on the tensor cores (mlp_tc.cu); launch errors surface
// at the pass's next error check, a wait that ran out of time through
// mlp_tc_take_error
template <bool TA, bool TB>
void gemm(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc,
          bool accumulate, cudaStream_t st)
{
    gemm_tc(TA, TB, M, N, K, A, lda, B, ldb, C, ldc, accumulate, st);
}

}  // namespace

// ---- network -------------------------------------------------------------------------
// parameter blob (FP32): W1 [64 x 128], b1 [128], W2 [128 x 128], b2 [128], W3 [128 x 3], b3 [3]
size_t mlp_param_count() { return (size_t)kMlpIn * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden +
                                  kMlpHidden * kMlpOut + kMlpOut; }

void mlp_refresh_bf16(MlpDev& m, cudaStream_t st)
{
    const float* w1 = m.params;
    const float* w2 = w1 + kMlpIn * kMlpHidden + kMlpHidden;
    const float* w3 = w2 + kMlpHidden * kMlpHidden + kMlpHidden;
    k_to_bf16<<<blocks_for(kMlpIn * kMlpHidden), 256, 0, st>>>(w1, kMlpIn, kMlpHidden, m.w1b, kMlpHidden);
    k_to_bf16<<<blocks_for(kMlpHidden * kMlpHidden), 256, 0, st>>>(w2, kMlpHidden, kMlpHidden, m.w2b, kMlpHidden);
    k_to_bf16<<<blocks_for(kMlpHidden * kMlpOutPad), 256, 0, st>>>(w3, kMlpHidden, kMlpOut, m.w3b, kMlpOutPad);
}

// Forward over B rows of X (BF16 [B x 64]); Y f32 [B x kMlpOutPad]; activations kept in ws.
void mlp_forward(const MlpDev& m, const __nv_bfloat16* X, int B, MlpWork& ws, float* Y, cudaStream_t st)
{
    const float* b1 = m.params + kMlpIn * kMlpHidden;
    const float* b2 = b1 + kMlpHidden + kMlpHidden * kMlpHidden;
    const float* b3 = b2 + kMlpHidden + kMlpHidden * kMlpOut;
    gemm<false, false>(B, kMlpHidden, kMlpIn, X, kMlpIn, m.w1b, kMlpHidden, ws.z1, kMlpHidden, false, st);
    k_bias_gelu<<<blocks_for((long long)B * kMlpHidden), 256, 0, st>>>(ws.z1, b1, ws.h1, B, kMlpHidden, kMlpHidden, 1);
    gemm<false, false>(B, kMlpHidden, kMlpHidden, ws.h1, kMlpHidden, m.w2b, kMlpHidden, ws.z2, kMlpHidden, false, st);
    k_bias_gelu<<<blocks_for((long long)B * kMlpHidden), 256, 0, st>>>(ws.z2, b2, ws.h2, B, kMlpHidden, kMlpHidden, 1);
    gemm<false, false>(B, kMlpOutPad, kMlpHidden, ws.h2, kMlpHidden, m.w3b, kMlpOutPad, Y, kMlpOutPad, false, st);
    k_bias_gelu<<<blocks_for((long long)B * kMlpOutPad), 256, 0, st>>>(Y, b3, nullptr, B, kMlpOutPad, kMlpOut, 0);
}

// Loss and gradients (into m.grad) for a batch; returns nothing, loss accumulates in *loss (device double).
void mlp_backward(const MlpDev& m, const __nv_bfloat16* X, const float* T, int B, MlpWork& ws, const float* Y,
                  double* loss, cudaStream_t st)
{
    float* gw1 = m.grad;
    float* gb1 = gw1 + kMlpIn * kMlpHidden;
    float* gw2 = gb1 + kMlpHidden;
    float* gb2 = gw2 + kMlpHidden * kMlpHidden;
    float* gw3 = gb2 + kMlpHidden;
    float* gb3 = gw3 + kMlpHidden * kMlpOut;
    // dY [B x 8] BF16
    k_mse_grad<<<blocks_for(B), 256, 0, st>>>(Y, kMlpOutPad, T, kMlpOut, B, ws.dy, kMlpOutPad, loss);
    // layer 3: dW3 = H2^T dY  [128 x 3], db3 = colsum(dY), dH2 = dY W3^T
    gemm<true, false>(kMlpHidden, kMlpOut, B, ws.h2, kMlpHidden, ws.dy, kMlpOutPad, gw3, kMlpOut, false, st);
    k_colsum<<<kMlpOut, 256, 0, st>>>(ws.dy, B, kMlpOut, kMlpOutPad, gb3);
    gemm<false, true>(B, kMlpHidden, kMlpOutPad, ws.dy, kMlpOutPad, m.w3b, kMlpOutPad, ws.dh, kMlpHidden, false, st);
    k_gelu_back<<<blocks_for((long long)B * kMlpHidden), 256, 0, st>>>(ws.dh, ws.z2, ws.dz, (long long)B * kMlpHidden);
    // layer 2
    gemm<true, false>(kMlpHidden, kMlpHidden, B, ws.h1, kMlpHidden, ws.dz, kMlpHidden, gw2, kMlpHidden, false, st);
    k_colsum<<<kMlpHidden, 256, 0, st>>>(ws.dz, B, kMlpHidden, kMlpHidden, gb2);
    gemm<false, true>(B, kMlpHidden, kMlpHidden, ws.dz, kMlpHidden, m.w2b, kMlpHidden, ws.dh, kMlpHidden, false, st);
    k_gelu_back<<<blocks_for((long long)B * kMlpHidden), 256, 0, st>>>(ws.dh, ws.z1, ws.dz, (long long)B * kMlpHidden);
    // layer 1
    gemm<true, false>(kMlpIn, kMlpHidden, B, X, kMlpIn, ws.dz, kMlpHidden, gw1, kMlpHidden, false, st);
    k_colsum<<<kMlpHidden, 256, 0, st>>>(ws.dz, B, kMlpHidden, kMlpHidden, gb1);
}

void mlp_adam(MlpDev& m, float lr, int t, cudaStream_t st)
{
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    const int n = (int)mlp_param_count();
    k_adam<<<blocks_for(n), 256, 0, st>>>(m.params, m.grad, m.m1, m.m2, n, lr, b1, b2, eps, c1, c2);
    mlp_refresh_bf16(m, st);
}

}  // namespace pdgb

// ---- allocation and host entry points ------------------------------------------------
namespace pdgb {

namespace {
__global__ void k_f32_to_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = __float2bfloat16_rn(src[i]);
}

__global__ void k_gather_rows(const __nv_bfloat16* __restrict__ X, const float* __restrict__ T, const int* __restrict__ idx,
                              int B, __nv_bfloat16* __restrict__ Xb, float* __restrict__ Tb)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * kMlpIn; i += gridDim.x * blockDim.x) {
        const int r = i / kMlpIn, c = i % kMlpIn;
        Xb[i] = X[(size_t)idx[r] * kMlpIn + c];
        if (c < kMlpOut) Tb[r * kMlpOut + c] = T[(size_t)idx[r] * kMlpOut + c];
    }
}

struct Xorshift {
    uint64_t s;
    explicit Xorshift(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull) {}
    uint64_t next()
    {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
    }
    float uniform() { return (float)((next() >> 11) * (1.0 / 9007199254740992.0)); }
};
}  // namespace

cudaError_t mlp_alloc(MlpDev* m, bool training)
{
    *m = MlpDev{};
    const size_t P = mlp_param_count();
    cudaError_t e;
    if ((e = cudaMalloc(&m->params, P * sizeof(float))) != cudaSuccess) return e;
    if (training) {
        if ((e = cudaMalloc(&m->grad, P * sizeof(float))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&m->m1, P * sizeof(float))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&m->m2, P * sizeof(float))) != cudaSuccess) return e;
        cudaMemset(m->grad, 0, P * sizeof(float));
        cudaMemset(m->m1, 0, P * sizeof(float));
        cudaMemset(m->m2, 0, P * sizeof(float));
    }
    if ((e = cudaMalloc(&m->w1b, sizeof(__nv_bfloat16) * kMlpIn * kMlpHidden)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&m->w2b, sizeof(__nv_bfloat16) * kMlpHidden * kMlpHidden)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&m->w3b, sizeof(__nv_bfloat16) * kMlpHidden * kMlpOutPad)) != cudaSuccess) return e;
    return cudaSuccess;
}

void mlp_free(MlpDev* m)
{
    void* p[] = {m->params, m->grad, m->m1, m->m2, m->w1b, m->w2b, m->w3b};
    for (void* q : p)
        if (q) cudaFree(q);
    *m = MlpDev{};
}

cudaError_t mlp_work_alloc(MlpWork* w, long long rows, bool training)
{
    *w = MlpWork{};
    w->rows = rows;
    const size_t r = (size_t)(rows > 0 ? rows : 1);
    cudaError_t e;
    if ((e = cudaMalloc(&w->z1, r * kMlpHidden * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&w->z2, r * kMlpHidden * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&w->h1, r * kMlpHidden * sizeof(__nv_bfloat16))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&w->h2, r * kMlpHidden * sizeof(__nv_bfloat16))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&w->y, r * kMlpOutPad * sizeof(float))) != cudaSuccess) return e;
    if (training) {
        if ((e = cudaMalloc(&w->dy, r * kMlpOutPad * sizeof(__nv_bfloat16))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->dh, r * kMlpHidden * sizeof(float))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->dz, r * kMlpHidden * sizeof(__nv_bfloat16))) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void mlp_work_free(MlpWork* w)
{
    void* p[] = {w->z1, w->z2, w->h1, w->h2, w->dy, w->dh, w->dz, w->y};
    for (void* q : p)
        if (q) cudaFree(q);
    *w = MlpWork{};
}

// Glorot-uniform weights, zero biases; the output layer is scaled by 0.1 so
// an untrained network predicts a guess close to the previous solution.
void mlp_init_params(float* w, unsigned seed)
{
    Xorshift rng(seed);
    const int fan[3][2] = {{kMlpIn, kMlpHidden}, {kMlpHidden, kMlpHidden}, {kMlpHidden, kMlpOut}};
    size_t off = 0;
    for (int l = 0; l < 3; ++l) {
        const float lim = std::sqrt(6.f / (float)(fan[l][0] + fan[l][1])) * (l == 2 ? 0.1f : 1.f);
        for (int i = 0; i < fan[l][0] * fan[l][1]; ++i) w[off++] = (2.f * rng.uniform() - 1.f) * lim;
        for (int i = 0; i < fan[l][1]; ++i) w[off++] = 0.f;
    }
}

}  // namespace pdgb

// ---- C ABI (no reference counterpart) --------------------------------------------------
namespace {

struct Session {
    cudaStream_t st = nullptr;
    pdgb::MlpDev m{};
    pdgb::MlpWork w{};
    __nv_bfloat16* X = nullptr;
    float* T = nullptr;
    float* Xf = nullptr;
    double* loss = nullptr;
    ~Session()
    {
        pdgb::mlp_work_free(&w);
        pdgb::mlp_free(&m);
        if (X) cudaFree(X);
        if (T) cudaFree(T);
        if (Xf) cudaFree(Xf);
        if (loss) cudaFree(loss);
        if (st) cudaStreamDestroy(st);
    }
};

pd_status mlp_fail(cudaError_t e)
{
    pdgb::set_handleless_error(std::string("mlp: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? PD_ERR_OUT_OF_MEMORY : PD_ERR_CUDA;
}

#define MLP_TRY(x)                                  \
    do {                                            \
        cudaError_t e_ = (x);                       \
        if (e_ != cudaSuccess) return mlp_fail(e_); \
    } while (0)

// uploads X (f32 -> BF16 on the device) and T
pd_status session_setup(Session& s, int device, const float* X, const float* T, long long rows, long long work_rows,
                        bool training, const float* params)
{
    MLP_TRY(cudaSetDevice(device));
    MLP_TRY(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    MLP_TRY(pdgb::mlp_alloc(&s.m, training));
    MLP_TRY(pdgb::mlp_work_alloc(&s.w, work_rows, training));
    const size_t nx = (size_t)rows * pdgb::kMlpIn;
    MLP_TRY(cudaMalloc(&s.X, (nx ? nx : 1) * sizeof(__nv_bfloat16)));
    MLP_TRY(cudaMalloc(&s.Xf, (nx ? nx : 1) * sizeof(float)));
    MLP_TRY(cudaMalloc(&s.T, ((size_t)rows * pdgb::kMlpOut + 1) * sizeof(float)));
    MLP_TRY(cudaMalloc(&s.loss, sizeof(double)));
    if (nx) MLP_TRY(cudaMemcpyAsync(s.Xf, X, nx * sizeof(float), cudaMemcpyHostToDevice, s.st));
    if (T && rows) MLP_TRY(cudaMemcpyAsync(s.T, T, (size_t)rows * pdgb::kMlpOut * sizeof(float), cudaMemcpyHostToDevice, s.st));
    if (nx) pdgb::k_f32_to_bf16<<<pdgb::blocks_for((long long)nx), 256, 0, s.st>>>(s.Xf, s.X, (long long)nx);
    MLP_TRY(cudaMemcpyAsync(s.m.params, params, pdgb::mlp_param_count() * sizeof(float), cudaMemcpyHostToDevice, s.st));
    pdgb::mlp_refresh_bf16(s.m, s.st);
    MLP_TRY(cudaGetLastError());
    return PD_OK;
}

}  // namespace

extern "C" size_t pd_mlp_param_count(void) { return pdgb::mlp_param_count(); }

extern "C" pd_status pd_mlp_init(unsigned seed, float* params)
{
    if (!params) return PD_ERR_INVALID_ARGUMENT;
    pdgb::mlp_init_params(params, seed);
    return PD_OK;
}

extern "C" pd_status pd_mlp_predict(int device, const float* X, long long rows, const float* params, float* Y)
{
    if (rows < 0 || (rows > 0 && (!X || !Y)) || !params) return PD_ERR_INVALID_ARGUMENT;
    Session s;
    const long long chunk = rows < 65536 ? (rows > 0 ? rows : 1) : 65536;
    pd_status st = session_setup(s, device, X, nullptr, rows, chunk, false, params);
    if (st != PD_OK) return st;
    std::vector<float> yb((size_t)chunk * pdgb::kMlpOutPad);
    for (long long r0 = 0; r0 < rows; r0 += chunk) {
        const int B = (int)std::min(chunk, rows - r0);
        MLP_TRY(pdgb::mlp_infer_tc(s.m, s.X + (size_t)r0 * pdgb::kMlpIn, B, s.w.y, s.st));
        MLP_TRY(cudaMemcpyAsync(yb.data(), s.w.y, (size_t)B * pdgb::kMlpOutPad * sizeof(float), cudaMemcpyDeviceToHost, s.st));
        MLP_TRY(cudaStreamSynchronize(s.st));
        if (pdgb::mlp_tc_take_error()) {
            pdgb::set_handleless_error("pd_mlp_predict: a tensor-core wait ran out of time");
            return PD_ERR_CUDA;
        }
        for (int i = 0; i < B; ++i)
            for (int c = 0; c < pdgb::kMlpOut; ++c) Y[(size_t)(r0 + i) * pdgb::kMlpOut + c] = yb[(size_t)i * pdgb::kMlpOutPad + c];
    }
    return PD_OK;
}

extern "C" pd_status pd_mlp_loss_grad(int device, const float* X, const float* T, int rows, const float* params,
                                      float* grad, double* loss)
{
    if (rows <= 0 || !X || !T || !params || !grad || !loss) return PD_ERR_INVALID_ARGUMENT;
    Session s;
    pd_status st = session_setup(s, device, X, T, rows, rows, true, params);
    if (st != PD_OK) return st;
    pdgb::mlp_forward(s.m, s.X, rows, s.w, s.w.y, s.st);
    MLP_TRY(cudaMemsetAsync(s.loss, 0, sizeof(double), s.st));
    pdgb::mlp_backward(s.m, s.X, s.T, rows, s.w, s.w.y, s.loss, s.st);
    MLP_TRY(cudaMemcpyAsync(grad, s.m.grad, pdgb::mlp_param_count() * sizeof(float), cudaMemcpyDeviceToHost, s.st));
    MLP_TRY(cudaMemcpyAsync(loss, s.loss, sizeof(double), cudaMemcpyDeviceToHost, s.st));
    MLP_TRY(cudaStreamSynchronize(s.st));
    MLP_TRY(cudaGetLastError());
    if (pdgb::mlp_tc_take_error()) {
        pdgb::set_handleless_error("pd_mlp_loss_grad: a tensor-core wait ran out of time");
        return PD_ERR_CUDA;
    }
    return PD_OK;
}

extern "C" pd_status pd_mlp_train(int device, const float* X, const float* T, long long rows, int iterations,
                                  int batch, float lr, unsigned seed, float* params, double* final_loss)
{
    if (rows <= 0 || !X || !T || !params || iterations < 0 || batch <= 0) return PD_ERR_INVALID_ARGUMENT;
    if (batch > rows) batch = (int)rows;
    Session s;
    pd_status st = session_setup(s, device, X, T, rows, std::max<long long>(batch, std::min<long long>(rows, 65536)),
                                 true, params);
    if (st != PD_OK) return st;
    __nv_bfloat16* Xb = nullptr;
    float* Tb = nullptr;
    int* idx = nullptr;
    struct Local {
        void *a, *b, *c;
        ~Local() { cudaFree(a); cudaFree(b); cudaFree(c); }
    } local{nullptr, nullptr, nullptr};
    MLP_TRY(cudaMalloc(&Xb, (size_t)batch * pdgb::kMlpIn * sizeof(__nv_bfloat16)));
    local.a = Xb;
    MLP_TRY(cudaMalloc(&Tb, (size_t)batch * pdgb::kMlpOut * sizeof(float)));
    local.b = Tb;
    MLP_TRY(cudaMalloc(&idx, (size_t)rows * sizeof(int)));
    local.c = idx;
    std::vector<int> perm((size_t)rows);
    for (long long i = 0; i < rows; ++i) perm[(size_t)i] = (int)i;
    pdgb::Xorshift rng(seed);
    long long cursor = rows;   // forces a shuffle first
    for (int it = 1; it <= iterations; ++it) {
        if (cursor + batch > rows) {
            for (long long i = rows - 1; i > 0; --i) std::swap(perm[(size_t)i], perm[(size_t)(rng.next() % (uint64_t)(i + 1))]);
            MLP_TRY(cudaMemcpyAsync(idx, perm.data(), (size_t)rows * sizeof(int), cudaMemcpyHostToDevice, s.st));
            MLP_TRY(cudaStreamSynchronize(s.st));
            cursor = 0;
        }
        pdgb::k_gather_rows<<<pdgb::blocks_for((long long)batch * pdgb::kMlpIn), 256, 0, s.st>>>(s.X, s.T, idx + cursor,
                                                                                                  batch, Xb, Tb);
        cursor += batch;
        pdgb::mlp_forward(s.m, Xb, batch, s.w, s.w.y, s.st);
        pdgb::mlp_backward(s.m, Xb, Tb, batch, s.w, s.w.y, s.loss, s.st);
        pdgb::mlp_adam(s.m, lr, it, s.st);
    }
    // loss over the whole dataset
    MLP_TRY(cudaMemsetAsync(s.loss, 0, sizeof(double), s.st));
    double total = 0.0;
    const long long chunk = s.w.rows;
    for (long long r0 = 0; r0 < rows; r0 += chunk) {
        const int B = (int)std::min(chunk, rows - r0);
        pdgb::mlp_forward(s.m, s.X + (size_t)r0 * pdgb::kMlpIn, B, s.w, s.w.y, s.st);
        MLP_TRY(cudaMemsetAsync(s.loss, 0, sizeof(double), s.st));
        pdgb::mlp_backward(s.m, s.X + (size_t)r0 * pdgb::kMlpIn, s.T + (size_t)r0 * pdgb::kMlpOut, B, s.w, s.w.y, s.loss,
                           s.st);
        double l = 0.0;
        MLP_TRY(cudaMemcpyAsync(&l, s.loss, sizeof(double), cudaMemcpyDeviceToHost, s.st));
        MLP_TRY(cudaStreamSynchronize(s.st));
        total += l * B;
    }
    if (final_loss) *final_loss = total / (double)rows;
    MLP_TRY(cudaMemcpyAsync(params, s.m.params, pdgb::mlp_param_count() * sizeof(float), cudaMemcpyDeviceToHost, s.st));
    MLP_TRY(cudaStreamSynchronize(s.st));
    MLP_TRY(cudaGetLastError());
    if (pdgb::mlp_tc_take_error()) {
        pdgb::set_handleless_error("pd_mlp_train: a tensor-core wait ran out of time");
        return PD_ERR_CUDA;
    }
    return PD_OK;
}
