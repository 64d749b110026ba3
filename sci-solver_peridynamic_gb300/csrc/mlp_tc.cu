// mlp_tc.cu -- inference of the learned warm start's network on the
// 5th-generation tensor cores (tcgen05), all three layers in one kernel.
//
// No reference counterpart.  The network (64 -> 128 -> 128 -> 3, GELU, BF16
// weights and activations, FP32 accumulation) is the one mlp.cu trains; this
// kernel runs it over every particle row of a step.  Per 128-row tile:
//   features (BF16, global) -> shared memory by TMA   (128-byte swizzle; the
//                              next tile's copy is issued as soon as layer 1
//                              has read this one, and overlaps the rest)
//   layer 1  tcgen05.mma  X[128x64]  W1^T -> TMEM columns   0..127 (FP32)
//   epilogue tcgen05.ld, + b1, GELU, BF16 -> shared memory H
//   layer 2  tcgen05.mma  H[128x128] W2^T -> TMEM columns 128..255
//   epilogue tcgen05.ld, + b2, GELU, BF16 -> H
//   layer 3  tcgen05.mma  H[128x128] W3^T (3 outputs padded to N = 16) -> TMEM 0..15
//   epilogue tcgen05.ld, + b3 -> Y (FP32, 8 columns per row, 3 used)
// One thread issues the MMAs; their completion arrives on an mbarrier
// (tcgen05.commit) that the whole block waits on.  Every wait is bounded in
// time: on expiry the kernel records an error, waits once more (bounded) for
// its MMAs in flight, frees its tensor memory and returns, leaving the rows it
// did not reach as they were.  The weights stay in shared memory for the
// CTA's whole run over its tiles; two CTAs share an SM (about 102 KB of
// shared memory and 256 TMEM columns each).
//
// Shared-memory operands: the feature tile as TMA writes it with the 128-byte
// swizzle (row r at r * 128 bytes, its 16-byte chunk c at chunk c ^ (r % 8);
// descriptor layout SWIZZLE_128B, 8-row groups 1024 bytes apart, an MMA's
// K = 16 slice 32 bytes further).  Weights and hidden activations, written by
// threads: SWIZZLE_NONE, K-major.  An R x K tile is a
// grid of 8 x 8 core matrices (8 rows of 16 bytes, 128 contiguous bytes);
// core (r/8, k/8) starts at ((r/8) * K/8 + k/8) * 128 bytes.  So the
// descriptors' leading-dimension byte offset (next core matrix along K) is
// 128 and the stride-dimension byte offset (next 8-row group) is K * 16; one
// MMA (K = 16) covers two core matrices along K, the next one starts 256
// bytes further.  Every byte an MMA reads lies inside its operand tile.
#include <cuda.h>   // CUtensorMap and its encoder's signature (called through the runtime's entry point)
#include <cuda_bf16.h>

#include <cstdint>
#include <mutex>

#include "pd_device.cuh"
#include "pd_kernels.h"

namespace pdgb {

namespace {

constexpr int kTcRows = 128;       // rows per tile = MMA M
constexpr int kTcThreads = 256;
constexpr uint32_t kTmemCols = 256;
constexpr int kOutN = 16;          // layer-3 MMA N
constexpr unsigned long long kTcWaitNs = 1000000000ull;   // 1 s per wait
constexpr int kMaxDevices = 64;

constexpr int kOffW1 = 0;                                  // W1^T: 128 x 64
constexpr int kOffW2 = kOffW1 + kMlpHidden * kMlpIn * 2;   // W2^T: 128 x 128
constexpr int kOffW3 = kOffW2 + kMlpHidden * kMlpHidden * 2;   // W3^T: 16 x 128
constexpr int kOffX = kOffW3 + kOutN * kMlpHidden * 2;     // features: 128 x 64
constexpr int kOffH = kOffX + kTcRows * kMlpIn * 2;        // hidden: 128 x 128
constexpr int kOffB = kOffH + kTcRows * kMlpHidden * 2;    // biases (f32): 128 + 128 + 16
constexpr int kOffBar = kOffB + (2 * kMlpHidden + kOutN) * 4;   // MMA mbarrier, TMA mbarrier, TMEM address
constexpr int kSmemUsed = kOffBar + 24;
constexpr uint32_t kTileBytes = kTcRows * kMlpIn * 2;      // one feature tile (16 KB)
static_assert(kOffX % 1024 == 0, "the swizzled feature tile needs 1024-byte alignment");
constexpr int kSmemBytes = kSmemUsed + 1024;               // + alignment of the base to 1024 B

__device__ int g_tc_error;   // 1: an mbarrier wait of the tensor-core kernel ran out of time

__device__ __forceinline__ uint32_t core_off(int r, int k, int K)
{
    return (uint32_t)(((((r >> 3) * (K >> 3)) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// shared-memory matrix descriptor: start, leading / stride byte offsets,
// descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// the same for the TMA-written feature tile: 128-byte swizzle (bits 61-63 =
// 2), 8-row groups 1024 bytes apart; the leading offset is not used by this
// layout (K of one MMA stays inside the 128-byte swizzle span)
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

// TMA: the 64 x 128 box at (0, row0) of the feature matrix into shared
// memory, completing on bar (whose expected bytes are set just before)
__device__ __forceinline__ void tma_load_tile(const CUtensorMap* tmap, uint32_t dst, uint32_t bar, int row0)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTileBytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"((uint64_t)tmap), "r"(0), "r"(row0), "r"(bar)
        : "memory");
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit
// 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t instr_desc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ unsigned long long now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const unsigned long long t0 = now_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (now_ns() - t0 > kTcWaitNs) return false;
    }
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// block barrier that orders tensor-core operations and generic shared-memory
// writes on both sides; returns the AND of every thread's ok
__device__ __forceinline__ bool tc_sync(bool ok)
{
    proxy_fence();
    tc_fence_before();
    const int all = __syncthreads_and(ok ? 1 : 0);
    tc_fence_after();
    return all != 0;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu_tc(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// hidden-layer epilogue: TMEM columns [col0, col0 + 128) of this warp's 32
// rows (quadrant w % 4), column half w / 4 -> + bias, GELU, BF16 into H
__device__ __forceinline__ void epilogue_hidden(uint32_t tmem, uint32_t col0, const float* bias, unsigned char* H,
                                                int warp, int lane)
{
    const int q = warp & 3, half = warp >> 2;
    const int row = 32 * q + lane;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int c0 = 64 * half + 32 * j;
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + col0 + (uint32_t)c0, v);
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            uint4 w;
            uint32_t* wp = reinterpret_cast<uint32_t*>(&w);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int i = 8 * g + 2 * e;
                wp[e] = pack2(gelu_tc(v[i] + bias[c0 + i]), gelu_tc(v[i + 1] + bias[c0 + i + 1]));
            }
            *reinterpret_cast<uint4*>(H + core_off(row, c0 + 8 * g, kMlpHidden)) = w;
        }
    }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_mlp_infer_tc(const __grid_constant__ CUtensorMap tmap_x, int B, const __nv_bfloat16* __restrict__ w1b,
                   const __nv_bfloat16* __restrict__ w2b, const __nv_bfloat16* __restrict__ w3b,
                   const float* __restrict__ b1, const float* __restrict__ b2, const float* __restrict__ b3,
                   float* __restrict__ Y)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float* sb1 = reinterpret_cast<float*>(sm + kOffB);
    float* sb2 = sb1 + kMlpHidden;
    float* sb3 = sb2 + kMlpHidden;
    const uint32_t bar = sbase + kOffBar;
    const uint32_t bar_x = sbase + kOffBar + 8;
    const uint32_t tmem_slot = sbase + kOffBar + 16;

    // weights as K-major B operands (row n of W^T = column n of W) and biases
    for (int i = tid; i < kMlpIn * kMlpHidden; i += blockDim.x) {
        const int k = i / kMlpHidden, n = i % kMlpHidden;
        *reinterpret_cast<__nv_bfloat16*>(sm + kOffW1 + core_off(n, k, kMlpIn)) = w1b[i];
    }
    for (int i = tid; i < kMlpHidden * kMlpHidden; i += blockDim.x) {
        const int k = i / kMlpHidden, n = i % kMlpHidden;
        *reinterpret_cast<__nv_bfloat16*>(sm + kOffW2 + core_off(n, k, kMlpHidden)) = w2b[i];
    }
    for (int i = tid; i < kOutN * kMlpHidden; i += blockDim.x) {
        const int n = i / kMlpHidden, k = i % kMlpHidden;
        const __nv_bfloat16 w = n < kMlpOut ? w3b[k * kMlpOutPad + n] : __float2bfloat16_rn(0.f);
        *reinterpret_cast<__nv_bfloat16*>(sm + kOffW3 + core_off(n, k, kMlpHidden)) = w;
    }
    for (int i = tid; i < kMlpHidden; i += blockDim.x) {
        sb1[i] = b1[i];
        sb2[i] = b2[i];
    }
    if (tid < kOutN) sb3[tid] = tid < kMlpOut ? b3[tid] : 0.f;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_x) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tmem_slot),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bool ok = tc_sync(true);
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + kOffBar + 16);
    uint32_t parity = 0, parity_x = 0;
    bool pending = false;     // an MMA group was committed and not yet waited for
    bool pending_x = false;   // a feature tile copy was issued and not yet waited for
    const int tiles0 = (B + kTcRows - 1) / kTcRows;
    if (tid == 0 && (int)blockIdx.x < tiles0) tma_load_tile(&tmap_x, sbase + kOffX, bar_x, (int)blockIdx.x * kTcRows);
    pending_x = (int)blockIdx.x < tiles0;

    constexpr uint32_t id_hidden = instr_desc(kTcRows, kMlpHidden);
    constexpr uint32_t id_out = instr_desc(kTcRows, kOutN);
    constexpr uint32_t lbo = 128;                    // next core matrix along K
    constexpr uint32_t sbo_k64 = kMlpIn * 16;        // next 8-row group, K = 64
    constexpr uint32_t sbo_k128 = kMlpHidden * 16;   // next 8-row group, K = 128
    const int tiles = (B + kTcRows - 1) / kTcRows;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const int row0 = t * kTcRows;
        // this tile's features (rows past B arrive as zeros)
        ok = mbar_wait(bar_x, parity_x);
        if (ok) { parity_x ^= 1u; pending_x = false; }
        ok = tc_sync(ok);
        if (!ok) break;
        // layer 1
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kMlpIn / 16; ++s)
                mma_bf16(tmem, smem_desc_sw128(sbase + kOffX + 32 * s),
                         smem_desc(sbase + kOffW1 + 2 * s * lbo, lbo, sbo_k64), id_hidden, s > 0);
            mma_commit(bar);
        }
        pending = true;
        ok = mbar_wait(bar, parity);
        if (ok) { parity ^= 1u; pending = false; }
        ok = tc_sync(ok);
        if (!ok) break;
        // layer 1 has read the feature tile: the next tile's copy overlaps the rest
        if (t + (int)gridDim.x < tiles) {
            if (tid == 0) tma_load_tile(&tmap_x, sbase + kOffX, bar_x, (t + (int)gridDim.x) * kTcRows);
            pending_x = true;
        }
        epilogue_hidden(tmem, 0, sb1, sm + kOffH, warp, lane);
        ok = tc_sync(ok);
        // layer 2
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kMlpHidden / 16; ++s)
                mma_bf16(tmem + kMlpHidden, smem_desc(sbase + kOffH + 2 * s * lbo, lbo, sbo_k128),
                         smem_desc(sbase + kOffW2 + 2 * s * lbo, lbo, sbo_k128), id_hidden, s > 0);
            mma_commit(bar);
        }
        pending = true;
        ok = mbar_wait(bar, parity);
        if (ok) { parity ^= 1u; pending = false; }
        ok = tc_sync(ok);
        if (!ok) break;
        epilogue_hidden(tmem, kMlpHidden, sb2, sm + kOffH, warp, lane);
        ok = tc_sync(ok);
        // layer 3 (accumulator in columns 0..15: layer 1's were read above)
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kMlpHidden / 16; ++s)
                mma_bf16(tmem, smem_desc(sbase + kOffH + 2 * s * lbo, lbo, sbo_k128),
                         smem_desc(sbase + kOffW3 + 2 * s * lbo, lbo, sbo_k128), id_out, s > 0);
            mma_commit(bar);
        }
        pending = true;
        ok = mbar_wait(bar, parity);
        if (ok) { parity ^= 1u; pending = false; }
        ok = tc_sync(ok);
        if (!ok) break;
        if (warp < 4) {
            const int row = 32 * warp + lane;
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
            if (row0 + row < B) {
                float4* y = reinterpret_cast<float4*>(Y + (size_t)(row0 + row) * kMlpOutPad);
                y[0] = make_float4(v[0] + sb3[0], v[1] + sb3[1], v[2] + sb3[2], v[3] + sb3[3]);
                y[1] = make_float4(v[4] + sb3[4], v[5] + sb3[5], v[6] + sb3[6], v[7] + sb3[7]);
            }
        }
        ok = tc_sync(ok);
    }
    if (!ok) {
        if (tid == 0) atomicExch(&g_tc_error, 1);
        if (pending) mbar_wait(bar, parity);       // the MMAs in flight, once more (bounded)
        if (pending_x) mbar_wait(bar_x, parity_x);   // and a feature copy in flight
    }
    tc_sync(true);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---- general GEMM of the training passes ----------------------------------------------
// C[M x N] (FP32, row-major, ldc) = op(A)[M x K] op(B)[K x N] (+ C), BF16
// operands; op(P) is P (row-major) or, with TA / TB, its transpose.  One CTA
// per 128 x 128 tile of C: K in slabs of 64, each slab's operands written by
// the threads into K-major core-matrix tiles (transposing where asked), four
// tcgen05.mma (K = 16) accumulating in TMEM, then the epilogue.
constexpr int kGemmSlab = 64;
constexpr int kGemmOffA = 0;                                   // 128 x 64
constexpr int kGemmOffB = kGemmOffA + 128 * kGemmSlab * 2;     // 128 x 64
constexpr int kGemmOffBar = kGemmOffB + 128 * kGemmSlab * 2;   // mbarrier, TMEM address
// requested shared memory: limits residency to 3 CTAs per SM (3 x 128 TMEM columns)
constexpr int kGemmSmemBytes = 58 * 1024;

template <bool TA, bool TB>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_gemm_tc(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda, const __nv_bfloat16* __restrict__ B,
              int ldb, float* __restrict__ C, int ldc, int accumulate)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * 128;
    const int nt = (N - n0 < 128 ? N - n0 : 128);
    const int nmma = (nt + 15) & ~15;   // MMA N: a multiple of 16
    const uint32_t bar = sbase + kGemmOffBar;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + kGemmOffBar + 8),
                     "r"(128u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bool ok = tc_sync(true);
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + kGemmOffBar + 8);
    const uint32_t idesc = instr_desc(128, nmma);
    uint32_t parity = 0;
    bool pending = false;
    for (int k0 = 0; k0 < K && ok; k0 += kGemmSlab) {
        // op(A) rows m0.., columns k0..: consecutive threads walk the
        // contiguous direction of A in memory
        for (int i = tid; i < 128 * kGemmSlab; i += blockDim.x) {
            const int m = TA ? (i & 127) : (i >> 6), kk = TA ? (i >> 7) : (i & 63);
            const int gm = m0 + m, gk = k0 + kk;
            __nv_bfloat16 v = __float2bfloat16_rn(0.f);
            if (gm < M && gk < K) v = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
            *reinterpret_cast<__nv_bfloat16*>(sm + kGemmOffA + core_off(m, kk, kGemmSlab)) = v;
        }
        // the B operand is op(B)^T: row n holds op(B)[k0.., n0 + n]
        for (int i = tid; i < 128 * kGemmSlab; i += blockDim.x) {
            const int n = TB ? (i >> 6) : (i & 127), kk = TB ? (i & 63) : (i >> 7);
            const int gn = n0 + n, gk = k0 + kk;
            __nv_bfloat16 v = __float2bfloat16_rn(0.f);
            if (gn < N && gk < K) v = TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
            *reinterpret_cast<__nv_bfloat16*>(sm + kGemmOffB + core_off(n, kk, kGemmSlab)) = v;
        }
        ok = tc_sync(ok);
        if (!ok) break;
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kGemmSlab / 16; ++s)
                mma_bf16(tmem, smem_desc(sbase + kGemmOffA + 256 * s, 128, kGemmSlab * 16),
                         smem_desc(sbase + kGemmOffB + 256 * s, 128, kGemmSlab * 16), idesc, (k0 > 0 || s > 0) ? 1u : 0u);
            mma_commit(bar);
        }
        pending = true;
        ok = mbar_wait(bar, parity);
        if (ok) { parity ^= 1u; pending = false; }
        ok = tc_sync(ok);
    }
    if (ok && warp < 4) {
        const int row = 32 * warp + lane, gm = m0 + row;
        for (int c0 = 0; c0 < nmma; c0 += 16) {
            float v[16];
            if (K > 0) tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            else
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            if (gm < M)
                for (int i = 0; i < 16; ++i) {
                    const int gn = n0 + c0 + i;
                    if (gn >= N) break;
                    float* dst = C + (size_t)gm * ldc + gn;
                    *dst = accumulate ? *dst + v[i] : v[i];
                }
        }
    }
    if (!ok) {
        if (tid == 0) atomicExch(&g_tc_error, 1);
        if (pending) mbar_wait(bar, parity);
    }
    tc_sync(true);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u) : "memory");
}

}  // namespace

template <bool TA, bool TB>
static cudaError_t gemm_tc_t(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb,
                             float* C, int ldc, bool accumulate, cudaStream_t st)
{
    static std::mutex mtx;
    static bool configured[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(mtx);
        if (!configured[dev]) {
            e = cudaFuncSetAttribute(k_gemm_tc<TA, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmemBytes);
            if (e != cudaSuccess) return e;
            configured[dev] = true;
        }
    }
    const dim3 grid((unsigned)((M + 127) / 128), (unsigned)((N + 127) / 128));
    k_gemm_tc<TA, TB><<<grid, kTcThreads, kGemmSmemBytes, st>>>(M, N, K, A, lda, B, ldb, C, ldc, accumulate ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t gemm_tc(bool ta, bool tb, int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B,
                    int ldb, float* C, int ldc, bool accumulate, cudaStream_t st)
{
    if (M <= 0 || N <= 0) return cudaSuccess;
    if (!ta && !tb) return gemm_tc_t<false, false>(M, N, K, A, lda, B, ldb, C, ldc, accumulate, st);
    if (ta && !tb) return gemm_tc_t<true, false>(M, N, K, A, lda, B, ldb, C, ldc, accumulate, st);
    if (!ta && tb) return gemm_tc_t<false, true>(M, N, K, A, lda, B, ldb, C, ldc, accumulate, st);
    return gemm_tc_t<true, true>(M, N, K, A, lda, B, ldb, C, ldc, accumulate, st);
}

// Y[B x kMlpOutPad] (columns 0..2 used) = network(X[B x 64]) on the tensor
// cores.  Launch errors are returned; a wait that ran out of time is reported
// by mlp_tc_take_error.
cudaError_t mlp_infer_tc(const MlpDev& m, const __nv_bfloat16* X, int B, float* Y, cudaStream_t st)
{
    if (B <= 0) return cudaSuccess;
    // once per device (the shared-memory opt-in is a per-device attribute);
    // the tensor-map encoder comes from the driver through the runtime
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static std::mutex mtx;
    static int sm_counts[kMaxDevices] = {};
    static EncodeFn encode_fn = nullptr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    int sm_count = 0;
    {
        std::lock_guard<std::mutex> lock(mtx);
        if (sm_counts[dev] == 0) {
            e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
            if (e != cudaSuccess) return e;
            int n = 0;
            e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            sm_counts[dev] = n;
        }
        sm_count = sm_counts[dev];
        if (!encode_fn) {
            void* fn = nullptr;
            cudaDriverEntryPointQueryResult q;
            e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
            if (e != cudaSuccess) return e;
            if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
            encode_fn = (EncodeFn)fn;
        }
    }
    const EncodeFn encode = encode_fn;
    // the feature matrix as a TMA tensor: 64 BF16 columns x B rows, boxes of
    // 64 x 128 with the 128-byte swizzle; rows past B read as zeros
    if (((uintptr_t)X & 15u) != 0) return cudaErrorInvalidValue;
    CUtensorMap tmap;
    {
        const cuuint64_t dims[2] = {(cuuint64_t)kMlpIn, (cuuint64_t)B};
        const cuuint64_t strides[1] = {(cuuint64_t)kMlpIn * sizeof(__nv_bfloat16)};
        const cuuint32_t box[2] = {(cuuint32_t)kMlpIn, (cuuint32_t)kTcRows};
        const cuuint32_t estr[2] = {1u, 1u};
        const CUresult r = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)X, dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    }
    const float* b1 = m.params + kMlpIn * kMlpHidden;
    const float* b2 = b1 + kMlpHidden + kMlpHidden * kMlpHidden;
    const float* b3 = b2 + kMlpHidden + kMlpHidden * kMlpOut;
    const int tiles = (B + kTcRows - 1) / kTcRows;
    const int grid = tiles < 2 * sm_count ? tiles : 2 * sm_count;
    k_mlp_infer_tc<<<grid, kTcThreads, kSmemBytes, st>>>(tmap, B, m.w1b, m.w2b, m.w3b, b1, b2, b3, Y);
    return cudaGetLastError();
}

// 1 if a tensor-core wait ran out of time since the last call (and clears it)
int mlp_tc_take_error()
{
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    if (v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
    }
    return v;
}

}  // namespace pdgb
