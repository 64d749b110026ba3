// tiles.cu -- the shared-memory tile SpMV of the mixed-precision operator.
//
// Rows (particles in Morton cell order) are grouped into tiles of tile_rows
// consecutive rows.  A tile occupies a compact region, so the distinct
// neighbours of all its rows -- its halo -- number only a few times the
// tile's rows (about 4.5x for 256 rows at 75 bonds per particle), while the
// tile has ~75 bonds per row.  The SpMV stages each halo entry's position
// (made relative to the tile's reference supercell, so the bond vector needs
// no per-bond decode) and its input-vector entry in shared memory once, then
// every bond reads both from shared memory through a 16-bit local index.
// Per bond the kernel streams 6 bytes (local index + 1/d0) instead of
// gathering 32 bytes from L1/L2.
//
// Built once per make_ready (bonds are never added; a broken bond only moves
// within its row, and its local index moves with it).
#include <vector>

#include "pd_device.cuh"
#include "pd_kernels.h"
#include "step_rows.cuh"

namespace pdgb {

namespace {

constexpr int kHashCap = 4096;                    // per-tile hash set of neighbour slots
constexpr int kHashLimit = (kHashCap * 3) / 4;    // larger halos use the global path
constexpr unsigned kEmpty = 0xffffffffu;

__device__ __forceinline__ unsigned hash_slot(unsigned q) { return (q * 2654435761u) >> (32 - 12); }

// Inserts the neighbour slots of rows [r0, r1) into the shared hash set;
// returns the number of distinct slots (kHashCap + 1 when the set is full).
__device__ int tile_collect(const DeviceState& S, int r0, int r1, unsigned* table)
{
    __shared__ int s_count;
    for (int i = threadIdx.x; i < kHashCap; i += blockDim.x) table[i] = kEmpty;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int p = r0 + warp; p < r1; p += nw) {
        const int rs = S.row_ptr[p], cn = S.cnt[p];
        for (int j = lane; j < cn; j += 32) {
            const unsigned q = (unsigned)S.col[rs + j];
            unsigned h = hash_slot(q);
            int probe = 0;
            for (; probe < kHashCap; ++probe) {
                const unsigned old = atomicCAS(&table[h], kEmpty, q);
                if (old == kEmpty) {
                    atomicAdd(&s_count, 1);
                    break;
                }
                if (old == q) break;
                h = (h + 1) & (kHashCap - 1);
            }
            if (probe == kHashCap) atomicExch(&s_count, kHashCap + 1);
        }
    }
    __syncthreads();
    const int c = s_count;
    __syncthreads();
    return c;
}

// Ascending bitonic sort of the kHashCap-entry table (empty = largest).
__device__ void sort_table(unsigned* t)
{
    for (int k = 2; k <= kHashCap; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < kHashCap; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned a = t[i], b = t[l];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        t[i] = b;
                        t[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_tile_count(DeviceState S, int n, unsigned* counts)
{
    __shared__ unsigned table[kHashCap];
    for (int t = blockIdx.x; t < S.n_tiles; t += gridDim.x) {
        const int r0 = t * S.tile_rows, r1 = min(n, r0 + S.tile_rows);
        const int c = tile_collect(S, r0, r1, table);
        if (threadIdx.x == 0) {
            const bool fits = c <= kHashLimit;
            S.tile_info[t] = fits ? c : -1;
            counts[t] = fits ? (unsigned)c : 0u;
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_tile_fill(DeviceState S, int n)
{
    __shared__ unsigned table[kHashCap];
    for (int t = blockIdx.x; t < S.n_tiles; t += gridDim.x) {
        const int info = S.tile_info[t];   // block-uniform
        if (info < 0) continue;
        const int r0 = t * S.tile_rows, r1 = min(n, r0 + S.tile_rows);
        tile_collect(S, r0, r1, table);
        sort_table(table);
        const int h0 = S.halo_ptr[t];
        for (int e = threadIdx.x; e < info; e += blockDim.x) S.halo[h0 + e] = (int)table[e];
        // local index of every bond: binary search in the sorted halo
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int p = r0 + warp; p < r1; p += nw) {
            const int rs = S.row_ptr[p], cn = S.cnt[p];
            for (int j = lane; j < cn; j += 32) {
                const unsigned q = (unsigned)S.col[rs + j];
                int lo = 0, hi = info - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (table[mid] < q) lo = mid + 1;
                    else hi = mid;
                }
                S.lidx[rs + j] = (uint16_t)lo;
            }
        }
        __syncthreads();
    }
}

// ---- the tile SpMV ------------------------------------------------------------------
template <int G, int U, bool DOT>
__device__ __forceinline__ void tile_row(const StepParams& P, const DeviceState& S, const float4* __restrict__ in,
                                         float4* __restrict__ out, const float4* sp, const float4* sw, int wref,
                                         int p, int lane, unsigned gmask, DotAcc32& acc)
{
    const uint8_t ab = S.act[p];
    if (is_dirichlet(ab & kActMask)) {
        if (lane == 0) out[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 w = __ldg(in + p);
    const float4 X = __ldg(S.xs4 + p);
    float dx, dy, dz;
    supercell_delta(__float_as_int(X.w), wref, (float)P.sup, dx, dy, dz);
    const float px = X.x + dx, py = X.y + dy, pz = X.z + dz;
    const int rs = S.row_ptr[p];
    const int cn = S.cnt[p];
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int j0 = lane; j0 < cn; j0 += G * U) {
        int e[U];
        float id0[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = j0 + u * G;
            e[u] = j < cn ? (int)__ldcs(S.lidx + rs + j) : -1;
            id0[u] = j < cn ? __ldcs(S.inv_d0 + rs + j) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e[u] < 0) continue;
            const float4 Xq = sp[e[u]];
            const float4 Wq = sw[e[u]];
            const float xs = Xq.x - px, ys = Xq.y - py, zs = Xq.z - pz;
            const float inv_d = rsqrtf(fmaf(xs, xs, fmaf(ys, ys, zs * zs)));
            const float wx = w.x - Wq.x, wy = w.y - Wq.y, wz = w.z - Wq.z;
            const float a1 = id0[u] - inv_d;
            const float g = fmaf(xs, wx, fmaf(ys, wy, zs * wz)) * (inv_d * inv_d * inv_d);
            ax = fmaf(a1, wx, fmaf(g, xs, ax));
            ay = fmaf(a1, wy, fmaf(g, ys, ay));
            az = fmaf(a1, wz, fmaf(g, zs, az));
        }
    }
    spmv_finish_mixed<G, DOT>(P, S, p, ab, w, ax, ay, az, lane, gmask, out, acc);
}

// Tiles are taken in any order (an atomic counter); each tile's rows are
// computed by one block with a fixed thread mapping and its <w, A w> partial
// is stored per tile, so results do not depend on the order.  The last block
// to finish resets the counters and, with DOT, sums the tile partials in
// tile order.
template <int G, int U, bool DOT>
__global__ void __launch_bounds__(kBlock) k_spmv_tile(StepParams P, DeviceState S, const float4* __restrict__ in,
                                                      float4* __restrict__ out, CgScalars* cg, double* dot_out)
{
    if (DOT && cg && ((volatile CgScalars*)cg)->done) return;
    extern __shared__ float4 smem[];
    float4* sp = smem;
    float4* sw = smem + S.halo_cap;
    __shared__ int s_tile;
    __shared__ double warp_sums[kBlock / 32];
    __shared__ bool is_last;
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    const float sup = (float)P.sup;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(S.tile_ctr, 1u);
        __syncthreads();
        const int t = s_tile;
        if (t >= S.n_tiles) break;
        const int r0 = t * S.tile_rows, r1 = min(P.n, r0 + S.tile_rows);
        const int h0 = S.halo_ptr[t];
        const int hn = S.halo_ptr[t + 1] - h0;
        const bool staged = S.tile_info[t] >= 0 && hn <= S.halo_cap;
        DotAcc32 acc;
        if (staged) {
            const int wref = __float_as_int(__ldg(S.xs4 + r0).w);
            for (int e = threadIdx.x; e < hn; e += blockDim.x) {
                const int q = __ldg(S.halo + h0 + e);
                const float4 X = __ldg(S.xs4 + q);
                float dx, dy, dz;
                supercell_delta(__float_as_int(X.w), wref, sup, dx, dy, dz);
                sp[e] = make_float4(X.x + dx, X.y + dy, X.z + dz, 0.f);
                sw[e] = __ldg(in + q);
            }
            __syncthreads();
            for (int p0 = r0; p0 < r1; p0 += gpb) {
                const int p = p0 + threadIdx.x / G;
                if (p < r1) tile_row<G, U, DOT>(P, S, in, out, sp, sw, wref, p, lane, gmask, acc);
            }
        } else {
            for (int p0 = r0; p0 < r1; p0 += gpb) {
                const int p = p0 + threadIdx.x / G;
                if (p < r1) spmv_row<G, false, DOT, U, kLdReadOnly>(P, S, in, out, p, lane, gmask, acc);
            }
        }
        if (DOT) {
            const double w = warp_total(acc);
            if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = w;
            __syncthreads();
            if (threadIdx.x == 0) {
                double tsum = 0.0;
                for (int i = 0; i < kBlock / 32; ++i) tsum += warp_sums[i];
                S.tile_partials[t] = tsum;
            }
        }
        __syncthreads();   // shared halo and s_tile are rewritten for the next tile
    }
    // arrival; the last block resets the counters and finishes the reduction
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(S.tile_ctr + 1, 1u);
        is_last = prev == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    if (DOT) {
        double v = 0.0;
        for (int i = threadIdx.x; i < S.n_tiles; i += blockDim.x) v += __ldcg(S.tile_partials + i);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = v;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        S.tile_ctr[0] = 0u;
        S.tile_ctr[1] = 0u;
        if (DOT) {
            double total = 0.0;
            for (int i = 0; i < kBlock / 32; ++i) total += warp_sums[i];
            if (cg) cg_fin_alpha(cg, total);
            if (dot_out) *dot_out = total;
        }
    }
}

template <int G, int U>
void tile_launch(bool dot, const StepParams& P, const DeviceState& S, int grid, cudaStream_t st)
{
    const size_t smem = sizeof(float4) * 2 * (size_t)S.halo_cap;
    if (dot) k_spmv_tile<G, U, true><<<grid, kBlock, smem, st>>>(P, S, (const float4*)S.p, (float4*)S.y, S.sc, nullptr);
    else k_spmv_tile<G, U, false><<<grid, kBlock, smem, st>>>(P, S, (const float4*)S.sol, (float4*)S.y, nullptr, nullptr);
}

template <int G, int U>
int tile_blocks(int halo_cap)
{
    const size_t smem = sizeof(float4) * 2 * (size_t)halo_cap;
    cudaFuncSetAttribute(k_spmv_tile<G, U, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_spmv_tile<G, U, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_spmv_tile<G, U, true>, kBlock, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_spmv_tile<G, U, false>, kBlock, smem);
    return a < b ? a : b;
}

}  // namespace

cudaError_t build_tiles(DeviceState& S, int n, int* max_halo, cudaStream_t st)
{
    free_tiles(S);
    *max_halo = 0;
    if (n <= 0 || S.tile_rows <= 0) return cudaSuccess;
    S.n_tiles = (n + S.tile_rows - 1) / S.tile_rows;
    const size_t nt = (size_t)S.n_tiles;
    unsigned* counts = nullptr;
    cudaError_t e = cudaMalloc((void**)&counts, sizeof(unsigned) * (nt + 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&S.tile_info, sizeof(int) * nt);
    if (e == cudaSuccess) e = cudaMalloc((void**)&S.halo_ptr, sizeof(int) * (nt + 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&S.tile_partials, sizeof(double) * nt);
    if (e == cudaSuccess) e = cudaMalloc((void**)&S.tile_ctr, sizeof(unsigned) * 2);
    if (e == cudaSuccess) e = cudaMemsetAsync(S.tile_ctr, 0, sizeof(unsigned) * 2, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(unsigned) * (nt + 1), st);
    const int grid = (int)(nt < 4096 ? nt : 4096);
    if (e == cudaSuccess) {
        k_tile_count<<<grid, kBlock, 0, st>>>(S, n, counts);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = scan_exclusive_u32(counts, (unsigned*)S.halo_ptr, (long long)nt + 1, st);
    int total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, S.halo_ptr + nt, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMalloc((void**)&S.halo, sizeof(int) * (size_t)(total > 0 ? total : 1));
    if (e == cudaSuccess) {
        k_tile_fill<<<grid, kBlock, 0, st>>>(S, n);
        e = cudaGetLastError();
    }
    std::vector<int> info(nt);
    if (e == cudaSuccess) e = cudaMemcpyAsync(info.data(), S.tile_info, sizeof(int) * nt, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(counts);
    if (e != cudaSuccess) return e;
    for (int v : info) *max_halo = v > *max_halo ? v : *max_halo;
    return cudaSuccess;
}

void free_tiles(DeviceState& S)
{
    cudaFree(S.halo);
    cudaFree(S.halo_ptr);
    cudaFree(S.tile_info);
    cudaFree(S.tile_partials);
    cudaFree(S.tile_ctr);
    S.halo = nullptr;
    S.halo_ptr = nullptr;
    S.tile_info = nullptr;
    S.tile_partials = nullptr;
    S.tile_ctr = nullptr;
    S.n_tiles = 0;
}

int tile_spmv_blocks_per_sm(int lanes, int unroll, int halo_cap)
{
    if (lanes == 4) return unroll == 4 ? tile_blocks<4, 4>(halo_cap) : unroll == 2 ? tile_blocks<4, 2>(halo_cap) : tile_blocks<4, 1>(halo_cap);
    return unroll == 4 ? tile_blocks<8, 4>(halo_cap) : unroll == 2 ? tile_blocks<8, 2>(halo_cap) : tile_blocks<8, 1>(halo_cap);
}

void launch_spmv_tiled(bool dot, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    const int g = L.grid_tiles;
    if (L.lanes == 4) {
        if (L.unroll == 4) tile_launch<4, 4>(dot, P, S, g, st);
        else if (L.unroll == 2) tile_launch<4, 2>(dot, P, S, g, st);
        else tile_launch<4, 1>(dot, P, S, g, st);
    } else {
        if (L.unroll == 4) tile_launch<8, 4>(dot, P, S, g, st);
        else if (L.unroll == 2) tile_launch<8, 2>(dot, P, S, g, st);
        else tile_launch<8, 1>(dot, P, S, g, st);
    }
}

}  // namespace pdgb
