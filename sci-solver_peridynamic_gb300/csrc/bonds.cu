// bonds.cu -- GPU bond construction: uniform-grid hashing and a CSR bond list.
//
// Replaces the reference's host kd-tree (src/core/kdtree.h:229-353, driven by
// Simulator::initPeridynamicsBonds, src/core/simulator.cu:825-943) with
//   bbox -> cell key (Morton order of cells of size >= horizon) -> LSD radix
//   sort (project-written, stable) -> cell start/end -> per-particle count ->
//   exclusive scan -> fill.
// The bond predicate is the reference's, evaluated in FP64 without
// contraction: howfar = (a-b).(a-b) summed x, y, z; bond iff sqrt(howfar) <
// horizon, q != p (kdtree.h:66-79, 319-326).  An FP32 test on positions
// relative to the box centre decides every pair that is clearly inside or
// outside; only pairs within a rounding margin of the horizon use FP64.
// Particle slots follow the sort (cells in Morton order, ties by caller
// index), which keeps bonded particles close in memory.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "pd_device.cuh"
#include "pd_kernels.h"

namespace pdgb {

namespace {

constexpr int kRowAlign = 8;        // row starts aligned to 8 ints (one 32-byte sector)
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

__device__ __forceinline__ unsigned spread3(unsigned v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

struct Grid {
    double lo[3];
    double inv_cs;
    int dim[3];
};

__device__ __forceinline__ void cell_of(const Grid& g, const dbl4& x, int c[3])
{
    const double v[3] = {x.x, x.y, x.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int ci = (int)floor((v[k] - g.lo[k]) * g.inv_cs);
        ci = ci < 0 ? 0 : (ci >= g.dim[k] ? g.dim[k] - 1 : ci);
        c[k] = ci;
    }
}

// ---- bounding box ---------------------------------------------------------------
__global__ void k_bbox(const dbl4* __restrict__ x, int n, double* __restrict__ part)
{
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 v = x[i];
        mn[0] = fmin(mn[0], v.x); mn[1] = fmin(mn[1], v.y); mn[2] = fmin(mn[2], v.z);
        mx[0] = fmax(mx[0], v.x); mx[1] = fmax(mx[1], v.y); mx[2] = fmax(mx[2], v.z);
    }
    __shared__ double s[6][kBlock];
    for (int k = 0; k < 3; ++k) { s[k][threadIdx.x] = mn[k]; s[3 + k][threadIdx.x] = mx[k]; }
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off)
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = fmin(s[k][threadIdx.x], s[k][threadIdx.x + off]);
                s[3 + k][threadIdx.x] = fmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + off]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) part[6 * blockIdx.x + k] = s[k][0];
}

// ---- keys -------------------------------------------------------------------------
__global__ void k_cell_keys(const dbl4* __restrict__ x, int n, Grid g, unsigned* __restrict__ key,
                            int* __restrict__ val)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int c[3];
        cell_of(g, x[i], c);
        key[i] = spread3((unsigned)c[0]) | (spread3((unsigned)c[1]) << 1) | (spread3((unsigned)c[2]) << 2);
        val[i] = i;
    }
}

// ---- stable LSD radix sort, 8-bit digits -------------------------------------------
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const unsigned* __restrict__ key, int n, int shift,
                                                             int tiles, unsigned* __restrict__ hist)
{
    __shared__ unsigned cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int e = base + r * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&cnt[(key[e] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const unsigned* __restrict__ key_in,
                                                                const int* __restrict__ val_in, int n, int shift,
                                                                int tiles, const unsigned* __restrict__ offs,
                                                                unsigned* __restrict__ key_out,
                                                                int* __restrict__ val_out)
{
    __shared__ unsigned running[256];
    __shared__ unsigned wcnt[kSortThreads / 32][257];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    running[threadIdx.x] = offs[threadIdx.x * tiles + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][threadIdx.x] = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][256] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; ++r) {
        const int e = base + r * kSortThreads + threadIdx.x;
        const bool valid = e < n;
        const unsigned k = valid ? key_in[e] : 0u;
        const int v = valid ? val_in[e] : 0;
        const unsigned d = valid ? ((k >> shift) & 0xffu) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned rank = __popc(peers & lt);
        if (rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned pos = running[d] + rank;
            for (int w = 0; w < warp; ++w) pos += wcnt[w][d];
            key_out[pos] = k;
            val_out[pos] = v;
        }
        __syncthreads();
        unsigned tot = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) {
            tot += wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = 0;
        }
        running[threadIdx.x] += tot;
        __syncthreads();
    }
}

// ---- exclusive scan (unsigned, 32-bit) --------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const unsigned* __restrict__ in,
                                                             unsigned* __restrict__ out, long long n,
                                                             unsigned* __restrict__ tile_sums)
{
    __shared__ unsigned s[kScanThreads];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned v[kScanItems];
    unsigned t = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        t += v[k];
    }
    s[threadIdx.x] = t;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        const unsigned o = (int)threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
        __syncthreads();
        s[threadIdx.x] += o;
        __syncthreads();
    }
    unsigned run = s[threadIdx.x] - t;   // exclusive prefix of this thread
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void k_scan_add(unsigned* __restrict__ out, long long n, const unsigned* __restrict__ tile_offs)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_offs[i / kScanTile];
}

// ---- cell ranges ----------------------------------------------------------------
__global__ void k_cell_ranges(const dbl4* __restrict__ xs, const unsigned* __restrict__ key, int n, Grid g,
                              int* __restrict__ cstart, int* __restrict__ cend)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int c[3];
        cell_of(g, xs[i], c);
        const long long lin = ((long long)c[2] * g.dim[1] + c[1]) * g.dim[0] + c[0];
        if (i == 0 || key[i] != key[i - 1]) cstart[lin] = i;
        if (i == n - 1 || key[i] != key[i + 1]) cend[lin] = i + 1;
    }
}

// ---- neighbour query --------------------------------------------------------------
struct Query {
    Grid g;
    double horizon;
    float h2_in, h2_out;   // FP32 certainly-inside / certainly-outside bounds on |dx|^2
};

// the reference predicate (kdtree.h:66-79): a = query particle, b = candidate
__device__ __forceinline__ bool exact_bond(const dbl4& a, const dbl4& b, double horizon)
{
    const double dx = dsub(a.x, b.x), dy = dsub(a.y, b.y), dz = dsub(a.z, b.z);
    const double howfar = dadd(dadd(dadd(0.0, dmul(dx, dx)), dmul(dy, dy)), dmul(dz, dz));
    return __dsqrt_rn(howfar) < horizon;
}

template <bool FILL>
__global__ void __launch_bounds__(kBlock) k_bond_query(const dbl4* __restrict__ xs, const float4* __restrict__ x32,
                                                       int n, Query Q, const int* __restrict__ cstart,
                                                       const int* __restrict__ cend, unsigned* __restrict__ count,
                                                       const int* __restrict__ row_ptr, int* __restrict__ col)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 a = xs[i];
        const float4 af = x32[i];
        int c[3];
        cell_of(Q.g, a, c);
        unsigned cntv = 0;
        const int out = FILL ? row_ptr[i] : 0;
        for (int dz = -1; dz <= 1; ++dz) {
            const int z = c[2] + dz;
            if (z < 0 || z >= Q.g.dim[2]) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int y = c[1] + dy;
                if (y < 0 || y >= Q.g.dim[1]) continue;
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = c[0] + dx;
                    if (x < 0 || x >= Q.g.dim[0]) continue;
                    const long long lin = ((long long)z * Q.g.dim[1] + y) * Q.g.dim[0] + x;
                    const int s = cstart[lin], e = cend[lin];
                    for (int j = s; j < e; ++j) {
                        if (j == i) continue;
                        const float4 bf = x32[j];
                        const float ex = af.x - bf.x, ey = af.y - bf.y, ez = af.z - bf.z;
                        const float d2 = ex * ex + ey * ey + ez * ez;
                        bool bonded;
                        if (d2 < Q.h2_in) bonded = true;
                        else if (d2 > Q.h2_out) bonded = false;
                        else bonded = exact_bond(a, xs[j], Q.horizon);
                        if (bonded) {
                            if (FILL) col[out + cntv] = j;
                            ++cntv;
                        }
                    }
                }
            }
        }
        if (!FILL) count[i] = cntv;
    }
}

__global__ void k_pad_counts(const unsigned* __restrict__ cnt, int n, int max_bonds, unsigned* __restrict__ padded,
                             int* __restrict__ cnt_out, int* __restrict__ flags)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned c = cnt[i];
        padded[i] = (c + kRowAlign - 1) / kRowAlign * kRowAlign;
        cnt_out[i] = (int)c;
        if ((int)c > max_bonds) flags[0] = 1;
        atomicMax(&flags[1], (int)c);
    }
}

__global__ void k_fill_padding(const int* __restrict__ row_ptr, const int* __restrict__ cnt, int n, int* __restrict__ col)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int j = row_ptr[i] + cnt[i]; j < row_ptr[i + 1]; ++j) col[j] = i;
}

__global__ void k_gather_d4(const dbl4* __restrict__ in, const int* __restrict__ perm, dbl4* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dbl4 v = in[perm[i]];
        v.w = 0.0;
        out[i] = v;
    }
}
__global__ void k_gather_d(const double* __restrict__ in, const int* __restrict__ perm, double* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[perm[i]];
}
__global__ void k_gather_i2u8(const int* __restrict__ in, const int* __restrict__ perm, uint8_t* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (uint8_t)(in[perm[i]] & kActMask);
}
__global__ void k_scatter_d4(const dbl4* __restrict__ in, const int* __restrict__ perm, dbl4* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[perm[i]] = in[i];
}
// exports: device slot order -> caller order, then one copy to the host
__global__ void k_scatter_words(const uint32_t* __restrict__ in, const int* __restrict__ perm,
                                uint32_t* __restrict__ out, int words, long long total)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long row = i / words;
        out[(long long)perm[row] * words + (i - row * words)] = in[i];
    }
}
__global__ void k_scatter_to_d4_w0(const void* __restrict__ in, bool is_float, const int* __restrict__ perm,
                                   dbl4* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dbl4 v;
        if (is_float) {
            const float4 f = ((const float4*)in)[i];
            v = make_dbl4(f.x, f.y, f.z, 0.0);
        } else {
            v = ((const dbl4*)in)[i];
            v.w = 0.0;
        }
        out[perm[i]] = v;
    }
}
__global__ void k_local32(const dbl4* __restrict__ X, double ox, double oy, double oz, float4* __restrict__ X32,
                          float4* __restrict__ u32, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 v = X[i];
        X32[i] = make_float4((float)(v.x - ox), (float)(v.y - oy), (float)(v.z - oz), 0.f);
        if (u32) u32[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

int grid_for(long long n, int threads = kBlock)
{
    long long g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 65535LL * 16) g = 65535LL * 16;
    return (int)g;
}

#define PD_TRY(x)                                  \
    do {                                           \
        cudaError_t e_ = (x);                      \
        if (e_ != cudaSuccess) return e_;          \
    } while (0)

// Exclusive scan of n unsigned values (in may equal out).  Temporary storage
// is allocated per level.
cudaError_t exclusive_scan(const unsigned* in, unsigned* out, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const long long tiles = (n + kScanTile - 1) / kScanTile;
    unsigned* sums = nullptr;
    PD_TRY(cudaMalloc(&sums, sizeof(unsigned) * (size_t)tiles));
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && tiles > 1) {
        e = exclusive_scan(sums, sums, tiles, st);
        if (e == cudaSuccess) {
            k_scan_add<<<grid_for(n), kBlock, 0, st>>>(out, n, sums);
            e = cudaGetLastError();
        }
    }
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFree(sums);
    return e != cudaSuccess ? e : e2;
}

}  // namespace

cudaError_t scan_exclusive_u32(const unsigned* in, unsigned* out, long long n, cudaStream_t st)
{
    return exclusive_scan(in, out, n, st);
}

cudaError_t sort_pairs_u32(unsigned* keys, int* vals, int n, int key_bits, cudaStream_t st)
{
    if (n <= 1) return cudaSuccess;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    unsigned *k1 = nullptr, *hist = nullptr;
    int* v1 = nullptr;
    PD_TRY(cudaMalloc(&k1, sizeof(unsigned) * n));
    PD_TRY(cudaMalloc(&v1, sizeof(int) * n));
    PD_TRY(cudaMalloc(&hist, sizeof(unsigned) * 256 * (size_t)tiles));
    unsigned *ka = keys, *kb = k1;
    int *va = vals, *vb = v1;
    cudaError_t e = cudaSuccess;
    for (int shift = 0; shift < key_bits && e == cudaSuccess; shift += 8) {
        k_radix_hist<<<tiles, kSortThreads, 0, st>>>(ka, n, shift, tiles, hist);
        e = exclusive_scan(hist, hist, 256LL * tiles, st);
        if (e != cudaSuccess) break;
        k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(ka, va, n, shift, tiles, hist, kb, vb);
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (e == cudaSuccess && ka != keys) {   // an odd number of passes: copy back
        e = cudaMemcpyAsync(keys, ka, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFree(k1);
    cudaFree(v1);
    cudaFree(hist);
    return e != cudaSuccess ? e : e2;
}

void gather_double4(const dbl4* in, const int* perm, dbl4* out, int n, cudaStream_t st)
{
    if (n > 0) k_gather_d4<<<grid_for(n), kBlock, 0, st>>>(in, perm, out, n);
}
void gather_double(const double* in, const int* perm, double* out, int n, cudaStream_t st)
{
    if (n > 0) k_gather_d<<<grid_for(n), kBlock, 0, st>>>(in, perm, out, n);
}
void gather_int_to_u8(const int* in, const int* perm, uint8_t* out, int n, cudaStream_t st)
{
    if (n > 0) k_gather_i2u8<<<grid_for(n), kBlock, 0, st>>>(in, perm, out, n);
}
void scatter_double4(const dbl4* in, const int* perm, dbl4* out, int n, cudaStream_t st)
{
    if (n > 0) k_scatter_d4<<<grid_for(n), kBlock, 0, st>>>(in, perm, out, n);
}
void scatter_words(const void* in, const int* perm, void* out, int words_per_row, int n, cudaStream_t st)
{
    if (n <= 0) return;
    const long long total = (long long)n * words_per_row;
    const int grid = (int)std::min<long long>((total + kBlock - 1) / kBlock, 65535LL * 8);
    k_scatter_words<<<grid, kBlock, 0, st>>>((const uint32_t*)in, perm, (uint32_t*)out, words_per_row, total);
}
void scatter_to_d4_w0(const void* in, bool is_float, const int* perm, dbl4* out, int n, cudaStream_t st)
{
    if (n > 0) k_scatter_to_d4_w0<<<grid_for(n), kBlock, 0, st>>>(in, is_float, perm, out, n);
}
void make_local32(const dbl4* X, double ox, double oy, double oz, float4* X32, float4* u32, int n, cudaStream_t st)
{
    if (n > 0) k_local32<<<grid_for(n), kBlock, 0, st>>>(X, ox, oy, oz, X32, u32, n);
}

cudaError_t build_bonds(const dbl4* pos_orig, int n, double horizon, int max_bonds, dbl4* pos_sorted,
                        float4* x32_sorted, double origin[3], BondBuildOut* out, cudaStream_t st)
{
    out->total = 0;
    out->bonds = 0;
    out->max_bonds = 0;
    out->overflow = 0;
    out->col = nullptr;
    if (n <= 0) return cudaSuccess;

    // bounding box
    const int bb_blocks = 256;
    double* d_part = nullptr;
    PD_TRY(cudaMalloc(&d_part, sizeof(double) * 6 * bb_blocks));
    k_bbox<<<bb_blocks, kBlock, 0, st>>>(pos_orig, n, d_part);
    std::vector<double> part(6 * bb_blocks);
    PD_TRY(cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, st));
    PD_TRY(cudaStreamSynchronize(st));
    cudaFree(d_part);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int b = 0; b < bb_blocks; ++b)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], part[6 * b + k]);
            hi[k] = std::max(hi[k], part[6 * b + 3 + k]);
        }
    for (int k = 0; k < 3; ++k) origin[k] = 0.5 * (lo[k] + hi[k]);

    // grid: cell size slightly above the horizon so rounding cannot push a
    // bonded pair two cells apart; at most 1024 cells per axis (30-bit Morton
    // key) and at most ~8 cells per particle
    Grid g;
    double cs = (horizon > 0 ? horizon : 1.0) * (1.0 + 1e-6);
    for (;;) {
        long long tot = 1;
        bool ok = true;
        for (int k = 0; k < 3; ++k) {
            const double span = hi[k] - lo[k];
            long long d = (long long)(span / cs) + 1;
            if (d > 1024) ok = false;
            g.dim[k] = (int)std::min<long long>(d, 1 << 20);
            tot *= g.dim[k];
        }
        if (ok && tot <= 8LL * n + 4096) break;
        cs *= 1.5;
    }
    for (int k = 0; k < 3; ++k) g.lo[k] = lo[k];
    g.inv_cs = 1.0 / cs;
    const long long ncell = (long long)g.dim[0] * g.dim[1] * g.dim[2];
    int maxdim = std::max(g.dim[0], std::max(g.dim[1], g.dim[2]));
    int bits = 0;
    while ((1 << bits) < maxdim) ++bits;
    const int key_bits = 3 * std::max(bits, 1);

    // keys + sort
    unsigned *k0 = nullptr, *k1 = nullptr, *hist = nullptr;
    int *v0 = nullptr, *v1 = nullptr;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    PD_TRY(cudaMalloc(&k0, sizeof(unsigned) * n));
    PD_TRY(cudaMalloc(&k1, sizeof(unsigned) * n));
    PD_TRY(cudaMalloc(&v0, sizeof(int) * n));
    PD_TRY(cudaMalloc(&v1, sizeof(int) * n));
    PD_TRY(cudaMalloc(&hist, sizeof(unsigned) * 256 * (size_t)tiles));
    k_cell_keys<<<grid_for(n), kBlock, 0, st>>>(pos_orig, n, g, k0, v0);
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_radix_hist<<<tiles, kSortThreads, 0, st>>>(k0, n, shift, tiles, hist);
        PD_TRY(exclusive_scan(hist, hist, 256LL * tiles, st));
        k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(k0, v0, n, shift, tiles, hist, k1, v1);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    PD_TRY(cudaGetLastError());
    cudaFree(hist);
    cudaFree(k1);
    cudaFree(v1);
    out->perm = v0;   // slot -> caller index (owned by the caller from here)
    gather_double4(pos_orig, out->perm, pos_sorted, n, st);
    make_local32(pos_sorted, origin[0], origin[1], origin[2], x32_sorted, nullptr, n, st);

    // cell ranges
    int *cstart = nullptr, *cend = nullptr;
    PD_TRY(cudaMalloc(&cstart, sizeof(int) * (size_t)ncell));
    PD_TRY(cudaMalloc(&cend, sizeof(int) * (size_t)ncell));
    PD_TRY(cudaMemsetAsync(cstart, 0, sizeof(int) * (size_t)ncell, st));
    PD_TRY(cudaMemsetAsync(cend, 0, sizeof(int) * (size_t)ncell, st));
    k_cell_ranges<<<grid_for(n), kBlock, 0, st>>>(pos_sorted, k0, n, g, cstart, cend);
    cudaFree(k0);

    // FP32 prefilter bounds: positions relative to the box centre carry a
    // rounding error below 2^-24 |x| per coordinate; the margin covers 4x the
    // resulting error on |dx|^2.
    double M = 0.0;
    for (int k = 0; k < 3; ++k) M = std::max(M, 0.5 * (hi[k] - lo[k]));
    Query Q;
    Q.g = g;
    Q.horizon = horizon;
    const double eps = 4.0 * (8.0 * std::ldexp(1.0, -24) * (M / (horizon > 0 ? horizon : 1.0) + 1.0));
    const double h2 = horizon * horizon;
    Q.h2_in = (float)(h2 * (1.0 - eps));
    Q.h2_out = (float)(h2 * (1.0 + eps));
    if (!(horizon > 0)) { Q.h2_in = -1.f; Q.h2_out = -1.f; }

    unsigned* cnt = nullptr;
    unsigned* padded = nullptr;
    int* flags = nullptr;
    PD_TRY(cudaMalloc(&cnt, sizeof(unsigned) * n));
    PD_TRY(cudaMalloc(&padded, sizeof(unsigned) * ((size_t)n + 1)));
    PD_TRY(cudaMalloc(&flags, sizeof(int) * 2));
    PD_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * 2, st));
    k_bond_query<false><<<grid_for(n), kBlock, 0, st>>>(pos_sorted, x32_sorted, n, Q, cstart, cend, cnt, nullptr, nullptr);
    k_pad_counts<<<grid_for(n), kBlock, 0, st>>>(cnt, n, max_bonds, padded, out->cnt, flags);
    PD_TRY(cudaMemsetAsync(padded + n, 0, sizeof(unsigned), st));
    PD_TRY(exclusive_scan(padded, padded, (long long)n + 1, st));
    int hflags[2] = {0, 0};
    unsigned total = 0;
    PD_TRY(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    PD_TRY(cudaMemcpyAsync(&total, padded + n, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    PD_TRY(cudaStreamSynchronize(st));
    out->overflow = hflags[0];
    out->max_bonds = hflags[1];
    // row_ptr (int) from the padded scan
    PD_TRY(cudaMemcpyAsync(out->row_ptr, padded, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
    out->total = total;
    if (!out->overflow && (long long)total < (1LL << 31) - 64) {
        PD_TRY(cudaMalloc(&out->col, sizeof(int) * ((size_t)total + kRowAlign)));
        k_bond_query<true><<<grid_for(n), kBlock, 0, st>>>(pos_sorted, x32_sorted, n, Q, cstart, cend, nullptr,
                                                           out->row_ptr, out->col);
        k_fill_padding<<<grid_for(n), kBlock, 0, st>>>(out->row_ptr, out->cnt, n, out->col);
        PD_TRY(cudaGetLastError());
    } else if ((long long)total >= (1LL << 31) - 64) {
        out->overflow = 2;
    }
    PD_TRY(cudaStreamSynchronize(st));
    // live bond count
    {
        std::vector<int> hc(n);
        PD_TRY(cudaMemcpy(hc.data(), out->cnt, sizeof(int) * n, cudaMemcpyDeviceToHost));
        long long b = 0;
        for (int i = 0; i < n; ++i) b += hc[i];
        out->bonds = b;
    }
    cudaFree(cnt);
    cudaFree(padded);
    cudaFree(flags);
    cudaFree(cstart);
    cudaFree(cend);
    return cudaGetLastError();
}

}  // namespace pdgb
