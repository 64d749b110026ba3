// lattice.cu -- the system product A w for bodies filled on a lattice
// (mixed precision).
//
// The reference fills every body on a simple-cubic lattice of spacing 2 r
// (src/examples/scene.cpp:33-135) and bonds each particle to the others within
// the horizon (src/core/kdtree.h:304-353); its product computeAx
// (src/core/cg_solver.cuh:343-383) then gathers one 3x3 block and one vector
// entry per bond.  Here, when every particle sits within 0.3 spacings of a
// distinct lattice site, each bond joins two sites whose offset lies in a
// small stencil (80 offsets for a horizon of 2.5 spacings).  The slots are
// renumbered brick by brick (bricks of 32 x 4 x bz sites, x fastest), and the
// product runs one brick per block iteration: the block stages the halo of
// the brick's sites (each particle's deviation from its site and its entry of
// w) in shared memory, then each thread walks its row's stencil.  Rows of a
// warp are x-consecutive sites, so the neighbours at one stencil entry are
// x-consecutive shared-memory words (no bank conflicts), and the only per-bond
// stream is 1/d0 per (row, stencil entry), 0 where there is no live bond
// (stored scaled by 2^100, see kLatScale).
//
// The per-bond arithmetic is the gather product's (step_rows.cuh,
// mixed_bond_chunk): the Jacobian applied to w_p - w_q is
//   c [ (1/d0 - 1/d) (w_p - w_q) + (xi . (w_p - w_q)) xi / d^3 ],
// with the bond vector xi = h v_k + (d_q - d_p) from the stencil offset v_k
// and the two deviations d from the lattice sites (per step, FP64 rounded
// once to FP32 within half a supercell), in pairs of FP32 lanes (f32x2).
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "step_rows.cuh"

namespace pdgb {

namespace {

#define LT_TRY(x)                              \
    do {                                       \
        cudaError_t e_ = (x);                  \
        if (e_ != cudaSuccess) return e_;      \
    } while (0)

constexpr int kLatBX = 32;
constexpr int kLatBY = 4;
constexpr float kLatEmpty = 1.0e4f;   // deviation of an empty site (any far, finite position)
// The table holds 2^100 / d0: then min(1/d, entry) is 1/d for a live bond (its
// entry is near 1e31 or more) and 0 for "no bond" (entry 0), one instruction,
// and 1/d0 - 1/d = fma(entry, 2^-100, -1/d) is exact scaling by a power of two.
constexpr float kLatScale = 1.2676506002282294e30f;     // 2^100
constexpr float kLatUnscale = 7.888609052210118e-31f;   // 2^-100
// the largest halo: R = 3, bricks of 32 x 4 x 2 sites -> 38 x 10 x 8 sites of 24 bytes
constexpr int kLatHaloMax = 38 * 10 * 8;
constexpr int kLatSiteBytes = sizeof(float4) + sizeof(float2);
constexpr int kLatSmemMax = kLatHaloMax * kLatSiteBytes;
constexpr int kLatHaloPerThread = (kLatHaloMax + kBlock - 1) / kBlock;

// The stencil of a horizon of 2.5 spacings (the benchmark's 5 r): every lattice
// offset with |v|^2 <= 6 (80 offsets, reach 2 per axis), in (dz, dy, dx)
// order.  Bodies whose bonds all fall in it use a product specialised for it:
// bricks of 32 x 4 x 4 sites, a 36 x 8 x 8 halo, and shared-memory offsets
// known at compile time.
constexpr int kS80 = 80;
constexpr int kS80Hx = kLatBX + 4, kS80Hy = kLatBY + 4, kS80Hz = 4 + 4;
struct Stencil80 {
    int off[kS80];
    int dx[kS80], dy[kS80], dz[kS80];
};
__host__ __device__ constexpr bool in_s80(int dx, int dy, int dz)
{
    return (dx || dy || dz) && dx * dx + dy * dy + dz * dz <= 6 && dx >= -2 && dx <= 2 && dy >= -2 && dy <= 2 &&
           dz >= -2 && dz <= 2;
}
__host__ __device__ constexpr Stencil80 make_stencil80()
{
    Stencil80 t{};
    int k = 0;
    for (int dz = -2; dz <= 2; ++dz)
        for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx)
                if (in_s80(dx, dy, dz)) {
                    t.off[k] = (dz * kS80Hy + dy) * kS80Hx + dx;
                    t.dx[k] = dx;
                    t.dy[k] = dy;
                    t.dz[k] = dz;
                    ++k;
                }
    return t;
}
__host__ __device__ constexpr int count_s80()
{
    int k = 0;
    for (int dz = -2; dz <= 2; ++dz)
        for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx)
                if (in_s80(dx, dy, dz)) ++k;
    return k;
}
static_assert(count_s80() == kS80, "the |v|^2 <= 6 stencil has 80 offsets");

// 1/sqrt(x) by the hardware approximation without a denormal path: a live
// bond's d^2 is far above the FP32 denormal range, and an empty or padding
// entry (d^2 = 0 -> +inf) is masked to 0 by its caller.  The file is built
// without flush-to-zero: the CG dot products of small right-hand sides
// (1e-20 entries, products near 1e-40) must keep their denormal terms.
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

int blocks_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + kBlock - 1) / kBlock, 8192)); }

// ---- detection ------------------------------------------------------------------------
// site = rint((X - anchor) / h) per axis; ext[0..2] = min, ext[3..5] = max,
// ext[6] != 0 when some coordinate lies more than 0.3 h from its site
__global__ void __launch_bounds__(kBlock) k_lat_sites(const dbl4* __restrict__ x, int n, double ax, double ay,
                                                      double az, double inv_h, int4* __restrict__ site,
                                                      int* __restrict__ ext)
{
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    int fail = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 p = x[i];
        const double f[3] = {(p.x - ax) * inv_h, (p.y - ay) * inv_h, (p.z - az) * inv_h};
        int s[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double r = rint(f[k]);
            if (!(fabs(f[k] - r) <= 0.3) || !(fabs(r) < 1.0e8)) {
                fail = 1;
                s[k] = 0;
            } else {
                s[k] = (int)r;
            }
            mn[k] = min(mn[k], s[k]);
            mx[k] = max(mx[k], s[k]);
        }
        site[i] = make_int4(s[0], s[1], s[2], 0);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = __reduce_min_sync(0xffffffffu, mn[k]);
        mx[k] = __reduce_max_sync(0xffffffffu, mx[k]);
    }
    fail = __reduce_or_sync(0xffffffffu, fail);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(&ext[k], mn[k]);
            atomicMax(&ext[3 + k], mx[k]);
        }
        if (fail) atomicOr(&ext[6], 1);
    }
}

// every live bond's site offset marked in the kLatTab^3 table (fail[0] set
// when an offset exceeds kLatRmax on some axis)
__global__ void __launch_bounds__(kBlock) k_lat_offsets(int n, const int4* __restrict__ site,
                                                        const int* __restrict__ row_ptr, const int* __restrict__ cnt,
                                                        const int* __restrict__ col, int* __restrict__ tab,
                                                        int* __restrict__ fail)
{
    __shared__ int stab[kLatTab * kLatTab * kLatTab];
    for (int i = threadIdx.x; i < kLatTab * kLatTab * kLatTab; i += blockDim.x) stab[i] = 0;
    __syncthreads();
    int bad = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int4 sp = site[p];
        const int rs = row_ptr[p], cn = cnt[p];
        for (int j = 0; j < cn; ++j) {
            const int4 sq = site[col[rs + j]];
            const int dx = sq.x - sp.x, dy = sq.y - sp.y, dz = sq.z - sp.z;
            if (abs(dx) > kLatRmax || abs(dy) > kLatRmax || abs(dz) > kLatRmax) {
                bad = 1;
                continue;
            }
            stab[((dz + kLatRmax) * kLatTab + (dy + kLatRmax)) * kLatTab + (dx + kLatRmax)] = 1;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kLatTab * kLatTab * kLatTab; i += blockDim.x)
        if (stab[i]) atomicOr(&tab[i], 1);
    if (bad) atomicOr(fail, 1);
}

// shifted sites and the brick-major sort key of every slot
__global__ void __launch_bounds__(kBlock) k_lat_keys(int n, int4* __restrict__ site, int3 lo, int bz, int3 nb,
                                                     unsigned* __restrict__ key, int* __restrict__ val)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int4 s = site[i];
        s.x -= lo.x;
        s.y -= lo.y;
        s.z -= lo.z;
        site[i] = s;
        const unsigned brick = ((unsigned)(s.z / bz) * (unsigned)nb.y + (unsigned)(s.y / kLatBY)) * (unsigned)nb.x +
                               (unsigned)(s.x / kLatBX);
        const unsigned local = ((unsigned)(s.z % bz) * kLatBY + (unsigned)(s.y % kLatBY)) * kLatBX +
                               (unsigned)(s.x % kLatBX);
        key[i] = brick * (unsigned)(kLatBX * kLatBY * bz) + local;
        val[i] = i;
    }
}

__global__ void k_lat_dups(const unsigned* __restrict__ key, int n, int* __restrict__ fail)
{
    for (int i = 1 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (key[i] == key[i - 1]) atomicOr(fail, 1);
}

// ---- renumbering (new slot i holds old slot n2o[i]) -------------------------------------
template <typename T>
__global__ void k_lat_gather(const T* __restrict__ in, const int* __restrict__ n2o, T* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[n2o[i]];
}

__global__ void k_lat_inverse(const int* __restrict__ n2o, int* __restrict__ o2n, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) o2n[n2o[i]] = i;
}

__global__ void k_lat_lengths(const int* __restrict__ row_ptr, const int* __restrict__ n2o, unsigned* __restrict__ len,
                              int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int o = n2o[i];
        len[i] = (unsigned)(row_ptr[o + 1] - row_ptr[o]);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) len[n] = 0u;
}

__global__ void k_lat_remap_col(const int* __restrict__ row_ptr_old, const int* __restrict__ col_old,
                                const unsigned* __restrict__ row_ptr_new, const int* __restrict__ n2o,
                                const int* __restrict__ o2n, int* __restrict__ col_new, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int o = n2o[i];
        const int a = row_ptr_old[o], len = row_ptr_old[o + 1] - a;
        const int b = (int)row_ptr_new[i];
        for (int j = 0; j < len; ++j) col_new[b + j] = o2n[col_old[a + j]];
    }
}

__global__ void k_lat_map(const int4* __restrict__ site, int n, int R, int mx, int my, int* __restrict__ map)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 s = site[i];
        map[((long long)(s.z + R) * my + (s.y + R)) * mx + (s.x + R)] = i;
    }
}

// ---- 1/d0 table ------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_lat_ell(DeviceState S, LatticeParams lp, int force)
{
    if (!force && ((volatile int*)S.flags)[1] == 0) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.n; p += gridDim.x * blockDim.x) {
        const int b = lp.row_brick[p];
        const int start = lp.brick_start[b];
        const int rows = lp.brick_start[b + 1] - start;
        const int l = p - start;
        float* e = lp.ell + (size_t)lp.K * start;
        for (int k4 = 0; k4 < lp.K / 4; ++k4)
            ((float4*)e)[(size_t)k4 * rows + l] = make_float4(0.f, 0.f, 0.f, 0.f);
        const int4 sp = lp.site[p];
        const int rs = S.row_ptr[p], cn = S.cnt[p];
        for (int j = 0; j < cn; ++j) {
            const int4 sq = lp.site[S.col[rs + j]];
            const int t = ((sq.z - sp.z + kLatRmax) * kLatTab + (sq.y - sp.y + kLatRmax)) * kLatTab +
                          (sq.x - sp.x + kLatRmax);
            const int k = lp.offk[t];
            e[((size_t)(k >> 2) * rows + l) * 4 + (k & 3)] = S.inv_d0[rs + j] * kLatScale;
        }
    }
}

// ---- deviations from the lattice sites ------------------------------------------------
// dl[i] = (d, n): x - (org + h site) = d + sup n per axis with n = rint(. / sup)
// (FP64, exact: sup is a power of two), d rounded once to FP32; n packed in
// 10 bits per axis (+512).  |n| stays below 512 for displacements below
// 500 supercells; larger ones are clamped (the deviation then loses digits).
__global__ void __launch_bounds__(kBlock) k_lat_delta(const dbl4* __restrict__ x64, int n, LatticeParams lp,
                                                      double sup, float4* __restrict__ dl)
{
    const double inv_sup = 1.0 / sup;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 x = x64[i];
        const int4 s = lp.site[i];
        const double dev[3] = {x.x - (lp.org[0] + lp.h * s.x), x.y - (lp.org[1] + lp.h * s.y),
                               x.z - (lp.org[2] + lp.h * s.z)};
        float d[3];
        int packed = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double m = fmin(fmax(rint(dev[k] * inv_sup), -511.0), 511.0);
            d[k] = (float)(dev[k] - m * sup);
            packed |= ((int)m + 512) << (10 * k);
        }
        dl[i] = make_float4(d[0], d[1], d[2], __int_as_float(packed));
    }
}

// ---- the product -----------------------------------------------------------------------
// Shared memory per halo site: A = (d.x, d.y, w.x, w.y), B = (d.z, w.z)
// (24 bytes), d the site particle's deviation re-referenced to the brick:
// d + sup (n - n_brick), n_brick the wrap counts of the brick's first slot
// (within a brick's halo they differ by at most one for any strain a bond
// survives, so |d| stays within 1.5 sup).  Entry k's bond vector is then
// xi = h v_k + (d_q - d_p), formed in FP32 pairs with the differences of w.
//
// Blocks take bricks from a counter (lp.sched[0]) in brick order, so that
// bricks of uneven fill balance over the blocks; the last block to finish
// resets the counter for the next launch.  (An L2 prefetch of the next
// brick's 1/d0 block, issued when the brick is taken, measured 3 % slower at
// three blocks per SM; ordering the bricks by row count made no difference.)
//
// FIXED: the 80-entry stencil with its compile-time halo (lp.K == 80, halo
// 36 x 8 x 8).  FUSE (a CG iteration): the direction is updated on the way
// in, w = r + beta p_prev for every halo site (beta = 0 on the first
// iteration, which cg_fin_residual sets), and each brick writes its rows' new
// direction to p_out (p_prev and p_out are different buffers, so blocks that
// still stage halos read the old direction).
__device__ __forceinline__ float wrap_delta(int nq, int nb, int shift, float sup)
{
    return sup * small_int_to_float(((nq >> shift) & 1023) - ((nb >> shift) & 1023));
}

// Three blocks per SM (80 registers, a 55 KB halo each): at 1M particles 173 us
// per product against 184 at two blocks (128 registers) and 178 at four (64).
template <bool DOT, bool FIXED, bool FUSE>
__global__ void __launch_bounds__(kBlock, 3) k_spmv_lattice(StepParams P, DeviceState S, LatticeParams lp,
                                                           const float4* __restrict__ in, float4* __restrict__ out,
                                                           ReduceSlot slot, CgScalars* cg, double* dot_out,
                                                           const float4* __restrict__ r_in, float4* __restrict__ p_out)
{
    if (DOT && cg && ((volatile CgScalars*)cg)->done) return;
    extern __shared__ float4 lat_smem[];
    __shared__ int s_next;
    const int H = FIXED ? kS80Hx * kS80Hy * kS80Hz : lp.hx * lp.hy * lp.hz;
    float4* sA = lat_smem;
    float2* sB = (float2*)(sA + H);
    const float sup = (float)P.sup;
    const int hx = FIXED ? kS80Hx : lp.hx, hxy = FIXED ? kS80Hx * kS80Hy : lp.hx * lp.hy;
    const int mx = lp.map_dim[0], mxy = lp.map_dim[0] * lp.map_dim[1];
    const int K = FIXED ? kS80 : lp.K;
    const float beta = FUSE ? (float)((volatile CgScalars*)cg)->beta : 0.f;
    const float2 m1 = make_float2(-1.f, -1.f);
    DotAcc32 acc;
    if (threadIdx.x == 0) {
        s_next = (int)atomicAdd(&lp.sched[0], 1u);
    }
    __syncthreads();
    int b = s_next;
    while (b < lp.n_bricks) {
        const int corner = lp.brick_corner[b];
        const int start = lp.brick_start[b];
        const int rows = lp.brick_start[b + 1] - start;
        const int nb = __float_as_int(__ldg(&lp.dl[start].w));
        // the map entries of this thread's halo sites first (independent
        // loads), then their deviations and w entries
        int qs[kLatHaloPerThread];
#pragma unroll
        for (int t = 0; t < kLatHaloPerThread; ++t) {
            const int h = threadIdx.x + t * kBlock;
            qs[t] = -1;
            if (h < H) {
                const int iz = h / hxy;
                const int r2 = h - iz * hxy;
                const int iy = r2 / hx;
                const int ix = r2 - iy * hx;
                qs[t] = __ldg(lp.map + corner + iz * mxy + iy * mx + ix);
            }
        }
#pragma unroll
        for (int t = 0; t < kLatHaloPerThread; ++t) {
            const int h = threadIdx.x + t * kBlock;
            if (h >= H) continue;
            const int q = qs[t];
            float4 a = make_float4(kLatEmpty, kLatEmpty, 0.f, 0.f);
            float2 bb = make_float2(kLatEmpty, 0.f);
            if (q >= 0) {
                const float4 dq = __ldg(lp.dl + q);
                float4 w = __ldg(in + q);
                if (FUSE) {   // xpby_elem: p = r + beta p
                    const float4 r = __ldg(r_in + q);
                    w.x = r.x + beta * w.x;
                    w.y = r.y + beta * w.y;
                    w.z = r.z + beta * w.z;
                }
                const int nq = __float_as_int(dq.w);
                a = make_float4(dq.x + wrap_delta(nq, nb, 0, sup), dq.y + wrap_delta(nq, nb, 10, sup), w.x, w.y);
                bb = make_float2(dq.z + wrap_delta(nq, nb, 20, sup), w.z);
            }
            sA[h] = a;
            sB[h] = bb;
        }
        __syncthreads();   // halo staged; every thread has read s_next
        if (threadIdx.x == 0) {
            s_next = (int)atomicAdd(&lp.sched[0], 1u);
        }
        for (int l = threadIdx.x; l < rows; l += blockDim.x) {
            const int p = start + l;
            const uint8_t ab = S.act[p];
            const int c = lp.row_local[p];
            const float4 pa = sA[c];
            const float2 pb = sB[c];
            const float4 w = make_float4(pa.z, pa.w, pb.y, 0.f);
            if (FUSE) p_out[p] = w;
            if (is_dirichlet(ab & kActMask)) {
                out[p] = make_float4(0.f, 0.f, 0.f, 0.f);
                continue;
            }
            const float2 pd = make_float2(pa.x, pa.y), pw = make_float2(pa.z, pa.w);
            // this row's 1/d0 stream: 16 bytes (4 stencil entries) per load
            const float4* __restrict__ e4 = (const float4*)(lp.ell + (size_t)K * start) + l;
            // sums of a1 (w_q - w_p) + g xi with g = xi . (w_q - w_p) / d^3: the
            // row's term with the sign of w_q - w_p, negated at the end
            float2 sxy = make_float2(0.f, 0.f);
            float sz = 0.f;
            constexpr Stencil80 s80 = make_stencil80();
            const auto bond = [&](int k, float s) {
                const int q = c + (FIXED ? s80.off[k] : lp.off[k]);
                const float4 qa = sA[q];
                const float2 qb = sB[q];
                float2 xy = __ffma2_rn(pd, m1, make_float2(qa.x, qa.y));    // d_q - d_p
                const float2 wxy = __ffma2_rn(pw, m1, make_float2(qa.z, qa.w));   // w_q - w_p
                const float2 zz = __ffma2_rn(pb, m1, qb);                        // (d_q - d_p, w_q - w_p).z
                float zs = zz.x;
                if (FIXED) {   // h v_k: compile-time zeros drop out
                    if (s80.dx[k] != 0) xy.x += lp.cx[k];
                    if (s80.dy[k] != 0) xy.y += lp.cy[k];
                    if (s80.dz[k] != 0) zs += lp.cz[k];
                } else {
                    xy.x += lp.cx[k];
                    xy.y += lp.cy[k];
                    zs += lp.cz[k];
                }
                const float2 sq = __fmul2_rn(xy, xy);
                float inv_d = rsqrt_ftz(fmaf(zs, zs, sq.x + sq.y));
                inv_d = fminf(inv_d, s);   // no live bond (s = 0): the term vanishes
                const float a1 = fmaf(s, kLatUnscale, -inv_d);
                const float2 t = __fmul2_rn(xy, wxy);
                const float g = fmaf(zs, zz.y, t.x + t.y) * (inv_d * inv_d * inv_d);
                sxy = __ffma2_rn(make_float2(a1, a1), wxy, __ffma2_rn(make_float2(g, g), xy, sxy));
                sz = fmaf(a1, zz.y, fmaf(g, zs, sz));
            };
            // (loading each table chunk one chunk ahead measured slower: 181 against 173 us)
            if constexpr (FIXED) {
#pragma unroll
                for (int k4 = 0; k4 < kS80 / 4; ++k4) {
                    const float4 s4 = __ldcs(e4 + (size_t)k4 * rows);
                    bond(4 * k4, s4.x);
                    bond(4 * k4 + 1, s4.y);
                    bond(4 * k4 + 2, s4.z);
                    bond(4 * k4 + 3, s4.w);
                }
            } else {
#pragma unroll 10   // 160 us at 1M against 163 (5), 168 (4), 171 (2) and 174 (20)
                for (int k4 = 0; k4 < K / 4; ++k4) {
                    const float4 s4 = __ldcs(e4 + (size_t)k4 * rows);
                    bond(4 * k4, s4.x);
                    bond(4 * k4 + 1, s4.y);
                    bond(4 * k4 + 2, s4.z);
                    bond(4 * k4 + 3, s4.w);
                }
            }
            spmv_finish_mixed<1, DOT>(P, S, p, ab, w, -sxy.x, -sxy.y, -sz, 0, 0xffffffffu, out, acc);
        }
        __syncthreads();   // the rows are done with the halo; s_next is visible
        b = s_next;
    }
    // every block has taken its last brick index: the last to arrive resets the counter
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&lp.sched[1], 1u) == gridDim.x - 1) {
            lp.sched[0] = 0u;
            lp.sched[1] = 0u;
        }
    }
    if (DOT) {
        block_reduce_finish(acc, slot, [cg, dot_out](double pAp) {
            if (cg) cg_fin_alpha(cg, pAp);
            if (dot_out) *dot_out = pAp;
        });
    }
}

}  // namespace

size_t lattice_smem_bytes(const LatticeParams& lp)
{
    return (size_t)lp.hx * lp.hy * lp.hz * kLatSiteBytes;
}

void launch_lattice_delta(const DeviceState& S, const LatticeParams& lp, double sup, cudaStream_t st)
{
    if (S.n > 0 && lp.dl) k_lat_delta<<<blocks_for(S.n), kBlock, 0, st>>>(S.x64, S.n, lp, sup, lp.dl);
}

template <bool FIXED>
int lattice_blocks(size_t smem)
{
    const void* ks[3] = {(const void*)k_spmv_lattice<false, FIXED, false>, (const void*)k_spmv_lattice<true, FIXED, false>,
                         (const void*)k_spmv_lattice<true, FIXED, true>};
    int m = 1 << 30;
    for (const void* k : ks) {
        // the attribute is per kernel and process: set to the largest halo any
        // handle can need, so that every handle's launch fits
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kLatSmemMax);
        int a = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k, kBlock, smem);
        m = std::min(m, a);
    }
    return m > 0 ? m : 1;
}

int lattice_spmv_blocks_per_sm(const LatticeParams& lp)
{
    // both variants get the shared-memory attribute: the autotuner may run
    // the general kernel on a stencil the compile-time one also covers
    const size_t smem = lattice_smem_bytes(lp);
    const int general = lattice_blocks<false>(smem);
    return lp.fixed ? std::min(general, lattice_blocks<true>(smem)) : general;
}

template <bool FIXED>
void launch_lattice_t(bool dot, const StepParams& P, const DeviceState& S, const LatticeParams& lp, const void* in,
                      void* out, ReduceSlot slot, CgScalars* cg, double* dot_out, const void* r_in, void* p_out,
                      int grid, size_t smem, cudaStream_t st)
{
    const float4* x = (const float4*)in;
    float4* y = (float4*)out;
    if (r_in)
        k_spmv_lattice<true, FIXED, true><<<grid, kBlock, smem, st>>>(P, S, lp, x, y, slot, cg, dot_out,
                                                                      (const float4*)r_in, (float4*)p_out);
    else if (dot)
        k_spmv_lattice<true, FIXED, false><<<grid, kBlock, smem, st>>>(P, S, lp, x, y, slot, cg, dot_out, nullptr,
                                                                       nullptr);
    else
        k_spmv_lattice<false, FIXED, false><<<grid, kBlock, smem, st>>>(P, S, lp, x, y, slot, nullptr, nullptr,
                                                                        nullptr, nullptr);
}

void launch_spmv_lattice(bool dot, const StepParams& P, const DeviceState& S, const LatticeParams& lp,
                         const void* in, void* out, ReduceSlot slot, CgScalars* cg, double* dot_out,
                         const void* r_in, void* p_out, cudaStream_t st)
{
    const size_t smem = lattice_smem_bytes(lp);
    const int grid = std::max(1, std::min(lp.grid, std::max(lp.n_bricks, 1)));
    if (lp.fixed) launch_lattice_t<true>(dot, P, S, lp, in, out, slot, cg, dot_out, r_in, p_out, grid, smem, st);
    else launch_lattice_t<false>(dot, P, S, lp, in, out, slot, cg, dot_out, r_in, p_out, grid, smem, st);
}

void launch_lattice_ell(const DeviceState& S, const LatticeParams& lp, int force, int grid, cudaStream_t st)
{
    k_lat_ell<<<grid, kBlock, 0, st>>>(S, lp, force);
}

void lattice_free(LatticeBuffers* lb)
{
    cudaFree(lb->brick_start);
    cudaFree(lb->brick_corner);
    cudaFree(lb->row_local);
    cudaFree(lb->row_brick);
    cudaFree(lb->site);
    cudaFree(lb->map);
    cudaFree(lb->offk);
    cudaFree(lb->ell);
    cudaFree(lb->dl);
    cudaFree(lb->sched);
    *lb = LatticeBuffers{};
}

cudaError_t lattice_build(int n, double spacing, dbl4* x64, float4* X32, int* perm, int* row_ptr, int* cnt, int** col,
                          long long total_slots, LatticeParams* lp, LatticeBuffers* lb, int* ok, cudaStream_t st)
{
    *ok = 0;
    // (spacings below 1e-6 would take 2^100 / d0 out of the FP32 range)
    if (n < 1 || !(spacing > 1e-6) || total_slots >= (1LL << 31) - 64) return cudaSuccess;
    // every temporary in one owner, freed on every return path
    struct Tmp {
        int* ext = nullptr;
        int* tab = nullptr;
        unsigned* key = nullptr;
        int* n2o = nullptr;
        int* o2n = nullptr;
        unsigned* len = nullptr;
        void* buf = nullptr;
        int* col_new = nullptr;
        LatticeBuffers lb{};
        ~Tmp()
        {
            cudaFree(ext); cudaFree(tab); cudaFree(key); cudaFree(n2o); cudaFree(o2n); cudaFree(len); cudaFree(buf);
            cudaFree(col_new);
            lattice_free(&lb);
        }
    } t;
    const int G = blocks_for(n);
    LT_TRY(cudaMalloc(&t.lb.site, sizeof(int4) * (size_t)n));
    LT_TRY(cudaMalloc(&t.ext, sizeof(int) * 8));
    LT_TRY(cudaMalloc(&t.tab, sizeof(int) * kLatTab * kLatTab * kLatTab));
    int ext_init[8] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 0, 0};
    LT_TRY(cudaMemcpyAsync(t.ext, ext_init, sizeof(ext_init), cudaMemcpyHostToDevice, st));
    LT_TRY(cudaMemsetAsync(t.tab, 0, sizeof(int) * kLatTab * kLatTab * kLatTab, st));
    // the lattice anchor: slot 0's position
    dbl4 anchor;
    LT_TRY(cudaMemcpyAsync(&anchor, x64, sizeof(dbl4), cudaMemcpyDeviceToHost, st));
    LT_TRY(cudaStreamSynchronize(st));
    k_lat_sites<<<G, kBlock, 0, st>>>(x64, n, anchor.x, anchor.y, anchor.z, 1.0 / spacing, t.lb.site, t.ext);
    LT_TRY(cudaGetLastError());
    int ext[8];
    LT_TRY(cudaMemcpyAsync(ext, t.ext, sizeof(ext), cudaMemcpyDeviceToHost, st));
    LT_TRY(cudaStreamSynchronize(st));
    if (ext[6]) return cudaSuccess;   // not a lattice fill
    k_lat_offsets<<<G, kBlock, 0, st>>>(n, t.lb.site, row_ptr, cnt, *col, t.tab, t.ext + 7);
    LT_TRY(cudaGetLastError());
    std::vector<int> tab(kLatTab * kLatTab * kLatTab);
    LT_TRY(cudaMemcpyAsync(tab.data(), t.tab, sizeof(int) * tab.size(), cudaMemcpyDeviceToHost, st));
    LT_TRY(cudaMemcpyAsync(ext, t.ext, sizeof(ext), cudaMemcpyDeviceToHost, st));
    LT_TRY(cudaStreamSynchronize(st));
    if (ext[7]) return cudaSuccess;   // a bond longer than the stencil reach
    // the stencil: offsets in (dz, dy, dx) order
    LatticeParams L{};
    int R = 1;
    std::vector<int> offk(tab.size(), -1);
    std::vector<int3> sten;
    // every offset inside the 80-entry stencil: take that stencil whole (absent
    // offsets get 1/d0 = 0) so that the specialised product applies
    bool in80 = true;
    for (int dz = -kLatRmax; dz <= kLatRmax; ++dz)
        for (int dy = -kLatRmax; dy <= kLatRmax; ++dy)
            for (int dx = -kLatRmax; dx <= kLatRmax; ++dx)
                if (tab[((dz + kLatRmax) * kLatTab + (dy + kLatRmax)) * kLatTab + (dx + kLatRmax)] && !in_s80(dx, dy, dz))
                    in80 = false;
    for (int dz = -kLatRmax; dz <= kLatRmax; ++dz)
        for (int dy = -kLatRmax; dy <= kLatRmax; ++dy)
            for (int dx = -kLatRmax; dx <= kLatRmax; ++dx) {
                const int i = ((dz + kLatRmax) * kLatTab + (dy + kLatRmax)) * kLatTab + (dx + kLatRmax);
                if (in80 ? !in_s80(dx, dy, dz) : !tab[i]) continue;
                if ((int)sten.size() >= kLatMaxK) return cudaSuccess;   // (kLatMaxK is a multiple of 4)
                offk[i] = (int)sten.size();
                sten.push_back(make_int3(dx, dy, dz));
                R = std::max(R, std::max(std::abs(dx), std::max(std::abs(dy), std::abs(dz))));
            }
    L.K = ((int)sten.size() + 3) / 4 * 4;   // padding entries: offset 0 (the row's own site), 1/d0 = 0
    if (in80) R = 2;
    L.R = R;
    L.fixed = in80 ? 1 : 0;
    L.bx = kLatBX;
    L.by = kLatBY;
    L.bz = R <= 2 ? 4 : 2;
    L.hx = L.bx + 2 * R;
    L.hy = L.by + 2 * R;
    L.hz = L.bz + 2 * R;
    for (int k = 0; k < L.K; ++k) {
        const int3 v = k < (int)sten.size() ? sten[k] : make_int3(0, 0, 0);
        L.off[k] = (v.z * L.hy + v.y) * L.hx + v.x;
        L.cx[k] = (float)(spacing * v.x);
        L.cy[k] = (float)(spacing * v.y);
        L.cz[k] = (float)(spacing * v.z);
    }
    // site s (from the minimum site) lies at anchor + h (s + min)
    L.h = spacing;
    L.org[0] = anchor.x + spacing * ext[0];
    L.org[1] = anchor.y + spacing * ext[1];
    L.org[2] = anchor.z + spacing * ext[2];
    const long long D[3] = {(long long)ext[3] - ext[0] + 1, (long long)ext[4] - ext[1] + 1,
                            (long long)ext[5] - ext[2] + 1};
    const long long NB[3] = {(D[0] + L.bx - 1) / L.bx, (D[1] + L.by - 1) / L.by, (D[2] + L.bz - 1) / L.bz};
    const long long M[3] = {NB[0] * L.bx + 2 * R, NB[1] * L.by + 2 * R, NB[2] * L.bz + 2 * R};
    const long long map_size = M[0] * M[1] * M[2];
    const long long bricks_total = NB[0] * NB[1] * NB[2];
    // a dense site map of modest size (the body fills a good part of its box)
    if (map_size > std::max<long long>(16LL * n, 1LL << 22) || map_size >= (1LL << 31) ||
        bricks_total * L.bx * L.by * L.bz >= (1LL << 32))
        return cudaSuccess;
    for (int k = 0; k < 3; ++k) L.map_dim[k] = (int)M[k];
    // brick-major keys, sorted; two particles on one site: not a lattice fill
    LT_TRY(cudaMalloc(&t.key, sizeof(unsigned) * (size_t)n));
    LT_TRY(cudaMalloc(&t.n2o, sizeof(int) * (size_t)n));
    k_lat_keys<<<G, kBlock, 0, st>>>(n, t.lb.site, make_int3(ext[0], ext[1], ext[2]), L.bz,
                                     make_int3((int)NB[0], (int)NB[1], (int)NB[2]), t.key, t.n2o);
    LT_TRY(cudaGetLastError());
    int key_bits = 0;
    while (key_bits < 32 && (1ULL << key_bits) < (unsigned long long)(bricks_total * L.bx * L.by * L.bz)) ++key_bits;
    key_bits = (key_bits + 7) / 8 * 8;
    LT_TRY(sort_pairs_u32(t.key, t.n2o, n, std::max(key_bits, 8), st));
    LT_TRY(cudaMemsetAsync(t.ext + 7, 0, sizeof(int), st));
    k_lat_dups<<<G, kBlock, 0, st>>>(t.key, n, t.ext + 7);
    LT_TRY(cudaMemcpyAsync(ext + 7, t.ext + 7, sizeof(int), cudaMemcpyDeviceToHost, st));
    std::vector<unsigned> keys(n);
    LT_TRY(cudaMemcpyAsync(keys.data(), t.key, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToHost, st));
    LT_TRY(cudaStreamSynchronize(st));
    if (ext[7]) return cudaSuccess;
    // ---- from here on the particles are renumbered: no more early returns ----
    LT_TRY(cudaMalloc(&t.o2n, sizeof(int) * (size_t)n));
    LT_TRY(cudaMalloc(&t.len, sizeof(unsigned) * ((size_t)n + 1)));
    LT_TRY(cudaMalloc(&t.buf, sizeof(dbl4) * (size_t)n));
    k_lat_inverse<<<G, kBlock, 0, st>>>(t.n2o, t.o2n, n);
    k_lat_gather<dbl4><<<G, kBlock, 0, st>>>(x64, t.n2o, (dbl4*)t.buf, n);
    LT_TRY(cudaMemcpyAsync(x64, t.buf, sizeof(dbl4) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    k_lat_gather<float4><<<G, kBlock, 0, st>>>(X32, t.n2o, (float4*)t.buf, n);
    LT_TRY(cudaMemcpyAsync(X32, t.buf, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    k_lat_gather<int4><<<G, kBlock, 0, st>>>(t.lb.site, t.n2o, (int4*)t.buf, n);
    LT_TRY(cudaMemcpyAsync(t.lb.site, t.buf, sizeof(int4) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    k_lat_gather<int><<<G, kBlock, 0, st>>>(perm, t.n2o, (int*)t.buf, n);
    LT_TRY(cudaMemcpyAsync(perm, t.buf, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    k_lat_gather<int><<<G, kBlock, 0, st>>>(cnt, t.n2o, (int*)t.buf, n);
    LT_TRY(cudaMemcpyAsync(cnt, t.buf, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    // CSR: rows keep their padded lengths and bond order; columns renamed
    k_lat_lengths<<<G, kBlock, 0, st>>>(row_ptr, t.n2o, t.len, n);
    LT_TRY(scan_exclusive_u32(t.len, t.len, (long long)n + 1, st));
    LT_TRY(cudaMalloc(&t.col_new, sizeof(int) * ((size_t)total_slots + 8)));
    LT_TRY(cudaMemsetAsync(t.col_new, 0, sizeof(int) * ((size_t)total_slots + 8), st));
    k_lat_remap_col<<<G, kBlock, 0, st>>>(row_ptr, *col, t.len, t.n2o, t.o2n, t.col_new, n);
    LT_TRY(cudaMemcpyAsync(row_ptr, t.len, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
    LT_TRY(cudaGetLastError());
    std::swap(*col, t.col_new);   // the old column array is freed with the temporaries
    // bricks, each row's halo index, the site map and the stencil lookup
    const unsigned bsz = (unsigned)(L.bx * L.by * L.bz);
    std::vector<int> bstart, bcorner, rlocal(n), rbrick(n);
    for (int i = 0; i < n; ++i) {
        const unsigned brick = keys[i] / bsz, local = keys[i] % bsz;
        if (i == 0 || brick != keys[i - 1] / bsz) {
            bstart.push_back(i);
            const long long bxi = brick % NB[0], byi = (brick / NB[0]) % NB[1], bzi = brick / (NB[0] * NB[1]);
            bcorner.push_back((int)(((bzi * L.bz) * M[1] + byi * L.by) * M[0] + bxi * L.bx));
        }
        const int lx = (int)(local % L.bx), ly = (int)((local / L.bx) % L.by), lz = (int)(local / (L.bx * L.by));
        rlocal[i] = ((lz + R) * L.hy + (ly + R)) * L.hx + (lx + R);
        rbrick[i] = (int)bstart.size() - 1;
    }
    L.n_bricks = (int)bstart.size();
    bstart.push_back(n);
    LT_TRY(cudaMalloc(&t.lb.brick_start, sizeof(int) * bstart.size()));
    LT_TRY(cudaMalloc(&t.lb.brick_corner, sizeof(int) * bcorner.size()));
    LT_TRY(cudaMalloc(&t.lb.row_local, sizeof(int) * (size_t)n));
    LT_TRY(cudaMalloc(&t.lb.row_brick, sizeof(int) * (size_t)n));
    LT_TRY(cudaMalloc(&t.lb.map, sizeof(int) * (size_t)map_size));
    LT_TRY(cudaMalloc(&t.lb.offk, sizeof(int) * offk.size()));
    LT_TRY(cudaMalloc(&t.lb.ell, sizeof(float) * (size_t)L.K * (size_t)n));
    LT_TRY(cudaMalloc(&t.lb.dl, sizeof(float4) * (size_t)n));
    LT_TRY(cudaMemsetAsync(t.lb.dl, 0, sizeof(float4) * (size_t)n, st));
    LT_TRY(cudaMalloc(&t.lb.sched, sizeof(unsigned) * 2));
    LT_TRY(cudaMemsetAsync(t.lb.sched, 0, sizeof(unsigned) * 2, st));
    LT_TRY(cudaMemcpyAsync(t.lb.brick_start, bstart.data(), sizeof(int) * bstart.size(), cudaMemcpyHostToDevice, st));
    LT_TRY(cudaMemcpyAsync(t.lb.brick_corner, bcorner.data(), sizeof(int) * bcorner.size(), cudaMemcpyHostToDevice, st));
    LT_TRY(cudaMemcpyAsync(t.lb.row_local, rlocal.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
    LT_TRY(cudaMemcpyAsync(t.lb.row_brick, rbrick.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
    LT_TRY(cudaMemcpyAsync(t.lb.offk, offk.data(), sizeof(int) * offk.size(), cudaMemcpyHostToDevice, st));
    LT_TRY(cudaMemsetAsync(t.lb.map, 0xff, sizeof(int) * (size_t)map_size, st));
    k_lat_map<<<G, kBlock, 0, st>>>(t.lb.site, n, R, (int)M[0], (int)M[1], t.lb.map);
    LT_TRY(cudaGetLastError());
    LT_TRY(cudaStreamSynchronize(st));   // the host vectors above are read by the copies
    L.brick_start = t.lb.brick_start;
    L.brick_corner = t.lb.brick_corner;
    L.row_local = t.lb.row_local;
    L.row_brick = t.lb.row_brick;
    L.site = t.lb.site;
    L.map = t.lb.map;
    L.offk = t.lb.offk;
    L.ell = t.lb.ell;
    L.dl = t.lb.dl;
    L.sched = t.lb.sched;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    L.grid = std::max(1, std::min(L.n_bricks, lattice_spmv_blocks_per_sm(L) * sms));
    *lp = L;
    *lb = t.lb;
    t.lb = LatticeBuffers{};
    *ok = 1;
    return cudaGetLastError();
}

}  // namespace pdgb
