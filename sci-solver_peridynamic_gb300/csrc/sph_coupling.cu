// sph_coupling.cu -- SPH <-> PD collision (the reference's
// collideDifferentParticles, src/core/simulator.cuh:1590-1733, run after the
// PD integration at simulator.cu:1188-1206).
//
// The SPH model itself (density, pressure, SPH integration) is not part of
// this library: the caller owns the SPH particles and passes their positions
// and velocities.  For every SPH particle i whose cell of the reference's
// uniform grid (edge cell_size from boundary_min, num_cell_x/y/z cells) is
// inside the grid, the nearest PD particle j of the 27 cells around it with
// |x_j - x_i| < r_sph + r_pd is found, and then, with e = (x_j - x_i) / |..|:
//   x_i <- x_j - (r_sph + r_pd) e
//   normal parts:     v_in' = v_jn' = (m_i v_in + m_j v_jn) / (m_i + m_j)
//   tangential parts: v_it' = ((m_i + m_j s) v_it + m_j (1 - s) v_jt) / (m_i + m_j)
//                     v_jt' = ((m_j + m_i s) v_jt + m_i (1 - s) v_it) / (m_i + m_j)
// (s = sph_pd_slip), in FP64 in the reference's operation order; the
// distance divisor is rounded to FP32 as the reference's fmaxf does.
//
// Where the reference differs (and why this does not follow it):
//  * it reads the PD velocity as _pdSortedVel[j] with j the scan loop's
//    final index instead of the nearest particle's index (an unrelated or
//    out-of-range entry); here it is the nearest particle's velocity;
//  * several SPH particles hitting one PD particle race on its velocity
//    (the last writer wins); here the SPH particle of the smallest index
//    writes it, and every SPH particle computes its own update from the PD
//    velocity before the call;
//  * it uses the PD positions and velocities sorted at the start of the step;
//    here those of the handle when the call is made (after pd_advance);
//  * equal distances go to the first particle of its scan order; here to the
//    smallest PD index (caller order);
//  * its cell-type filter (findCellParticleType / propagateMixedCell) only
//    skips SPH particles with no PD particle in the 27 cells around them,
//    which find nothing here either.
#include <algorithm>
#include <climits>

#include "pd_device.cuh"
#include "pd_kernels.h"
#include "step_rows.cuh"

namespace pdgb {

namespace {

constexpr double kSmall = 1.0e-10;   // SMALL, src/core/definitions.h:61

// calcGridPos / calcGridHash (simulator.cuh:61-87): -1 outside the grid
__device__ __forceinline__ int grid_cell(const SphGrid& g, double x, double y, double z, int c[3])
{
    c[0] = (int)floor(ddiv(dsub(x, g.lo[0]), g.cell));
    c[1] = (int)floor(ddiv(dsub(y, g.lo[1]), g.cell));
    c[2] = (int)floor(ddiv(dsub(z, g.lo[2]), g.cell));
    if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= g.n[0] || c[1] >= g.n[1] || c[2] >= g.n[2]) return -1;
    return (c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
}

__global__ void __launch_bounds__(kBlock) k_sph_pd_keys(int n, const dbl4* __restrict__ x64, SphGrid g,
                                                        unsigned* __restrict__ key, int* __restrict__ val)
{
    const unsigned none = (unsigned)g.n[0] * g.n[1] * g.n[2];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 x = x64[i];
        int c[3];
        const int h = grid_cell(g, x.x, x.y, x.z, c);
        key[i] = h < 0 ? none : (unsigned)h;
        val[i] = i;
    }
}

__global__ void __launch_bounds__(kBlock) k_sph_pd_ranges(int n, const unsigned* __restrict__ key, unsigned none,
                                                          int* __restrict__ start, int* __restrict__ end)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned k = key[i];
        if (k == none) continue;
        if (i == 0 || key[i - 1] != k) start[k] = i;
        if (i == n - 1 || key[i + 1] != k) end[k] = i + 1;
    }
}

struct SphCollideArgs {
    int n_sph;
    SphGrid g;
    double min_dist;   // r_sph + r_pd
    double mi, mj, slip;
    const dbl4* x64;   // PD positions (slots)
    const dbl4* v64;   // PD velocities (slots)
    const int* perm;   // slot -> caller index
    const int* sorted; // slots by cell
    const int* start;  // per cell, -1 empty
    const int* end;
    dbl4* pos;      // SPH positions (caller order), updated
    dbl4* vel;      // SPH velocities, updated
    int* hit;          // per SPH particle: PD slot, or -1
    dbl4* vnew;     // per SPH particle: the PD particle's new velocity
    int* winner;       // per PD slot: smallest SPH index that hit it (INT_MAX: none)
    int* count;        // SPH particles corrected
};

__global__ void __launch_bounds__(kBlock) k_sph_collide(SphCollideArgs a)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_sph; i += gridDim.x * blockDim.x) {
        a.hit[i] = -1;
        const dbl4 pi = a.pos[i];
        int c[3];
        if (grid_cell(a.g, pi.x, pi.y, pi.z, c) < 0) continue;
        double best = a.min_dist;
        int bj = -1, bcaller = INT_MAX;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int cx = c[0] + dx, cy = c[1] + dy, cz = c[2] + dz;
                    if (cx < 0 || cy < 0 || cz < 0 || cx >= a.g.n[0] || cy >= a.g.n[1] || cz >= a.g.n[2]) continue;
                    const int cell = (cz * a.g.n[1] + cy) * a.g.n[0] + cx;
                    const int s0 = a.start[cell];
                    if (s0 < 0) continue;
                    const int s1 = a.end[cell];
                    for (int t = s0; t < s1; ++t) {
                        const int j = a.sorted[t];
                        const dbl4 pj = a.x64[j];
                        const double ex = dsub(pj.x, pi.x), ey = dsub(pj.y, pi.y), ez = dsub(pj.z, pi.z);
                        const double d = __dsqrt_rn(dadd(dadd(dmul(ex, ex), dmul(ey, ey)), dmul(ez, ez)));
                        const int caller = a.perm[j];
                        if (d < best || (d == best && bj >= 0 && caller < bcaller)) {
                            best = d;
                            bj = j;
                            bcaller = caller;
                        }
                    }
                }
        if (bj < 0) continue;
        const dbl4 pj = a.x64[bj];
        const double D = (double)fmaxf((float)best, (float)kSmall);
        const double e[3] = {ddiv(dsub(pj.x, pi.x), D), ddiv(dsub(pj.y, pi.y), D), ddiv(dsub(pj.z, pi.z), D)};
        const double pjv[3] = {pj.x, pj.y, pj.z};
        const dbl4 vi4 = a.vel[i];
        const dbl4 vj4 = a.v64[bj];
        const double vi[3] = {vi4.x, vi4.y, vi4.z}, vj[3] = {vj4.x, vj4.y, vj4.z};
        const double di = dadd(dadd(dmul(e[0], vi[0]), dmul(e[1], vi[1])), dmul(e[2], vi[2]));
        const double dj = dadd(dadd(dmul(e[0], vj[0]), dmul(e[1], vj[1])), dmul(e[2], vj[2]));
        const double mm = dadd(a.mi, a.mj);
        const double ci = dadd(a.mi, dmul(a.mj, a.slip)), cj = dadd(a.mj, dmul(a.mi, a.slip));
        const double ti = dmul(a.mj, dsub(1.0, a.slip)), tj = dmul(a.mi, dsub(1.0, a.slip));
        double xo[3], vo[3], wo[3];
        for (int k = 0; k < 3; ++k) {
            xo[k] = dsub(pjv[k], dmul(a.min_dist, e[k]));
            const double vin = dmul(e[k], di), vit = dsub(vi[k], vin);
            const double vjn = dmul(e[k], dj), vjt = dsub(vj[k], vjn);
            const double vn2 = ddiv(dadd(dmul(a.mi, vin), dmul(a.mj, vjn)), mm);
            const double vit2 = ddiv(dadd(dmul(ci, vit), dmul(ti, vjt)), mm);
            const double vjt2 = ddiv(dadd(dmul(cj, vjt), dmul(tj, vit)), mm);
            vo[k] = dadd(vn2, vit2);
            wo[k] = dadd(vn2, vjt2);
        }
        a.pos[i] = make_dbl4(xo[0], xo[1], xo[2], pi.w);
        a.vel[i] = make_dbl4(vo[0], vo[1], vo[2], vi4.w);
        a.vnew[i] = make_dbl4(wo[0], wo[1], wo[2], 0.0);
        a.hit[i] = bj;
        atomicMin(a.winner + bj, i);
        atomicAdd(a.count, 1);
    }
}

__global__ void __launch_bounds__(kBlock) k_sph_apply(int n_sph, const int* __restrict__ hit,
                                                      const int* __restrict__ winner, const dbl4* __restrict__ vnew,
                                                      dbl4* __restrict__ v64)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_sph; i += gridDim.x * blockDim.x) {
        const int j = hit[i];
        if (j < 0 || winner[j] != i) continue;
        const dbl4 w = vnew[i];
        v64[j] = make_dbl4(w.x, w.y, w.z, 0.0);
    }
}

int grid_blocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + kBlock - 1) / kBlock, 4096)); }

}  // namespace

cudaError_t sph_pd_collide(const DeviceState& S, const int* perm, const SphGrid& g, double min_dist, double m_sph,
                           double m_pd, double slip, int n_sph, dbl4* d_pos, dbl4* d_vel, SphBuffers* b,
                           int* collided, cudaStream_t st)
{
    const int n = S.n;
    const long long cells = (long long)g.n[0] * g.n[1] * g.n[2];
    if (cells <= 0 || cells >= INT_MAX) return cudaErrorInvalidValue;
    // buffers grow to the largest call
    auto grow = [](void** p, size_t* cap, size_t bytes) -> cudaError_t {
        if (*cap >= bytes) return cudaSuccess;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *cap = 0;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) *cap = bytes;
        return e;
    };
    const size_t np = (size_t)std::max(n, 1), ns = (size_t)std::max(n_sph, 1);
    cudaError_t e;
    if ((e = grow((void**)&b->key, &b->key_cap, sizeof(unsigned) * np)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->sorted, &b->sorted_cap, sizeof(int) * np)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->winner, &b->winner_cap, sizeof(int) * np)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->start, &b->start_cap, sizeof(int) * (size_t)cells)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->end, &b->end_cap, sizeof(int) * (size_t)cells)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->hit, &b->hit_cap, sizeof(int) * ns)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->vnew, &b->vnew_cap, sizeof(dbl4) * ns)) != cudaSuccess) return e;
    if ((e = grow((void**)&b->count, &b->count_cap, sizeof(int))) != cudaSuccess) return e;
    int bits = 1;
    while (bits < 32 && (1ULL << bits) <= (unsigned long long)cells) ++bits;
    if (n > 0) {
        k_sph_pd_keys<<<grid_blocks(n), kBlock, 0, st>>>(n, S.x64, g, b->key, b->sorted);
        if ((e = sort_pairs_u32(b->key, b->sorted, n, bits, st)) != cudaSuccess) return e;
    }
    if ((e = cudaMemsetAsync(b->start, 0xff, sizeof(int) * (size_t)cells, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b->end, 0xff, sizeof(int) * (size_t)cells, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b->winner, 0x7f, sizeof(int) * np, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b->count, 0, sizeof(int), st)) != cudaSuccess) return e;
    if (n > 0) k_sph_pd_ranges<<<grid_blocks(n), kBlock, 0, st>>>(n, b->key, (unsigned)cells, b->start, b->end);
    if (n_sph > 0) {
        SphCollideArgs a{n_sph, g, min_dist, m_sph, m_pd, slip, S.x64, S.v64, perm, b->sorted, b->start, b->end,
                         d_pos, d_vel, b->hit, b->vnew, b->winner, b->count};
        k_sph_collide<<<grid_blocks(n_sph), kBlock, 0, st>>>(a);
        k_sph_apply<<<grid_blocks(n_sph), kBlock, 0, st>>>(n_sph, b->hit, b->winner, b->vnew, S.v64);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int c = 0;
    if ((e = cudaMemcpyAsync(&c, b->count, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if (collided) *collided = c;
    return cudaSuccess;
}

void sph_buffers_free(SphBuffers* b)
{
    void* ptrs[] = {b->key, b->sorted, b->winner, b->start, b->end, b->hit, b->vnew, b->count, b->pos, b->vel};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    *b = SphBuffers{};
}

}  // namespace pdgb
