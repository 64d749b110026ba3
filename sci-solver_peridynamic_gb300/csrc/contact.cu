// contact.cu -- PD-PD contact: a short-range repulsion between any two
// particles closer than a contact distance, bonded or not (the reference's
// collectPDParticles / collidePDParticles, src/core/simulator.cuh:606-768,
// compiled out there with #if 0 at simulator.cu:410-426 and 581-597; here an
// option, off by default).
//
// For each particle p and every other particle q with 0 < r = |x_p - x_q| <
// d_c (FP64, start-of-step positions):
//     f_p += (K_c (r - d_c)^2 / V) (x_p - x_q) / r
// added to p's force after the force pass (it enters the right-hand side;
// no Jacobian term), skipped when |f_p| <= 1e-10, as the reference does.
//
// Neighbours come from a spatial hash of cell edge d_c rebuilt every step:
// counts per bucket, a prefix sum, then the particles of each bucket; a
// particle scans the buckets of the 27 cells around it (each bucket once).
// The reference hashes into num_pd_particle lists of at most 128 entries,
// dropping particles of an overflowing list and visiting a list twice when
// two of the 27 cells hash to it; here no particle is dropped and each pair
// counts once.  Contributions are summed in neighbour-slot order, so the
// result does not depend on the order atomics filled the buckets.
#include "pd_device.cuh"
#include "pd_kernels.h"
#include "step_rows.cuh"

namespace pdgb {

namespace {

constexpr unsigned kP1 = 73856093u, kP2 = 19349663u, kP3 = 83492791u;
constexpr int kMaxContacts = 64;

__device__ __forceinline__ void cell_of(const dbl4& x, double inv_d, long long c[3])
{
    c[0] = (long long)floor(x.x * inv_d);
    c[1] = (long long)floor(x.y * inv_d);
    c[2] = (long long)floor(x.z * inv_d);
}

__device__ __forceinline__ unsigned bucket_of(long long cx, long long cy, long long cz, unsigned mask)
{
    return (((unsigned)cx * kP1) ^ ((unsigned)cy * kP2) ^ ((unsigned)cz * kP3)) & mask;
}

__global__ void k_contact_count(const DeviceState S, int n, double inv_d, unsigned mask, unsigned* counts,
                                unsigned* bucket)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        if ((S.act[p] & kActMask) == ACT_INVISIBLE) {
            bucket[p] = 0xffffffffu;
            continue;
        }
        long long c[3];
        cell_of(S.x64[p], inv_d, c);
        const unsigned b = bucket_of(c[0], c[1], c[2], mask);
        bucket[p] = b;
        atomicAdd(counts + b, 1u);
    }
}

__global__ void k_contact_fill(int n, const unsigned* bucket, unsigned* cursor, int* list)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const unsigned b = bucket[p];
        if (b == 0xffffffffu) continue;
        list[atomicAdd(cursor + b, 1u)] = p;
    }
}

template <bool FP64>
__global__ void k_contact_force(const DeviceState S, int n, double dc, double inv_d, double kc, double vol,
                                unsigned mask, const unsigned* start, const int* list)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    V4* force = (V4*)S.force;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        if ((S.act[p] & kActMask) == ACT_INVISIBLE) continue;
        const dbl4 xp = S.x64[p];
        long long c[3];
        cell_of(xp, inv_d, c);
        unsigned seen[27];
        int nseen = 0;
        int qs[kMaxContacts];
        double fs[kMaxContacts][3];
        int nc = 0;
        double fx = 0.0, fy = 0.0, fz = 0.0;   // beyond kMaxContacts: summed in scan order
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const unsigned b = bucket_of(c[0] + dx, c[1] + dy, c[2] + dz, mask);
                    bool dup = false;
                    for (int k = 0; k < nseen; ++k) dup = dup || seen[k] == b;
                    if (dup) continue;
                    seen[nseen++] = b;
                    for (unsigned k = start[b]; k < start[b + 1]; ++k) {
                        const int q = list[k];
                        if (q == p) continue;
                        const dbl4 xq = S.x64[q];
                        const double px = dsub(xp.x, xq.x), py = dsub(xp.y, xq.y), pz = dsub(xp.z, xq.z);
                        const double r = dsqrt(dadd(dadd(dmul(px, px), dmul(py, py)), dmul(pz, pz)));
                        if (r >= dc || r == 0.0) continue;
                        const double howfar = dsub(r, dc);
                        const double mag = ddiv(dmul(kc, dmul(howfar, howfar)), vol);
                        const double gx = dmul(mag, ddiv(px, r)), gy = dmul(mag, ddiv(py, r)), gz = dmul(mag, ddiv(pz, r));
                        if (nc < kMaxContacts) {
                            // insertion by slot: the sum below runs in neighbour order
                            int at = nc++;
                            while (at > 0 && qs[at - 1] > q) {
                                qs[at] = qs[at - 1];
                                fs[at][0] = fs[at - 1][0]; fs[at][1] = fs[at - 1][1]; fs[at][2] = fs[at - 1][2];
                                --at;
                            }
                            qs[at] = q;
                            fs[at][0] = gx; fs[at][1] = gy; fs[at][2] = gz;
                        } else {
                            fx = dadd(fx, gx); fy = dadd(fy, gy); fz = dadd(fz, gz);
                        }
                    }
                }
        if (nc == 0 && fx == 0.0 && fy == 0.0 && fz == 0.0) continue;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int k = 0; k < nc; ++k) {
            sx = dadd(sx, fs[k][0]);
            sy = dadd(sy, fs[k][1]);
            sz = dadd(sz, fs[k][2]);
        }
        sx = dadd(sx, fx); sy = dadd(sy, fy); sz = dadd(sz, fz);
        if (!(dsqrt(dadd(dadd(dmul(sx, sx), dmul(sy, sy)), dmul(sz, sz))) > 1e-10)) continue;
        V4 f = force[p];
        f.x = (Real)((double)f.x + sx);
        f.y = (Real)((double)f.y + sy);
        f.z = (Real)((double)f.z + sz);
        force[p] = f;
    }
}

}  // namespace

cudaError_t launch_contact(bool fp64, const DeviceState& S, int n, const ContactParams& C, const ContactBuffers& B,
                           cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const unsigned mask = B.buckets - 1u;
    const double inv_d = 1.0 / C.distance;
    const int grid = (int)std::min<long long>(((long long)n + kBlock - 1) / kBlock, 65535LL * 8);
    cudaError_t e = cudaMemsetAsync(B.counts, 0, sizeof(unsigned) * (B.buckets + 1), st);
    if (e != cudaSuccess) return e;
    k_contact_count<<<grid, kBlock, 0, st>>>(S, n, inv_d, mask, B.counts, B.bucket);
    e = scan_exclusive_u32(B.counts, B.start, (long long)B.buckets + 1, st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(B.cursor, B.start, sizeof(unsigned) * B.buckets, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    k_contact_fill<<<grid, kBlock, 0, st>>>(n, B.bucket, B.cursor, B.list);
    if (fp64)
        k_contact_force<true><<<grid, kBlock, 0, st>>>(S, n, C.distance, inv_d, C.stiffness, C.volume, mask, B.start,
                                                       B.list);
    else
        k_contact_force<false><<<grid, kBlock, 0, st>>>(S, n, C.distance, inv_d, C.stiffness, C.volume, mask,
                                                        B.start, B.list);
    return cudaGetLastError();
}

}  // namespace pdgb
