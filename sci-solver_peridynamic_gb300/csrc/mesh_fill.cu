// mesh_fill.cu -- lattice points inside a closed triangle mesh, on the GPU.
//
// The reference fills its example scene on the host (Scene::fillParticlesToMesh,
// src/examples/scene.cpp:537-598): every point of a regular lattice over the
// mesh's bounding box is tested with mesh_query's point_inside_mesh (Robert
// Bridson's mesh_query 0.1, shipped in src/examples/mesh_query0.1: a ray cast
// along +z, the parity of the triangles crossed decides, with exact
// orientation predicates and half-open rules for rays through edges and
// vertices so that every crossing is counted exactly once).  Here one thread
// tests one lattice point against the triangles of its xy bin (the only ones
// a +z ray from it can cross), with the same decision rules evaluated by
// exact predicates, and a prefix sum keeps the inside points in lattice order.
#include "pd_device.cuh"
#include "pd_kernels.h"
#include "predicates.cuh"
#include "mesh.h"

namespace pdgb {

namespace {

// Does the ray from p along +z cross triangle q, r, s (counterclockwise in xy)?
// The decision rules of mesh_query's tri_zcast_inner (mesh_query.cpp): no
// crossing when p is on or above the triangle; strictly inside the xy
// projection: a crossing; on an edge or a vertex: a crossing for exactly one
// of the triangles sharing it, chosen by the edge's / vertex's y (then x) order.
__device__ bool zcast_inner(const double* p, const double* q, const double* r, const double* s)
{
    if (pred::orient3d(p, q, r, s) >= 0) return false;
    const int pqr = pred::orient2d(p, q, r);
    if (pqr < 0) return false;
    const int prs = pred::orient2d(p, r, s);
    if (prs < 0) return false;
    const int psq = pred::orient2d(p, s, q);
    if (psq < 0) return false;
    if (pqr > 0 && prs > 0 && psq > 0) return true;
    auto edge_rule = [](const double* a, const double* b) {
        if (a[1] < b[1]) return false;
        if (a[1] > b[1]) return true;
        return a[0] < b[0];
    };
    if (pqr == 0 && prs > 0 && psq > 0) return edge_rule(q, r);
    if (prs == 0 && pqr > 0 && psq > 0) return edge_rule(r, s);
    if (psq == 0 && pqr > 0 && prs > 0) return edge_rule(s, q);
    if (p[0] == q[0] && p[1] == q[1]) return q[1] >= r[1] && q[1] < s[1];
    if (p[0] == r[0] && p[1] == r[1]) return r[1] >= s[1] && r[1] < q[1];
    if (p[0] == s[0] && p[1] == s[1]) return s[1] >= q[1] && s[1] < r[1];
    return false;
}

__device__ bool zcast(const double* p, const double* q, const double* r, const double* s)
{
    const int qrs = pred::orient2d(q, r, s);
    if (qrs > 0) return zcast_inner(p, q, r, s);
    if (qrs < 0) return zcast_inner(p, q, s, r);
    return false;   // degenerate in the xy projection
}

__device__ __forceinline__ int bin_of(double v, double v0, double inv, int nb)
{
    const double t = __dmul_rn(__dsub_rn(v, v0), inv);
    int b = (int)floor(t);
    return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

__global__ void k_mesh_inside(MeshGrid M, unsigned* flags)
{
    const long long total = (long long)M.nx * M.ny * M.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % M.nx);
        const int y = (int)((i / M.nx) % M.ny);
        const int z = (int)(i / ((long long)M.nx * M.ny));
        double p[3];
        const int c[3] = {x, y, z};
        for (int k = 0; k < 3; ++k) {
            p[k] = __dadd_rn(M.lat_min[k], __dmul_rn((double)c[k], M.spacing));
            if (M.jitter) p[k] = __dadd_rn(p[k], M.jitter[3 * i + k]);
        }
        bool inside = false;
        if (M.box_lo[0] <= p[0] && p[0] <= M.box_hi[0] && M.box_lo[1] <= p[1] && p[1] <= M.box_hi[1] &&
            M.box_lo[2] <= p[2] && p[2] <= M.box_hi[2]) {
            const int bx = bin_of(p[0], M.bin_x0, M.bin_inv_w, M.bins_x);
            const int by = bin_of(p[1], M.bin_y0, M.bin_inv_h, M.bins_y);
            const int b = by * M.bins_x + bx;
            int crossings = 0;
            for (int k = M.bin_start[b]; k < M.bin_start[b + 1]; ++k) {
                const int t = M.bin_tri[k];
                const double* q = M.vtx + 3 * M.tri[3 * t];
                const double* r = M.vtx + 3 * M.tri[3 * t + 1];
                const double* s = M.vtx + 3 * M.tri[3 * t + 2];
                // the ray misses triangles below p or beside it (mesh_query's box_zcast)
                if (fmax(q[2], fmax(r[2], s[2])) < p[2]) continue;
                if (zcast(p, q, r, s)) ++crossings;
            }
            inside = (crossings & 1) != 0;
        }
        flags[i] = inside ? 1u : 0u;
    }
}

__global__ void k_mesh_emit(MeshGrid M, const unsigned* flags, const unsigned* offs, double* out)
{
    const long long total = (long long)M.nx * M.ny * M.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        if (!flags[i]) continue;
        const int c[3] = {(int)(i % M.nx), (int)((i / M.nx) % M.ny), (int)(i / ((long long)M.nx * M.ny))};
        double* o = out + 4 * (size_t)offs[i];
        for (int k = 0; k < 3; ++k) {
            double v = __dadd_rn(M.lat_min[k], __dmul_rn((double)c[k], M.spacing));
            if (M.jitter) v = __dadd_rn(v, M.jitter[3 * i + k]);
            v = v < M.clamp_lo[k] ? M.clamp_lo[k] : v;
            v = v > M.clamp_hi[k] ? M.clamp_hi[k] : v;
            o[k] = v;
        }
        o[3] = 0.0;
    }
}

}  // namespace

// Tests every lattice point of M (device pointers in M), writes the inside
// points' positions (double4, lattice order) to a device buffer allocated
// here (*d_out, caller frees) and their number to *count.
cudaError_t mesh_fill(const MeshGrid& M, double** d_out, long long* count, cudaStream_t st)
{
    *d_out = nullptr;
    *count = 0;
    const long long total = (long long)M.nx * M.ny * M.nz;
    if (total <= 0) return cudaSuccess;
    if (total >= (1ll << 31)) return cudaErrorInvalidValue;
    unsigned* flags = nullptr;
    unsigned* offs = nullptr;
    cudaError_t e = cudaMalloc((void**)&flags, sizeof(unsigned) * (size_t)(total + 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&offs, sizeof(unsigned) * (size_t)(total + 1));
    const int grid = (int)std::min<long long>((total + kBlock - 1) / kBlock, 65535LL * 8);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags + total, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) {
        k_mesh_inside<<<grid, kBlock, 0, st>>>(M, flags);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = scan_exclusive_u32(flags, offs, total + 1, st);
    unsigned n = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n, offs + total, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && n > 0) e = cudaMalloc((void**)d_out, sizeof(double) * 4 * (size_t)n);
    if (e == cudaSuccess && n > 0) {
        k_mesh_emit<<<grid, kBlock, 0, st>>>(M, flags, offs, *d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(flags);
    cudaFree(offs);
    if (e == cudaSuccess) *count = n;
    return e;
}

}  // namespace pdgb
