// mesh.h -- lattice fill of a closed triangle mesh (mesh_fill.cu, scene.cpp).
#pragma once

#include <cuda_runtime.h>

namespace pdgb {

struct MeshGrid {
    const double* vtx;     // 3 per vertex (transformed)
    const int* tri;        // 3 per triangle
    const int* bin_start;  // xy bins: triangles of bin b are bin_tri[bin_start[b] .. bin_start[b+1])
    const int* bin_tri;
    int bins_x, bins_y;
    double bin_x0, bin_y0, bin_inv_w, bin_inv_h;
    double box_lo[3], box_hi[3];   // bounding box of the triangles' vertices
    // lattice: point (x, y, z) = lat_min + (x, y, z) * spacing + jitter
    double lat_min[3];
    double spacing;
    int nx, ny, nz;
    const double* jitter;  // 3 offsets per lattice point, or null
    double clamp_lo[3], clamp_hi[3];   // position correction of fillParticlesToMesh
};

cudaError_t mesh_fill(const MeshGrid& M, double** d_out, long long* count, cudaStream_t st);

}  // namespace pdgb
