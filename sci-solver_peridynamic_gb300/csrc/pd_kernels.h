// pd_kernels.h -- host-visible interface between the engine and the CUDA kernels.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pdgb {

constexpr int kBlock = 256;          // threads per block of the per-particle kernels
constexpr int kMaxPartials = 4096;   // upper bound on blocks of a reducing launch

// 32-byte aligned FP64 4-vector (CUDA 13 deprecates the unaligned double4).
struct __align__(32) dbl4 {
    double x, y, z, w;
};
__host__ __device__ inline dbl4 make_dbl4(double x, double y, double z, double w)
{
    dbl4 v;
    v.x = x; v.y = y; v.z = z; v.w = w;
    return v;
}

// Activity byte: low 3 bits = pd_activity, bit 3 = in contact with the sphere
// during the current step (set by the force pass, read by the SpMV).
constexpr int kTileRows = 256;      // rows per tile of the shared-memory SpMV
constexpr int kMaxHaloCap = 2048;   // halo entries a tile may stage (64 KB of shared memory)
constexpr uint8_t kActMask = 7;
constexpr uint8_t kActContact = 8;

// Scalars of the device-resident CG (one instance per handle, device memory).
struct CgScalars {
    double bnorm2;     // ||P b||^2 over free rows
    double tol;        // rel_tol * ||P b||
    double rz;         // <r, r>
    double pAp;        // <p, A p>
    double alpha;
    double beta;
    double rnorm;      // sqrt(rz) at the last check
    double rel_tol;
    int iter;
    int done;
    int converged;
    int max_iter;
    double rr;             // preconditioned CG: <r, r> of the stopping test (rz is then <r, z>)
    double rz_plain;       // <r, r> of the previous-solution guess (learned warm start)
    double rz_learned;     // <r, r> of the learned guess
    int ws_revert;         // 1: the learned guess was worse and was replaced
    int ws_kept;           // learned guesses kept so far
    int ws_rejects;        // batch: consecutive rejected guesses (and paused steps since)
    int ws_skip;           // batch: 1 while this step's learned pass is paused
    int ws_skipped;        // batch: steps whose learned pass was paused
};

// Partial-sum scratch of a reducing launch: one double per block and an
// arrival counter that is zero before the launch (the last block resets it).
struct ReduceSlot {
    double* partials;
    unsigned int* counter;
};

// Per-step constants, passed by value to the step kernels.
struct StepParams {
    int n;
    int integrator;            // 0 implicit Euler, 1 Newmark-beta
    int ticks;                 // pd_time_step
    int box_enabled;
    int sphere_on;
    double cs;                 // clockScale
    double bond_coeff;         // c: pd_C_times_V * PD_K or override
    double horizon, radius;
    double vs_threshold;       // horizon - radius
    double mass;
    double dt_base;
    double h;                  // ticks * dt_base
    double t2;                 // h^2 (IE) or h^2/4 (Newmark)
    double gravity[3];
    double stretch_a, stretch_b, alpha;
    double bmin[3], bmax[3];
    double restitution;
    double sphere_c[3];        // centre at the start of this step (absolute coordinates)
    double sphere_c_local[3];  // same, relative to the FP32 coordinate origin
    double sphere_r, sphere_k;
    // supercells of edge sup (a power of two >= horizon) anchored at sup_lo:
    // x = sup_lo + sup * ijk + offset, ijk in [0, 1023]^3
    double sup_lo[3];
    double sup, inv_sup;
};

// Device pointers of one handle (particles in cell-sorted order).
struct DeviceState {
    int n;
    uint8_t* act;
    dbl4* x64;      // positions (FP64 master)
    dbl4* v64;      // velocities (FP64 master)
    dbl4* X64;      // original positions
    dbl4* x64_bk;
    dbl4* v64_bk;
    double* st;        // pd_stretch
    double* ost;       // pd_original_stretch
    double* nst;       // pd_new_stretch
    float4* lim;       // mixed: limits of the squared break test per particle (limit_pair of st), double-float
    int* row_ptr;      // CSR row starts (32-byte aligned rows), n+1
    int* cnt;          // live bonds per particle (pd_bond_list_top + 1)
    int* cnt_bk;
    int* col;          // neighbour slots
    float4* X32;       // original positions relative to origin (mixed)
    float4* u32;       // displacement x - X (mixed)
    float4* xs4;       // mixed: position as FP32 offset in its supercell, w = packed supercell coords
    float4* xlo4;      // mixed: the offset's low-order FP32 word (double-float with xs4)
    float* inv_d0;     // mixed: 1 / |X_q - X_p| per bond slot (from FP64)
    float2* d0sq;      // mixed: |X_p - X_q|^2 per bond slot, formed as the reference's stretch test forms it,
                       // as a double-float pair
    // mixed mode, tiles of tile_rows consecutive rows for the shared-memory
    // SpMV: halo[halo_ptr[t] .. halo_ptr[t+1]) = sorted distinct neighbour
    // slots of tile t's rows; lidx[slot] = the bond's neighbour as an index
    // into its tile's halo (swapped with col on breakage); tile_info[t] = halo
    // size, or -1 when the tile's halo did not fit the builder's hash set
    uint16_t* lidx;
    int* halo;
    int* halo_ptr;
    int* tile_info;
    int tile_rows;
    int n_tiles;
    int halo_cap;          // halo entries staged in shared memory (larger tiles use the global path)
    double* tile_partials; // one FP64 partial per tile
    unsigned* tile_ctr;    // [0] next tile, [1] arrivals (zero between launches)
    double* jac;       // FP64 mode: symmetric bond Jacobians, 6 per bond slot
    double* jdiag;     // FP64 mode: 6 per particle (sum of bond Jacobians + contact)
    void* force;       // Real4 per particle: pd_force
    void* rhs;         // Real4: b
    void* sol;         // Real4: x (pd_system_solution)
    void* r;           // Real4
    void* p;           // Real4
    void* y;           // Real4
    void* z;           // Real4: preconditioned residual M^-1 r (preconditioner on)
    void* pc;          // Real4 x 2 per particle: M^-1, the inverse diagonal block of A
                       // (m00 m11 m22 m01 | m02 m12 0 0)
    CgScalars* sc;
    double* partials;
    unsigned int* counters;  // 8 reduction counters
    int* flags;              // [0] has_broken, [1] broken bonds this pass, [2] overflow
};

// ---- lattice-stencil SpMV (lattice.cu) ---------------------------------------
// Bodies filled on a simple-cubic lattice (the reference's Scene fills every
// body that way, src/examples/scene.cpp:33-135) keep each particle within a
// fraction of a spacing of its lattice site, and every bond joins two sites
// whose offset lies in a small stencil.  For such bodies the slots are
// renumbered brick by brick (bricks of bx x by x bz sites, x fastest), and the
// product runs brick-wise with the brick's halo of sites staged in shared
// memory: a row's neighbour at stencil entry k sits at a fixed shared-memory
// offset, and 1/d0 per (row, stencil entry) streams from a table in which 0
// marks "no live bond" (no particle there, beyond the horizon, or broken).
constexpr int kLatMaxK = 160;        // stencil entries at most
constexpr int kLatticeMinRows = 20000;   // automatic choice: smaller bodies keep the gather product
constexpr int kLatticeOnlyRows = 250000; // automatic choice: larger lattice bodies time only the stencil variants
constexpr int kLatRmax = 3;          // largest offset per axis (sites)
constexpr int kLatTab = 2 * kLatRmax + 1;

struct LatticeParams {
    int K;                    // stencil entries, padded to a multiple of 4 (padding: offset 0, 1/d0 = 0)
    int R;                    // halo width (sites)
    int bx, by, bz;           // brick extent (sites)
    int hx, hy, hz;           // halo extent = brick + 2R
    int n_bricks;
    int grid;                 // blocks of the product
    int fixed;                // 1: the 80-entry stencil of a 2.5-spacing horizon (compile-time offsets)
    int map_dim[3];           // site map extent (bricks + R on each side)
    const int* brick_start;   // n_bricks + 1: slot range of each brick
    const int* brick_corner;  // n_bricks: map index of the halo's first site
    const int* row_local;     // n: halo index of the row's own site
    const int* row_brick;     // n: brick of each slot
    const int4* site;         // n: site coordinates (x, y, z) of each slot, from the map's first site
    const int* map;           // site map: slot or -1
    const int* offk;          // kLatTab^3: stencil entry of an offset, or -1
    unsigned* sched;          // [0] next brick, [1] blocks finished (zero between launches)
    float* ell;               // K per row, brick-major, in chunks of 4 entries:
                              // [K * start_b + (k / 4) * 4 rows_b + 4 l + k % 4]
    float4* dl;               // n, per step: the particle's deviation from its site, x - (org + h site)
                              // = d + sup n (|d| <= sup / 2 per axis): (d.x, d.y, d.z, packed n + 512)
    double org[3];            // position of site (0, 0, 0)
    double h;                 // lattice spacing
    int off[kLatMaxK];        // halo index offset of each stencil entry
    float cx[kLatMaxK], cy[kLatMaxK], cz[kLatMaxK];   // h * (lattice offset) of each stencil entry
};

struct LatticeBuffers {       // device allocations owned by the engine
    int* brick_start = nullptr;
    int* brick_corner = nullptr;
    int* row_local = nullptr;
    int* row_brick = nullptr;
    int4* site = nullptr;
    int* map = nullptr;
    int* offk = nullptr;
    float* ell = nullptr;
    float4* dl = nullptr;
    unsigned* sched = nullptr;
};

// ---- step kernels (step.cu) --------------------------------------------------
struct LaunchCfg {
    int lanes;          // SpMV lanes per particle row (4, 8, 16, 32)
    int unroll;         // SpMV bonds loaded per lane before computing (1, 2, 4)
    int tiled;          // 1: shared-memory tile SpMV (mixed mode)
    int grid_tiles;     // blocks of the tile SpMV
    int grid_bonds;     // SpMV blocks
    int force_lanes;    // force-pass lanes per particle row
    int grid_force;     // force-pass blocks
    int grid_vec;       // blocks for per-particle vector kernels
    int lattice;        // 1: lattice-stencil SpMV (mixed mode, lat set)
    const LatticeParams* lat;
};

// Lattice detection and slot renumbering, after build_bonds (the arrays are
// the builder's, in its slot order, and are permuted in place): returns
// cudaSuccess with *ok = 0 when the particles are not a lattice fill whose
// bonds fit the stencil (nothing is changed then).  spacing: the lattice
// spacing (2 r).  On success fills *lp (without `ell`) and *lb.
cudaError_t lattice_build(int n, double spacing, dbl4* x64, float4* X32, int* perm, int* row_ptr, int* cnt, int** col,
                          long long total_slots, LatticeParams* lp, LatticeBuffers* lb, int* ok, cudaStream_t st);
// 1/d0 table from the live CSR bonds (force = 0: only when the force pass
// reported a broken bond, read from S.flags[1] on the device)
void launch_lattice_ell(const DeviceState& S, const LatticeParams& lp, int force, int grid, cudaStream_t st);
// y = A(in) by the lattice stencil; dot as launch_operator (cg: CG iteration).
// r_in set (a CG iteration): the direction p = r_in + beta in is formed on the
// way in (beta from cg) and written to p_out (a buffer other than in); y = A p.
void launch_spmv_lattice(bool dot, const StepParams& P, const DeviceState& S, const LatticeParams& lp,
                         const void* in, void* out, ReduceSlot slot, CgScalars* cg, double* dot_out,
                         const void* r_in, void* p_out, cudaStream_t st);
// lp.dl from the positions x64 (with the supercell edge sup): after every
// change of the positions the product's operator is taken at
void launch_lattice_delta(const DeviceState& S, const LatticeParams& lp, double sup, cudaStream_t st);
int lattice_spmv_blocks_per_sm(const LatticeParams& lp);
size_t lattice_smem_bytes(const LatticeParams& lp);
void lattice_free(LatticeBuffers* lb);

void launch_force(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
void launch_cg_init(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
// y = A(x) (dot = false) or y = A(p) with <p,y> reduced into alpha (dot = true)
void launch_spmv(bool fp64, bool dot, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
// y = A(in) with the reduction slot given by the caller; dot_out (device,
// may be null) receives <in, A in>.  Used by the operator entry points.
void launch_operator(bool fp64, const StepParams& P, const DeviceState& S, int lanes, int grid, const void* in,
                     void* out, ReduceSlot slot, double* dot_out, cudaStream_t st);
void launch_cg_residual(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
// Preconditioned CG (no reference counterpart in use: the reference's
// cusp::precond::diagonal is commented out, simulator.cu:767-769): mode 1 =
// inverse diagonal of A, 2 = inverse 3x3 diagonal blocks; the stopping test
// stays on the unpreconditioned ||r||.
void launch_pc_build(bool fp64, int mode, const StepParams& P, const DeviceState& S, const LaunchCfg& L,
                     cudaStream_t st);
// z = M^-1 r, p = z, rz = <r, z>, rr = <r, r> (after the residual of the guess)
void launch_pcg_start(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
// x += alpha p ; r -= alpha A p ; z = M^-1 r ; rr, rz ; beta = rz'/rz ; test
void launch_cg_axpy_pc(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st,
                       cudaGraphConditionalHandle cond = 0);
// cond: the while node's condition handle when launched inside the CG graph, else 0
void launch_cg_axpy(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st,
                    cudaGraphConditionalHandle cond = 0);
void launch_cg_xpby(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
void launch_update(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
void launch_refresh(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
void launch_bond_geometry(const DeviceState& S, int grid, cudaStream_t st);
// mixed: lim[p] = limit_pair(st[p]) for every particle (after st is set)
void launch_stretch_limits(const DeviceState& S, int grid, cudaStream_t st);
// mixed mode: live bonds of each row reordered from the (g_from, u_from)
// SpMV shape's slot order to (g_to, u_to)'s (u = 1: build order)
void launch_bond_relayout(const DeviceState& S, int grid, int g_from, int u_from, int g_to, int u_to,
                          cudaStream_t st);
// Shared-memory tile SpMV (tiles.cu).  build_tiles fills halo / halo_ptr /
// tile_info / lidx of S (allocating them) for tiles of S.tile_rows rows and
// returns the largest halo in *max_halo.
cudaError_t build_tiles(DeviceState& S, int n, int* max_halo, cudaStream_t st);
void free_tiles(DeviceState& S);
// Tile SpMV: blocks per SM for a shared-memory halo of halo_cap entries, and the launch.
int tile_spmv_blocks_per_sm(int lanes, int unroll, int halo_cap);
void launch_spmv_tiled(bool dot, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st);
cudaError_t scan_exclusive_u32(const unsigned* in, unsigned* out, long long n, cudaStream_t st);
// Stable LSD radix sort of (key, value) pairs on the low key_bits bits, in place.
cudaError_t sort_pairs_u32(unsigned* keys, int* vals, int n, int key_bits, cudaStream_t st);

// PD-PD contact (contact.cu)
struct ContactParams {
    double distance;    // d_c
    double stiffness;   // K_c
    double volume;      // V
};
struct ContactBuffers {
    unsigned buckets;   // power of two
    unsigned* counts;   // buckets + 1
    unsigned* start;    // buckets + 1
    unsigned* cursor;   // buckets
    unsigned* bucket;   // n
    int* list;          // n
};
cudaError_t launch_contact(bool fp64, const DeviceState& S, int n, const ContactParams& C, const ContactBuffers& B,
                           cudaStream_t st);
// Max resident blocks per SM of the SpMV / force kernels (for grid sizing).
int row_kernel_blocks_per_sm(bool fp64, int lanes, int unroll);

// ---- SPH <-> PD collision (sph_coupling.cu) ------------------------------------------
struct SphGrid {              // the reference's uniform grid (calcGridPos, simulator.cuh:61-87)
    double lo[3];             // boundary_min
    double cell;              // cell_size
    int n[3];                 // num_cell_x, y, z
};
struct SphBuffers {           // device scratch of the collision, grown to the largest call
    unsigned* key = nullptr; size_t key_cap = 0;
    int* sorted = nullptr; size_t sorted_cap = 0;
    int* winner = nullptr; size_t winner_cap = 0;
    int* start = nullptr; size_t start_cap = 0;
    int* end = nullptr; size_t end_cap = 0;
    int* hit = nullptr; size_t hit_cap = 0;
    dbl4* vnew = nullptr; size_t vnew_cap = 0;
    int* count = nullptr; size_t count_cap = 0;
    dbl4* pos = nullptr; size_t pos_cap = 0;   // the caller's SPH arrays on the device
    dbl4* vel = nullptr; size_t vel_cap = 0;
};
// d_pos / d_vel: the SPH particles (caller order), corrected in place; the
// PD velocities S.v64 of the particles hit; collided = SPH particles corrected
cudaError_t sph_pd_collide(const DeviceState& S, const int* perm, const SphGrid& g, double min_dist, double m_sph,
                           double m_pd, double slip, int n_sph, dbl4* d_pos, dbl4* d_vel, SphBuffers* b,
                           int* collided, cudaStream_t st);
void sph_buffers_free(SphBuffers* b);

// ---- history-projection initial guess (history.cu) --------------------------------
constexpr int kHistMax = 8;                 // history vectors kept at most
struct HistPtrs { const void* v[kHistMax]; };
// the m x m solve's result, in device memory: coefficients, columns used
// (0: no guess), whether the network's column got a nonzero weight, and <r,r>
// of the previous solution's residual
struct HistSolve {
    double y[kHistMax];
    int used;
    int net_used;
    double rz1;
};
// entries of a Gram pass: 0 -> S = H^T H (upper) then c = H^T r; 1 -> G = H^T W (upper)
int hist_dots_count(int pass);
// the block partials of a Gram pass (blocks x hist_dots_count(pass), a row per block)
void launch_hist_dots(bool fp64, int pass, int n, int m, const HistPtrs& H, const HistPtrs& W, const void* r,
                      double* partials, int blocks, cudaStream_t st);
// the m x m solve on the host (a stream callback): the block partials of both
// Gram passes (blocks x hist_dots_count(0), then blocks x hist_dots_count(1))
// summed in block order, the scalars of x1's residual, the result
struct HistHostSolve {
    int m;
    int blocks;
    int net_col;              // the network's column, or -1
    double rel_tol;
    const double* partials;   // pinned
    const CgScalars* sc;      // pinned
    HistSolve* out;           // pinned
};
void hist_host_solve(const HistHostSolve& a);
// x += H y where out->used > 0
void launch_hist_apply(bool fp64, int n, int m, const HistPtrs& H, const HistSolve* Y, void* x, int blocks,
                       cudaStream_t st);
void launch_hist_push(bool fp64, int n, const uint8_t* act, const void* x, void* dst, int blocks, cudaStream_t st);
// coefficients y of x1 + H y (Galerkin over the well-conditioned part of span
// H); returns the number of history columns used, 0 for no guess (host,
// history.cu).
int hist_solve(int m, const double* S_up, const double* G_up, const double* c, double rel_tol, double* y);
int force_kernel_blocks_per_sm(bool fp64, int lanes);
void launch_operator_u(bool fp64, const StepParams& P, const DeviceState& S, int lanes, int unroll, int grid,
                       const void* in, void* out, ReduceSlot slot, double* dot_out, cudaStream_t st);

// ---- bond construction kernels (bonds.cu) --------------------------------------
struct BondBuildOut {
    int* perm;        // slot -> original index (device, n)
    int* row_ptr;     // device, n+1
    int* col;         // device, allocated by the builder (cudaMalloc), caller frees
    int* cnt;         // device, n
    long long total;  // padded bond slots
    long long bonds;  // live bonds
    int max_bonds;    // largest row
    int overflow;     // 1 if some row exceeded max_bonds
};

// Sorts particles by Morton cell key and builds the CSR bond list over the
// exact predicate sqrt((a-b).(a-b)) < horizon.  pos_orig: n dbl4 in caller
// order (device).  Writes the sorted positions to pos_sorted (n dbl4).
// x32_sorted receives FP32 positions relative to origin (the box centre).
cudaError_t build_bonds(const dbl4* pos_orig, int n, double horizon, int max_bonds,
                        dbl4* pos_sorted, float4* x32_sorted, double origin[3], BondBuildOut* out,
                        cudaStream_t st);

// out[i] = in[perm[i]] for 4-double, 1-double, int32 and uint8 records
void gather_double4(const dbl4* in, const int* perm, dbl4* out, int n, cudaStream_t st);
void gather_double(const double* in, const int* perm, double* out, int n, cudaStream_t st);
void gather_int_to_u8(const int* in, const int* perm, uint8_t* out, int n, cudaStream_t st);
// out[perm[i]] = in[i]
void scatter_double4(const dbl4* in, const int* perm, dbl4* out, int n, cudaStream_t st);
// out[perm[i]] = in[i] for rows of words_per_row 32-bit words
void scatter_words(const void* in, const int* perm, void* out, int words_per_row, int n, cudaStream_t st);
// out[perm[i]] = (x, y, z, 0) of a float4 (is_float) or double4 row
void scatter_to_d4_w0(const void* in, bool is_float, const int* perm, dbl4* out, int n, cudaStream_t st);
// FP32 copies relative to an origin
void make_local32(const dbl4* X, double ox, double oy, double oz, float4* X32, float4* u32, int n,
                  cudaStream_t st);

// ---- learned warm start (mlp.cu, warmstart.cu) -----------------------------------
constexpr int kMlpIn = 64;
constexpr int kMlpHidden = 128;
constexpr int kMlpOut = 3;
constexpr int kMlpOutPad = 8;

struct MlpDev {
    float* params;            // FP32 master parameters (mlp_param_count())
    float* grad;
    float* m1;                // Adam moments
    float* m2;
    __nv_bfloat16* w1b;       // [64 x 128]
    __nv_bfloat16* w2b;       // [128 x 128]
    __nv_bfloat16* w3b;       // [128 x 8] (3 used)
};

struct MlpWork {              // activations for up to `rows` rows
    float* z1;
    float* z2;
    __nv_bfloat16* h1;
    __nv_bfloat16* h2;
    __nv_bfloat16* dy;        // [rows x 8]
    float* dh;
    __nv_bfloat16* dz;
    float* y;                 // [rows x 8]
    long long rows;
};

struct WsScalars {
    double sum_x2, sum_r2, sum_v2;   // over free particles
    int n_free;
};

struct WsState {
    float* diag;                  // n
    float4* dj;                   // n: Jacobi step r / D
    __nv_bfloat16* features;      // n x 64
    float4* hist2;                // solution two steps back
    float4* hist3;                // three steps back
    float4* xsave;                // previous solution (x1) saved before the CG
    __nv_bfloat16* ds_x;          // dataset features (capacity x 64)
    float* ds_t;                  // dataset targets (capacity x 3)
    WsScalars* sc;
    int* free_list;               // slots of the free (non-Dirichlet) particles
    int n_free_host;
    int max_bonds;
};

size_t mlp_param_count();
void mlp_refresh_bf16(MlpDev& m, cudaStream_t st);
void mlp_forward(const MlpDev& m, const __nv_bfloat16* X, int B, MlpWork& ws, float* Y, cudaStream_t st);
// C[M x N] (f32, ldc) = op(A) op(B) (+ C) on tcgen05, op = transpose when ta / tb (mlp_tc.cu)
cudaError_t gemm_tc(bool ta, bool tb, int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B,
                    int ldb, float* C, int ldc, bool accumulate, cudaStream_t st);
// inference only (mlp_tc.cu): all layers in one tcgen05 kernel, Y [B x 8]
cudaError_t mlp_infer_tc(const MlpDev& m, const __nv_bfloat16* X, int B, float* Y, cudaStream_t st);
// 1 if a wait of the tensor-core kernel ran out of time since the last call
int mlp_tc_take_error();
void mlp_backward(const MlpDev& m, const __nv_bfloat16* X, const float* T, int B, MlpWork& ws, const float* Y,
                  double* loss, cudaStream_t st);
void mlp_adam(MlpDev& m, float lr, int t, cudaStream_t st);
cudaError_t mlp_alloc(MlpDev* m, bool training);
void mlp_free(MlpDev* m);
cudaError_t mlp_work_alloc(MlpWork* w, long long rows, bool training);
void mlp_work_free(MlpWork* w);
void mlp_init_params(float* host_params, unsigned seed);

void launch_ws_jacobi(const StepParams& P, const DeviceState& S, const WsState& W, int lanes, int grid,
                      ReduceSlot s0, ReduceSlot s1, ReduceSlot s2, cudaStream_t st);
void launch_ws_features(const StepParams& P, const DeviceState& S, const WsState& W, int grid, cudaStream_t st);
void launch_ws_apply(const StepParams& P, const DeviceState& S, const WsState& W, const float* Y, int grid,
                     cudaStream_t st);
void launch_ws_column(const StepParams& P, const DeviceState& S, const WsState& W, const float* Y, float4* h,
                      int grid, cudaStream_t st);
void launch_ws_collect(const StepParams& P, const DeviceState& S, const WsState& W, int count, int stride, int offset,
                       long long pos, long long cap, cudaStream_t st);
void launch_count_free(const uint8_t* act, int n, int* out, cudaStream_t st);
// learned-guess guard: keep the guess with the smaller residual
void launch_ws_save_plain(const DeviceState& S, cudaStream_t st);
void launch_ws_guard(const StepParams& P, const DeviceState& S, const float4* xsave, const float4* rsave, int grid,
                     cudaStream_t st);

}  // namespace pdgb
