// step.cu -- the implicit PD step on sm_103a.
//
// One step (reference: Simulator::integratePeridynamicsImplicitEuler /
// NewmarkBeta, src/core/simulator.cu:297-652) is
//   k_force      bond stretch, breakage, force, right-hand side      (cg_solver.cuh:200-339,
//                                                                     implicit_euler.cuh:62-86,
//                                                                     newmark_beta.cuh:62-86)
//   k_cg_init / k_spmv / k_cg_residual                               CG set-up
//   { k_spmv(dot) ; k_cg_axpy ; k_cg_xpby } x iterations              CUSP krylov::cg restated
//   k_update     position / velocity update + box reflection        (implicit_euler.cuh:90-176,
//                                                                     newmark_beta.cuh:89-199)
// The reference assembles A = M + beta h^2 K as 3x3 blocks in a 528-slot
// bond-major array (cg_solver.cuh:307, implicit_euler.cuh:19-59); here the
// mixed-precision path never forms A: k_spmv recomputes each bond's Jacobian
// from the positions inside the product.  The FP64 path stores the six
// independent entries of each symmetric bond Jacobian.
//
// Rows of G lanes ("lanes per particle") walk a particle's CSR row; the
// per-particle sums are shuffled within the group.
#include "step_rows.cuh"

namespace pdgb {

// ---- force / breakage ----------------------------------------------------------
// mixed precision: every particle's supercell words from x64, read by the
// force pass for the particle's own row and as a neighbour
__global__ void __launch_bounds__(kBlock) k_supercell_words(StepParams P, DeviceState S)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        supercell_elem(P, S, i);
}

template <int G, bool FP64>
__global__ void __launch_bounds__(kBlock) k_force(StepParams P, DeviceState S)
{
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    const int stride = gridDim.x * gpb;
    for (int p = blockIdx.x * gpb + threadIdx.x / G; p < P.n; p += stride) force_row<G, FP64>(P, S, p, lane, gmask);
}

// ---- A u: mass + (beta h^2) stiffness, Dirichlet rows projected out --------------
// Mixed precision: per bond, with xi the current bond vector (FP32, from the
// supercell positions) and d0 the reference length, the bond Jacobian applied
// to w = u_p - u_q is
//   c [ (1/d0 - 1/d) w + (xi . w) xi / d^3 ]
// which equals (c/d0)[(1 - d0/d) I + (d0/d) e e^T] w of cg_solver.cuh:292-299.
// DOT: reduce <in, A in>; with `cg` set (CG iteration) the result becomes
// alpha = rz / <p, A p> and the launch is skipped once the CG has finished;
// with `dot_out` set the result is also stored there.
// U: bonds each lane loads before it computes (memory-level parallelism).
// Mixed mode keeps 4 blocks (32 warps) resident per SM: the kernel is
// latency-bound on its gathers, and at 1M particles 64 registers and 4
// blocks beat 73 registers and 3 blocks by 7 % (254 vs 272 us per product).
constexpr int kSpmvMinBlocks = 4;
template <int G, bool FP64, bool DOT, int U>
__global__ void __launch_bounds__(kBlock, FP64 ? 1 : kSpmvMinBlocks) k_spmv(StepParams P, DeviceState S, const void* __restrict__ in_,
                                                  void* __restrict__ out_, ReduceSlot slot, CgScalars* cg,
                                                  double* dot_out)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    using Acc = typename DotAccFor<Real>::type;
    if (DOT && cg && ((volatile CgScalars*)cg)->done) return;
    const V4* __restrict__ in = (const V4*)in_;
    V4* __restrict__ out = (V4*)out_;
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    constexpr int gpb = kBlock / G;
    const int stride = gridDim.x * gpb;
    Acc acc;
    // every group runs the same number of loop trips so that whole blocks reach the reduction
    // Each block walks one contiguous run of rows: consecutive trips touch
    // overlapping neighbourhoods (slots are in Morton cell order), so the
    // gathered data stays in L1 between trips.
    const int trips = (P.n + stride - 1) / stride;
    const int run_begin = blockIdx.x * trips * gpb;
    for (int t = 0; t < trips; ++t) {
        const int p = run_begin + t * gpb + threadIdx.x / G;
        if (p >= P.n) continue;
        spmv_row<G, FP64, DOT, U, kLdReadOnly>(P, S, in, out, p, lane, gmask, acc);
    }
    if (DOT) {
        block_reduce_finish(acc, slot, [cg, dot_out](double pAp) {
            if (cg) cg_fin_alpha(cg, pAp);
            if (dot_out) *dot_out = pAp;
        });
    }
}

// ---- CG vector kernels --------------------------------------------------------------
template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_cg_init(StepParams P, DeviceState S, ReduceSlot slot)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    typename DotAccFor<Real>::type acc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        cg_init_elem<FP64>(P, S, i, acc);
    CgScalars* sc = S.sc;
    block_reduce_finish(acc, slot, [sc](double bb) { cg_fin_init(sc, bb); });
}

// r = b - A x0 (free rows), p = r, rz = <r,r>; convergence test before the first iteration
template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_cg_residual(StepParams P, DeviceState S, ReduceSlot slot)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    typename DotAccFor<Real>::type acc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        residual_elem<FP64>(S, i, acc);
    CgScalars* sc = S.sc;
    block_reduce_finish(acc, slot, [sc](double rr) { cg_fin_residual(sc, rr); });
}

// x += alpha p ; r -= alpha A p ; rz' = <r,r> ; beta = rz'/rz ; test
//
// Inside the CG graph (cond != 0) this kernel also sets the while node's
// condition: its finisher to "not done" after the test, or, when the solve
// had already finished before the launch, block 0 to 0.  Exactly one thread of
// each launch sets it: `done` only changes in the finisher, which runs after
// every block has read it, so all blocks of one launch take the same branch.
template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_cg_axpy(StepParams P, DeviceState S, ReduceSlot slot,
                                                   cudaGraphConditionalHandle cond)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    CgScalars* sc = S.sc;
    if (((volatile CgScalars*)sc)->done) {
        if (cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
        return;
    }
    const Real alpha = (Real)sc->alpha;
    typename DotAccFor<Real>::type acc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        axpy_elem<FP64>(S, i, alpha, acc);
    block_reduce_finish(acc, slot, [sc, cond](double rr) {
        cg_fin_axpy(sc, rr);
        if (cond) cudaGraphSetConditional(cond, sc->done ? 0u : 1u);
    });
}

// p = r + beta p
template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_cg_xpby(StepParams P, DeviceState S)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    const CgScalars* sc = S.sc;
    if (((volatile const CgScalars*)sc)->done) return;
    const Real beta = (Real)sc->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        xpby_elem<FP64>(S, i, beta);
}

// ---- preconditioned CG -----------------------------------------------------------
// FP64: D = m I + t2 jdiag (the bond Jacobians' sum and the contact term, as
// the product uses them); one thread per particle.
__global__ void __launch_bounds__(kBlock) k_pc_build64(StepParams P, DeviceState S, int mode)
{
    dbl4* pc = (dbl4*)S.pc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        double M[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (!is_dirichlet(S.act[i] & kActMask)) {
            const double* J = S.jdiag + 6ll * i;
            const double D[6] = {P.mass + P.t2 * J[0], P.mass + P.t2 * J[1], P.mass + P.t2 * J[2],
                                 P.t2 * J[3], P.t2 * J[4], P.t2 * J[5]};
            pc_invert(mode, P.mass, D, M);
        }
        pc[2 * i] = make_dbl4(M[0], M[1], M[2], M[3]);
        pc[2 * i + 1] = make_dbl4(M[4], M[5], 0.0, 0.0);
    }
}

// Mixed precision: D = m I + t2 (c sum_q [(1/d0 - 1/d) I + xi xi^T / d^3] + k n n^T)
// over the particle's live bonds (the product's bond term, from the same
// supercell positions), G lanes per particle.
template <int G>
__global__ void __launch_bounds__(kBlock) k_pc_build32(StepParams P, DeviceState S, int mode)
{
    const unsigned gmask = group_mask<G>();
    const int lane = threadIdx.x & (G - 1);
    const int groups = gridDim.x * (kBlock / G);
    float4* pc = (float4*)S.pc;
    const float sup = (float)P.sup;
    for (int p = blockIdx.x * (kBlock / G) + threadIdx.x / G; p < P.n; p += groups) {
        const uint8_t ab = S.act[p];
        if (is_dirichlet(ab & kActMask)) {
            if (lane == 0) {
                pc[2 * p] = make_float4(0.f, 0.f, 0.f, 0.f);
                pc[2 * p + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            continue;
        }
        const float4 xp4 = S.xs4[p];
        const int wp = __float_as_int(xp4.w);
        const int rs = S.row_ptr[p];
        const int cn = S.cnt[p];
        float sa = 0.f, sxx = 0.f, syy = 0.f, szz = 0.f, sxy = 0.f, sxz = 0.f, syz = 0.f;
        for (int j = lane; j < cn; j += G) {
            const int q = S.col[rs + j];
            const float4 Xq = S.xs4[q];
            float cx, cy, cz;
            supercell_delta(__float_as_int(Xq.w), wp, sup, cx, cy, cz);
            const float xs = (Xq.x - xp4.x) + cx, ys = (Xq.y - xp4.y) + cy, zs = (Xq.z - xp4.z) + cz;
            const float inv_d = rsqrtf(fmaf(xs, xs, fmaf(ys, ys, zs * zs)));
            const float i3 = inv_d * inv_d * inv_d;
            sa += S.inv_d0[rs + j] - inv_d;
            sxx = fmaf(xs * xs, i3, sxx); syy = fmaf(ys * ys, i3, syy); szz = fmaf(zs * zs, i3, szz);
            sxy = fmaf(xs * ys, i3, sxy); sxz = fmaf(xs * zs, i3, sxz); syz = fmaf(ys * zs, i3, syz);
        }
        sa = group_sum<G>(sa, gmask);
        sxx = group_sum<G>(sxx, gmask); syy = group_sum<G>(syy, gmask); szz = group_sum<G>(szz, gmask);
        sxy = group_sum<G>(sxy, gmask); sxz = group_sum<G>(sxz, gmask); syz = group_sum<G>(syz, gmask);
        if (lane != 0) continue;
        const double c = P.bond_coeff, t2 = P.t2, m = P.mass;
        double D[6] = {m + t2 * c * ((double)sa + sxx), m + t2 * c * ((double)sa + syy),
                       m + t2 * c * ((double)sa + szz), t2 * c * sxy, t2 * c * sxz, t2 * c * syz};
        if (ab & kActContact) {
            const float4 Xp = S.X32[p];
            const float4 Up = S.u32[p];
            const double dx = (double)(Xp.x + Up.x) - P.sphere_c_local[0];
            const double dy = (double)(Xp.y + Up.y) - P.sphere_c_local[1];
            const double dz = (double)(Xp.z + Up.z) - P.sphere_c_local[2];
            const double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
            const double nx = dx * inv, ny = dy * inv, nz = dz * inv, k = t2 * P.sphere_k;
            D[0] += k * nx * nx; D[1] += k * ny * ny; D[2] += k * nz * nz;
            D[3] += k * nx * ny; D[4] += k * nx * nz; D[5] += k * ny * nz;
        }
        double M[6];
        pc_invert(mode, m, D, M);
        pc[2 * p] = make_float4((float)M[0], (float)M[1], (float)M[2], (float)M[3]);
        pc[2 * p + 1] = make_float4((float)M[4], (float)M[5], 0.f, 0.f);
    }
}

template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_pcg_start(StepParams P, DeviceState S, ReduceSlot slot, double* partials_b)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    typename DotAccFor<Real>::type rr, rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        pcg_start_elem<FP64>(S, i, rr, rz);
    CgScalars* sc = S.sc;
    block_reduce_finish2(rr, rz, slot, partials_b, [sc](double a, double b) { cg_fin_pcg_start(sc, a, b); });
}

// as k_cg_axpy (the graph's condition included), with z = M r and <r, z>
template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_cg_axpy_pc(StepParams P, DeviceState S, ReduceSlot slot,
                                                      double* partials_b, cudaGraphConditionalHandle cond)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    CgScalars* sc = S.sc;
    if (((volatile CgScalars*)sc)->done) {
        if (cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
        return;
    }
    const Real alpha = (Real)sc->alpha;
    typename DotAccFor<Real>::type rr, rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        axpy_pc_elem<FP64>(S, i, alpha, rr, rz);
    block_reduce_finish2(rr, rz, slot, partials_b, [sc, cond](double a, double b) {
        cg_fin_axpy_pc(sc, a, b);
        if (cond) cudaGraphSetConditional(cond, sc->done ? 0u : 1u);
    });
}

// ---- position / velocity update ------------------------------------------------
template <bool FP64>
__global__ void __launch_bounds__(kBlock) k_update(StepParams P, DeviceState S)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        update_elem<FP64>(P, S, i);
}

// FP32 displacement from the FP64 master positions (after a rollback restore)
__global__ void __launch_bounds__(kBlock) k_refresh(StepParams P, DeviceState S)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x)
        refresh_elem(P, S, i);
}

// 1 / d0 and d0^2 per bond slot from the FP64 original positions (once, after the bond build)
__global__ void __launch_bounds__(kBlock) k_bond_geometry(int n, DeviceState S)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const dbl4 Xp = S.X64[p];
        const int rs = S.row_ptr[p], cn = S.cnt[p];
        for (int j = 0; j < cn; ++j) {
            const dbl4 Xq = S.X64[S.col[rs + j]];
            const double dx = dsub(Xp.x, Xq.x), dy = dsub(Xp.y, Xq.y), dz = dsub(Xp.z, Xq.z);
            const double d0s = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
            S.inv_d0[rs + j] = (float)(1.0 / sqrt(d0s));
            const F2 w = f2_of(d0s);
            S.d0sq[rs + j] = make_float2(w.h, w.l);
        }
    }
}

void launch_bond_geometry(const DeviceState& S, int grid, cudaStream_t st)
{
    k_bond_geometry<<<grid, kBlock, 0, st>>>(S.n, S);
}

__global__ void __launch_bounds__(kBlock) k_stretch_limits(int n, DeviceState S)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        S.lim[p] = limit_pair(S.st[p]);
}

void launch_stretch_limits(const DeviceState& S, int grid, cudaStream_t st)
{
    k_stretch_limits<<<grid, kBlock, 0, st>>>(S.n, S);
}

// Reorders the live bonds of each row for a (lanes G, unroll U) SpMV shape.
// The SpMV's lane k loads U consecutive slots 16-byte-wise (slots b*GU + kU +
// u, u < U) and gathers their neighbours as U instructions; so that the
// neighbours gathered by one instruction are the row's G consecutive bonds of
// the build order (the build scans neighbour cells, so consecutive bonds are
// close in memory), every full block of GU live slots stores build-order bond
// uG + k at slot kU + u.  `from` undoes a previous shape's order first.  Only
// whole blocks inside [0, cnt) move, so the live set of every row is unchanged.
template <typename T>
__device__ __forceinline__ void permute_block(T* a, int G, int U, bool to_shape)
{
    T t[128];
    const int B = G * U;
    for (int i = 0; i < B; ++i) t[i] = a[i];
    for (int k = 0; k < G; ++k)
        for (int u = 0; u < U; ++u) {
            if (to_shape) a[k * U + u] = t[u * G + k];
            else a[u * G + k] = t[k * U + u];
        }
}

__global__ void __launch_bounds__(kBlock) k_bond_relayout(int n, DeviceState S, int g_from, int u_from, int g_to,
                                                          int u_to)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int rs = S.row_ptr[p], cn = S.cnt[p];
        for (int pass = 0; pass < 2; ++pass) {
            const int G = pass == 0 ? g_from : g_to, U = pass == 0 ? u_from : u_to;
            if (U <= 1 || G * U > 128) continue;
            const int B = G * U;
            for (int b = 0; b + B <= cn; b += B) {
                permute_block(S.col + rs + b, G, U, pass == 1);
                permute_block(S.inv_d0 + rs + b, G, U, pass == 1);
                permute_block(S.d0sq + rs + b, G, U, pass == 1);
                if (S.lidx) permute_block(S.lidx + rs + b, G, U, pass == 1);
            }
        }
    }
}

void launch_bond_relayout(const DeviceState& S, int grid, int g_from, int u_from, int g_to, int u_to,
                          cudaStream_t st)
{
    k_bond_relayout<<<grid, kBlock, 0, st>>>(S.n, S, g_from, u_from, g_to, u_to);
}

// ---- launchers ------------------------------------------------------------------
static ReduceSlot slot_of(const DeviceState& S, int k) { return ReduceSlot{S.partials, S.counters + k}; }

template <int G>
static void force_g(bool fp64, const StepParams& P, const DeviceState& S, int grid, cudaStream_t st)
{
    if (fp64) k_force<G, true><<<grid, kBlock, 0, st>>>(P, S);
    else k_force<G, false><<<grid, kBlock, 0, st>>>(P, S);
}

void launch_force(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (!fp64 && P.n > 0) k_supercell_words<<<L.grid_vec, kBlock, 0, st>>>(P, S);
    // the lattice product's deviations from the same positions
    if (!fp64 && L.lattice && L.lat) launch_lattice_delta(S, *L.lat, P.sup, st);
    switch (L.force_lanes) {
    case 4: force_g<4>(fp64, P, S, L.grid_force, st); break;
    case 16: force_g<16>(fp64, P, S, L.grid_force, st); break;
    case 32: force_g<32>(fp64, P, S, L.grid_force, st); break;
    default: force_g<8>(fp64, P, S, L.grid_force, st); break;
    }
}

template <int G, bool DOT, int U>
static void spmv_g(bool fp64, const StepParams& P, const DeviceState& S, int grid, const void* in, void* out,
                   ReduceSlot slot, CgScalars* cg, double* dot_out, cudaStream_t st)
{
    if (fp64) k_spmv<G, true, DOT, 1><<<grid, kBlock, 0, st>>>(P, S, in, out, slot, cg, dot_out);
    else k_spmv<G, false, DOT, U><<<grid, kBlock, 0, st>>>(P, S, in, out, slot, cg, dot_out);
}

template <bool DOT, int U>
static void spmv_lanes(bool fp64, const StepParams& P, const DeviceState& S, int lanes, int grid, const void* in,
                       void* out, ReduceSlot slot, CgScalars* cg, double* dot_out, cudaStream_t st)
{
    switch (lanes) {
    case 4: spmv_g<4, DOT, U>(fp64, P, S, grid, in, out, slot, cg, dot_out, st); break;
    case 16: spmv_g<16, DOT, U>(fp64, P, S, grid, in, out, slot, cg, dot_out, st); break;
    case 32: spmv_g<32, DOT, U>(fp64, P, S, grid, in, out, slot, cg, dot_out, st); break;
    default: spmv_g<8, DOT, U>(fp64, P, S, grid, in, out, slot, cg, dot_out, st); break;
    }
}

template <bool DOT>
static void spmv_d(bool fp64, const StepParams& P, const DeviceState& S, int lanes, int unroll, int grid,
                   const void* in, void* out, ReduceSlot slot, CgScalars* cg, double* dot_out, cudaStream_t st)
{
    switch (unroll) {
    case 2: spmv_lanes<DOT, 2>(fp64, P, S, lanes, grid, in, out, slot, cg, dot_out, st); break;
    case 4: spmv_lanes<DOT, 4>(fp64, P, S, lanes, grid, in, out, slot, cg, dot_out, st); break;
    default: spmv_lanes<DOT, 1>(fp64, P, S, lanes, grid, in, out, slot, cg, dot_out, st); break;
    }
}

void launch_spmv(bool fp64, bool dot, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (!fp64 && L.lattice && L.lat) {
        if (dot) launch_spmv_lattice(true, P, S, *L.lat, S.p, S.y, slot_of(S, 1), S.sc, nullptr, nullptr, nullptr, st);
        else launch_spmv_lattice(false, P, S, *L.lat, S.sol, S.y, slot_of(S, 1), nullptr, nullptr, nullptr, nullptr, st);
        return;
    }
    if (!fp64 && L.tiled) {
        launch_spmv_tiled(dot, P, S, L, st);
        return;
    }
    if (dot) spmv_d<true>(fp64, P, S, L.lanes, L.unroll, L.grid_bonds, S.p, S.y, slot_of(S, 1), S.sc, nullptr, st);
    else spmv_d<false>(fp64, P, S, L.lanes, L.unroll, L.grid_bonds, S.sol, S.y, slot_of(S, 1), nullptr, nullptr, st);
}

void launch_operator(bool fp64, const StepParams& P, const DeviceState& S, int lanes, int grid, const void* in,
                     void* out, ReduceSlot slot, double* dot_out, cudaStream_t st)
{
    launch_operator_u(fp64, P, S, lanes, 1, grid, in, out, slot, dot_out, st);
}

void launch_operator_u(bool fp64, const StepParams& P, const DeviceState& S, int lanes, int unroll, int grid,
                       const void* in, void* out, ReduceSlot slot, double* dot_out, cudaStream_t st)
{
    if (dot_out) spmv_d<true>(fp64, P, S, lanes, unroll, grid, in, out, slot, nullptr, dot_out, st);
    else spmv_d<false>(fp64, P, S, lanes, unroll, grid, in, out, slot, nullptr, nullptr, st);
}

void launch_cg_init(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (fp64) k_cg_init<true><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 0));
    else k_cg_init<false><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 0));
}

void launch_cg_residual(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (fp64) k_cg_residual<true><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 2));
    else k_cg_residual<false><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 2));
}

void launch_cg_axpy(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st,
                    cudaGraphConditionalHandle cond)
{
    if (fp64) k_cg_axpy<true><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 3), cond);
    else k_cg_axpy<false><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 3), cond);
}

void launch_pc_build(bool fp64, int mode, const StepParams& P, const DeviceState& S, const LaunchCfg& L,
                     cudaStream_t st)
{
    if (fp64) k_pc_build64<<<L.grid_vec, kBlock, 0, st>>>(P, S, mode);
    else k_pc_build32<8><<<L.grid_vec, kBlock, 0, st>>>(P, S, mode);
}

void launch_pcg_start(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (fp64) k_pcg_start<true><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 2), S.partials + kMaxPartials);
    else k_pcg_start<false><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 2), S.partials + kMaxPartials);
}

void launch_cg_axpy_pc(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st,
                       cudaGraphConditionalHandle cond)
{
    if (fp64) k_cg_axpy_pc<true><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 3), S.partials + kMaxPartials, cond);
    else k_cg_axpy_pc<false><<<L.grid_vec, kBlock, 0, st>>>(P, S, slot_of(S, 3), S.partials + kMaxPartials, cond);
}

void launch_cg_xpby(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (fp64) k_cg_xpby<true><<<L.grid_vec, kBlock, 0, st>>>(P, S);
    else k_cg_xpby<false><<<L.grid_vec, kBlock, 0, st>>>(P, S);
}

void launch_update(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    if (fp64) k_update<true><<<L.grid_vec, kBlock, 0, st>>>(P, S);
    else k_update<false><<<L.grid_vec, kBlock, 0, st>>>(P, S);
}

void launch_refresh(bool fp64, const StepParams& P, const DeviceState& S, const LaunchCfg& L, cudaStream_t st)
{
    k_refresh<<<L.grid_vec, kBlock, 0, st>>>(P, S);
    if (!fp64 && L.lattice && L.lat) launch_lattice_delta(S, *L.lat, P.sup, st);
}

template <int G, int U>
static int blocks_gu(bool fp64)
{
    int a = 0, b = 0, c = 0;
    if (fp64) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_spmv<G, true, true, 1>, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_force<G, true>, kBlock, 0);
        c = a;
    } else {
        cudaFuncSetAttribute(k_spmv<G, false, true, U>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaFuncSetAttribute(k_spmv<G, false, false, U>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_spmv<G, false, true, U>, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_spmv<G, false, false, U>, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_force<G, false>, kBlock, 0);
    }
    int m = a < c ? a : c;
    (void)b;
    return m > 0 ? m : 1;
}

template <int G>
static int blocks_g(bool fp64, int unroll)
{
    switch (unroll) {
    case 2: return blocks_gu<G, 2>(fp64);
    case 4: return blocks_gu<G, 4>(fp64);
    default: return blocks_gu<G, 1>(fp64);
    }
}

int row_kernel_blocks_per_sm(bool fp64, int lanes, int unroll)
{
    switch (lanes) {
    case 4: return blocks_g<4>(fp64, unroll);
    case 16: return blocks_g<16>(fp64, unroll);
    case 32: return blocks_g<32>(fp64, unroll);
    default: return blocks_g<8>(fp64, unroll);
    }
}

int force_kernel_blocks_per_sm(bool fp64, int lanes)
{
    int b = 0;
    switch (lanes) {
    case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fp64 ? (const void*)k_force<4, true> : (const void*)k_force<4, false>, kBlock, 0); break;
    case 16: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fp64 ? (const void*)k_force<16, true> : (const void*)k_force<16, false>, kBlock, 0); break;
    case 32: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fp64 ? (const void*)k_force<32, true> : (const void*)k_force<32, false>, kBlock, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fp64 ? (const void*)k_force<8, true> : (const void*)k_force<8, false>, kBlock, 0); break;
    }
    return b > 0 ? b : 1;
}

}  // namespace pdgb
