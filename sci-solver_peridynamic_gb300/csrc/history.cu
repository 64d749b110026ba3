// history.cu -- the history-projection initial guess of the CG solve.
//
// No reference counterpart: the reference starts each solve from the
// previous step's solution (Simulator::solveLinearSystem,
// src/core/simulator.cu:745-770), and so does this library by default.  With
// warm_start = 2 the guess is instead x1 + H y, where the columns of H are the
// last m accepted solutions (Dirichlet rows zeroed) and y makes the residual
// orthogonal to span(H) (a Galerkin projection, the successive right-hand-side
// method of P. F. Fischer, "Projection techniques for iterative solution of
// Ax = b with successive right-hand sides", CMAME 163, 1998).  The CG then runs
// to the same tolerance as always.
//
// Per solve: one product A h_j per history vector (the operator changes every
// step), the block partials of the small Gram matrices below, the m x m solve
// on the host in a stream callback (the partials summed there in block order;
// the calling thread does not wait, and one FP64 thread on the device took
// 0.5-0.9 ms for it), x += H y, and a fresh residual.
#include <cmath>

#include "pd_device.cuh"
#include "pd_kernels.h"

namespace pdgb {

namespace {

constexpr int kPairs = kHistMax * (kHistMax + 1) / 2;

// One accumulator per entry: pass 0 -> S (upper, kPairs) then c (kHistMax);
// pass 1 -> G (upper, kPairs).
template <typename Real, int PASS>
__global__ void __launch_bounds__(kBlock) k_hist_dots(int n, int m, HistPtrs H, HistPtrs W, const void* r_,
                                                      double* partials)
{
    using V4 = typename Vec4<Real>::type;
    using Acc = typename DotAccFor<Real>::type;
    constexpr int NA = PASS == 0 ? kPairs + kHistMax : kPairs;
    Acc acc[NA];
    const V4* r = (const V4*)r_;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        V4 h[kHistMax], w[kHistMax];
#pragma unroll
        for (int k = 0; k < kHistMax; ++k) {
            if (k < m) {
                h[k] = ((const V4*)H.v[k])[i];
                if (PASS == 1) w[k] = ((const V4*)W.v[k])[i];
            }
        }
        V4 rv;
        if (PASS == 0) rv = r[i];
        int e = 0;
#pragma unroll
        for (int a = 0; a < kHistMax; ++a) {
#pragma unroll
            for (int b = a; b < kHistMax; ++b, ++e) {
                if (b < m) {
                    const V4& y = PASS == 0 ? h[b] : w[b];
                    acc[e].fma(h[a].x, y.x);
                    acc[e].fma(h[a].y, y.y);
                    acc[e].fma(h[a].z, y.z);
                }
            }
        }
        if (PASS == 0) {
#pragma unroll
            for (int a = 0; a < kHistMax; ++a) {
                if (a < m) {
                    acc[kPairs + a].fma(h[a].x, rv.x);
                    acc[kPairs + a].fma(h[a].y, rv.y);
                    acc[kPairs + a].fma(h[a].z, rv.z);
                }
            }
        }
    }
    // block totals in FP64, fixed order: warps by shuffles, then warp 0 over warps
    __shared__ double s_w[kBlock / 32][NA];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NA; ++k) {
        double v = acc[k].value();
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) s_w[warp][k] = v;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < NA; k += blockDim.x) {
        double v = 0.0;
        for (int w = 0; w < kBlock / 32; ++w) v += s_w[w][k];
        partials[(size_t)blockIdx.x * NA + k] = v;
    }
}

// x += H y, formed in FP64 (the coefficients of nearly parallel history
// vectors can be large and of opposite sign)
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_hist_apply(int n, int m, HistPtrs H, const HistSolve* Y, void* x_)
{
    using V4 = typename Vec4<Real>::type;
    V4* x = (V4*)x_;
    if (((const volatile HistSolve*)Y)->used == 0) return;
    double yk[kHistMax];
#pragma unroll
    for (int k = 0; k < kHistMax; ++k) yk[k] = Y->y[k];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double ax = 0.0, ay = 0.0, az = 0.0;
#pragma unroll
        for (int k = 0; k < kHistMax; ++k) {
            if (k < m) {
                const V4 h = ((const V4*)H.v[k])[i];
                ax = fma(yk[k], (double)h.x, ax);
                ay = fma(yk[k], (double)h.y, ay);
                az = fma(yk[k], (double)h.z, az);
            }
        }
        V4 xi = x[i];
        xi.x = (Real)((double)xi.x + ax);
        xi.y = (Real)((double)xi.y + ay);
        xi.z = (Real)((double)xi.z + az);
        x[i] = xi;
    }
}

// dst = x with Dirichlet rows zeroed (the correction never moves them)
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_hist_push(int n, const uint8_t* act, const void* x_, void* dst_)
{
    using V4 = typename Vec4<Real>::type;
    const V4* x = (const V4*)x_;
    V4* dst = (V4*)dst_;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        V4 v = x[i];
        if (is_dirichlet(act[i] & kActMask)) v = make_v4<V4>(0.0, 0.0, 0.0);
        v.w = 0;
        dst[i] = v;
    }
}

}  // namespace

int hist_dots_count(int pass) { return pass == 0 ? kPairs + kHistMax : kPairs; }

void launch_hist_dots(bool fp64, int pass, int n, int m, const HistPtrs& H, const HistPtrs& W, const void* r,
                      double* partials, int blocks, cudaStream_t st)
{
    if (pass == 0) {
        if (fp64) k_hist_dots<double, 0><<<blocks, kBlock, 0, st>>>(n, m, H, W, r, partials);
        else k_hist_dots<float, 0><<<blocks, kBlock, 0, st>>>(n, m, H, W, r, partials);
    } else {
        if (fp64) k_hist_dots<double, 1><<<blocks, kBlock, 0, st>>>(n, m, H, W, r, partials);
        else k_hist_dots<float, 1><<<blocks, kBlock, 0, st>>>(n, m, H, W, r, partials);
    }
}

void hist_host_solve(const HistHostSolve& a)
{
    const int na0 = hist_dots_count(0), na1 = hist_dots_count(1);
    double dots[kPairs + kHistMax + kPairs];
    const double* p0 = a.partials;
    const double* p1 = a.partials + (size_t)a.blocks * na0;
    for (int k = 0; k < na0; ++k) {   // block order
        double v = 0.0;
        for (int b = 0; b < a.blocks; ++b) v += p0[(size_t)b * na0 + k];
        dots[k] = v;
    }
    for (int k = 0; k < na1; ++k) {
        double v = 0.0;
        for (int b = 0; b < a.blocks; ++b) v += p1[(size_t)b * na1 + k];
        dots[na0 + k] = v;
    }
    double y[kHistMax];
    int used = hist_solve(a.m, dots, dots + na0, dots + kPairs, a.rel_tol, y);
    // a solve that had already converged from the previous solution keeps it
    if (a.sc->done) used = 0;
    for (int k = 0; k < kHistMax; ++k) a.out->y[k] = (used > 0 && k < a.m) ? y[k] : 0.0;
    a.out->used = used;
    a.out->net_used = (used > 0 && a.net_col >= 0 && a.net_col < a.m && y[a.net_col] != 0.0) ? 1 : 0;
    a.out->rz1 = a.sc->rz;
}

void launch_hist_apply(bool fp64, int n, int m, const HistPtrs& H, const HistSolve* Y, void* x, int blocks,
                       cudaStream_t st)
{
    if (fp64) k_hist_apply<double><<<blocks, kBlock, 0, st>>>(n, m, H, Y, x);
    else k_hist_apply<float><<<blocks, kBlock, 0, st>>>(n, m, H, Y, x);
}

void launch_hist_push(bool fp64, int n, const uint8_t* act, const void* x, void* dst, int blocks, cudaStream_t st)
{
    if (fp64) k_hist_push<double><<<blocks, kBlock, 0, st>>>(n, act, x, dst);
    else k_hist_push<float><<<blocks, kBlock, 0, st>>>(n, act, x, dst);
}

// ---- the m x m solve (host) ------------------------------------------------------------
// S = H^T H, G = H^T A H (upper triangles, row-major pairs a <= b), c = H^T r1.
// A pivoted Cholesky of S selects a well-conditioned subset of the history
// (columns whose remaining component is below rel_tol of the largest are
// dropped: in FP32 storage they are rounding noise); in the orthonormal basis
// Q = H_sel R^-1 the projected system G_Q z = c_Q is solved by Cholesky and
// y = R^-1 z.  Returns the number of columns used (0: no usable guess).
int hist_solve(int m, const double* S_up, const double* G_up, const double* c, double rel_tol, double* y)
{
    double S[kHistMax][kHistMax], G[kHistMax][kHistMax];
    int e = 0;
    for (int a = 0; a < kHistMax; ++a)
        for (int b = a; b < kHistMax; ++b, ++e) {
            if (a < m && b < m) {
                S[a][b] = S[b][a] = S_up[e];
                G[a][b] = G[b][a] = G_up[e];
            }
        }
    for (int k = 0; k < m; ++k) y[k] = 0.0;
    // pivoted Cholesky on a copy of S: choose columns in order of largest remaining norm
    double W[kHistMax][kHistMax];
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b) W[a][b] = S[a][b];
    double dmax = 0.0;
    for (int a = 0; a < m; ++a) dmax = W[a][a] > dmax ? W[a][a] : dmax;
    if (!(dmax > 0.0)) return 0;
    int sel[kHistMax];
    bool used[kHistMax] = {};
    int r = 0;
    for (; r < m; ++r) {
        int piv = -1;
        double best = rel_tol * dmax;
        for (int a = 0; a < m; ++a)
            if (!used[a] && W[a][a] > best) best = W[a][a], piv = a;
        if (piv < 0) break;
        used[piv] = true;
        sel[r] = piv;
        const double d = W[piv][piv];
        // the pivot's column and row are copied first: the update zeroes row
        // piv, and every row after it must still be downdated by the old row
        double col[kHistMax], prow[kHistMax];
        for (int a = 0; a < m; ++a) col[a] = W[a][piv] / d;
        for (int b = 0; b < m; ++b) prow[b] = W[piv][b];
        for (int a = 0; a < m; ++a)
            for (int b = 0; b < m; ++b) W[a][b] -= col[a] * prow[b];
    }
    if (r == 0) return 0;
    // R: upper Cholesky factor of S restricted to the selected columns
    double R[kHistMax][kHistMax] = {};
    for (int i = 0; i < r; ++i) {
        for (int j = i; j < r; ++j) {
            double s = S[sel[i]][sel[j]];
            for (int k = 0; k < i; ++k) s -= R[k][i] * R[k][j];
            if (i == j) {
                if (!(s > 0.0)) return 0;
                R[i][i] = sqrt(s);
            } else {
                R[i][j] = s / R[i][i];
            }
        }
    }
    // Rinv (upper triangular)
    double Ri[kHistMax][kHistMax] = {};
    for (int j = 0; j < r; ++j) {
        Ri[j][j] = 1.0 / R[j][j];
        for (int i = j - 1; i >= 0; --i) {
            double s = 0.0;
            for (int k = i + 1; k <= j; ++k) s += R[i][k] * Ri[k][j];
            Ri[i][j] = -s / R[i][i];
        }
    }
    // G_Q = Ri^T G_sel Ri, c_Q = Ri^T c_sel
    double T[kHistMax][kHistMax], GQ[kHistMax][kHistMax], cQ[kHistMax];
    for (int i = 0; i < r; ++i)
        for (int j = 0; j < r; ++j) {
            double s = 0.0;
            for (int k = 0; k < r; ++k) s += G[sel[i]][sel[k]] * Ri[k][j];
            T[i][j] = s;
        }
    for (int i = 0; i < r; ++i) {
        for (int j = 0; j < r; ++j) {
            double s = 0.0;
            for (int k = 0; k < r; ++k) s += Ri[k][i] * T[k][j];
            GQ[i][j] = s;
        }
        double s = 0.0;
        for (int k = 0; k < r; ++k) s += Ri[k][i] * c[sel[k]];
        cQ[i] = s;
    }
    for (int i = 0; i < r; ++i)
        for (int j = i + 1; j < r; ++j) GQ[i][j] = GQ[j][i] = 0.5 * (GQ[i][j] + GQ[j][i]);
    // Cholesky solve of G_Q z = c_Q (SPD for an SPD operator)
    double L[kHistMax][kHistMax] = {};
    for (int j = 0; j < r; ++j) {
        double s = GQ[j][j];
        for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
        if (!(s > 0.0)) return 0;
        L[j][j] = sqrt(s);
        for (int i = j + 1; i < r; ++i) {
            double t = GQ[i][j];
            for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
            L[i][j] = t / L[j][j];
        }
    }
    double z[kHistMax];
    for (int i = 0; i < r; ++i) {
        double s = cQ[i];
        for (int k = 0; k < i; ++k) s -= L[i][k] * z[k];
        z[i] = s / L[i][i];
    }
    for (int i = r - 1; i >= 0; --i) {
        double s = z[i];
        for (int k = i + 1; k < r; ++k) s -= L[k][i] * z[k];
        z[i] = s / L[i][i];
    }
    for (int i = 0; i < r; ++i) {
        double s = 0.0;
        for (int k = i; k < r; ++k) s += Ri[i][k] * z[k];
        if (!(fabs(s) <= 1.7976931348623157e308)) {   // NaN or infinite
            for (int q = 0; q < m; ++q) y[q] = 0.0;
            return 0;
        }
        y[sel[i]] = s;
    }
    return r;
}

}  // namespace pdgb
