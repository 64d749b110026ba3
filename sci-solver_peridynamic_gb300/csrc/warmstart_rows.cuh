// warmstart_rows.cuh -- per-particle bodies of the learned CG warm start,
// shared by the one-scene kernels (warmstart.cu) and the batched persistent
// kernels (batch.cu), so both paths compute the same features.
//
// No reference counterpart.  With x1 = the previous solution (the reference's
// warm start), x2, x3 the two before it and r = b - A x1:
//   ws_jacobi_row    D_p = m + beta h^2 c sum_q (1/d0 - 2/(3d)) (trace/3 of
//                    the diagonal block), dj_p = r_p / D_p, and the squares
//                    summed for the RMS scales of x1, dj and v;
//   ws_features_row  64 BF16 features: solution history, Jacobi step and its
//                    neighbour averages, bond-projected differences, velocity,
//                    stretch statistics, stiffness ratio, contact/boundary flags;
//   ws_apply_elem    x0 = x1 + sigma_o * MLP(features) on free rows.
// LD selects the load path of data other rows wrote (kLdReadOnly in kernels
// that do not write it, kLdCoherent in a persistent kernel after a barrier).
#pragma once

#include <cuda_bf16.h>

#include "pd_device.cuh"
#include "pd_kernels.h"
#include "step_rows.cuh"

namespace pdgb {

__device__ __forceinline__ float safe_scale(double sum2, int n)
{
    const double s = sqrt(sum2 / (double)(n > 0 ? n : 1));
    return (float)(s > 1e-30 ? s : 1e-30);
}

template <int G, int LD>
__device__ __forceinline__ void ws_jacobi_row(const StepParams& P, const DeviceState& S, const WsState& W, int p,
                                              int lane, unsigned gmask, DotAcc32& ax, DotAcc32& ar, DotAcc32& av)
{
    const int a = S.act[p] & kActMask;
    const int rs = S.row_ptr[p], cn = S.cnt[p];
    const float4 Xp = S.X32[p], Up = ld_in<LD>(S.u32 + p);
    float ksum = 0.f;
    for (int j = lane; j < cn; j += G) {
        const int q = S.col[rs + j];
        const float4 Xq = S.X32[q], Uq = ld_in<LD>(S.u32 + q);
        const float x0 = Xq.x - Xp.x, y0 = Xq.y - Xp.y, z0 = Xq.z - Xp.z;
        const float xs = x0 + (Uq.x - Up.x), ys = y0 + (Uq.y - Up.y), zs = z0 + (Uq.z - Up.z);
        ksum += rsqrtf(x0 * x0 + y0 * y0 + z0 * z0) - (2.f / 3.f) * rsqrtf(xs * xs + ys * ys + zs * zs);
    }
    ksum = group_sum<G>(ksum, gmask);
    if (lane == 0) {
        const float D = (float)P.mass + (float)(P.t2 * P.bond_coeff) * ksum;
        W.diag[p] = D;
        float4 dj = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!is_dirichlet(a)) {
            const float4 rv = ((const float4*)S.r)[p];
            const float inv = 1.f / D;
            dj = make_float4(rv.x * inv, rv.y * inv, rv.z * inv, 0.f);
            const float4 xv = ld_in<LD>((const float4*)S.sol + p);
            const dbl4 v = S.v64[p];
            ax.fma(xv.x, xv.x); ax.fma(xv.y, xv.y); ax.fma(xv.z, xv.z);
            ar.fma(dj.x, dj.x); ar.fma(dj.y, dj.y); ar.fma(dj.z, dj.z);
            av.fma((float)v.x, (float)v.x); av.fma((float)v.y, (float)v.y); av.fma((float)v.z, (float)v.z);
        }
        W.dj[p] = dj;
    }
}

template <int G, int LD>
__device__ __forceinline__ void ws_features_row(const StepParams& P, const DeviceState& S, const WsState& W, int p,
                                                int lane, unsigned gmask, float sx, float sr, float sv)
{
    const float so = sx + sr;
    const float4* x1 = (const float4*)S.sol;
    const int a = S.act[p] & kActMask;
    __nv_bfloat16* f = W.features + (size_t)p * kMlpIn;
    if (is_dirichlet(a)) {
        for (int k = lane; k < kMlpIn; k += G) f[k] = __float2bfloat16_rn(0.f);
        return;
    }
    const int rs = S.row_ptr[p], cn = S.cnt[p];
    const float4 Xp = S.X32[p], Up = ld_in<LD>(S.u32 + p);
    const float4 djp = ld_in<LD>(W.dj + p);
    const float4 xp = ld_in<LD>(x1 + p);
    float mdj[3] = {0, 0, 0}, mx[3] = {0, 0, 0}, pdj[3] = {0, 0, 0}, px[3] = {0, 0, 0};
    float smean = 0.f, smin = 1e30f, smax = -1e30f, kstiff = 0.f;
    for (int j = lane; j < cn; j += G) {
        const int q = S.col[rs + j];
        const float4 Xq = S.X32[q], Uq = ld_in<LD>(S.u32 + q);
        const float4 djq = ld_in<LD>(W.dj + q);
        const float4 xq = ld_in<LD>(x1 + q);
        const float x0 = Xq.x - Xp.x, y0 = Xq.y - Xp.y, z0 = Xq.z - Xp.z;
        const float dx = Uq.x - Up.x, dy = Uq.y - Up.y, dz = Uq.z - Up.z;
        const float xs = x0 + dx, ys = y0 + dy, zs = z0 + dz;
        const float d02 = x0 * x0 + y0 * y0 + z0 * z0;
        const float inv_d0 = rsqrtf(d02), inv_d = rsqrtf(xs * xs + ys * ys + zs * zs);
        const float d0 = d02 * inv_d0, d = 1.f / inv_d;
        const float s = ((2.f * x0 + dx) * dx + (2.f * y0 + dy) * dy + (2.f * z0 + dz) * dz) / (d0 * (d + d0));
        smean += s;
        smin = fminf(smin, s);
        smax = fmaxf(smax, s);
        kstiff += inv_d0;
        const float ex = xs * inv_d, ey = ys * inv_d, ez = zs * inv_d;
        mdj[0] += djq.x; mdj[1] += djq.y; mdj[2] += djq.z;
        mx[0] += xq.x - xp.x; mx[1] += xq.y - xp.y; mx[2] += xq.z - xp.z;
        const float pj = ex * (djq.x - djp.x) + ey * (djq.y - djp.y) + ez * (djq.z - djp.z);
        const float pxv = ex * (xq.x - xp.x) + ey * (xq.y - xp.y) + ez * (xq.z - xp.z);
        pdj[0] += pj * ex; pdj[1] += pj * ey; pdj[2] += pj * ez;
        px[0] += pxv * ex; px[1] += pxv * ey; px[2] += pxv * ez;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mdj[k] = group_sum<G>(mdj[k], gmask);
        mx[k] = group_sum<G>(mx[k], gmask);
        pdj[k] = group_sum<G>(pdj[k], gmask);
        px[k] = group_sum<G>(px[k], gmask);
    }
    smean = group_sum<G>(smean, gmask);
    kstiff = group_sum<G>(kstiff, gmask);
    for (int off = G / 2; off > 0; off >>= 1) {
        smin = fminf(smin, __shfl_xor_sync(gmask, smin, off, G));
        smax = fmaxf(smax, __shfl_xor_sync(gmask, smax, off, G));
    }
    if (lane == 0) {
        const float inv_c = cn > 0 ? 1.f / (float)cn : 0.f;
        const float4 x2 = W.hist2[p], x3 = W.hist3[p];
        const dbl4 v = S.v64[p];
        float fv[kMlpIn];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) fv[k] = 0.f;
        fv[0] = xp.x / sx; fv[1] = xp.y / sx; fv[2] = xp.z / sx;
        fv[3] = x2.x / sx; fv[4] = x2.y / sx; fv[5] = x2.z / sx;
        fv[6] = x3.x / sx; fv[7] = x3.y / sx; fv[8] = x3.z / sx;
        fv[9] = djp.x / sr; fv[10] = djp.y / sr; fv[11] = djp.z / sr;
        for (int k = 0; k < 3; ++k) {
            fv[12 + k] = mdj[k] * inv_c / sr;
            fv[15 + k] = mx[k] * inv_c / sx;
            fv[18 + k] = pdj[k] * inv_c / sr;
            fv[21 + k] = px[k] * inv_c / sx;
        }
        fv[24] = (float)v.x / sv; fv[25] = (float)v.y / sv; fv[26] = (float)v.z / sv;
        fv[27] = cn > 0 ? 100.f * smean * inv_c : 0.f;
        fv[28] = cn > 0 ? 100.f * smin : 0.f;
        fv[29] = cn > 0 ? 100.f * smax : 0.f;
        fv[30] = (float)cn / (float)(W.max_bonds > 0 ? W.max_bonds : 1);
        fv[31] = log1pf((float)(P.t2 * P.bond_coeff / P.mass) * kstiff);
        fv[32] = (S.act[p] & kActContact) ? 1.f : 0.f;
        fv[33] = log10f(sx / so);
        fv[34] = log10f(sr / so);
        fv[35] = P.integrator ? 1.f : 0.f;
        fv[36] = W.diag[p] / (float)P.mass;
        fv[37] = (xp.x * djp.x + xp.y * djp.y + xp.z * djp.z) / (sx * sr);
        fv[38] = 1.f;
        for (int k = 0; k < kMlpIn; ++k) f[k] = __float2bfloat16_rn(fminf(fmaxf(fv[k], -64.f), 64.f));
    }
}

// x0 = x1 + sigma_o * y on a free row (y: the network's output row)
__device__ __forceinline__ void ws_apply_elem(const DeviceState& S, const float* __restrict__ Y, int p, float so)
{
    if (is_dirichlet(S.act[p] & kActMask)) return;
    const float* y = Y + (size_t)p * kMlpOutPad;
    float4* x = (float4*)S.sol;
    float4 v = x[p];
    v.x += so * y[0];
    v.y += so * y[1];
    v.z += so * y[2];
    x[p] = v;
}

// The guard after the learned guess's residual: keeps the guess when its
// <r, r> is not above the previous solution's, otherwise flags the rows for
// the previous solution and restores the plain scalars (thread 0, once per
// solve).
__device__ __forceinline__ void ws_decide(CgScalars* sc)
{
    sc->rz_learned = sc->rz;
    if (!(sc->rz <= sc->rz_plain)) {   // worse, or not a number: back to the previous solution
        sc->ws_revert = 1;
        sc->ws_rejects += 1;
        sc->rz = sc->rz_plain;
        sc->rnorm = sqrt(sc->rz_plain);
        sc->done = 0;
        sc->converged = 0;
        if (sc->rnorm <= sc->tol) {
            sc->done = 1;
            sc->converged = 1;
        } else if (sc->iter >= sc->max_iter) {
            sc->done = 1;
        }
    } else {
        sc->ws_revert = 0;
        sc->ws_rejects = 0;
        sc->ws_kept += 1;
    }
}

}  // namespace pdgb
