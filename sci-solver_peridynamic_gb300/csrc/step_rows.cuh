// step_rows.cuh -- per-particle bodies of the step kernels.
//
// Each function does one particle's (or one row group's) share of a kernel,
// so the same arithmetic runs in the one-scene launches of step.cu and in the
// persistent multi-scene kernels of batch.cu.  Reference formulas and their
// file:line are cited at each body.
#pragma once

#include <type_traits>

#include "pd_device.cuh"
#include "pd_kernels.h"

namespace pdgb {

// ---- FP64 operations the compiler must not contract ---------------------------
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

// Bond geometry exactly as calculatePDForceDerivative evaluates it
// (cg_solver.cuh:254-260): eij = x_q - x_p, dij = sqrt(x*x + y*y + z*z),
// d0 = length(X_p - X_q), drdivd = dij / d0 - 1.
struct BondEval {
    double ex, ey, ez, dij, d0, s;
};

__device__ __forceinline__ BondEval eval_bond(const dbl4& xp, const dbl4& Xp, const dbl4& xq,
                                              const dbl4& Xq)
{
    BondEval b;
    b.ex = dsub(xq.x, xp.x);
    b.ey = dsub(xq.y, xp.y);
    b.ez = dsub(xq.z, xp.z);
    b.dij = dsqrt(dadd(dadd(dmul(b.ex, b.ex), dmul(b.ey, b.ey)), dmul(b.ez, b.ez)));
    const double ox = dsub(Xp.x, Xq.x), oy = dsub(Xp.y, Xq.y), oz = dsub(Xp.z, Xq.z);
    b.d0 = dsqrt(dadd(dadd(dmul(ox, ox), dmul(oy, oy)), dmul(oz, oz)));
    b.s = dsub(ddiv(b.dij, b.d0), 1.0);
    return b;
}

// Position as an FP32 offset inside its supercell plus the supercell's integer
// coordinates (10 bits each) in the w lane.  A bond vector is then
// (off_q - off_p) + sup * (ijk_q - ijk_p): the offsets are small, so the FP32
// bond vector keeps ~2^-23 * sup / |xi| relative accuracy wherever the body is.
__device__ __forceinline__ float4 encode_supercell(const StepParams& P, const dbl4& x)
{
    const double v[3] = {x.x - P.sup_lo[0], x.y - P.sup_lo[1], x.z - P.sup_lo[2]};
    int c[3];
    float o[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int ck = (int)floor(v[k] * P.inv_sup);
        ck = ck < 0 ? 0 : (ck > 1023 ? 1023 : ck);
        c[k] = ck;
        o[k] = (float)(v[k] - P.sup * (double)ck);
    }
    return make_float4(o[0], o[1], o[2], __int_as_float(c[0] | (c[1] << 10) | (c[2] << 20)));
}

// The same offset split into two FP32 words, x = sup_lo + sup * ijk + hi + lo:
// x - sup_lo is formed error-free (two-difference in FP64), the offset inside
// the supercell is then exact in FP64, hi is it rounded to FP32 (the
// encode_supercell word, so the SpMV sees the same positions) and lo the rest
// rounded to FP32.  The representation error is below 2^-48 sup, so a bond
// vector built from (hi, lo) words carries ~1e-14 relative error -- double-float
// accuracy without FP64 arithmetic per bond.  A position outside the 1024^3
// supercell window (its cell index clamped) has an offset of many supercells
// and no such bound: lo.w = 1 marks it, and its bonds take the exact test.
__device__ __forceinline__ void encode_supercell_df(const StepParams& P, const dbl4& x, float4& hi, float4& lo)
{
    const double xv[3] = {x.x, x.y, x.z};
    int c[3];
    float o[3], l[3];
    bool clamped = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double v = dsub(xv[k], P.sup_lo[k]);
        const double bb = dsub(v, xv[k]);
        const double ve = dadd(dsub(xv[k], dsub(v, bb)), dsub(-P.sup_lo[k], bb));   // v + ve == x - sup_lo
        int ck = (int)floor(v * P.inv_sup);
        if (ck < 0 || ck > 1023) clamped = true;
        ck = ck < 0 ? 0 : (ck > 1023 ? 1023 : ck);
        c[k] = ck;
        const double off = dsub(v, dmul(P.sup, (double)ck));   // exact
        o[k] = (float)off;
        l[k] = (float)dadd(dsub(off, (double)o[k]), ve);
    }
    hi = make_float4(o[0], o[1], o[2], __int_as_float(c[0] | (c[1] << 10) | (c[2] << 20)));
    lo = make_float4(l[0], l[1], l[2], clamped ? 1.f : 0.f);
}

// A small integer as float without an int-to-float conversion (those issue
// at 1/8 of the FP32 rate): the integer added to the mantissa of 1.5 * 2^23,
// then 1.5 * 2^23 subtracted -- exact for |i| < 2^22.
__device__ __forceinline__ float small_int_to_float(int i)
{
    return __fsub_rn(__int_as_float(0x4B400000 + i), 12582912.0f);
}

__device__ __forceinline__ void supercell_delta(int wq, int wp, float sup, float& dx, float& dy, float& dz)
{
    dx = sup * small_int_to_float((wq & 1023) - (wp & 1023));
    dy = sup * small_int_to_float(((wq >> 10) & 1023) - ((wp >> 10) & 1023));
    dz = sup * small_int_to_float(((wq >> 20) & 1023) - ((wp >> 20) & 1023));
}

// ---- double-float (unevaluated sum of two FP32 words) -------------------------------
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return F2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ F2 quick_two_sum(float a, float b)   // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return F2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b)
{
    const F2 s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b)
{
    const float p = __fmul_rn(a.h, b.h);
    const float e = __fmaf_rn(a.h, b.h, -p);
    return quick_two_sum(p, __fadd_rn(e, __fadd_rn(__fmul_rn(a.h, b.l), __fmul_rn(a.l, b.h))));
}
__device__ __forceinline__ F2 f2_sqr(F2 a)
{
    const float p = __fmul_rn(a.h, a.h);
    const float e = __fmaf_rn(a.h, a.h, -p);
    return quick_two_sum(p, __fadd_rn(e, __fmul_rn(2.f * a.h, a.l)));
}
__device__ __forceinline__ F2 f2_of(double d)   // FP64 to double-float: per particle, or per bond at set-up
{
    const float h = (float)d;
    return F2{h, (float)(d - (double)h)};
}
__device__ __forceinline__ float f2_sign_diff(F2 a, F2 b)   // the sign of a - b
{
    return __fadd_rn(__fsub_rn(a.h, b.h), __fsub_rn(a.l, b.l));
}

// fmaxf(stretch_p, stretch_q) of cg_solver.cuh:264: both limits rounded to float.
__device__ __forceinline__ double break_threshold(float thp, double stq)
{
    const float thq = (float)stq;
    return (double)(thp > thq ? thp : thq);
}

// ---- force / breakage ----------------------------------------------------------
// Mixed precision: the reference's stretch test s = sqrt(dij2)/sqrt(d0_2) - 1 >
// threshold costs two FP64 square roots and a division per bond, and GB300
// runs FP64 at ~1/64 of its FP32 rate.  The test is decided instead on the
// squares, dij2 > (1 + threshold)^2 d0_2, evaluated in double-float from the
// (hi, lo) position words (relative error ~1e-13); only when the two sides are
// within 1e-12 relative (far above that error and the rounding difference of
// the two forms) is the reference FP64 expression itself evaluated.
// Broken-bond sets stay bit-exact, and no FP64 arithmetic runs per bond.
struct MixedBond {
    float ex, ey, ez;    // x_q - x_p
    float dd;            // dij^2
    float num;           // dij^2 - d0^2, from the double-float difference (no cancellation)
    bool live;
};

// Limits of the squared break test of a particle with stretch limit st:
// with t = st rounded to float and L = (1 + t)^2, {L (1 - 1e-12), L (1 + 1e-12)}
// as double-float words {lo.h, lo.l, hi.h, hi.l} ({-1, 0, -1, 0} when
// 1 + t <= 0).  A bond's limit is the larger of its two particles' t, and
// (1 + t)^2 grows with t, so the bond's pair is the element-wise maximum of
// the particles' pairs.
__device__ __forceinline__ float4 limit_pair(double st)
{
    const double l1 = dadd(1.0, (double)(float)st);
    if (!(l1 > 0.0)) return make_float4(-1.f, 0.f, -1.f, 0.f);
    const double L = dmul(l1, l1);
    const F2 lo = f2_of(dmul(L, 1.0 - 1e-12)), hi = f2_of(dmul(L, 1.0 + 1e-12));
    return make_float4(lo.h, lo.l, hi.h, hi.l);
}

__device__ __forceinline__ F2 f2_max(F2 a, F2 b) { return f2_sign_diff(a, b) >= 0.f ? a : b; }

// One component of the bond vector from the (hi, lo) words and the supercell
// coordinates: (hi_q - hi_p) + sup (c_q - c_p) + (lo_q - lo_p) in double-float.
__device__ __forceinline__ F2 bond_component(float hq, float hp, float lq, float lp, float cdelta)
{
    const F2 d = two_sum(hq, -hp);          // exact
    const F2 s = two_sum(d.h, cdelta);      // exact (cdelta is a power of two times a small integer)
    return quick_two_sum(s.h, __fadd_rn(__fadd_rn(d.l, s.l), __fsub_rn(lq, lp)));
}

// The break test s > fmaxf(st_p, st_q) (s = dij / d0 - 1 in FP64) decided on
// squares: broken when dij^2 > (1 + t)^2 d0^2 (1 + 1e-12), live when
// dij^2 < (1 + t)^2 d0^2 (1 - 1e-12); a bond in between takes the reference
// expression.
__device__ __forceinline__ MixedBond classify_mixed(float sup, const DeviceState& S, const float4& hp,
                                                    const float4& lp, const dbl4& xp, const dbl4& Xp, float thp,
                                                    const float4& limp, int slot, int q)
{
    MixedBond m;
    const float4 hq = S.xs4[q], lq = S.xlo4[q];
    float cx, cy, cz;
    supercell_delta(__float_as_int(hq.w), __float_as_int(hp.w), sup, cx, cy, cz);
    const F2 ex = bond_component(hq.x, hp.x, lq.x, lp.x, cx);
    const F2 ey = bond_component(hq.y, hp.y, lq.y, lp.y, cy);
    const F2 ez = bond_component(hq.z, hp.z, lq.z, lp.z, cz);
    const F2 dd = f2_add(f2_add(f2_sqr(ex), f2_sqr(ey)), f2_sqr(ez));
    const float2 d0w = S.d0sq[slot];
    const F2 d0s{d0w.x, d0w.y};
    const float4 limq = S.lim[q];
    const F2 lo = f2_max(F2{limp.x, limp.y}, F2{limq.x, limq.y});
    const F2 hi = f2_max(F2{limp.z, limp.w}, F2{limq.z, limq.w});
    const bool exact_only = lp.w != 0.f || lq.w != 0.f;   // outside the supercell window
    if (!exact_only && hi.h > 0.f && f2_sign_diff(dd, f2_mul(hi, d0s)) > 0.f) m.live = false;
    else if (!exact_only && lo.h > 0.f && f2_sign_diff(dd, f2_mul(lo, d0s)) < 0.f) m.live = true;
    else m.live = !(eval_bond(xp, Xp, S.x64[q], S.X64[q]).s > break_threshold(thp, S.st[q]));
    m.ex = ex.h;
    m.ey = ey.h;
    m.ez = ez.h;
    m.dd = dd.h;
    m.num = f2_sign_diff(dd, d0s);
    return m;
}


// Force pass of particle p by its G-lane group: stretch test and breakage,
// bond force, new stretch limit, gravity and contact; FP64 mode also stores the
// bond Jacobians and their diagonal sum.
template <int G, bool FP64>
__device__ __forceinline__ void force_row(const StepParams& P, const DeviceState& S, int p, int lane,
                                          unsigned gmask)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    V4* force = (V4*)S.force;
    const int a = S.act[p] & kActMask;
    const dbl4 xp = S.x64[p];
    const dbl4 Xp = S.X64[p];
    // FP32 displacement of this step's linear system (read by k_spmv).  The
    // supercell words of the positions (xs4, xlo4) were written from x64 by
    // the launch before this one (supercell_elem), as the neighbours read them.
    if (!FP64 && lane == 0)
        S.u32[p] = make_float4((float)(xp.x - Xp.x), (float)(xp.y - Xp.y), (float)(xp.z - Xp.z), 0.f);
    if (a == ACT_INVISIBLE) return;
    const float thp = (float)S.st[p];
    const int rs = S.row_ptr[p];
    const int c = S.cnt[p];
    Real fx = 0, fy = 0, fz = 0;
    double j0 = 0, j1 = 0, j2 = 0, j3 = 0, j4 = 0, j5 = 0;   // FP64: diagonal block sum
    double smin = 0.0;
    int nb = 0;
    if constexpr (FP64) {
        for (int j = lane; j < c; j += G) {
            const int q = S.col[rs + j];
            const dbl4 xq = S.x64[q];
            const dbl4 Xq = S.X64[q];
            const BondEval b = eval_bond(xp, Xp, xq, Xq);
            if (b.s > break_threshold(thp, S.st[q])) {
                ++nb;
                continue;
            }
            smin = b.s < smin ? b.s : smin;
            if (FP64) {
                // reference formulas: eij /= fmaxf(dij, SMALL) (float-rounded), vscale,
                // J = (c/d0) [ (1 - d0/dij) I + (d0/dij) e e^T ]   (cg_solver.cuh:256-303)
                const double D = (double)fmaxf((float)b.dij, (float)1e-10);
                const double ex = ddiv(b.ex, D), ey = ddiv(b.ey, D), ez = ddiv(b.ez, D);
                double vscale = 1.0;
                if (b.d0 > P.vs_threshold) vscale = dadd(0.5, ddiv(ddiv(dsub(P.horizon, b.d0), 2.0), P.radius));
                const double kk = dmul(b.s, vscale);
                fx = dadd(fx, dmul(kk, ex));
                fy = dadd(fy, dmul(kk, ey));
                fz = dadd(fz, dmul(kk, ez));
                const double r = ddiv(b.d0, b.dij);
                const double dg = dsub(1.0, r);
                const double cc = ddiv(P.bond_coeff, b.d0);
                const double jxx = dmul(dadd(dg, dmul(dmul(ex, ex), r)), cc);
                const double jyy = dmul(dadd(dg, dmul(dmul(ey, ey), r)), cc);
                const double jzz = dmul(dadd(dg, dmul(dmul(ez, ez), r)), cc);
                const double jxy = dmul(dmul(dmul(ex, ey), r), cc);
                const double jxz = dmul(dmul(dmul(ex, ez), r), cc);
                const double jyz = dmul(dmul(dmul(ey, ez), r), cc);
                double* J = S.jac + 6ll * (rs + j);
                J[0] = jxx; J[1] = jyy; J[2] = jzz; J[3] = jxy; J[4] = jxz; J[5] = jyz;
                j0 += jxx; j1 += jyy; j2 += jzz; j3 += jxy; j4 += jxz; j5 += jyz;
            } else {
                const float inv = 1.0f / (float)b.dij;
                const float d0f = (float)b.d0;
                float vs = 1.0f;
                if (b.d0 > P.vs_threshold) vs = 0.5f + ((float)P.horizon - d0f) * 0.5f / (float)P.radius;
                const float kk = (float)b.s * vs * inv;
                fx = fmaf(kk, (float)b.ex, (float)fx);
                fy = fmaf(kk, (float)b.ey, (float)fy);
                fz = fmaf(kk, (float)b.ez, (float)fz);
            }
        }
    } else {
        // live bonds: FP32 force from the FP64 bond vector; the stretch comes
        // from dij2 - d0^2 (no cancellation) as s = (dij2 - d0^2) / (d0 (dij + d0))
        const float* id0r = S.inv_d0 + rs;
        const float4 limp = S.lim[p];
        const float4 hp = S.xs4[p], lp = S.xlo4[p];
        const float supf = (float)P.sup, hor = (float)P.horizon, radf = (float)P.radius;
        // (double)d0 > vs_threshold  <=>  d0 > (vs_threshold rounded down to float)
        const float vs_thr = __double2float_rd(P.vs_threshold);
        float r1 = 3.0e38f, r2 = 3.0e38f;   // the lane's two smallest (dij2 - d0^2) / d0^2
        int j1 = -1;
        for (int j = lane; j < c; j += G) {
            const int q = S.col[rs + j];
            const MixedBond m = classify_mixed(supf, S, hp, lp, xp, Xp, thp, limp, rs + j, q);
            if (!m.live) {
                ++nb;
                continue;
            }
            const float idd0 = id0r[j];
            const float d = sqrtf((float)m.dd);
            const float d0 = 1.0f / idd0;
            const float sf = (float)m.num * idd0 / (d + d0);
            const float r = (float)m.num * (idd0 * idd0);
            if (r < r1) {
                r2 = r1;
                r1 = r;
                j1 = j;
            } else if (r < r2) {
                r2 = r;
            }
            float vs = 1.0f;
            if (d0 > vs_thr) vs = 0.5f + (hor - d0) * 0.5f / radf;
            const float kk = sf * vs / fmaxf(d, 1e-10f);   // eij /= fmaxf(dij, SMALL)
            fx = fmaf(kk, (float)m.ex, (float)fx);
            fy = fmaf(kk, (float)m.ey, (float)fy);
            fz = fmaf(kk, (float)m.ez, (float)fz);
        }
        // smin = min(0, smallest stretch of a live bond), bit for bit: if no
        // live bond is shorter than at rest every stretch is >= 0; otherwise
        // the bonds whose estimate lies within its error (1e-6 relative) of the
        // smallest are evaluated with the reference expression.  A bond at its
        // rest length (dij^2 == d0^2 exactly, r == 0) has stretch exactly 0 and
        // cannot lower smin, so rows at rest skip the exact evaluation; an r
        // that underflows to -0 stands for a stretch below 1e-45, which moves
        // the new limit (10 - 9 cs) s0 - 0.25 min(0, smin) by less than an ulp.
        const float rmin = group_minf<G>(r1, gmask);
        if (rmin < 0.f) {
            const float band = rmin + 1e-6f * fabsf(rmin) + 1e-30f;
            if (!__any_sync(gmask, r2 <= band)) {
                if (r1 <= band) {
                    const int q = S.col[rs + j1];
                    const double s1 = eval_bond(xp, Xp, S.x64[q], S.X64[q]).s;
                    smin = s1 < smin ? s1 : smin;
                }
            } else {
                // several candidates in one lane: walk the row again
                for (int j = lane; j < c; j += G) {
                    const int q = S.col[rs + j];
                    const MixedBond m = classify_mixed(supf, S, hp, lp, xp, Xp, thp, limp, rs + j, q);
                    if (!m.live) continue;
                    const float idd0 = id0r[j];
                    if ((float)m.num * (idd0 * idd0) > band) continue;
                    const double sj = eval_bond(xp, Xp, S.x64[q], S.X64[q]).s;
                    smin = sj < smin ? sj : smin;
                }
            }
        }
    }
    fx = group_sum<G>(fx, gmask);
    fy = group_sum<G>(fy, gmask);
    fz = group_sum<G>(fz, gmask);
    smin = group_min<G>(smin, gmask);
    nb = group_sum<G>(nb, gmask);
    if (FP64) {
        j0 = group_sum<G>(j0, gmask); j1 = group_sum<G>(j1, gmask); j2 = group_sum<G>(j2, gmask);
        j3 = group_sum<G>(j3, gmask); j4 = group_sum<G>(j4, gmask); j5 = group_sum<G>(j5, gmask);
    }
    if (nb > 0) {
        // Rare path: partition the row as the reference does (swap the broken
        // bond with the last live one and retest the swapped-in bond,
        // cg_solver.cuh:264-275), so live bonds occupy the first cnt slots.
        int top = c - 1;
        if (lane == 0) {
            int bond = 0;
            while (bond <= top) {
                const int q = S.col[rs + bond];
                const BondEval b = eval_bond(xp, Xp, S.x64[q], S.X64[q]);
                if (b.s > break_threshold(thp, S.st[q])) {
                    S.col[rs + bond] = S.col[rs + top];
                    S.col[rs + top] = q;
                    if (!FP64) {
                        const float t = S.inv_d0[rs + bond];
                        S.inv_d0[rs + bond] = S.inv_d0[rs + top];
                        S.inv_d0[rs + top] = t;
                        const float2 t2 = S.d0sq[rs + bond];
                        S.d0sq[rs + bond] = S.d0sq[rs + top];
                        S.d0sq[rs + top] = t2;
                        if (S.lidx) {
                            const uint16_t l = S.lidx[rs + bond];
                            S.lidx[rs + bond] = S.lidx[rs + top];
                            S.lidx[rs + top] = l;
                        }
                    }
                    --top;
                    continue;
                }
                ++bond;
            }
            S.cnt[p] = top + 1;
            S.flags[0] = 1;
            atomicAdd(&S.flags[1], nb);
        }
        __syncwarp(gmask);
        if (FP64) {
            // bond slots moved: store each live bond's Jacobian at its new slot
            top = __shfl_sync(gmask, top, 0, G);
            for (int j = lane; j <= top; j += G) {
                const int q = S.col[rs + j];
                const BondEval b = eval_bond(xp, Xp, S.x64[q], S.X64[q]);
                const double D = (double)fmaxf((float)b.dij, (float)1e-10);
                const double ex = ddiv(b.ex, D), ey = ddiv(b.ey, D), ez = ddiv(b.ez, D);
                const double r = ddiv(b.d0, b.dij);
                const double dg = dsub(1.0, r);
                const double cc = ddiv(P.bond_coeff, b.d0);
                double* J = S.jac + 6ll * (rs + j);
                J[0] = dmul(dadd(dg, dmul(dmul(ex, ex), r)), cc);
                J[1] = dmul(dadd(dg, dmul(dmul(ey, ey), r)), cc);
                J[2] = dmul(dadd(dg, dmul(dmul(ez, ez), r)), cc);
                J[3] = dmul(dmul(dmul(ex, ey), r), cc);
                J[4] = dmul(dmul(dmul(ex, ez), r), cc);
                J[5] = dmul(dmul(dmul(ey, ez), r), cc);
            }
        }
    }
    if (lane == 0) {
        // force *= C*V*PD_K; new stretch limit; gravity (cg_solver.cuh:325-331)
        double f0 = (double)fx * P.bond_coeff, f1 = (double)fy * P.bond_coeff, f2 = (double)fz * P.bond_coeff;
        if (FP64) {
            f0 = dmul((double)fx, P.bond_coeff);
            f1 = dmul((double)fy, P.bond_coeff);
            f2 = dmul((double)fz, P.bond_coeff);
        }
        const double ss0 = dmul(dsub(P.stretch_a, dmul(P.stretch_b, P.cs)), S.ost[p]);
        S.nst[p] = dsub(ss0, dmul(P.alpha, smin));
        if (P.gravity[0] != 0.0) f0 = dsub(f0, dmul(dmul(P.cs, -P.gravity[0]), P.mass));
        if (P.gravity[1] != 0.0) f1 = dsub(f1, dmul(dmul(P.cs, -P.gravity[1]), P.mass));
        if (P.gravity[2] != 0.0) f2 = dsub(f2, dmul(dmul(P.cs, -P.gravity[2]), P.mass));
        // rigid-sphere penalty contact at the start-of-step position (extension)
        uint8_t actb = (uint8_t)a;
        if (P.sphere_on) {
            const double dx = xp.x - P.sphere_c[0], dy = xp.y - P.sphere_c[1], dz = xp.z - P.sphere_c[2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            const double pen = (P.sphere_r + P.radius) - d;
            if (pen > 0.0 && d > 0.0) {
                const double nx = dx / d, ny = dy / d, nz = dz / d;
                f0 += P.sphere_k * pen * nx;
                f1 += P.sphere_k * pen * ny;
                f2 += P.sphere_k * pen * nz;
                actb |= kActContact;
                if (FP64) {
                    j0 += P.sphere_k * nx * nx; j1 += P.sphere_k * ny * ny; j2 += P.sphere_k * nz * nz;
                    j3 += P.sphere_k * nx * ny; j4 += P.sphere_k * nx * nz; j5 += P.sphere_k * ny * nz;
                }
            }
        }
        S.act[p] = actb;
        force[p] = make_v4<V4>(f0, f1, f2);
        if (FP64) {
            double* D = S.jdiag + 6ll * p;
            D[0] = j0; D[1] = j1; D[2] = j2; D[3] = j3; D[4] = j4; D[5] = j5;
        }
    }
}

// ---- A w -------------------------------------------------------------------------
// Load paths of the SpMV gathers.  The read-only (non-coherent) path may only
// read data that no thread writes during the kernel: a persistent kernel that
// rewrites the CG vector or the positions between its phases (separated by a
// gpu-scope acquire) reads them with ordinary cached loads (ld.global.ca).
enum : int { kLdCoherent = 0, kLdCoherentIn = 1, kLdReadOnly = 2 };

template <int LD, typename T>
__device__ __forceinline__ T ld_pos(const T* p)
{
    if (LD == kLdCoherent) return __ldca(p);
    return __ldg(p);
}
template <int LD, typename T>
__device__ __forceinline__ T ld_in(const T* p)
{
    if (LD == kLdReadOnly) return __ldg(p);
    return __ldca(p);
}
template <int LD>
__device__ __forceinline__ dbl4 ld_in(const dbl4* p)
{
    const double2* q = (const double2*)p;
    const double2 a = LD == kLdReadOnly ? __ldg(q) : __ldca(q);
    const double2 b = LD == kLdReadOnly ? __ldg(q + 1) : __ldca(q + 1);
    return make_dbl4(a.x, a.y, b.x, b.y);
}

// Mixed-precision row result from the group's partial bond sums:
// y_p = m w_p + t2 (c sum_q J'(w_p - w_q) + k_contact n n^T w_p).
template <int G, bool DOT, typename Acc>
__device__ __forceinline__ void spmv_finish_mixed(const StepParams& P, const DeviceState& S, int p, uint8_t ab,
                                                  const float4& w, float ax, float ay, float az, int lane,
                                                  unsigned gmask, float4* __restrict__ out, Acc& acc)
{
    const float c = (float)P.bond_coeff;
    const float t2 = (float)P.t2;
    const float m = (float)P.mass;
    ax = group_sum<G>(ax, gmask);
    ay = group_sum<G>(ay, gmask);
    az = group_sum<G>(az, gmask);
    if (lane == 0) {
        float kx = c * ax, ky = c * ay, kz = c * az;
        if (ab & kActContact) {
            const float4 Xp = S.X32[p];
            const float4 Up = S.u32[p];
            const float dx = Xp.x + Up.x - (float)P.sphere_c_local[0];
            const float dy = Xp.y + Up.y - (float)P.sphere_c_local[1];
            const float dz = Xp.z + Up.z - (float)P.sphere_c_local[2];
            const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
            const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
            const float kn = (float)P.sphere_k * (nx * w.x + ny * w.y + nz * w.z);
            kx += kn * nx; ky += kn * ny; kz += kn * nz;
        }
        const float yx = m * w.x + t2 * kx;
        const float yy = m * w.y + t2 * ky;
        const float yz = m * w.z + t2 * kz;
        out[p] = make_float4(yx, yy, yz, 0.f);
        if (DOT) {
            acc.fma(w.x, yx);
            acc.fma(w.y, yy);
            acc.fma(w.z, yz);
        }
    }
}

// U bonds of one lane in mixed precision: gathers of the neighbours'
// supercell positions and CG entries (every load issued before any
// arithmetic), then each bond's Jacobian applied to w_p - w_q and added to
// (ax, ay, az).  qq[u] < 0 marks an empty slot.
template <int U, int LD, typename Real>
__device__ __forceinline__ void mixed_bond_chunk(const float4* __restrict__ xs4, const float4* __restrict__ in32,
                                                 const float4& xp4, int wp, float sup, const float4& w, int p,
                                                 const int (&qq)[U], const float (&id0)[U], Real& ax, Real& ay,
                                                 Real& az)
{
    float4 Xq[U], Wq[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int q = qq[u] < 0 ? p : qq[u];
        Xq[u] = ld_pos<LD>(xs4 + q);
        Wq[u] = ld_in<LD>(in32 + q);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (qq[u] < 0) continue;
        float cx, cy, cz;
        supercell_delta(__float_as_int(Xq[u].w), wp, sup, cx, cy, cz);
        const float xs = (Xq[u].x - xp4.x) + cx, ys = (Xq[u].y - xp4.y) + cy, zs = (Xq[u].z - xp4.z) + cz;
        const float inv_d0 = id0[u];
        const float inv_d = rsqrtf(fmaf(xs, xs, fmaf(ys, ys, zs * zs)));
        const float wx = w.x - Wq[u].x, wy = w.y - Wq[u].y, wz = w.z - Wq[u].z;
        const float a1 = inv_d0 - inv_d;
        const float g = fmaf(xs, wx, fmaf(ys, wy, zs * wz)) * (inv_d * inv_d * inv_d);
        ax = fmaf(a1, wx, fmaf(g, xs, (float)ax));
        ay = fmaf(a1, wy, fmaf(g, ys, (float)ay));
        az = fmaf(a1, wz, fmaf(g, zs, (float)az));
    }
}

// y_p = (A w)_p by particle p's G-lane group: mass + (beta h^2) stiffness with
// Dirichlet rows projected out.  DOT: lane 0 adds w_p . y_p to acc.
// LD: load path of the positions and of w (kLd*).
template <int G, bool FP64, bool DOT, int U, int LD, typename V4, typename Acc>
__device__ __forceinline__ void spmv_row(const StepParams& P, const DeviceState& S, const V4* __restrict__ in,
                                         V4* __restrict__ out, int p, int lane, unsigned gmask, Acc& acc)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    const Real c = (Real)P.bond_coeff;
    const Real t2 = (Real)P.t2;
    const Real m = (Real)P.mass;
    const uint8_t ab = S.act[p];
    if (is_dirichlet(ab & kActMask)) {
        if (lane == 0) out[p] = make_v4<V4>(0.0, 0.0, 0.0);
        return;
    }
    const V4 w = ld_in<LD>(in + p);
    const int rs = S.row_ptr[p];
    const int cn = S.cnt[p];
    Real ax = 0, ay = 0, az = 0;
    if (FP64) {
        for (int j = lane; j < cn; j += G) {
            const int q = S.col[rs + j];
            const V4 wq = ld_in<LD>(in + q);
            const double* J = S.jac + 6ll * (rs + j);
            ax += J[0] * wq.x + J[3] * wq.y + J[4] * wq.z;
            ay += J[3] * wq.x + J[1] * wq.y + J[5] * wq.z;
            az += J[4] * wq.x + J[5] * wq.y + J[2] * wq.z;
        }
    } else {
        // per bond: the column index and 1/d0 stream in coalesced; the
        // neighbour's supercell position and its CG entry are gathered
        const float4 xp4 = ld_pos<LD>(S.xs4 + p);
        const int wp = __float_as_int(xp4.w);
        const float sup = (float)P.sup;
        const float4* __restrict__ xs4 = S.xs4;
        const float4* __restrict__ in32 = (const float4*)in;
        // lane k takes the U consecutive slots j0 .. j0 + U - 1 of each block
        // of G*U (one 8- or 16-byte load per stream; the bond order of the
        // slots is arranged by launch_bond_relayout for this shape).  Rows
        // start 32-byte aligned and hold a multiple of 8 slots, so the vector
        // loads stay inside the row.
        for (int j0 = lane * U; j0 < cn; j0 += G * U) {
            // issue every load of U bonds before any arithmetic
            int qq[U];
            float id0[U];
            if constexpr (U == 4) {
                const int4 c4 = __ldcs((const int4*)(S.col + rs + j0));
                const float4 d4 = __ldcs((const float4*)(S.inv_d0 + rs + j0));
                qq[0] = c4.x; qq[1] = c4.y; qq[2] = c4.z; qq[3] = c4.w;
                id0[0] = d4.x; id0[1] = d4.y; id0[2] = d4.z; id0[3] = d4.w;
            } else if constexpr (U == 2) {
                const int2 c2 = __ldcs((const int2*)(S.col + rs + j0));
                const float2 d2 = __ldcs((const float2*)(S.inv_d0 + rs + j0));
                qq[0] = c2.x; qq[1] = c2.y;
                id0[0] = d2.x; id0[1] = d2.y;
            } else {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    qq[u] = __ldcs(S.col + rs + j0 + u);
                    id0[u] = __ldcs(S.inv_d0 + rs + j0 + u);
                }
            }
#pragma unroll
            for (int u = 1; u < U; ++u)
                if (j0 + u >= cn) qq[u] = -1;
            mixed_bond_chunk<U, LD>(xs4, in32, xp4, wp, sup, make_float4((float)w.x, (float)w.y, (float)w.z, 0.f), p,
                                    qq, id0, ax, ay, az);
        }
    }
    if constexpr (!FP64) {
        spmv_finish_mixed<G, DOT>(P, S, p, ab, w, ax, ay, az, lane, gmask, out, acc);
        return;
    }
    ax = group_sum<G>(ax, gmask);
    ay = group_sum<G>(ay, gmask);
    az = group_sum<G>(az, gmask);
    if (lane == 0) {
        Real kx, ky, kz;
        if (FP64) {
            const double* D = S.jdiag + 6ll * p;
            kx = D[0] * w.x + D[3] * w.y + D[4] * w.z - ax;
            ky = D[3] * w.x + D[1] * w.y + D[5] * w.z - ay;
            kz = D[4] * w.x + D[5] * w.y + D[2] * w.z - az;
        } else {
            kx = c * ax; ky = c * ay; kz = c * az;
            if (ab & kActContact) {
                const float4 Xp = S.X32[p];
                const float4 Up = S.u32[p];
                const float dx = Xp.x + Up.x - (float)P.sphere_c_local[0];
                const float dy = Xp.y + Up.y - (float)P.sphere_c_local[1];
                const float dz = Xp.z + Up.z - (float)P.sphere_c_local[2];
                const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
                const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
                const float kn = (float)P.sphere_k * (nx * (float)w.x + ny * (float)w.y + nz * (float)w.z);
                kx += kn * nx; ky += kn * ny; kz += kn * nz;
            }
        }
        const Real yx = m * (Real)w.x + t2 * kx;
        const Real yy = m * (Real)w.y + t2 * ky;
        const Real yz = m * (Real)w.z + t2 * kz;
        V4 yv;
        yv.x = yx; yv.y = yy; yv.z = yz; yv.w = 0;
        out[p] = yv;
        if (DOT) {
            acc.fma(w.x, yx);
            acc.fma(w.y, yy);
            acc.fma(w.z, yz);
        }
    }
}

// ---- CG vector bodies (CUSP krylov::cg, identity preconditioner) -----------------
// Right-hand side with this step's final time step (the adaptive scheme may
// have changed it after the force pass, simulator.cu:540-572, before
// fillVectorB*): b = m v + h f (implicit_euler.cuh:83-84) or
// b = h (m v + (h/2) f) (newmark_beta.cuh:264-265).
// Dirichlet values: clamped and invisible particles 0, prescribed particles their
// velocity (implicit Euler) or h * velocity (Newmark); ||b|| over free rows.
template <bool FP64, typename Acc>
__device__ __forceinline__ void cg_init_elem(const StepParams& P, const DeviceState& S, int i, Acc& acc)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    V4* x = (V4*)S.sol;
    V4* b = (V4*)S.rhs;
    const V4* force = (const V4*)S.force;
    const int a = S.act[i] & kActMask;
    const dbl4 v = S.v64[i];
    const V4 f = force[i];
    double b0, b1, b2;
    if (P.integrator == 0) {
        b0 = dadd(dmul(P.mass, v.x), dmul(P.h, (double)f.x));
        b1 = dadd(dmul(P.mass, v.y), dmul(P.h, (double)f.y));
        b2 = dadd(dmul(P.mass, v.z), dmul(P.h, (double)f.z));
    } else {
        const double hh = dmul(0.5, P.h);
        b0 = dmul(P.h, dadd(dmul(P.mass, v.x), dmul(hh, (double)f.x)));
        b1 = dmul(P.h, dadd(dmul(P.mass, v.y), dmul(hh, (double)f.y)));
        b2 = dmul(P.h, dadd(dmul(P.mass, v.z), dmul(hh, (double)f.z)));
    }
    const V4 bv = make_v4<V4>(b0, b1, b2);
    b[i] = bv;
    if (is_dirichlet(a)) {
        double ux = 0, uy = 0, uz = 0;
        if (a == ACT_PRESCRIBED) {
            const double s = P.integrator == 0 ? 1.0 : P.h;
            ux = v.x * s; uy = v.y * s; uz = v.z * s;
        }
        x[i] = make_v4<V4>(ux, uy, uz);
    } else {
        acc.fma(bv.x, bv.x);
        acc.fma(bv.y, bv.y);
        acc.fma(bv.z, bv.z);
    }
}

// r = b - A x0 on free rows (y holds A x0), p = r
template <bool FP64, typename Acc>
__device__ __forceinline__ void residual_elem(const DeviceState& S, int i, Acc& acc)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    const V4* b = (const V4*)S.rhs;
    const V4* y = (const V4*)S.y;
    V4 rv;
    if (is_dirichlet(S.act[i] & kActMask)) {
        rv.x = 0; rv.y = 0; rv.z = 0; rv.w = 0;
    } else {
        const V4 bv = b[i], yv = y[i];
        rv.x = bv.x - yv.x; rv.y = bv.y - yv.y; rv.z = bv.z - yv.z; rv.w = 0;
        acc.fma(rv.x, rv.x);
        acc.fma(rv.y, rv.y);
        acc.fma(rv.z, rv.z);
    }
    ((V4*)S.r)[i] = rv;
    ((V4*)S.p)[i] = rv;
}

// x += alpha p ; r -= alpha A p ; acc += <r, r>
template <bool FP64, typename Real, typename Acc>
__device__ __forceinline__ void axpy_elem(const DeviceState& S, int i, Real alpha, Acc& acc)
{
    using V4 = typename Vec4<Real>::type;
    V4* x = (V4*)S.sol;
    V4* r = (V4*)S.r;
    const V4 pi = ((const V4*)S.p)[i], yi = ((const V4*)S.y)[i];
    V4 xi = x[i], ri = r[i];
    xi.x += alpha * pi.x; xi.y += alpha * pi.y; xi.z += alpha * pi.z;
    ri.x -= alpha * yi.x; ri.y -= alpha * yi.y; ri.z -= alpha * yi.z;
    x[i] = xi;
    r[i] = ri;
    acc.fma(ri.x, ri.x);
    acc.fma(ri.y, ri.y);
    acc.fma(ri.z, ri.z);
}

// p = r + beta p
template <bool FP64, typename Real>
__device__ __forceinline__ void xpby_elem(const DeviceState& S, int i, Real beta)
{
    using V4 = typename Vec4<Real>::type;
    V4* pv = (V4*)S.p;
    const V4 ri = ((const V4*)S.r)[i];
    V4 pi = pv[i];
    pi.x = ri.x + beta * pi.x;
    pi.y = ri.y + beta * pi.y;
    pi.z = ri.z + beta * pi.z;
    pv[i] = pi;
}

// Scalar updates of the CG state, run once per reduction by its finisher.
__device__ __forceinline__ void cg_fin_init(CgScalars* sc, double bb)
{
    sc->bnorm2 = bb;
    sc->tol = 0.0 + sc->rel_tol * sqrt(bb);
    sc->iter = 0;
    sc->done = 0;
    sc->converged = 0;
}

// rz = <r,r>; convergence test before the first iteration
__device__ __forceinline__ void cg_fin_residual(CgScalars* sc, double rr)
{
    sc->rz = rr;
    sc->beta = 0.0;   // p = r: a direction update fused into the next product keeps p as it is
    sc->rnorm = sqrt(rr);
    if (sc->rnorm <= sc->tol) {
        sc->done = 1;
        sc->converged = 1;
    } else if (sc->iter >= sc->max_iter) {
        sc->done = 1;
    }
}

__device__ __forceinline__ void cg_fin_alpha(CgScalars* sc, double pAp)
{
    sc->pAp = pAp;
    sc->alpha = sc->rz / pAp;
}

// rz' = <r,r> ; beta = rz'/rz ; iteration count and test
__device__ __forceinline__ void cg_fin_axpy(CgScalars* sc, double rr)
{
    const double rz_old = sc->rz;
    sc->rz = rr;
    sc->beta = rr / rz_old;
    sc->iter += 1;
    sc->rnorm = sqrt(rr);
    if (sc->rnorm <= sc->tol) {
        sc->done = 1;
        sc->converged = 1;
    } else if (sc->iter >= sc->max_iter) {
        sc->done = 1;
    }
}

// ---- preconditioner ---------------------------------------------------------------
// M = D^-1 from the symmetric diagonal block D = (xx yy zz xy xz yz) of A:
// mode 2 inverts the block (adjugate over determinant) where it is positive
// definite, mode 1 -- and mode 2 elsewhere -- inverts its diagonal; a
// non-positive diagonal entry takes 1 / mass.
__device__ __forceinline__ void pc_invert(int mode, double mass, const double (&D)[6], double (&M)[6])
{
    const double a = D[0], b = D[1], c = D[2], d = D[3], e = D[4], f = D[5];
    if (mode == 2) {
        const double c00 = b * c - f * f, c11 = a * c - e * e, c22 = a * b - d * d;
        const double c01 = e * f - d * c, c02 = d * f - b * e, c12 = d * e - a * f;
        const double det = a * c00 + d * c01 + e * c02;
        if (a > 0.0 && c22 > 0.0 && det > 0.0) {
            const double id = 1.0 / det;
            M[0] = c00 * id; M[1] = c11 * id; M[2] = c22 * id;
            M[3] = c01 * id; M[4] = c02 * id; M[5] = c12 * id;
            return;
        }
    }
    const double im = 1.0 / mass;
    M[0] = a > 0.0 ? 1.0 / a : im;
    M[1] = b > 0.0 ? 1.0 / b : im;
    M[2] = c > 0.0 ? 1.0 / c : im;
    M[3] = M[4] = M[5] = 0.0;
}

template <typename V4>
__device__ __forceinline__ V4 pc_apply(const V4* __restrict__ pc, int i, const V4& r)
{
    const V4 m0 = pc[2 * i], m1 = pc[2 * i + 1];
    V4 z;
    z.x = m0.x * r.x + m0.w * r.y + m1.x * r.z;
    z.y = m0.w * r.x + m0.y * r.y + m1.y * r.z;
    z.z = m1.x * r.x + m1.y * r.y + m0.z * r.z;
    z.w = 0;
    return z;
}

// z = M r, p = z; rr += <r, r>, rz += <r, z>
template <bool FP64, typename Acc>
__device__ __forceinline__ void pcg_start_elem(const DeviceState& S, int i, Acc& rr, Acc& rz)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    const V4 ri = ((const V4*)S.r)[i];
    const V4 zi = pc_apply((const V4*)S.pc, i, ri);
    ((V4*)S.z)[i] = zi;
    ((V4*)S.p)[i] = zi;
    rr.fma(ri.x, ri.x); rr.fma(ri.y, ri.y); rr.fma(ri.z, ri.z);
    rz.fma(ri.x, zi.x); rz.fma(ri.y, zi.y); rz.fma(ri.z, zi.z);
}

// x += alpha p ; r -= alpha A p ; z = M r ; rr += <r, r>, rz += <r, z>
template <bool FP64, typename Real, typename Acc>
__device__ __forceinline__ void axpy_pc_elem(const DeviceState& S, int i, Real alpha, Acc& rr, Acc& rz)
{
    using V4 = typename Vec4<Real>::type;
    V4* x = (V4*)S.sol;
    V4* r = (V4*)S.r;
    const V4 pi = ((const V4*)S.p)[i], yi = ((const V4*)S.y)[i];
    V4 xi = x[i], ri = r[i];
    xi.x += alpha * pi.x; xi.y += alpha * pi.y; xi.z += alpha * pi.z;
    ri.x -= alpha * yi.x; ri.y -= alpha * yi.y; ri.z -= alpha * yi.z;
    x[i] = xi;
    r[i] = ri;
    const V4 zi = pc_apply((const V4*)S.pc, i, ri);
    ((V4*)S.z)[i] = zi;
    rr.fma(ri.x, ri.x); rr.fma(ri.y, ri.y); rr.fma(ri.z, ri.z);
    rz.fma(ri.x, zi.x); rz.fma(ri.y, zi.y); rz.fma(ri.z, zi.z);
}

// rho = <r, z> for the direction, ||r|| for the test (as the plain CG)
__device__ __forceinline__ void cg_fin_pcg_start(CgScalars* sc, double rr, double rz)
{
    sc->rr = rr;
    sc->rz = rz;
    sc->beta = 0.0;
    sc->rnorm = sqrt(rr);
    if (sc->rnorm <= sc->tol) {
        sc->done = 1;
        sc->converged = 1;
    } else if (sc->iter >= sc->max_iter) {
        sc->done = 1;
    }
}

__device__ __forceinline__ void cg_fin_axpy_pc(CgScalars* sc, double rr, double rz)
{
    const double rz_old = sc->rz;
    sc->rr = rr;
    sc->rz = rz;
    sc->beta = rz / rz_old;
    sc->iter += 1;
    sc->rnorm = sqrt(rr);
    if (sc->rnorm <= sc->tol) {
        sc->done = 1;
        sc->converged = 1;
    } else if (sc->iter >= sc->max_iter) {
        sc->done = 1;
    }
}

// ---- position / velocity update ------------------------------------------------
// box reflection of updatePDPosition* (implicit_euler.cuh:116-168), FP64, same order
__device__ __forceinline__ void reflect(const StepParams& P, double& np, double& nv, int k)
{
    const double mn = dadd(P.bmin[k], P.radius);
    const double mx = dsub(P.bmax[k], P.radius);
    if (np > mx) {
        nv = dmul(nv, -P.restitution);
        np = dsub(mx, dmul(P.restitution, dsub(np, mx)));
    }
    if (np < mn) {
        nv = dmul(nv, -P.restitution);
        np = dadd(mn, dmul(P.restitution, dsub(mn, np)));
    }
}

template <bool FP64>
__device__ __forceinline__ void update_elem(const StepParams& P, const DeviceState& S, int i)
{
    using Real = typename std::conditional<FP64, double, float>::type;
    using V4 = typename Vec4<Real>::type;
    const V4* sol = (const V4*)S.sol;
    S.st[i] = S.nst[i];   // updatePDStretchNeighborList (simulator.cuh:2601-2620)
    if constexpr (!FP64) S.lim[i] = limit_pair(S.nst[i]);
    const int a = S.act[i] & kActMask;
    const dbl4 x = S.x64[i];
    dbl4 v = S.v64[i];
    if (a == ACT_INVISIBLE) {
        if (P.integrator == 0) S.v64[i] = make_dbl4(0.0, 0.0, 0.0, 0.0);
        return;
    }
    double nv[3], np[3];
    const double xs[3] = {x.x, x.y, x.z};
    const double vs[3] = {v.x, v.y, v.z};
    if (P.integrator == 0) {
        // transferData(PD_VELOCITY <- PD_SYSTEM_SOLUTION); x += v * base * ticks
        if (a == ACT_PRESCRIBED) {
            nv[0] = vs[0]; nv[1] = vs[1]; nv[2] = vs[2];
        } else if (a == ACT_CLAMPED) {
            nv[0] = nv[1] = nv[2] = 0.0;
        } else {
            const V4 s = sol[i];
            nv[0] = (double)s.x; nv[1] = (double)s.y; nv[2] = (double)s.z;
        }
        for (int k = 0; k < 3; ++k) np[k] = dadd(xs[k], dmul(dmul(nv[k], P.dt_base), (double)P.ticks));
    } else {
        // v = 2/h dx - v ; x += dx
        double dx[3];
        if (a == ACT_PRESCRIBED) {
            for (int k = 0; k < 3; ++k) { dx[k] = dmul(P.h, vs[k]); nv[k] = vs[k]; }
        } else if (a == ACT_CLAMPED) {
            for (int k = 0; k < 3; ++k) { dx[k] = 0.0; nv[k] = 0.0; }
        } else {
            const V4 s = sol[i];
            dx[0] = (double)s.x; dx[1] = (double)s.y; dx[2] = (double)s.z;
            const double two_h = ddiv(2.0, P.h);
            for (int k = 0; k < 3; ++k) nv[k] = dsub(dmul(two_h, dx[k]), vs[k]);
        }
        for (int k = 0; k < 3; ++k) np[k] = dadd(xs[k], dx[k]);
    }
    if (P.box_enabled)
        for (int k = 0; k < 3; ++k) reflect(P, np[k], nv[k], k);
    S.x64[i] = make_dbl4(np[0], np[1], np[2], 0.0);
    S.v64[i] = make_dbl4(nv[0], nv[1], nv[2], 0.0);
}

// The supercell words of one particle's position, before a force pass
__device__ __forceinline__ void supercell_elem(const StepParams& P, const DeviceState& S, int i)
{
    encode_supercell_df(P, S.x64[i], S.xs4[i], S.xlo4[i]);
}

// FP32 displacement and supercell position from the FP64 master positions
// (after a rollback restore); the contact bit is cleared
__device__ __forceinline__ void refresh_elem(const StepParams& P, const DeviceState& S, int i)
{
    const dbl4 x = S.x64[i], X = S.X64[i];
    S.u32[i] = make_float4((float)(x.x - X.x), (float)(x.y - X.y), (float)(x.z - X.z), 0.f);
    if (S.xs4) encode_supercell_df(P, x, S.xs4[i], S.xlo4[i]);
    S.act[i] &= kActMask;
}

}  // namespace pdgb
