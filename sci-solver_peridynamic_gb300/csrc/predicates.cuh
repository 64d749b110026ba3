// predicates.cuh -- exact signs of the 2D and 3D orientation determinants
// (host and device).
//
// The method is Shewchuk's (Adaptive Precision Floating-Point Arithmetic and
// Fast Robust Geometric Predicates, 1997): evaluate the determinant in FP64
// with a forward error bound; when the result is too close to zero for its
// sign to be certain, evaluate the determinant exactly as a nonoverlapping
// expansion (a sum of doubles) built with error-free transformations -- the
// two-sum of Knuth and the FMA two-product -- and take the sign of its
// largest component.  Only the sign is returned: that is all the ray-casting
// inside test uses (a zero sign means "exactly on").
//
// Every FP64 operation here is an explicitly rounded one (no contraction), so
// the host and device evaluations are identical.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define PD_HD __host__ __device__ __forceinline__
#else
#define PD_HD inline
#endif

namespace pdgb {
namespace pred {

#if defined(__CUDA_ARCH__)
PD_HD double add(double a, double b) { return __dadd_rn(a, b); }
PD_HD double sub(double a, double b) { return __dsub_rn(a, b); }
PD_HD double mul(double a, double b) { return __dmul_rn(a, b); }
PD_HD double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
#else
PD_HD double add(double a, double b) { return a + b; }
PD_HD double sub(double a, double b) { return a - b; }
PD_HD double mul(double a, double b) { return a * b; }
PD_HD double fma_(double a, double b, double c) { return std::fma(a, b, c); }
#endif

// x + y = a + b exactly, |y| <= ulp(x) / 2 (Knuth)
PD_HD void two_sum(double a, double b, double& x, double& y)
{
    x = add(a, b);
    const double bv = sub(x, a);
    const double av = sub(x, bv);
    y = add(sub(a, av), sub(b, bv));
}

// x + y = a * b exactly
PD_HD void two_prod(double a, double b, double& x, double& y)
{
    x = mul(a, b);
    y = fma_(a, b, -x);
}

// e[0..n) nonoverlapping, increasing magnitude, no zeros; e += b (in place,
// into out which may alias e only when out has room for n + 1).  Returns the
// new length.  (Grow-Expansion with zero elimination.)
PD_HD int grow(const double* e, int n, double b, double* out)
{
    double q = b;
    int k = 0;
    for (int i = 0; i < n; ++i) {
        double qn, h;
        two_sum(q, e[i], qn, h);
        if (h != 0.0) out[k++] = h;
        q = qn;
    }
    if (q != 0.0 || k == 0) out[k++] = q;
    return k;
}

PD_HD int sign_of(const double* e, int n)
{
    for (int i = n - 1; i >= 0; --i)
        if (e[i] != 0.0) return e[i] > 0.0 ? 1 : -1;
    return 0;
}

// Adds the exact product a * b (a, b given as two-term sums a0 + a1, b0 + b1)
// times sign s into the expansion acc.
PD_HD int add_product2(double* acc, int n, double a0, double a1, double b0, double b1, double s)
{
    const double av[2] = {a0, a1}, bv[2] = {b0, b1};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            if (av[i] == 0.0 || bv[j] == 0.0) continue;
            double x, y;
            two_prod(av[i], bv[j], x, y);
            n = grow(acc, n, s * x, acc);
            if (y != 0.0) n = grow(acc, n, s * y, acc);
        }
    return n;
}

// Adds the exact product a * b * c of two-term sums, times sign s.
PD_HD int add_product3(double* acc, int n, const double* a, const double* b, const double* c, double s)
{
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            if (a[i] == 0.0 || b[j] == 0.0) continue;
            double x, y;
            two_prod(a[i], b[j], x, y);
            const double xy[2] = {x, y};
            for (int u = 0; u < 2; ++u)
                for (int k = 0; k < 2; ++k) {
                    if (xy[u] == 0.0 || c[k] == 0.0) continue;
                    double p, q;
                    two_prod(xy[u], c[k], p, q);
                    n = grow(acc, n, s * p, acc);
                    if (q != 0.0) n = grow(acc, n, s * q, acc);
                }
        }
    return n;
}

// Exact difference a - b as a two-term sum (hi, lo).
PD_HD void diff2(double a, double b, double* d)
{
    double x, y;
    x = sub(a, b);
    const double bv = sub(a, x);
    const double av = add(x, bv);
    y = add(sub(a, av), sub(bv, b));
    d[0] = x;
    d[1] = y;
}

constexpr double kEps = 1.1102230246251565e-16;   // 2^-53
constexpr double kCcwErrA = (3.0 + 16.0 * kEps) * kEps;
constexpr double kO3dErrA = (7.0 + 56.0 * kEps) * kEps;

// sign of (ax - cx)(by - cy) - (ay - cy)(bx - cx): > 0 when a, b, c turn
// counterclockwise in the xy projection
PD_HD int orient2d(const double* a, const double* b, const double* c)
{
    const double detl = mul(sub(a[0], c[0]), sub(b[1], c[1]));
    const double detr = mul(sub(a[1], c[1]), sub(b[0], c[0]));
    const double det = sub(detl, detr);
    const double bound = mul(kCcwErrA, add(fabs(detl), fabs(detr)));
    if (det > bound) return 1;
    if (-det > bound) return -1;
    double ax[2], ay[2], bx[2], by[2];
    diff2(a[0], c[0], ax);
    diff2(a[1], c[1], ay);
    diff2(b[0], c[0], bx);
    diff2(b[1], c[1], by);
    double acc[20];
    int n = 0;
    n = add_product2(acc, n, ax[0], ax[1], by[0], by[1], 1.0);
    n = add_product2(acc, n, ay[0], ay[1], bx[0], bx[1], -1.0);
    return sign_of(acc, n);
}

// sign of det [a - d; b - d; c - d] (rows): > 0 when d lies below the plane
// of a, b, c, with a, b, c counterclockwise seen from above
PD_HD int orient3d(const double* a, const double* b, const double* c, const double* d)
{
    const double adx = sub(a[0], d[0]), ady = sub(a[1], d[1]), adz = sub(a[2], d[2]);
    const double bdx = sub(b[0], d[0]), bdy = sub(b[1], d[1]), bdz = sub(b[2], d[2]);
    const double cdx = sub(c[0], d[0]), cdy = sub(c[1], d[1]), cdz = sub(c[2], d[2]);
    const double bdxcdy = mul(bdx, cdy), cdxbdy = mul(cdx, bdy);
    const double cdxady = mul(cdx, ady), adxcdy = mul(adx, cdy);
    const double adxbdy = mul(adx, bdy), bdxady = mul(bdx, ady);
    const double det = add(add(mul(adz, sub(bdxcdy, cdxbdy)), mul(bdz, sub(cdxady, adxcdy))),
                           mul(cdz, sub(adxbdy, bdxady)));
    const double perm = add(add(mul(add(fabs(bdxcdy), fabs(cdxbdy)), fabs(adz)),
                                mul(add(fabs(cdxady), fabs(adxcdy)), fabs(bdz))),
                            mul(add(fabs(adxbdy), fabs(bdxady)), fabs(cdz)));
    const double bound = mul(kO3dErrA, perm);
    if (det > bound) return 1;
    if (-det > bound) return -1;
    double A[3][2], B[3][2], C[3][2];
    for (int k = 0; k < 3; ++k) {
        diff2(a[k], d[k], A[k]);
        diff2(b[k], d[k], B[k]);
        diff2(c[k], d[k], C[k]);
    }
    // 6 triple products, each at most 32 terms
    double acc[200];
    int n = 0;
    n = add_product3(acc, n, A[2], B[0], C[1], 1.0);
    n = add_product3(acc, n, A[2], C[0], B[1], -1.0);
    n = add_product3(acc, n, B[2], C[0], A[1], 1.0);
    n = add_product3(acc, n, B[2], A[0], C[1], -1.0);
    n = add_product3(acc, n, C[2], A[0], B[1], 1.0);
    n = add_product3(acc, n, C[2], B[0], A[1], -1.0);
    return sign_of(acc, n);
}

}  // namespace pred
}  // namespace pdgb
