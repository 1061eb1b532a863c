// Device readouts of the 18 reference attributes (+ bounding-box elongation) from
// the accumulated records.  Each expression keeps the reference's operand order and
// float/double mix (attributes.c:102-880), because filter thresholds and spectrum
// bin edges are compared against these values exactly.  Build with --fmad=false.
#pragma once
#include "dcf_kernels.cuh"

namespace dcf {

// ---- double-double helpers (Dekker / Knuth error-free transformations) ----
struct dd {
    double hi, lo;
};
__device__ __forceinline__ dd two_sum(double a, double b)
{
    double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dd two_prod(double a, double b)
{
    double p = a * b;
    return {p, fma(a, b, -p)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    double lo = s.lo + a.lo + b.lo;
    return two_sum(s.hi, lo);
}
__device__ __forceinline__ dd dd_mul(dd a, dd b)
{
    dd p = two_prod(a.hi, b.hi);
    double lo = p.lo + (a.hi * b.lo + a.lo * b.hi);
    return two_sum(p.hi, lo);
}
__device__ __forceinline__ dd dd_div_d(dd a, double b)
{
    double q1 = a.hi / b;
    dd r = dd_add(a, two_prod(-q1, b));
    double q2 = r.hi / b;
    return two_sum(q1, q2);
}

// pow(x, 5.0/3.0) for x > 0 as glibc computes it (~0.52 ulp, i.e. correctly
// rounded almost always).  The exponent is the double nearest 5/3, which exceeds
// 5/3 by delta = 7.4014868308343770e-17, so x^e = x^(5/3) * (1 + delta*ln x + ...).
// x^(5/3) is formed in double-double (Newton steps t <- t - (t^3 - x)/(3 t^2) for the
// cube root, then x*t*t) and the delta term is added before the single final
// rounding.  CUDA's own pow (2 ulp) would move non-compactness thresholds.
__device__ __forceinline__ double pow_5_3(double x)
{
    const double delta = 7.4014868308343770e-17;
    double t0 = cbrt(x);
    dd t = {t0, 0.0};
    for (int it = 0; it < 2; it++) {
        dd t2 = dd_mul(t, t);
        dd t3 = dd_mul(t2, t);
        dd f = dd_add(t3, {-x, 0.0});
        dd d = dd_div_d(f, 3.0 * t2.hi);
        t = dd_add(t, {-d.hi, -d.lo});
    }
    dd r = dd_mul(dd_mul({x, 0.0}, t), t);
    return r.hi + (r.lo + r.hi * (delta * log(x)));
}

__device__ __forceinline__ double gsum(const AttrBufs &a, int d, int u)
{
    return a.exact_g ? (double)(long long)((const unsigned long long *)a.gw[d])[u] : ((const double *)a.gw[d])[u];
}

// the group's `area` readout (AttribsArray[i].area)
__device__ __forceinline__ double area_value(const AttrBufs &a, int u, const float *pd)
{
    const unsigned ar = a.area[u];
    switch (a.group) {
    case 0: /* area_attribute: float product times (float) area (attributes.c:105) */
        return (double)__fmul_rn(__fmul_rn(__fmul_rn(pd[0], pd[1]), pd[2]), __uint2float_rn(ar));
    case 1: /* extent_area_attribute (attributes.c:213) */
        return (double)ar;
    case 2: /* mean_area_attribute (attributes.c:348) */
        return (double)__fmul_rn(__fmul_rn(pd[0], pd[1]), pd[2]) * (double)ar;
    case 3: /* wmean_area_attribute (attributes.c:465) */
        return (double)ar;
    default: /* inertia_area_attribute (attributes.c:700) */
        return (double)pd[0] * (double)pd[1] * (double)pd[2] * (double)ar;
    }
}

// inertia_arr (attributes.c:628-648)
__device__ __forceinline__ void inertia_arr(const AttrBufs &a, int u, const float *pd, double in[15])
{
    in[0] = (double)pd[0] * (double)pd[1] * (double)pd[2] * (double)a.area[u];
    in[1] = (double)pd[0] * (double)a.s1[0][u];
    in[2] = (double)pd[1] * (double)a.s1[1][u];
    in[3] = (double)pd[2] * (double)a.s1[2][u];
    in[4] = (double)__fmul_rn(pd[0], pd[0]) * (double)a.s2[0][u];
    in[5] = (double)__fmul_rn(pd[1], pd[1]) * (double)a.s2[1][u];
    in[6] = (double)__fmul_rn(pd[2], pd[2]) * (double)a.s2[2][u];
    in[7] = (double)__fmul_rn(pd[0], pd[1]) * (double)a.s2[3][u];
    in[8] = (double)__fmul_rn(pd[1], pd[2]) * (double)a.s2[4][u];
    in[9] = (double)__fmul_rn(pd[0], pd[2]) * (double)a.s2[5][u];
    in[10] = gsum(a, 0, u);
    in[11] = gsum(a, 1, u);
    in[12] = (double)pd[0] * gsum(a, 2, u);
    in[13] = (double)pd[1] * gsum(a, 3, u);
    in[14] = (double)pd[2] * gsum(a, 4, u);
}

// Centroids as the inertia group reports them in the tree file
// (inertia_attribute_arr, attributes.c:629-641): k = 0..2 mean x, y, z =
// in[1+k] / in[0]; k = 3..5 grey-weighted means in[12+k-3] / in[10].  They differ
// from the mean and weighted-mean attributes (6-11) when the pixel size is not 1.
__device__ __forceinline__ double inertia_column(const AttrBufs &a, int k, int u, const float *pd)
{
    double in[15];
    inertia_arr(a, u, pd, in);
    return k < 3 ? in[1 + k] / in[0] : in[12 + k - 3] / in[10];
}

__device__ __forceinline__ double attr_value(const AttrBufs &a, int attr, int u, const float *pd)
{
    switch (attr) {
    case 0: /* area_attribute (attributes.c:105); every group's record has the area count */
        return (double)__fmul_rn(__fmul_rn(__fmul_rn(pd[0], pd[1]), pd[2]), __uint2float_rn(a.area[u]));
    case 1: { /* extent_rectarea_attribute (attributes.c:218) */
        double v = (double)(a.bmax[0][u] - a.bmin[0][u]) * (double)(a.bmax[1][u] - a.bmin[1][u]) *
                   (double)(a.bmax[2][u] - a.bmin[2][u]);
        return v * (double)__fmul_rn(__fmul_rn(pd[0], pd[1]), pd[2]);
    }
    case 2: { /* extent_rectdiag_attribute (attributes.c:234) */
        double mnx = (double)pd[0] * (double)a.bmin[0][u], mny = (double)pd[1] * (double)a.bmin[1][u];
        double mnz = (double)pd[2] * (double)a.bmin[2][u];
        double mxx = (double)pd[0] * (double)a.bmax[0][u], mxy = (double)pd[1] * (double)a.bmax[1][u];
        double mxz = (double)pd[2] * (double)a.bmax[2][u];
        return (mxx - mnx) * (mxx - mnx) + (mxy - mny) * (mxy - mny) + (mxz - mnz) * (mxz - mnz);
    }
    case 3: return (double)pd[0] * (double)(a.bmax[0][u] - a.bmin[0][u]);
    case 4: return (double)pd[1] * (double)(a.bmax[1][u] - a.bmin[1][u]);
    case 5: return (double)pd[2] * (double)(a.bmax[2][u] - a.bmin[2][u]);
    case 6: return (double)pd[0] * (double)a.s1[0][u] / (double)a.area[u];
    case 7: return (double)pd[1] * (double)a.s1[1][u] / (double)a.area[u];
    case 8: return (double)pd[2] * (double)a.s1[2][u] / (double)a.area[u];
    case 9: return (double)pd[0] * gsum(a, 2, u) / gsum(a, 0, u);
    case 10: return (double)pd[1] * gsum(a, 3, u) / gsum(a, 0, u);
    case 11: return (double)pd[2] * gsum(a, 4, u) / gsum(a, 0, u);
    case 12: return gsum(a, 0, u);
    case 18: { /* bounding-box elongation (not a reference attribute) */
        double xe = (double)pd[0] * (double)(a.bmax[0][u] - a.bmin[0][u]);
        double ye = (double)pd[1] * (double)(a.bmax[1][u] - a.bmin[1][u]);
        double hi = xe > ye ? xe : ye, lo = xe < ye ? xe : ye;
        return hi / (lo > 1.0 ? lo : 1.0);
    }
    default:
        break;
    }
    double in[15];
    inertia_arr(a, u, pd, in);
    const double corr = in[0] / 12;
    double mat[6];
    mat[0] = in[4] - in[1] * in[1] / in[0] + (double)pd[0] * corr;
    mat[1] = in[5] - in[2] * in[2] / in[0] + (double)pd[1] * corr;
    mat[2] = in[6] - in[3] * in[3] / in[0] + (double)pd[2] * corr;
    mat[3] = in[7] - in[1] * in[2] / in[0];
    mat[4] = in[8] - in[2] * in[3] / in[0];
    mat[5] = in[9] - in[1] * in[3] / in[0];
    const bool flat2d = in[3] == 0;
    switch (attr) {
    case 13:
        return flat2d ? (mat[0] + mat[1]) : (mat[0] + mat[1] + mat[2]);
    case 14:
    case 15:
    case 16: {
        if (flat2d) {
            if (attr == 15) return -1;
            double m2[4] = {mat[0], mat[3], mat[3], mat[1]}, ev[2];
            dcf_sym_eigenvalues(2, m2, ev);
            if (attr == 14) return ev[1] / ev[0];
            double ax0 = sqrt(4 * ev[1] / in[0]), ax1 = sqrt(4 * ev[0] / in[0]);
            return M_PI * ax0 * ax1 / (in[0]);
        }
        double m3[9] = {mat[0], mat[3], mat[5], mat[3], mat[1], mat[4], mat[5], mat[4], mat[2]}, ev[3];
        dcf_sym_eigenvalues(3, m3, ev);
        if (attr == 14) return ev[2] / ev[1];
        if (attr == 15) return ev[1] / ev[0];
        double ax0 = sqrt(20 * ev[2] / in[0]), ax1 = sqrt(20 * ev[1] / in[0]), ax2 = sqrt(20 * ev[0] / in[0]);
        return M_PI * ax0 * ax1 * ax2 / (6 * in[0]);
    }
    case 17:
        // pow(area, 2.0) is exactly area*area whenever that is representable
        if (flat2d) return (mat[0] + mat[1]) / (in[0] * in[0]);
        return (mat[0] + mat[1] + mat[2]) / pow_5_3(in[0]);
    default:
        return __longlong_as_double(0x7ff8000000000000LL);
    }
}

}  // namespace dcf
