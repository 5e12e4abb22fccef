// FP64 helpers shared by the singular and nearly singular kernels: the
// accumulator, a short-argument sincos, the plane frame of a flat element and
// its side geometry, the corner angles seen from an interior point, and the
// scaled FP64 store.
#pragma once

#include <cmath>

#include "geom.cuh"

namespace nihu {

constexpr double INV_FOUR_PI = 1.0 / FOUR_PI;

struct Acc {
    double sr = 0, si = 0, dr = 0, di = 0;
};

// Maclaurin series of cos and sin truncated after x^22 / x^23: on
// |x| <= pi/2 the first omitted terms are below 1e-19, so these agree with the
// correctly rounded values to a few ulp at a fraction of the cost of the
// general routines (which reduce arbitrary arguments).  Coefficients are
// (-1)^n / (2n)! and (-1)^n / (2n+1)!.
struct TaylorCoeffs {
    double c[12], s[12];
    constexpr TaylorCoeffs() : c(), s()
    {
        double fc = 1.0, fs = 1.0;  // (2n)! and (2n+1)!
        for (int n = 0; n < 12; ++n) {
            if (n > 0) {
                fc *= (2.0 * n - 1.0) * (2.0 * n);
                fs *= (2.0 * n) * (2.0 * n + 1.0);
            }
            c[n] = (n % 2 ? -1.0 : 1.0) / fc;
            s[n] = (n % 2 ? -1.0 : 1.0) / fs;
        }
    }
};
__device__ constexpr TaylorCoeffs TAYLOR{};
constexpr double HALF_PI = 1.57079632679489661923;

// sin and cos for |x| <= pi/2 (general routine beyond).  `short_series`
// is a launch-wide promise that every argument has |x| <= 3/4 (nearly
// singular pairs at small k D): the terms up to x^18 / x^19 then leave an
// error below 2e-21.
__device__ __forceinline__ void sincos_bounded(double x, double *s, double *c, bool short_series)
{
    const double ax = fabs(x);
    if (ax > HALF_PI || (short_series && ax > 0.75)) {
        sincos(x, s, c);
        return;
    }
    const double u = x * x;
    double pc, ps;
    if (short_series) {
        pc = TAYLOR.c[9];
        ps = TAYLOR.s[9];
#pragma unroll
        for (int n = 8; n >= 0; --n) {
            pc = fma(pc, u, TAYLOR.c[n]);
            ps = fma(ps, u, TAYLOR.s[n]);
        }
    } else {
        pc = TAYLOR.c[11];
        ps = TAYLOR.s[11];
#pragma unroll
        for (int n = 10; n >= 0; --n) {
            pc = fma(pc, u, TAYLOR.c[n]);
            ps = fma(ps, u, TAYLOR.s[n]);
        }
    }
    *c = pc;
    *s = ps * x;
}

// cos of an angle difference known to lie within pi/2 of 0 modulo 2 pi
__device__ __forceinline__ double cos_angle(double x)
{
    x -= (2.0 * PI) * rint(x * (0.5 / PI));
    if (fabs(x) > HALF_PI) return cos(x);
    const double u = x * x;
    double pc = TAYLOR.c[11];
#pragma unroll
    for (int n = 10; n >= 0; --n) pc = fma(pc, u, TAYLOR.c[n]);
    return pc;
}

// rotate the element parallel to the x-y plane (nihu/library/plane_element_helper.hpp:112-126):
// T rows t0 = v1^, t1 = (v1 x v2)^ x t0, t2 = (v1 x v2)^; loc = T (c - x0) in
// the plane, z = height of x0 above the plane
__device__ __forceinline__ void plane_local_frame(const Elem64 &e, const double x0in[3], double loc[4][2], double &z,
                                                  double T[3][3])
{
    double v1[3], v2[3];
    for (int d = 0; d < 3; ++d) { v1[d] = e.c[1][d] - e.c[0][d]; v2[d] = e.c[2][d] - e.c[0][d]; }
    double n1 = 1.0 / norm3(v1);
    for (int d = 0; d < 3; ++d) T[0][d] = v1[d] * n1;
    cross3(v1, v2, T[2]);
    double n2 = 1.0 / norm3(T[2]);
    for (int d = 0; d < 3; ++d) T[2][d] *= n2;
    cross3(T[2], T[0], T[1]);
    double n3 = 1.0 / norm3(T[1]);
    for (int d = 0; d < 3; ++d) T[1][d] *= n3;
    for (int a = 0; a < e.nc; ++a) {
        double dv[3] = {e.c[a][0] - x0in[0], e.c[a][1] - x0in[1], e.c[a][2] - x0in[2]};
        loc[a][0] = dot3(T[0], dv);
        loc[a][1] = dot3(T[1], dv);
    }
    double dv[3] = {x0in[0] - e.c[0][0], x0in[1] - e.c[0][1], x0in[2] - e.c[0][2]};
    z = dot3(T[2], dv);
}

__device__ __forceinline__ void plane_local(const Elem64 &e, const double x0in[3], double loc[4][2], double &z)
{
    double T[3][3];
    plane_local_frame(e, x0in, loc, z, T);
}

// first column of trial element j >= j0 whose pairs include list entry p:
// the largest j < j1 with col_ptr[j] <= p
__device__ __forceinline__ int near_column(const int64_t *col_ptr, int j0, int j1, int64_t p)
{
    int lo = j0, hi = j1 - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (col_ptr[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// corner angle, foot angle and distance of a side (c1 -> c2) seen from the
// origin of the local frame (nihu/library/plane_element_helper.hpp:76-99)
__device__ __forceinline__ void side_geometry(const double c1[2], const double c2[2], double &th_lim, double &th0,
                                              double &dref, bool guard_short)
{
    double l0 = 1.0, l1 = 0.0;
    double d0 = c2[0] - c1[0], d1 = c2[1] - c1[1];
    double ln = sqrt(d0 * d0 + d1 * d1);
    if (!guard_short || ln > 1e-3) { double il = 1.0 / ln; l0 = d0 * il; l1 = d1 * il; }
    double pr = c1[0] * l0 + c1[1] * l1;
    double f0 = c1[0] - l0 * pr, f1 = c1[1] - l1 * pr;
    th_lim = atan2(c1[1], c1[0]);
    th0 = atan2(f1, f0);
    dref = sqrt(f0 * f0 + f1 * f1);
}

__device__ __forceinline__ void wrap_limits(double &t1, double &t2)
{
    if (fabs(t2 - t1) > PI) {
        if (t2 > t1) t1 += 2.0 * PI;
        else t2 += 2.0 * PI;
    }
}

// radii r, subtended angles theta and corner angles alpha of the sides of a
// flat element seen from an interior point
// (nihu/library/plane_element_helper.hpp:42-74)
__device__ __forceinline__ void corner_angles(const Elem64 &e, const double x0[3], double r[4], double theta[4],
                                              double alpha[4])
{
    const int N = e.nc;
    double R[4][3];
    for (int i = 0; i < N; ++i) {
        for (int d = 0; d < 3; ++d) R[i][d] = e.c[i][d] - x0[d];
        r[i] = norm3(R[i]);
        double ir = 1.0 / r[i];
        for (int d = 0; d < 3; ++d) R[i][d] *= ir;
    }
    for (int i = 0; i < N; ++i) {
        int i1 = (i + 1) % N;
        double C[3] = {e.c[i][0] - e.c[i1][0], e.c[i][1] - e.c[i1][1], e.c[i][2] - e.c[i1][2]};
        double ic = 1.0 / norm3(C);
        for (int d = 0; d < 3; ++d) C[d] *= ic;
        double cs = dot3(R[i], R[i1]);
        theta[i] = cs >= 1.0 ? 0.0 : acos(cs);
        alpha[i] = acos(dot3(R[i], C));
    }
}

// analytic static part of the flat-element 1/r integral from an interior point
// (nihu/library/laplace_singular_integrals.hpp:465-479), times 4 pi
__device__ inline double self_static(const Elem64 &e, const double x0[3])
{
    double r[4], theta[4], alpha[4];
    corner_angles(e, x0, r, theta, alpha);
    double v = 0.0;
    for (int i = 0; i < e.nc; ++i)
        v += r[i] * sin(alpha[i]) * log(tan((alpha[i] + theta[i]) / 2.0) / tan(alpha[i] / 2.0));
    return v;
}

__device__ __forceinline__ double sinc_ref(double x)
{
    if (fabs(x) > 1e-3) return sin(x) / x;
    return 1.0 - x * x / 6.0 * (1.0 - x * x / 20.0);
}

// the dynamic part sum_13 w J (e^{-ikr} - 1)/r of a constant triangle's SLP
// self term for a complex (lossy) wave number, in the reference's form
// -ik e^{-ikr/2} sinc(kr/2) (finite at r = 0: the rule holds the centroid),
// with z = kr/2 complex:
//   e^{-iz} = e^{Im z} (cos Re z - i sin Re z),
//   sin z = sin Re z cosh Im z + i cos Re z sinh Im z,
//   sinc z = sin z / z, or 1 - z^2/6 (1 - z^2/20) for |z| <= 1e-3 (nihu/util/math_functions.hpp:54-61)
__device__ inline cd tria_self_slp_dynamic_ck(const Elem64 &e, cd k, const double x0[3])
{
    double e1[3], e2[3], nt[3];
    for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
    cross3(e1, e2, nt);
    const double J = norm3(nt);
    const cd mik{k.im, -k.re};  // -i k
    cd sum{0.0, 0.0};
    for (int p = 0; p < 13; ++p) {
        double xi, eta, w;
        tri_pt(7, p, xi, eta, w);
        double rv[3];
        for (int d = 0; d < 3; ++d) rv[d] = e.c[0][d] + xi * e1[d] + eta * e2[d] - x0[d];
        const double r = norm3(rv);
        const cd z{0.5 * k.re * r, 0.5 * k.im * r};
        double sr, cr;
        sincos(z.re, &sr, &cr);
        const double ez = exp(z.im);
        const cd em{ez * cr, -ez * sr};  // e^{-iz}
        cd sc;
        if (sqrt(z.re * z.re + z.im * z.im) > 1e-3) {
            const cd sz{sr * cosh(z.im), cr * sinh(z.im)};
            const double den = z.re * z.re + z.im * z.im;  // sz / z = sz conj(z) / |z|^2
            sc = {(sz.re * z.re + sz.im * z.im) / den, (sz.im * z.re - sz.re * z.im) / den};
        } else {
            const cd z2 = cmul(z, z);
            const cd t = {1.0 - z2.re / 20.0, -z2.im / 20.0};
            const cd u = cmul(z2, t);
            sc = {1.0 - u.re / 6.0, -u.im / 6.0};
        }
        sum = cadd(sum, cscale(cmul(mik, cmul(em, sc)), w * J));
    }
    return sum;
}

template <typename Out>
__device__ __forceinline__ void store64(Out *p, double re, double im, double are, double aim, int accumulate)
{
    double vr = are * re - aim * im, vi = are * im + aim * re;
    Out o;
    if (accumulate) {
        o = *p;
        o.x += vr;
        o.y += vi;
    } else {
        o.x = vr;
        o.y = vi;
    }
    *p = o;
}

// The 42-point degree-14 Dunavant rule in FP32, (xi, eta, w) per point
struct Tri14 {
    float p[42][3];
    constexpr Tri14() : p()
    {
        constexpr double d[NIHU_TRI_DATA_LEN] = NIHU_TRI_DATA;
        constexpr int off[15] = NIHU_TRI_OFFSETS;
        for (int q = 0; q < 42; ++q)
            for (int c = 0; c < 3; ++c) p[q][c] = (float)d[3 * (off[14] + q) + c];
    }
};
__device__ constexpr Tri14 TRI14{};

// an n-point Gauss-Legendre rule on [-1, 1] in FP32, (x, w) per point
template <int N>
struct GaussF {
    float x[N], w[N];
    constexpr GaussF() : x(), w()
    {
        constexpr double d[NIHU_GAUSS_DATA_LEN] = NIHU_GAUSS_DATA;
        constexpr int off[NIHU_GAUSS_MAX_N] = NIHU_GAUSS_OFFSETS;
        for (int q = 0; q < N; ++q) {
            x[q] = (float)d[2 * (off[N - 1] + q)];
            w[q] = (float)d[2 * (off[N - 1] + q) + 1];
        }
    }
};
__device__ constexpr GaussF<6> GAUSS6F{};
__device__ constexpr GaussF<8> GAUSS8F{};

}  // namespace nihu
