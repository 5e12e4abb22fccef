// Burton-Miller point kernels and FP64 nearly singular / self schemes of all
// four operators (SLP, DLP, DLPt, HSP) on constant triangles, shared by the
// dense kernels (assemble_bm.cu) and the pair-list kernels (assemble_pairs.cu).
// References are paths inside the NiHu project.
#pragma once

#include "planar.cuh"

namespace nihu {

template <typename R>
struct BmSum {
    R sr = 0, si = 0, dr = 0, di = 0, tr = 0, ti = 0, hr = 0, hi = 0;
};

// one quadrature point of all four kernels sharing r, 1/r and one sincos;
// ws / wd / wt / wh select the operators whose rule holds this point
// CK: a complex (lossy) wave number k + i ki: with z = ikr = -ki r + i k r and
// E = e^{-ikr} = e^{ki r} (cos kr - i sin kr), the SLP takes E, the DLP and
// DLPt (1 + z) E and the HSP [m (1 + z) + a z^2] E, which are the real-k
// expressions below at ki = 0 (nihu/library/helmholtz_kernel.hpp:42-54)
template <int FAM, bool ALL4, typename R, bool CK = false>
__device__ __forceinline__ void eval_bm(R rx, R ry, R rz, R wj, R ny0, R ny1, R ny2, R nx0, R nx1, R nx2, R k, R ws,
                                        R wd, R wt, R wh, BmSum<R> &o, R ki = R(0))
{
    constexpr R INV4PI = R(1.0 / (4.0 * 3.14159265358979323846));
    const R r2 = rx * rx + ry * ry + rz * rz;
    R rinv;
    if constexpr (sizeof(R) == 4) rinv = rsqrtf(r2);
    else rinv = rsqrt(r2);
    const R g = wj * rinv * INV4PI;  // w J / (4 pi r)
    const R g2 = g * rinv;
    const R g3 = g2 * rinv;
    const R rdny = (rx * ny0 + ry * ny1 + rz * ny2) * rinv;
    const R rdnx = -(rx * nx0 + ry * nx1 + rz * nx2) * rinv;
    const R aa = rdnx * rdny;
    const R m = R(3) * aa + (nx0 * ny0 + nx1 * ny1 + nx2 * ny2);
    if constexpr (FAM == FAM_HELMHOLTZ && CK) {
        const R r = r2 * rinv;
        const R kr = k * r;
        R s, c, damp;
        if constexpr (sizeof(R) == 4) {
            sincos_reduced(kr, s, c);
            damp = expf(ki * r);
        } else {
            sincos(kr, &s, &c);
            damp = exp(ki * r);
        }
        c *= damp;
        s *= damp;
        const R zr = -ki * r, zi = kr;
        // (1 + z) E = p + i q
        const R p = (R(1) + zr) * c + zi * s, q = zi * c - (R(1) + zr) * s;
        if constexpr (ALL4) {
            o.sr += ws * g * c;
            o.si -= ws * g * s;
            const R fd = -wd * g2 * rdny;
            o.dr += fd * p;
            o.di += fd * q;
        }
        const R ft = -wt * g2 * rdnx;
        o.tr += ft * p;
        o.ti += ft * q;
        // m (1 + z) + a z^2 = u + i v
        const R u = m * (R(1) + zr) + aa * (zr * zr - zi * zi), v = m * zi + R(2) * aa * zr * zi;
        const R fh = wh * g3;
        o.hr += fh * (u * c + v * s);
        o.hi += fh * (v * c - u * s);
    } else if constexpr (FAM == FAM_HELMHOLTZ) {
        const R kr = k * (r2 * rinv);
        R s, c;
        if constexpr (sizeof(R) == 4) sincos_reduced(kr, s, c);
        else sincos(kr, &s, &c);
        // (1 + ikr) e^{-ikr} = p + i q
        const R p = c + kr * s, q = kr * c - s;
        if constexpr (ALL4) {
            o.sr += ws * g * c;
            o.si -= ws * g * s;
            const R fd = -wd * g2 * rdny;
            o.dr += fd * p;
            o.di += fd * q;
        }
        const R ft = -wt * g2 * rdnx;
        o.tr += ft * p;
        o.ti += ft * q;
        // HSP: g3 e^{-ikr} [(3a + b - a (kr)^2) + i kr (3a + b)], a = rdnx rdny, b = nx.ny
        const R u = m - aa * kr * kr, v = kr * m;
        const R fh = wh * g3;
        o.hr += fh * (u * c + v * s);
        o.hi += fh * (v * c - u * s);
    } else {
        if constexpr (ALL4) {
            o.sr += ws * g;
            o.dr -= wd * g2 * rdny;
        }
        o.tr -= wt * g2 * rdnx;
        o.hr += wh * g3 * m;
    }
}

// HSP alone at one point (levels that no other operator of the pair uses)
template <int FAM, typename R, bool CK = false>
__device__ __forceinline__ void eval_h(R rx, R ry, R rz, R wj, R ny0, R ny1, R ny2, R nx0, R nx1, R nx2, R k,
                                       BmSum<R> &o, R ki = R(0))
{
    constexpr R INV4PI = R(1.0 / (4.0 * 3.14159265358979323846));
    const R r2 = rx * rx + ry * ry + rz * rz;
    R rinv;
    if constexpr (sizeof(R) == 4) rinv = rsqrtf(r2);
    else rinv = rsqrt(r2);
    const R g3 = wj * rinv * rinv * rinv * INV4PI;
    const R rdny = (rx * ny0 + ry * ny1 + rz * ny2) * rinv;
    const R rdnx = -(rx * nx0 + ry * nx1 + rz * nx2) * rinv;
    const R aa = rdnx * rdny;
    const R m = R(3) * aa + (nx0 * ny0 + nx1 * ny1 + nx2 * ny2);
    if constexpr (FAM == FAM_HELMHOLTZ && CK) {
        const R r = r2 * rinv;
        const R kr = k * r;
        R s, c, damp;
        if constexpr (sizeof(R) == 4) {
            sincos_reduced(kr, s, c);
            damp = expf(ki * r);
        } else {
            sincos(kr, &s, &c);
            damp = exp(ki * r);
        }
        c *= damp;
        s *= damp;
        const R zr = -ki * r, zi = kr;
        const R u = m * (R(1) + zr) + aa * (zr * zr - zi * zi), v = m * zi + R(2) * aa * zr * zi;
        o.hr += g3 * (u * c + v * s);
        o.hi += g3 * (v * c - u * s);
    } else if constexpr (FAM == FAM_HELMHOLTZ) {
        const R kr = k * (r2 * rinv);
        R s, c;
        if constexpr (sizeof(R) == 4) sincos_reduced(kr, s, c);
        else sincos(kr, &s, &c);
        const R u = m - aa * kr * kr, v = kr * m;
        o.hr += g3 * (u * c + v * s);
        o.hi += g3 * (v * c - u * s);
    } else {
        o.hr += g3 * m;
    }
}

// The Dunavant rules of degree 6 (12 points) and 7 (13 points) in FP32 for
// the HSP fourth level: (xi, eta, w) per point
struct Tri67 {
    float p6[12][3], p7[13][3];
    constexpr Tri67() : p6(), p7()
    {
        constexpr double d[NIHU_TRI_DATA_LEN] = NIHU_TRI_DATA;
        constexpr int off[15] = NIHU_TRI_OFFSETS;
        for (int q = 0; q < 12; ++q)
            for (int c = 0; c < 3; ++c) p6[q][c] = (float)d[3 * (off[6] + q) + c];
        for (int q = 0; q < 13; ++q)
            for (int c = 0; c < 3; ++c) p7[q][c] = (float)d[3 * (off[7] + q) + c];
    }
};
__device__ constexpr Tri67 TRI67{};

// ------------------------------------------------- nearly singular and self

// The four operators of one pair in FP64
struct Acc4 {
    double sr = 0, si = 0, dr = 0, di = 0, tr = 0, ti = 0, hr = 0, hi = 0;
};

// which operators a launch evaluates (uniform over the launch)
struct OpSet {
    bool s, d, t, h;
};

// Static (Laplace) parts of all four operators over a flat triangle seen from
// x0 with unit normal nx.  In the element's plane frame (x0 projected to the
// origin, height z) each side is integrated over its angle theta with
// R(theta) = dref / cos(theta - t0), r = sqrt(R^2 + z^2), r_vec = (R cos, R sin, -z):
//   SLP, 6 Gauss points:  r - |z|
//   DLP, 6 Gauss points:  sgn(z) (1 - |z|/r)
//   DLPt, 6 Gauss points: -nx.r_vec/r + (nx_0 cos + nx_1 sin) ln(R + r) - nx_2 sgn(z)
//   HSP, 21 Gauss points: -R^2/(r^2 z) (-r_vec.nx/r), or -nx_2/R when |z| <= 1e-12
// all over 4 pi (nihu/library/laplace_nearly_singular_integrals.hpp:62-209, :212-298, :301-380).
// With phi = theta - t0 (|phi| < pi/2 on the side), cos(theta) and sin(theta)
// follow from the foot direction (cos t0, sin t0) and one short-argument sincos
// of phi, which also gives R.
__device__ inline void near_static4(const Elem64 &e, const double x0[3], const double nxg[3], OpSet ops, Acc4 &a)
{
    double loc[4][2], z, T[3][3];
    plane_local_frame(e, x0, loc, z, T);
    const double n0 = dot3(T[0], nxg), n1 = dot3(T[1], nxg), n2 = dot3(T[2], nxg);
    const double sg = (0.0 < z) - (z < 0.0);
    const double az = fabs(z), z2 = z * z;
    const bool in_plane = !(az > 1e-12);
    const double iz = in_plane ? 0.0 : 1.0 / z;
    const bool six = ops.s || ops.d || ops.t;
    double s_sum = 0.0, d_sum = 0.0, t_sum = 0.0, h_sum = 0.0;
    double tl[3], t0[3], dref[3], fc[3], fs[3];
    for (int s = 0; s < 3; ++s) {
        side_geometry(loc[s], loc[(s + 1) % 3], tl[s], t0[s], dref[s], false);
        // foot direction; atan2(0, 0) = 0 when x0 lies on the side's line
        double f0 = loc[s][0], f1 = loc[s][1];
        {
            const double d0 = loc[(s + 1) % 3][0] - loc[s][0], d1 = loc[(s + 1) % 3][1] - loc[s][1];
            const double il = 1.0 / sqrt(d0 * d0 + d1 * d1);
            const double l0 = d0 * il, l1 = d1 * il;
            const double pr = f0 * l0 + f1 * l1;
            f0 -= l0 * pr;
            f1 -= l1 * pr;
        }
        if (dref[s] > 0.0) {
            fc[s] = f0 / dref[s];
            fs[s] = f1 / dref[s];
        } else {
            fc[s] = 1.0;
            fs[s] = 0.0;
        }
    }
    for (int s = 0; s < 3; ++s) {
        double t1 = tl[s], t2 = tl[(s + 1) % 3];
        wrap_limits(t1, t2);
        const double jac = (t2 - t1) / 2.0;
        // nx_0 cos(theta) + nx_1 sin(theta) = pa cos(phi) + pb sin(phi)
        const double pa = n0 * fc[s] + n1 * fs[s], pb = n1 * fc[s] - n0 * fs[s];
        const double dr = dref[s];
        for (int pass = 0; pass < 2; ++pass) {
            // pass 0: the 6-point rule of SLP, DLP and DLPt; pass 1: HSP's 21 points
            const int ng = pass == 0 ? 6 : 21;
            if (pass == 0 ? !six : !ops.h) continue;
            for (int q = 0; q < ng; ++q) {
                double xi, w;
                gauss_pt(ng, q, xi, w);
                const double th = t1 * (1.0 - xi) / 2.0 + t2 * (1.0 + xi) / 2.0;
                double phi = th - t0[s];
                phi -= (2.0 * PI) * rint(phi * (0.5 / PI));
                double sp, cp;
                sincos_bounded(phi, &sp, &cp, false);
                const double R = dr / cp;
                const double rnx = R * (pa * cp + pb * sp) - n2 * z;  // r_vec.nx
                const double jw = jac * w;
                if (pass == 0) {
                    const double r2 = R * R + z2;
                    const double rinv = rsqrt(r2);
                    const double r = r2 * rinv;
                    if (ops.s) s_sum += (r - az) * jw;
                    if (ops.d) d_sum += (1.0 - az * rinv) * jw;
                    if (ops.t) t_sum += (-rnx * rinv + (pa * cp + pb * sp) * log(R + r) - n2 * sg) * jw;
                } else if (in_plane) {
                    h_sum += -n2 / R * jw;
                } else {
                    const double r2 = R * R + z2;
                    const double rinv = rsqrt(r2);
                    // -R^2/(r^2 z) (-r_vec.nx/r)
                    h_sum += R * R * rinv * rinv * rinv * rnx * iz * jw;
                }
            }
        }
    }
    a.sr += s_sum * INV_FOUR_PI;
    a.dr += sg * d_sum * INV_FOUR_PI;
    a.tr += t_sum * INV_FOUR_PI;
    a.hr += h_sum * INV_FOUR_PI;
}

// dynamic parts K_k - K_0 of the four operators with the 42-point rule
// (y, w J), sharing 1/r and one sincos per point
// (nihu/library/helmholtz_nearly_singular_integrals.hpp:48-220)
__device__ inline void near_dynamic4(const Elem64 &e, double k, const double x0[3], const double nx[3], OpSet ops, Acc4 &a,
                              const Pt4 *__restrict__ pts42, bool short_series)
{
    double en[3];
    enormal(e, 1.0 / 3.0, 1.0 / 3.0, en);
    const double nn = 1.0 / norm3(en);
    for (int d = 0; d < 3; ++d) en[d] *= nn;
    const double nxny = dot3(nx, en);
    for (int p = 0; p < 42; ++p) {
        const Pt4 v = pts42[p];
        const double rv0 = v.x - x0[0], rv1 = v.y - x0[1], rv2 = v.z - x0[2];
        const double r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
        const double rinv = rsqrt(r2);
        const double kr = k * (r2 * rinv);
        double sn, cs;
        sincos_bounded(kr, &sn, &cs, short_series);
        const double t = v.w * rinv * INV_FOUR_PI;  // w J / (4 pi r)
        const double rdnx = -(rv0 * nx[0] + rv1 * nx[1] + rv2 * nx[2]) * rinv;
        const double rdny = (rv0 * en[0] + rv1 * en[1] + rv2 * en[2]) * rinv;
        // (1 + ikr) e^{-ikr} - 1 = pm + i qm
        const double pm = cs + kr * sn - 1.0, qm = kr * cs - sn;
        if (ops.s) {
            a.sr += t * (cs - 1.0);
            a.si -= t * sn;
        }
        if (ops.d) {
            const double u = t * rinv * rdny;
            a.dr -= u * pm;
            a.di -= u * qm;
        }
        if (ops.t) {
            const double u = t * rinv * rdnx;
            a.tr -= u * pm;
            a.ti -= u * qm;
        }
        if (ops.h) {
            const double g3 = t * rinv * rinv;
            const double aa = rdnx * rdny;
            const double m = 3.0 * aa + nxny;
            const double uu = m - aa * kr * kr, vv = kr * m;
            a.hr += g3 * (uu * cs + vv * sn - m);
            a.hi += g3 * (vv * cs - uu * sn);
        }
    }
}


// The same dynamic parts in FP32 (regular quadrature in FP32): K_k - K_0 is
// smooth and, for a nearly singular pair, of relative size (kr)^2 against the
// FP64 static part, so FP32 point sums keep the entry within a few 1e-7 of
// the FP64 value while taking the narrow FP64 pipe out of 42 points per pair.
// The points are formed in FP32 relative to x0 from the corners.
__device__ inline void near_dynamic4_f32(const Elem64 &e, double k, const double x0[3], const double nx[3], OpSet ops,
                                  Acc4 &a)
{
    double e1[3], e2[3], nt[3];
    for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
    cross3(e1, e2, nt);
    const double J = norm3(nt);
    float b[3], f1[3], f2[3], en[3], xn[3];
    for (int d = 0; d < 3; ++d) {
        b[d] = (float)(e.c[0][d] - x0[d]);
        f1[d] = (float)e1[d];
        f2[d] = (float)e2[d];
        en[d] = (float)(nt[d] / J);
        xn[d] = (float)nx[d];
    }
    const float kf = (float)k;
    const float wj = (float)(J * INV_FOUR_PI);
    const float nxny = xn[0] * en[0] + xn[1] * en[1] + xn[2] * en[2];
    float sr = 0, si = 0, dr = 0, di = 0, tr = 0, ti = 0, hr = 0, hi = 0;
    for (int p = 0; p < 42; ++p) {
        const float xi = TRI14.p[p][0], eta = TRI14.p[p][1], w = TRI14.p[p][2];
        const float rv0 = b[0] + xi * f1[0] + eta * f2[0];
        const float rv1 = b[1] + xi * f1[1] + eta * f2[1];
        const float rv2 = b[2] + xi * f1[2] + eta * f2[2];
        const float r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
        const float rinv = rsqrtf(r2);
        const float kr = kf * (r2 * rinv);
        float sn, cs;
        sincosf(kr, &sn, &cs);
        // cos(kr) - 1 without cancellation
        const float hs = sinf(0.5f * kr);
        const float cm1 = -2.0f * hs * hs;
        const float t = w * wj * rinv;
        const float rdnx = -(rv0 * xn[0] + rv1 * xn[1] + rv2 * xn[2]) * rinv;
        const float rdny = (rv0 * en[0] + rv1 * en[1] + rv2 * en[2]) * rinv;
        const float pm = cm1 + kr * sn, qm = kr * cs - sn;
        if (ops.s) {
            sr += t * cm1;
            si -= t * sn;
        }
        if (ops.d) {
            const float u = t * rinv * rdny;
            dr -= u * pm;
            di -= u * qm;
        }
        if (ops.t) {
            const float u = t * rinv * rdnx;
            tr -= u * pm;
            ti -= u * qm;
        }
        if (ops.h) {
            const float g3 = t * rinv * rinv;
            const float aa = rdnx * rdny;
            const float m = 3.0f * aa + nxny;
            // uu cs + vv sn - m with uu = m - aa kr^2, vv = kr m
            hr += g3 * (m * cm1 - aa * kr * kr * cs + kr * m * sn);
            hi += g3 * (kr * m * cs - (m - aa * kr * kr) * sn);
        }
    }
    a.sr += sr;
    a.si += si;
    a.dr += dr;
    a.di += di;
    a.tr += tr;
    a.ti += ti;
    a.hr += hr;
    a.hi += hi;
}

// near_dynamic4 for a complex (lossy) wave number, in FP64 in both modes:
// with z = ikr and E = e^{-ikr}, E - 1 = expm1(ki r) cos(kr) - 2 sin^2(kr/2)
// - i e^{ki r} sin(kr) (no cancellation as r -> 0), the DLP / DLPt part
// (1 + z) E - 1 = (E - 1) + z E and the HSP part [m (1 + z) + a z^2] E - m
// = m (E - 1) + [m z + a z^2] E
__device__ inline void near_dynamic4_ck(const Elem64 &e, cd k, const double x0[3], const double nx[3], OpSet ops,
                                        Acc4 &a, const Pt4 *__restrict__ pts42)
{
    double en[3];
    enormal(e, 1.0 / 3.0, 1.0 / 3.0, en);
    const double nn = 1.0 / norm3(en);
    for (int d = 0; d < 3; ++d) en[d] *= nn;
    const double nxny = dot3(nx, en);
    for (int p = 0; p < 42; ++p) {
        const Pt4 v = pts42[p];
        const double rv0 = v.x - x0[0], rv1 = v.y - x0[1], rv2 = v.z - x0[2];
        const double r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
        const double rinv = rsqrt(r2);
        const double r = r2 * rinv;
        double sn, cs, sh, chh;
        sincos(k.re * r, &sn, &cs);
        sincos(0.5 * k.re * r, &sh, &chh);
        const double ea = exp(k.im * r);
        const cd em1{expm1(k.im * r) * cs - 2.0 * sh * sh, -ea * sn};  // E - 1
        const cd E{ea * cs, -ea * sn};
        const cd z{-k.im * r, k.re * r};
        const double t = v.w * rinv * INV_FOUR_PI;  // w J / (4 pi r)
        const double rdnx = -(rv0 * nx[0] + rv1 * nx[1] + rv2 * nx[2]) * rinv;
        const double rdny = (rv0 * en[0] + rv1 * en[1] + rv2 * en[2]) * rinv;
        const cd pm = cadd(em1, cmul(z, E));  // (1 + z) E - 1
        if (ops.s) {
            a.sr += t * em1.re;
            a.si += t * em1.im;
        }
        if (ops.d) {
            const double u = t * rinv * rdny;
            a.dr -= u * pm.re;
            a.di -= u * pm.im;
        }
        if (ops.t) {
            const double u = t * rinv * rdnx;
            a.tr -= u * pm.re;
            a.ti -= u * pm.im;
        }
        if (ops.h) {
            const double g3 = t * rinv * rinv;
            const double aa = rdnx * rdny;
            const double m = 3.0 * aa + nxny;
            const cd w = cadd(cscale(z, m), cscale(cmul(z, z), aa));  // m z + a z^2
            const cd hv = cadd(cscale(em1, m), cmul(w, E));
            a.hr += g3 * hv.re;
            a.hi += g3 * hv.im;
        }
    }
}

// the bounded remainder (e^{-ikr}(1 + ikr) - 1 + (ikr)^2/2) / r^3 of the HSP
// kernel's expansion, its series below r = 1e-3
// (nihu/library/helmholtz_singular_integrals.hpp:768-777)
__device__ __forceinline__ cd hsp_remainder(double r, double k, double sn, double cs)
{
    if (fabs(r) > 1e-3) {
        const double kr = k * r;
        const double ir3 = 1.0 / (r * r * r);
        return {(cs + kr * sn - 1.0 - kr * kr / 2.0) * ir3, (kr * cs - sn) * ir3};
    }
    // -i k^3 (1/3 - z (1/8 - z (1/30 - z (1/144 - z (1/840 - z / 5760))))), z = ikr
    const cd z{0.0, k * r};
    cd h{1.0 / 840.0, 0.0};
    h = cadd(h, cscale(z, -1.0 / 5760.0));
    h = cadd(cd{1.0 / 144.0, 0.0}, cscale(cmul(z, h), -1.0));
    h = cadd(cd{1.0 / 30.0, 0.0}, cscale(cmul(z, h), -1.0));
    h = cadd(cd{1.0 / 8.0, 0.0}, cscale(cmul(z, h), -1.0));
    h = cadd(cd{1.0 / 3.0, 0.0}, cscale(cmul(z, h), -1.0));
    return cmul(cd{0.0, -k * k * k}, h);
}

// constant flat triangle over itself, from its centre:
//   SLP: (IG0 + sum_13 w J (e^{-ikr} - 1)/r) / (4 pi), IG0 over every side
//        (nihu/library/helmholtz_singular_integrals.hpp:703-762)
//   DLP = DLPt = 0 (nihu/library/normal_derivative_singular_integrals.hpp:13-56)
//   HSP: (IddG0 + k^2/2 IG0' + sum_13 w J rem(r)) / (4 pi),
//        IddG0 = sum (cos(alpha + theta) - cos(alpha)) / (r sin(alpha)),
//        IG0' = IG0 without the sides of theta < 1e-3 (skipped by the reference)
//        (nihu/library/helmholtz_singular_integrals.hpp:779-839)
__device__ inline void self_tria4(const Elem64 &e, int fam, double k, const double x0[3], OpSet ops, Acc4 &a)
{
    double r[4], th[4], al[4];
    corner_angles(e, x0, r, th, al);
    double IG0 = 0.0, IG0h = 0.0, IddG0 = 0.0;
    for (int i = 0; i < 3; ++i) {
        const double g = r[i] * sin(al[i]) * log(tan((al[i] + th[i]) / 2.0) / tan(al[i] / 2.0));
        IG0 += g;
        if (th[i] < 1e-3) continue;
        IG0h += g;
        IddG0 += (cos(al[i] + th[i]) - cos(al[i])) / (r[i] * sin(al[i]));
    }
    double s_dr = 0.0, s_di = 0.0, h_dr = 0.0, h_di = 0.0;
    if (fam == FAM_HELMHOLTZ) {
        double e1[3], e2[3], nt[3];
        for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
        cross3(e1, e2, nt);
        const double J = norm3(nt);
        for (int p = 0; p < 13; ++p) {
            double xi, eta, w;
            tri_pt(7, p, xi, eta, w);
            double rv[3];
            for (int d = 0; d < 3; ++d) rv[d] = e.c[0][d] + xi * e1[d] + eta * e2[d] - x0[d];
            const double rr = norm3(rv);
            const double wj = w * J;
            if (ops.s) {
                // (e^{-ikr} - 1)/r = -ik e^{-ikr/2} sinc(kr/2)
                double s, c;
                sincos_bounded(k * rr / 2.0, &s, &c, false);
                const double sc = sinc_ref(k * rr / 2.0);
                s_dr += -k * s * sc * wj;
                s_di += -k * c * sc * wj;
            }
            if (ops.h) {
                double s = 0.0, c = 1.0;
                if (fabs(rr) > 1e-3) sincos(k * rr, &s, &c);
                const cd h = hsp_remainder(rr, k, s, c);
                h_dr += h.re * wj;
                h_di += h.im * wj;
            }
        }
    }
    if (ops.s) {
        a.sr += (IG0 + s_dr) * INV_FOUR_PI;
        a.si += s_di * INV_FOUR_PI;
    }
    if (ops.h) {
        if (fam == FAM_LAPLACE) {
            a.hr += IddG0 * INV_FOUR_PI;
        } else {
            a.hr += (IddG0 + k * k / 2.0 * IG0h + h_dr) * INV_FOUR_PI;
            a.hi += h_di * INV_FOUR_PI;
        }
    }
}

// hsp_remainder for a complex wave number: the same expression with z = ikr
// complex, its series below r = 1e-3 times -i k^3
__device__ __forceinline__ cd hsp_remainder_ck(double r, cd k)
{
    const cd z{-k.im * r, k.re * r};
    if (fabs(r) > 1e-3) {
        double sn, cs;
        sincos(k.re * r, &sn, &cs);
        const double ea = exp(k.im * r);
        const cd E{ea * cs, -ea * sn};
        const cd z2 = cmul(z, z);
        const cd v = cadd(cadd(cmul(cd{1.0 + z.re, z.im}, E), cd{-1.0, 0.0}), cscale(z2, 0.5));
        return cscale(v, 1.0 / (r * r * r));
    }
    cd h{1.0 / 840.0, 0.0};
    h = cadd(h, cscale(z, -1.0 / 5760.0));
    h = cadd(cd{1.0 / 144.0, 0.0}, cscale(cmul(z, h), -1.0));
    h = cadd(cd{1.0 / 30.0, 0.0}, cscale(cmul(z, h), -1.0));
    h = cadd(cd{1.0 / 8.0, 0.0}, cscale(cmul(z, h), -1.0));
    h = cadd(cd{1.0 / 3.0, 0.0}, cscale(cmul(z, h), -1.0));
    const cd k3 = cmul(k, cmul(k, k));
    return cmul(cd{k3.im, -k3.re}, h);  // -i k^3 h
}

// self_tria4 for a complex (lossy) wave number: the SLP's dynamic part in the
// complex sinc form (tria_self_slp_dynamic_ck), the HSP's IddG0 + k^2/2 IG0'
// with complex k^2 and the complex remainder
__device__ inline void self_tria4_ck(const Elem64 &e, int fam, cd k, const double x0[3], OpSet ops, Acc4 &a)
{
    double r[4], th[4], al[4];
    corner_angles(e, x0, r, th, al);
    double IG0 = 0.0, IG0h = 0.0, IddG0 = 0.0;
    for (int i = 0; i < 3; ++i) {
        const double g = r[i] * sin(al[i]) * log(tan((al[i] + th[i]) / 2.0) / tan(al[i] / 2.0));
        IG0 += g;
        if (th[i] < 1e-3) continue;
        IG0h += g;
        IddG0 += (cos(al[i] + th[i]) - cos(al[i])) / (r[i] * sin(al[i]));
    }
    cd sdyn{0.0, 0.0}, hdyn{0.0, 0.0};
    if (fam == FAM_HELMHOLTZ) {
        if (ops.s) sdyn = tria_self_slp_dynamic_ck(e, k, x0);
        if (ops.h) {
            double e1[3], e2[3], nt[3];
            for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
            cross3(e1, e2, nt);
            const double J = norm3(nt);
            for (int p = 0; p < 13; ++p) {
                double xi, eta, w;
                tri_pt(7, p, xi, eta, w);
                double rv[3];
                for (int d = 0; d < 3; ++d) rv[d] = e.c[0][d] + xi * e1[d] + eta * e2[d] - x0[d];
                hdyn = cadd(hdyn, cscale(hsp_remainder_ck(norm3(rv), k), w * J));
            }
        }
    }
    if (ops.s) {
        a.sr += (IG0 + sdyn.re) * INV_FOUR_PI;
        a.si += sdyn.im * INV_FOUR_PI;
    }
    if (ops.h) {
        if (fam == FAM_LAPLACE) {
            a.hr += IddG0 * INV_FOUR_PI;
        } else {
            const cd k2h = cscale(cmul(k, k), 0.5 * IG0h);
            a.hr += (IddG0 + k2h.re + hdyn.re) * INV_FOUR_PI;
            a.hi += (k2h.im + hdyn.im) * INV_FOUR_PI;
        }
    }
}

// out = c0 v0 + c1 v1 (+ out), FP64
template <typename Out>
__device__ __forceinline__ void store2(Out *p, bool use0, double r0, double i0, double c0r, double c0i, bool use1,
                                       double r1, double i1, double c1r, double c1i, int accumulate)
{
    double vr = 0.0, vi = 0.0;
    if (use0) {
        vr += c0r * r0 - c0i * i0;
        vi += c0r * i0 + c0i * r0;
    }
    if (use1) {
        vr += c1r * r1 - c1i * i1;
        vi += c1r * i1 + c1i * r1;
    }
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

}  // namespace nihu
