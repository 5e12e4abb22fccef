// FP64 nearly singular and self schemes of the SLP and DLP kernels shared by
// the dense singular kernel (assemble_singular.cu) and the pair-list kernels
// (assemble_pairs.cu): the planar constant-element scheme, the inverse
// mapping with polar and Telles quadrature for quads, and the Duffy self term
// of quads.  References are paths inside the NiHu project.
#pragma once

#include "planar.cuh"

namespace nihu {

// G(r) and dG/dr of the Helmholtz kernel sharing one sincos and 1/r:
//   G = e^{-ikr}/(4 pi r), dG/dr = -(1 + ikr) e^{-ikr}/(4 pi r^2)
__device__ __forceinline__ void helm_g_dg(double k, double r, double rinv, cd &g, cd &dg)
{
    double s, c;
    sincos_bounded(k * r, &s, &c, false);
    double a = rinv * INV_FOUR_PI;
    g = {c * a, -s * a};
    double b = a * rinv, kr = k * r;
    dg = {-(c + kr * s) * b, -(kr * c - s) * b};
}

// the same for a complex (lossy) wave number k = k.re + i k.im:
// e^{-ikr} = e^{k.im r} (cos k.re r - i sin k.re r), 1 + ikr = (1 - k.im r) + i k.re r
__device__ __forceinline__ void helm_g_dg(cd k, double r, double rinv, cd &g, cd &dg)
{
    double s, c;
    sincos(k.re * r, &s, &c);
    const double a = rinv * INV_FOUR_PI * exp(k.im * r);
    g = {c * a, -s * a};
    const double p = 1.0 - k.im * r, q = k.re * r;
    dg = {-(p * g.re - q * g.im) * rinv, -(p * g.im + q * g.re) * rinv};
}

// kernel values times the Jacobian at a point y with (unnormalised) normal n:
// SLP = G J, DLP = dG/dr (r.n)/r (n = N/J, so the J cancels); K is the wave
// number's type (double, or cd for a complex one)
template <class K>
__device__ __forceinline__ void kern_point(int fam, K k, const double x0[3], const double y[3], const double n[3],
                                           double J, bool do_s, bool do_d, cd &ks, cd &kd)
{
    double rv0 = y[0] - x0[0], rv1 = y[1] - x0[1], rv2 = y[2] - x0[2];
    double r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
    double rinv = rsqrt(r2);
    double r = r2 * rinv;
    double rn = (rv0 * n[0] + rv1 * n[1] + rv2 * n[2]) * rinv;  // (r.N)/r = J (r.n)/r
    if (fam == FAM_LAPLACE) {
        double a = rinv * INV_FOUR_PI;
        if (do_s) ks = {a * J, 0.0};
        if (do_d) kd = {-a * rinv * rn, 0.0};
        return;
    }
    cd g, dg;
    helm_g_dg(k, r, rinv, g, dg);
    if (do_s) ks = cscale(g, J);
    if (do_d) kd = cscale(dg, rn);
}

template <class K>
__device__ __forceinline__ void kern_on_elem(const Elem64 &e, int fam, K k, const double x0[3], double xi,
                                             double eta, bool do_s, bool do_d, cd &ks, cd &kd)
{
    double y[3], n[3];
    ex(e, xi, eta, y);
    enormal(e, xi, eta, n);
    kern_point(fam, k, x0, y, n, norm3(n), do_s, do_d, ks, kd);
}

// ------------------------------------------------------------------ planar

// static (Laplace) nearly singular part over a flat element: radial integral
// analytic, angular integral with 6 Gauss points per side
// (nihu/library/laplace_nearly_singular_integrals.hpp:62-209); adds the SLP and
// DLP (real) results to a.sr / a.dr
__device__ inline void near_static(const Elem64 &e, const double x0[3], bool do_s, bool do_d, Acc &a)
{
    double loc[4][2], z;
    plane_local(e, x0, loc, z);
    const int N = e.nc;
    double tl[4], t0[4], dr[4];
    for (int s = 0; s < N; ++s) side_geometry(loc[s], loc[(s + 1) % N], tl[s], t0[s], dr[s], false);
    const double az = fabs(z), z2 = z * z;
    double s_sum = 0.0, d_sum = 0.0;
    for (int s = 0; s < N; ++s) {
        double t1 = tl[s], t2 = tl[(s + 1) % N];
        wrap_limits(t1, t2);
        const double jac = (t2 - t1) / 2.0;
        for (int q = 0; q < 6; ++q) {
            double xi, w;
            gauss_pt(6, q, xi, w);
            double th = t1 * (1.0 - xi) / 2.0 + t2 * (1.0 + xi) / 2.0;
            double R = dr[s] / cos_angle(th - t0[s]);
            double r2 = R * R + z2;
            double rinv = rsqrt(r2);
            double jw = jac * w;
            if (do_s) s_sum += (r2 * rinv - az) * jw;  // r - |z|
            if (do_d) d_sum += (1.0 - az * rinv) * jw;  // 1 - |z|/r
        }
    }
    const double sg = (0.0 < z) - (z < 0.0);
    a.sr += s_sum * INV_FOUR_PI;
    a.dr += sg * d_sum * INV_FOUR_PI;
}

// near_static with the angular point sums in FP32 (the FP32 regular
// quadrature mode), for a triangle whose plane frame is precomputed (frame:
// the element's DevMesh::frame record).  The plane coordinates and the foot
// vectors stay FP64.  Per side, with the reference's 6 points: the SLP sums
// r - |z| = R^2 / (r + |z|) (positive, no cancellation) and the DLP sums
// 1 - |z|/r as sum(w) (t2 - t1)/2 - sum(w |z|/r) (t2 - t1)/2.  Over the sides
// the first part adds up to sum(w)/2 times the winding angle of the polygon
// around the foot point: 2 pi inside, 0 outside, which an FP64
// point-in-polygon test gives exactly (summed in FP32, those O(1) terms would
// leave FP32 rounding of that size in a DLP entry whose foot point lies
// outside the element, where the sides cancel).  A foot point within rounding
// of a side takes near_static itself.
__device__ inline void near_static_f32(const Elem64 &e, const double *__restrict__ frame, const double x0[3],
                                       bool do_s, bool do_d, Acc &a)
{
    // plane_local with the element's own frame: corner a at (u_a + u0, v_a + v0)
    const double dv0 = e.c[0][0] - x0[0], dv1 = e.c[0][1] - x0[1], dv2 = e.c[0][2] - x0[2];
    const double u0 = frame[0] * dv0 + frame[1] * dv1 + frame[2] * dv2;
    const double v0 = frame[3] * dv0 + frame[4] * dv1 + frame[5] * dv2;
    const double z = -(frame[6] * dv0 + frame[7] * dv1 + frame[8] * dv2);
    double loc[3][2];
    for (int c = 0; c < 3; ++c) {
        loc[c][0] = frame[9 + 2 * c] + u0;
        loc[c][1] = frame[10 + 2 * c] + v0;
    }
    constexpr int N = 3;
    // winding of the (counter-clockwise) polygon around the foot point
    double scale = 0.0;
    for (int s = 0; s < N; ++s) scale = fmax(scale, loc[s][0] * loc[s][0] + loc[s][1] * loc[s][1]);
    int pos = 0, neg = 0;
    for (int s = 0; s < N; ++s) {
        const double *c1 = loc[s], *c2 = loc[(s + 1) % N];
        const double cr = c1[0] * c2[1] - c1[1] * c2[0];
        if (fabs(cr) <= 1e-9 * scale) {
            near_static(e, x0, do_s, do_d, a);
            return;
        }
        if (cr > 0.0) ++pos;
        else ++neg;
    }
    const double wind = pos == N ? 2.0 * PI : (neg == N ? -2.0 * PI : 0.0);
    const float az = (float)fabs(z), z2 = az * az;
    double s_sum = 0.0, dz_sum = 0.0;
    for (int s = 0; s < N; ++s) {
        const double *c1 = loc[s], *c2 = loc[(s + 1) % N];
        // side s seen from the foot point: the foot vector f (distance ds) and
        // the corners' angles measured from it, p = atan2(f x c, f . c) in
        // (-pi/2, pi/2), so that the reference's th - t0 = p1 (1 - x)/2 +
        // p2 (1 + x)/2 and t2 - t1 = p2 - p1 come without cancellation.  f is
        // a difference of nearly equal vectors when ds is small against the
        // corners' distance, so it and the angle arguments are FP64; the
        // angles themselves and the point sums are FP32.
        const double d0 = c2[0] - c1[0], d1 = c2[1] - c1[1];
        const double il = rsqrt(d0 * d0 + d1 * d1);
        const double l0 = d0 * il, l1 = d1 * il;
        const double pr = c1[0] * l0 + c1[1] * l1;
        const double f0 = c1[0] - l0 * pr, f1 = c1[1] - l1 * pr;
        const float ds = sqrtf((float)(f0 * f0 + f1 * f1));
        const float p1 = atan2f((float)(f0 * c1[1] - f1 * c1[0]), (float)(f0 * c1[0] + f1 * c1[1]));
        const float p2 = atan2f((float)(f0 * c2[1] - f1 * c2[0]), (float)(f0 * c2[0] + f1 * c2[1]));
        const float jac = (p2 - p1) * 0.5f;
        float ss = 0.0f, sz = 0.0f;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float xf = GAUSS6F.x[q], wf = GAUSS6F.w[q];
            const float ph = p1 * (1.0f - xf) * 0.5f + p2 * (1.0f + xf) * 0.5f;
            const float R = __fdividef(ds, cosf(ph));
            const float R2 = R * R;
            const float r = sqrtf(R2 + z2);
            ss += wf * __fdividef(R2, r + az);  // r - |z|
            sz += wf * __fdividef(az, r);       // |z| / r
        }
        s_sum += (double)(jac * ss);
        dz_sum += (double)(jac * sz);
    }
    // sum(w) = 2 for the 6-point rule
    const double d_sum = wind - dz_sum;
    const double sg = (0.0 < z) - (z < 0.0);
    if (do_s) a.sr += s_sum * INV_FOUR_PI;
    if (do_d) a.dr += sg * d_sum * INV_FOUR_PI;
}

// dynamic part (K_k - K_0) of the planar nearly singular scheme with the
// degree-14 rule (42-point Dunavant on triangles, 8x8 Gauss on quads)
__device__ inline void near_dynamic(const Elem64 &e, double k, const double x0[3], bool do_s, bool do_d, Acc &a,
                             const Pt4 *__restrict__ pts42, bool short_series)
{
    double en[3];
    {
        double xi, eta;
        domain_center(e.nc, xi, eta);
        enormal(e, xi, eta, en);
        double nn = 1.0 / norm3(en);
        for (int d = 0; d < 3; ++d) en[d] *= nn;
    }
    const int np = e.nc == 3 ? 42 : 64;
    for (int p = 0; p < np; ++p) {
        double xi, eta, w, J;
        double y[3];
        if (pts42) {
            // precomputed per triangle: (y, w J) of the 42-point rule
            const Pt4 v = pts42[p];
            y[0] = v.x; y[1] = v.y; y[2] = v.z;
            w = v.w;
            J = 1.0;
        } else if (e.nc == 3) {
            double e1[3], e2[3], nt[3];
            for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
            cross3(e1, e2, nt);
            tri_pt(14, p, xi, eta, w);
            for (int d = 0; d < 3; ++d) y[d] = e.c[0][d] + xi * e1[d] + eta * e2[d];
            J = norm3(nt);
        } else {
            double w0, w1, n[3];
            gauss_pt(8, p / 8, xi, w0);
            gauss_pt(8, p % 8, eta, w1);
            w = w0 * w1;
            ex(e, xi, eta, y);
            enormal(e, xi, eta, n);
            J = norm3(n);
        }
        double rv0 = y[0] - x0[0], rv1 = y[1] - x0[1], rv2 = y[2] - x0[2];
        double r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
        double rinv = rsqrt(r2);
        double kr = k * (r2 * rinv);
        double sn, cs;
        sincos_bounded(kr, &sn, &cs, short_series);
        // t = w J / (4 pi r); e^{-ikr} = cs - i sn
        //   SLP: (G_k - G_0) w J = t (cs - 1 - i sn)
        //   DLP: (dG_k - dG_0)/dr (r.n)/r w J = -t/r (r.n)/r ((cs + kr sn - 1) + i (kr cs - sn))
        const double t = w * J * rinv * INV_FOUR_PI;
        if (do_s) {
            a.sr += t * (cs - 1.0);
            a.si -= t * sn;
        }
        if (do_d) {
            double u = t * rinv * ((rv0 * en[0] + rv1 * en[1] + rv2 * en[2]) * rinv);
            a.dr -= u * (cs + kr * sn - 1.0);
            a.di -= u * (kr * cs - sn);
        }
    }
}

// near_dynamic for a complex (lossy) wave number: the same points, with
// e^{-ikr} - 1 = expm1(k.im r) cos(k.re r) - 2 sin^2(k.re r / 2) - i e^{k.im r} sin(k.re r)
// (no cancellation as k r -> 0) and the DLP's (e^{-ikr} - 1) + ikr e^{-ikr}
__device__ inline void near_dynamic_ck(const Elem64 &e, cd k, const double x0[3], bool do_s, bool do_d, Acc &a,
                                       const Pt4 *__restrict__ pts42)
{
    double en[3];
    {
        double xi, eta;
        domain_center(e.nc, xi, eta);
        enormal(e, xi, eta, en);
        double nn = 1.0 / norm3(en);
        for (int d = 0; d < 3; ++d) en[d] *= nn;
    }
    const int np = e.nc == 3 ? 42 : 64;
    for (int p = 0; p < np; ++p) {
        double xi, eta, w, J;
        double y[3];
        if (pts42) {
            const Pt4 v = pts42[p];
            y[0] = v.x; y[1] = v.y; y[2] = v.z;
            w = v.w;
            J = 1.0;
        } else if (e.nc == 3) {
            double e1[3], e2[3], nt[3];
            for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
            cross3(e1, e2, nt);
            tri_pt(14, p, xi, eta, w);
            for (int d = 0; d < 3; ++d) y[d] = e.c[0][d] + xi * e1[d] + eta * e2[d];
            J = norm3(nt);
        } else {
            double w0, w1, n[3];
            gauss_pt(8, p / 8, xi, w0);
            gauss_pt(8, p % 8, eta, w1);
            w = w0 * w1;
            ex(e, xi, eta, y);
            enormal(e, xi, eta, n);
            J = norm3(n);
        }
        double rv0 = y[0] - x0[0], rv1 = y[1] - x0[1], rv2 = y[2] - x0[2];
        double r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
        double rinv = rsqrt(r2);
        double r = r2 * rinv;
        double sn, cs, sh, chh;
        sincos(k.re * r, &sn, &cs);
        sincos(0.5 * k.re * r, &sh, &chh);
        const double ea = exp(k.im * r);
        const double em1_re = expm1(k.im * r) * cs - 2.0 * sh * sh, em1_im = -ea * sn;  // e^{-ikr} - 1
        const double E_re = ea * cs, E_im = -ea * sn;                                      // e^{-ikr}
        const double t = w * J * rinv * INV_FOUR_PI;
        if (do_s) {
            a.sr += t * em1_re;
            a.si += t * em1_im;
        }
        if (do_d) {
            // ikr = -k.im r + i k.re r
            const double ar = -k.im * r, ai = k.re * r;
            const double d_re = em1_re + (ar * E_re - ai * E_im), d_im = em1_im + (ar * E_im + ai * E_re);
            double u = t * rinv * ((rv0 * en[0] + rv1 * en[1] + rv2 * en[2]) * rinv);
            a.dr -= u * d_re;
            a.di -= u * d_im;
        }
    }
}

// The same dynamic part in FP32 (triangles, regular quadrature in FP32):
// K_k - K_0 is smooth and, for a nearly singular pair, of relative size
// (kr)^2 against the FP64 static part, so FP32 point sums keep the entry
// within a few 1e-7 of the FP64 value while taking the narrow FP64 pipe out
// of 42 points per pair.  The points are formed in FP32 relative to x0 from
// the corners (the corner offsets in FP64), and cos(kr) - 1 as
// -2 sin^2(kr/2), without cancellation.
__device__ inline void near_dynamic_f32(const Elem64 &e, double k, const double x0[3], bool do_s, bool do_d, Acc &a)
{
    double e1[3], e2[3], nt[3];
    for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
    cross3(e1, e2, nt);
    const double J = norm3(nt);
    float b[3], f1[3], f2[3], en[3];
    for (int d = 0; d < 3; ++d) {
        b[d] = (float)(e.c[0][d] - x0[d]);
        f1[d] = (float)e1[d];
        f2[d] = (float)e2[d];
        en[d] = (float)(nt[d] / J);
    }
    const float kf = (float)k;
    const float wj = (float)(J * INV_FOUR_PI);
    float sr = 0, si = 0, dr = 0, di = 0;
    // six points in flight: one warp per scheduler leaves the loop latency-bound
#pragma unroll 6
    for (int p = 0; p < 42; ++p) {
        const float xi = TRI14.p[p][0], eta = TRI14.p[p][1], w = TRI14.p[p][2];
        const float rv0 = b[0] + xi * f1[0] + eta * f2[0];
        const float rv1 = b[1] + xi * f1[1] + eta * f2[1];
        const float rv2 = b[2] + xi * f1[2] + eta * f2[2];
        const float r2 = rv0 * rv0 + rv1 * rv1 + rv2 * rv2;
        const float rinv = rsqrtf(r2);
        const float kr = kf * (r2 * rinv);
        // the half angle by the hardware approximation after a reduction by
        // the nearest multiple of 2 pi (absolute error about 4e-7): the
        // dynamic part is of relative size (kr)^2 against the static one, so
        // that stays far below the entries' 1e-5
        float hs, hc;
        sincos_reduced(0.5f * kr, hs, hc);
        const float cm1 = -2.0f * hs * hs;  // cos kr - 1
        const float sn = 2.0f * hs * hc;    // sin kr
        const float cs = 1.0f + cm1;
        const float t = w * wj * rinv;
        if (do_s) {
            sr += t * cm1;
            si -= t * sn;
        }
        if (do_d) {
            const float u = t * rinv * ((rv0 * en[0] + rv1 * en[1] + rv2 * en[2]) * rinv);
            dr -= u * (cm1 + kr * sn);
            di -= u * (kr * cs - sn);
        }
    }
    a.sr += sr;
    a.si += si;
    a.dr += dr;
    a.di += di;
}

// full planar constant-element nearly singular integral
__device__ inline void near_plane(const Elem64 &e, int fam, double k, const double x0[3], bool do_s, bool do_d, Acc &a,
                           const Pt4 *__restrict__ pts42 = nullptr, bool short_series = false)
{
    if (fam == FAM_HELMHOLTZ) near_dynamic(e, k, x0, do_s, do_d, a, pts42, short_series);
    near_static(e, x0, do_s, do_d, a);
}

// ------------------------------------------------------------ inverse mapping

// Newton iteration (nihu/core/inverse_mapping.hpp:52-112).  Records the first
// iterate with |f| < 1e-5 (polar scheme) and with |f| < 1e-6 (Telles); both
// come from the same iteration sequence the reference runs separately.
__device__ inline bool inverse_mapping(const Elem64 &e, const double x0[3], bool need6, double r5[3], double r6[3])
{
    double res[3] = {0.0, 0.0, 0.0};
    bool got5 = false;
    double dxe[3] = {0, 0, 0};
    if (e.nc == 4)
        for (int d = 0; d < 3; ++d) dxe[d] = (e.c[0][d] - e.c[1][d] + e.c[2][d] - e.c[3][d]) * 0.25;
    for (int it = 0; it < 100; ++it) {
        double dxi[3], deta[3], n[3], y[3];
        ex(e, res[0], res[1], y);
        edx(e, res[0], res[1], dxi, deta);
        cross3(dxi, deta, n);
        double sq = sqrt(norm3(n));
        for (int d = 0; d < 3; ++d) n[d] /= sq;
        double f[3];
        for (int d = 0; d < 3; ++d) f[d] = y[d] + n[d] * res[2] - x0[d];
        double err = norm3(f);
        if (!got5 && err < 1e-5) {
            got5 = true;
            for (int d = 0; d < 3; ++d) r5[d] = res[d];
            if (!need6) return true;
        }
        if (need6 && err < 1e-6) {
            for (int d = 0; d < 3; ++d) r6[d] = res[d];
            return got5;
        }
        // d n / d xi = (x_xixi x x_eta + x_xi x x_xieta) / sq, x_xixi = x_etaeta = 0
        double t2[3], dnxi[3], dneta[3];
        cross3(dxi, dxe, t2);
        for (int d = 0; d < 3; ++d) dnxi[d] = t2[d] / sq;
        cross3(dxe, deta, t2);
        for (int d = 0; d < 3; ++d) dneta[d] = t2[d] / sq;
        double M[3][4];
        for (int d = 0; d < 3; ++d) {
            M[d][0] = dxi[d] + dnxi[d] * res[2];
            M[d][1] = deta[d] + dneta[d] * res[2];
            M[d][2] = n[d];
            M[d][3] = f[d];
        }
        for (int c = 0; c < 3; ++c) {
            int p = c;
            for (int r = c + 1; r < 3; ++r)
                if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
            if (p != c)
                for (int q = 0; q < 4; ++q) { double t = M[c][q]; M[c][q] = M[p][q]; M[p][q] = t; }
            for (int r = c + 1; r < 3; ++r) {
                double fct = M[r][c] / M[c][c];
                for (int q = c; q < 4; ++q) M[r][q] -= fct * M[c][q];
            }
        }
        double s[3];
        for (int r = 2; r >= 0; --r) {
            double v = M[r][3];
            for (int q = r + 1; q < 3; ++q) v -= M[r][q] * s[q];
            s[r] = v / M[r][r];
        }
        for (int d = 0; d < 3; ++d) res[d] -= s[d];
    }
    return false;
}

__device__ inline void linearized(const Elem64 &e, double xi0, double eta0, Elem64 &lin)
{
    double x0[3], dxi[3], deta[3];
    ex(e, xi0, eta0, x0);
    edx(e, xi0, eta0, dxi, deta);
    lin.nc = e.nc;
    for (int a = 0; a < 4; ++a) {
        double ci, ce;
        domain_corner(e.nc, a < e.nc ? a : e.nc - 1, ci, ce);
        for (int d = 0; d < 3; ++d) lin.c[a][d] = x0[d] + dxi[d] * (ci - xi0) + deta[d] * (ce - eta0);
    }
}

// polar scheme around (xi0, eta0) with linearized-element subtraction
template <class K>
__device__ inline void near_polar_sum(const Elem64 &e, const Elem64 &lin, int fam, K k, const double x0[3], double xi0,
                               double eta0, bool do_s, bool do_d, Acc &a)
{
    const int N = e.nc;
    double tl[4], t0[4], dr[4];
    for (int n = 0; n < N; ++n) {
        double c1[2], c2[2];
        domain_corner(N, n, c1[0], c1[1]);
        domain_corner(N, (n + 1) % N, c2[0], c2[1]);
        c1[0] -= xi0; c1[1] -= eta0;
        c2[0] -= xi0; c2[1] -= eta0;
        side_geometry(c1, c2, tl[n], t0[n], dr[n], true);
    }
    // the linearized element is affine: one normal for all points
    double ln[3];
    enormal(lin, xi0, eta0, ln);
    const double lJ = norm3(ln);
    for (int n = 0; n < N; ++n) {
        double t1 = tl[n], t2 = tl[(n + 1) % N];
        wrap_limits(t1, t2);
        if (fabs(t2 - t1) < 1e-3) continue;
        for (int ia = 0; ia < 8; ++ia) {
            double xx, wa;
            gauss_pt(8, ia, xx, wa);
            double th = ((1.0 - xx) * t1 + (1.0 + xx) * t2) / 2.0;
            double wth = wa * (t2 - t1) / 2.0;
            double cth, sth;
            sincos(th, &sth, &cth);
            double rho_lim = dr[n] / cos_angle(th - t0[n]);
            for (int ib = 0; ib < 8; ++ib) {
                double xr, wb;
                gauss_pt(8, ib, xr, wb);
                double rho = (1.0 + xr) * rho_lim / 2.0;
                double wrho = wb * rho_lim / 2.0;
                double xi = xi0 + rho * cth, eta = eta0 + rho * sth;
                cd fs{0, 0}, fd{0, 0}, ls{0, 0}, ld{0, 0};
                kern_on_elem(e, fam, k, x0, xi, eta, do_s, do_d, fs, fd);
                double yl[3];
                ex(lin, xi, eta, yl);
                kern_point(fam, k, x0, yl, ln, lJ, do_s, do_d, ls, ld);
                double wt = wth * wrho * rho;
                a.sr += wt * (fs.re - ls.re);
                a.si += wt * (fs.im - ls.im);
                a.dr += wt * (fd.re - ld.re);
                a.di += wt * (fd.im - ld.im);
            }
        }
    }
}

// Telles-transformed 16x16 Gauss rule (DLP only)
template <class K>
__device__ inline void near_telles_sum(const Elem64 &e, int fam, K k, const double x0[3], const double im[3], Acc &a)
{
    double dist = im[2];
    double rb;
    if (dist < 0.05) rb = 0.0;
    else if (dist <= 1.3) rb = 0.85 + 0.24 * log(dist);
    else if (dist <= 3.618) rb = 0.893 + 0.0832 * log(dist);
    else rb = 1.0;
    double ca[2], cb[2], cc[2], cdd[2];
    for (int dim = 0; dim < 2; ++dim) {
        double eb = im[dim];
        double f = 1.0 + 2.0 * rb;
        double q = 1.0 / (2.0 * f) * ((eb * (3.0 - 2.0 * rb) - 2.0 * eb * eb * eb / f) * 1.0 / f - eb);
        double p = 1.0 / (3.0 * f * f) * (4.0 * rb * (1.0 - rb) + 3.0 * (1.0 - eb * eb));
        double s = sqrt(q * q + p * p * p);
        double gb = cbrt(-q + s) + cbrt(-q - s) + eb / f;
        double Q = 1.0 + 3.0 * gb * gb;
        ca[dim] = (1.0 - rb) / Q;
        cb[dim] = -3.0 * (1.0 - rb) * gb / Q;
        cc[dim] = (3.0 * gb * gb + rb) / Q;
        cdd[dim] = -cb[dim];
    }
    double tv[16], tw[16];  // transformed eta nodes and Jacobians (second dimension)
    for (int b = 0; b < 16; ++b) {
        double x, w;
        gauss_pt(16, b, x, w);
        tv[b] = ca[1] * x * x * x + cb[1] * x * x + cc[1] * x + cdd[1];
        tw[b] = w * (3.0 * ca[1] * x * x + 2.0 * cb[1] * x + cc[1]);
    }
    for (int ia = 0; ia < 16; ++ia) {
        double x, w;
        gauss_pt(16, ia, x, w);
        double t0 = ca[0] * x * x * x + cb[0] * x * x + cc[0] * x + cdd[0];
        double w0 = w * (3.0 * ca[0] * x * x + 2.0 * cb[0] * x + cc[0]);
        for (int ib = 0; ib < 16; ++ib) {
            cd ks{0, 0}, kd{0, 0};
            kern_on_elem(e, fam, k, x0, t0, tv[ib], false, true, ks, kd);
            double wt = w0 * tw[ib];
            a.dr += kd.re * wt;
            a.di += kd.im * wt;
        }
    }
}

// ------------------------------------------------- FP32 sums of the quad schemes
// Under FP32 regular quadrature the sums of the nearly singular quad schemes
// run in FP32 while the rule stays FP64 (inverse mapping, side limits and
// angles, Telles coefficients, the planar static part).  A bilinear quad
// around the parameter point (xi0, eta0) is exactly
//   y - x0 = p + u t1 + v t2 + u v d,   u = xi - xi0, v = eta - eta0,
// p = y(xi0, eta0) - x0, t1, t2 the tangents there, d = (c0 - c1 + c2 - c3)/4,
// with normal N = t1 x t2 + u (t1 x d) + v (d x t2); its linearisation at
// (xi0, eta0) drops the u v d term and has normal t1 x t2.  Formed from these
// FP64-made vectors, r = y - x0 keeps FP32 relative accuracy as r -> 0, and so
// does the element-minus-linearisation difference of the polar scheme.
struct QuadAround32 {
    float p[3], t1[3], t2[3], d[3], n0[3], nu[3], nv[3];
};

__device__ inline void quad_around32(const Elem64 &e, const double x0[3], double xi0, double eta0, QuadAround32 &q)
{
    double y[3], a[3], b[3];
    ex(e, xi0, eta0, y);
    edx(e, xi0, eta0, a, b);
    double d[3], n0[3], nu[3], nv[3];
    for (int k = 0; k < 3; ++k) d[k] = 0.25 * (e.c[0][k] - e.c[1][k] + e.c[2][k] - e.c[3][k]);
    cross3(a, b, n0);
    cross3(a, d, nu);
    cross3(d, b, nv);
    for (int k = 0; k < 3; ++k) {
        q.p[k] = (float)(y[k] - x0[k]);
        q.t1[k] = (float)a[k];
        q.t2[k] = (float)b[k];
        q.d[k] = (float)d[k];
        q.n0[k] = (float)n0[k];
        q.nu[k] = (float)nu[k];
        q.nv[k] = (float)nv[k];
    }
}

// kernel values times the Jacobian at r = y - x0 with unnormalised normal N
// (|N| = J): SLP = G J, DLP = dG/dr (r.N)/r; kern_point in FP32
__device__ __forceinline__ void kern32(int fam, float k, const float rv[3], const float N[3], bool do_s, bool do_d,
                                       float &sr, float &si, float &dr, float &di)
{
    constexpr float INV4PI = (float)INV_FOUR_PI;
    const float r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
    const float rinv = rsqrtf(r2);
    const float a = rinv * INV4PI;
    const float rn = (rv[0] * N[0] + rv[1] * N[1] + rv[2] * N[2]) * rinv;
    if (fam == FAM_LAPLACE) {
        sr = do_s ? a * sqrtf(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]) : 0.0f;
        si = 0.0f;
        dr = do_d ? -a * rinv * rn : 0.0f;
        di = 0.0f;
        return;
    }
    const float kr = k * (r2 * rinv);
    float s, c;
    sincos_reduced(kr, s, c);
    if (do_s) {
        const float J = sqrtf(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        sr = c * a * J;
        si = -s * a * J;
    } else {
        sr = si = 0.0f;
    }
    if (do_d) {
        const float b = a * rinv * rn;
        dr = -(c + kr * s) * b;
        di = -(kr * c - s) * b;
    } else {
        dr = di = 0.0f;
    }
}

// near_polar_sum with the FP32 sums (quads)
static __device__ __noinline__ void near_polar_sum_f32(const Elem64 &e, int fam, double k, const double x0[3], double xi0,
                                          double eta0, bool do_s, bool do_d, Acc &a)
{
    const int N = e.nc;
    double tl[4], t0[4], dr[4];
    for (int n = 0; n < N; ++n) {
        double c1[2], c2[2];
        domain_corner(N, n, c1[0], c1[1]);
        domain_corner(N, (n + 1) % N, c2[0], c2[1]);
        c1[0] -= xi0; c1[1] -= eta0;
        c2[0] -= xi0; c2[1] -= eta0;
        side_geometry(c1, c2, tl[n], t0[n], dr[n], true);
    }
    QuadAround32 q;
    quad_around32(e, x0, xi0, eta0, q);
    const float kf = (float)k;
    float sr = 0, si = 0, dsr = 0, dsi = 0;
    for (int n = 0; n < N; ++n) {
        double t1 = tl[n], t2 = tl[(n + 1) % N];
        wrap_limits(t1, t2);
        if (fabs(t2 - t1) < 1e-3) continue;
        for (int ia = 0; ia < 8; ++ia) {
            double xx, wa;
            gauss_pt(8, ia, xx, wa);
            const double th = ((1.0 - xx) * t1 + (1.0 + xx) * t2) / 2.0;
            double cth, sth;
            sincos(th, &sth, &cth);
            const float wth = (float)(wa * (t2 - t1) / 2.0);
            const float rho_lim = (float)(dr[n] / cos_angle(th - t0[n]));
            const float cf = (float)cth, sf = (float)sth;
            float ps = 0, pi = 0, pds = 0, pdi = 0;
            for (int ib = 0; ib < 8; ++ib) {
                double xr, wb;
                gauss_pt(8, ib, xr, wb);
                const float rho = (1.0f + (float)xr) * rho_lim * 0.5f;
                const float wt = (float)wb * rho_lim * 0.5f * rho;
                const float u = rho * cf, v = rho * sf, uv = u * v;
                float rl[3], re[3], ne[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    rl[c] = q.p[c] + u * q.t1[c] + v * q.t2[c];
                    re[c] = rl[c] + uv * q.d[c];
                    ne[c] = q.n0[c] + u * q.nu[c] + v * q.nv[c];
                }
                float fsr, fsi, fdr, fdi, lsr, lsi, ldr, ldi;
                kern32(fam, kf, re, ne, do_s, do_d, fsr, fsi, fdr, fdi);
                kern32(fam, kf, rl, q.n0, do_s, do_d, lsr, lsi, ldr, ldi);
                ps += wt * (fsr - lsr);
                pi += wt * (fsi - lsi);
                pds += wt * (fdr - ldr);
                pdi += wt * (fdi - ldi);
            }
            sr += wth * ps;
            si += wth * pi;
            dsr += wth * pds;
            dsi += wth * pdi;
        }
    }
    a.sr += sr;
    a.si += si;
    a.dr += dsr;
    a.di += dsi;
}

// near_telles_sum with the FP32 sums (quads): the Telles coefficients in FP64,
// the points expanded around the inverse-mapped point
static __device__ __noinline__ void near_telles_sum_f32(const Elem64 &e, int fam, double k, const double x0[3], const double im[3],
                                           Acc &a)
{
    double dist = im[2];
    double rb;
    if (dist < 0.05) rb = 0.0;
    else if (dist <= 1.3) rb = 0.85 + 0.24 * log(dist);
    else if (dist <= 3.618) rb = 0.893 + 0.0832 * log(dist);
    else rb = 1.0;
    double ca[2], cb[2], cc[2], cdd[2];
    for (int dim = 0; dim < 2; ++dim) {
        double eb = im[dim];
        double f = 1.0 + 2.0 * rb;
        double qq = 1.0 / (2.0 * f) * ((eb * (3.0 - 2.0 * rb) - 2.0 * eb * eb * eb / f) * 1.0 / f - eb);
        double p = 1.0 / (3.0 * f * f) * (4.0 * rb * (1.0 - rb) + 3.0 * (1.0 - eb * eb));
        double s = sqrt(qq * qq + p * p * p);
        double gb = cbrt(-qq + s) + cbrt(-qq - s) + eb / f;
        double Q = 1.0 + 3.0 * gb * gb;
        ca[dim] = (1.0 - rb) / Q;
        cb[dim] = -3.0 * (1.0 - rb) * gb / Q;
        cc[dim] = (3.0 * gb * gb + rb) / Q;
        cdd[dim] = -cb[dim];
    }
    QuadAround32 q;
    quad_around32(e, x0, im[0], im[1], q);
    float vv[16], tw[16];  // eta - eta0 at the transformed nodes, and their weights
    for (int b = 0; b < 16; ++b) {
        double x, w;
        gauss_pt(16, b, x, w);
        vv[b] = (float)(ca[1] * x * x * x + cb[1] * x * x + cc[1] * x + cdd[1] - im[1]);
        tw[b] = (float)(w * (3.0 * ca[1] * x * x + 2.0 * cb[1] * x + cc[1]));
    }
    const float kf = (float)k;
    float sdr = 0, sdi = 0;
    for (int ia = 0; ia < 16; ++ia) {
        double x, w;
        gauss_pt(16, ia, x, w);
        const float u = (float)(ca[0] * x * x * x + cb[0] * x * x + cc[0] * x + cdd[0] - im[0]);
        const float w0 = (float)(w * (3.0 * ca[0] * x * x + 2.0 * cb[0] * x + cc[0]));
        float pr = 0, pim = 0;
        for (int ib = 0; ib < 16; ++ib) {
            const float v = vv[ib], uv = u * v;
            float rv[3], nv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                rv[c] = q.p[c] + u * q.t1[c] + v * q.t2[c] + uv * q.d[c];
                nv[c] = q.n0[c] + u * q.nu[c] + v * q.nv[c];
            }
            float sr, si, dr, di;
            kern32(fam, kf, rv, nv, false, true, sr, si, dr, di);
            pr += dr * tw[ib];
            pim += di * tw[ib];
        }
        sdr += w0 * pr;
        sdi += w0 * pim;
    }
    a.dr += sdr;
    a.di += sdi;
}

// the dynamic part K_k - K_0 of near_plane over a flat (linearised) quad in
// FP32: 8 x 8 Gauss as near_dynamic, points expanded around the centre
static __device__ __noinline__ void near_dynamic_quad_f32(const Elem64 &e, double k, const double x0[3], bool do_s, bool do_d,
                                             Acc &a)
{
    QuadAround32 q;
    quad_around32(e, x0, 0.0, 0.0, q);
    const float J0 = sqrtf(q.n0[0] * q.n0[0] + q.n0[1] * q.n0[1] + q.n0[2] * q.n0[2]);
    float en[3];
    for (int c = 0; c < 3; ++c) en[c] = q.n0[c] / J0;  // centre normal (near_dynamic's en)
    constexpr float INV4PI = (float)INV_FOUR_PI;
    const float kf = (float)k;
    float sr = 0, si = 0, dr = 0, di = 0;
    for (int p = 0; p < 64; ++p) {
        double xi, eta, w0, w1;
        gauss_pt(8, p / 8, xi, w0);
        gauss_pt(8, p % 8, eta, w1);
        const float u = (float)xi, v = (float)eta, uv = u * v;
        float rv[3], nv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            rv[c] = q.p[c] + u * q.t1[c] + v * q.t2[c] + uv * q.d[c];
            nv[c] = q.n0[c] + u * q.nu[c] + v * q.nv[c];
        }
        const float J = sqrtf(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        const float r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
        const float rinv = rsqrtf(r2);
        const float kr = kf * (r2 * rinv);
        float hs, hc;  // the half angle, as in near_dynamic_f32
        sincos_reduced(0.5f * kr, hs, hc);
        const float cm1 = -2.0f * hs * hs;  // cos kr - 1 without cancellation
        const float sn = 2.0f * hs * hc;
        const float cs = 1.0f + cm1;
        const float t = (float)(w0 * w1) * J * rinv * INV4PI;
        if (do_s) {
            sr += t * cm1;
            si -= t * sn;
        }
        if (do_d) {
            const float uu = t * rinv * ((rv[0] * en[0] + rv[1] * en[1] + rv[2] * en[2]) * rinv);
            dr -= uu * (cm1 + kr * sn);
            di -= uu * (kr * cs - sn);
        }
    }
    a.sr += sr;
    a.si += si;
    a.dr += dr;
    a.di += di;
}


template <class K>
__device__ inline void self_quad(const Elem64 &e, int fam, K k, const double x0[3], bool do_s, bool do_d, Acc &a)
{
    for (int d = 0; d < 4; ++d) {
        double P2[2], P3[2];
        domain_corner(4, d, P2[0], P2[1]);
        domain_corner(4, (d + 1) % 4, P3[0], P3[1]);
        for (int ia = 0; ia < 4; ++ia)
            for (int ib = 0; ib < 4; ++ib) {
                double u, wu, v, wv;
                gauss_pt(4, ia, u, wu);
                gauss_pt(4, ib, v, wv);
                // corners P0 = P1 = (0,0) (the collocation point), P2, P3
                double N[4], dN[4][2];
                shape(4, u, v, N);
                dshape(4, u, v, dN);
                double xi = N[2] * P2[0] + N[3] * P3[0];
                double eta = N[2] * P2[1] + N[3] * P3[1];
                double j00 = dN[2][0] * P2[0] + dN[3][0] * P3[0];
                double j01 = dN[2][0] * P2[1] + dN[3][0] * P3[1];
                double j10 = dN[2][1] * P2[0] + dN[3][1] * P3[0];
                double j11 = dN[2][1] * P2[1] + dN[3][1] * P3[1];
                double wd = wu * wv * (j00 * j11 - j01 * j10);
                cd ks{0, 0}, kd{0, 0};
                kern_on_elem(e, fam, k, x0, xi, eta, do_s, do_d, ks, kd);
                a.sr += ks.re * wd;
                a.si += ks.im * wd;
                a.dr += kd.re * wd;
                a.di += kd.im * wd;
            }
    }
}

}  // namespace nihu
