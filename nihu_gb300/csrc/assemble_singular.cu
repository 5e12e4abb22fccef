// FP64 singular (self) and nearly singular collocational entries.
//
// One thread evaluates one (test, trial) pair.  GB300's FP64 pipe is narrow,
// so the per-pair set-up (plane transform, side angles, inverse mapping) is
// done exactly once per pair -- never replicated across lanes -- and every
// quadrature point shares one sincos and one reciprocal square root between
// the SLP and the DLP and between the Helmholtz and Laplace parts of the
// kernel difference.  Threads of a warp take consecutive pairs of the
// column-sorted list, so they share the trial element and the code path.
//
// Schemes (all restated from the reference, paths inside the NiHu project):
//  self, constant tria, SLP: analytic static part + (e^{-ikr}-1)/r with the
//      13-point degree-7 rule  (nihu/library/helmholtz_singular_integrals.hpp:703-762,
//      laplace_singular_integrals.hpp:456-480, plane_element_helper.hpp:42-74)
//  self, constant tria, DLP: 0 (nihu/library/normal_derivative_singular_integrals.hpp:13-33)
//  self, quad: Duffy splitting into 4 collapsed quads x 4x4 Gauss
//      (nihu/core/duffy_quadrature.hpp:82-141, singular_accelerator.hpp:440-448)
//  near, constant tria: static Laplace part semi-analytic (6 Gauss points per
//      side) + dynamic part with the 42-point degree-14 rule
//      (nihu/library/helmholtz_nearly_singular_integrals.hpp:48-129,
//       laplace_nearly_singular_integrals.hpp:62-209)
//  near, quad, SLP and Laplace DLP: polar quadrature around the inverse-mapped
//      image with linearized-element subtraction (8 x 8 per side) plus the
//      planar formula on the linearized element
//      (nihu/library/nearly_singular_collocational.hpp:87-198, inverse_mapping.hpp:52-112)
//  near, quad, Helmholtz DLP: Telles-transformed 16x16 Gauss
//      (nihu/library/nearly_singular_collocational_telles.hpp:85-110, telles_1987.hpp:44-113)
// A frequency batch on a triangle evaluates the same 42-point dynamic sums
// through their power series in k (near_moments / near_series below).
#include <cmath>

#include "kernels.h"
#include "planar.cuh"

namespace nihu {

constexpr int SING_THREADS = 128;
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

// kernel values times the Jacobian at a point y with (unnormalised) normal n:
// SLP = G J, DLP = dG/dr (r.n)/r (n = N/J, so the J cancels)
__device__ __forceinline__ void kern_point(int fam, double k, const double x0[3], const double y[3], const double n[3],
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

__device__ __forceinline__ void kern_on_elem(const Elem64 &e, int fam, double k, const double x0[3], double xi,
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
__device__ void near_static(const Elem64 &e, const double x0[3], bool do_s, bool do_d, Acc &a)
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

// dynamic part (K_k - K_0) of the planar nearly singular scheme with the
// degree-14 rule (42-point Dunavant on triangles, 8x8 Gauss on quads)
__device__ void near_dynamic(const Elem64 &e, double k, const double x0[3], bool do_s, bool do_d, Acc &a,
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

// full planar constant-element nearly singular integral
__device__ void near_plane(const Elem64 &e, int fam, double k, const double x0[3], bool do_s, bool do_d, Acc &a,
                           const Pt4 *__restrict__ pts42 = nullptr, bool short_series = false)
{
    if (fam == FAM_HELMHOLTZ) near_dynamic(e, k, x0, do_s, do_d, a, pts42, short_series);
    near_static(e, x0, do_s, do_d, a);
}

// ------------------------------------------------ frequency-batch moments
//
// With W_p = w_p J_p / (4 pi) and x = k r_p, the 42-point dynamic sums of a
// triangle are power series in k with k-independent coefficients (term by
// term expansions of e^{-ix} - 1 and 1 - (1 + ix) e^{-ix}):
//   SLP(k) = sum_{j>=1} (-ik)^j / j!        S_j,  S_j = sum_p W_p r_p^{j-1}
//   DLP(k) = sum_{j>=2} (-ik)^j (j - 1)/j!  T_j,  T_j = sum_p W_p (r_p.n) r_p^{j-3}
// The moments are formed once per pair; each wave number then costs one
// Horner evaluation in u = -k^2 ((-ik)^{2m} = u^m, (-ik)^{2m+1} = -ik u^m)
// instead of 42 complex exponentials.  Wave number k uses the first J with
// x^{J+1} / J! < 1e-15 for x = |k| max_p r_p, which bounds the truncation of
// every point's term by 1e-15 times that point's static contribution; the
// moments are formed up to the J of the batch's largest |k|.  J depends only
// on the pair and k, so an entry does not depend on the other wave numbers
// of its batch; where x is beyond the longest series the points are summed
// directly for that wave number.

constexpr int MOM_J = 64;  // most series terms (shared memory per thread: 2 x MOM_J doubles)
constexpr size_t MOM_SMEM = 2 * sizeof(double) * MOM_J * SING_THREADS;

// c_series_x[J] = (1e-15 J!)^{1/(J+1)} (1 - 1e-5): the largest x that J terms serve
__constant__ float c_series_x[MOM_J];

// terms for x = k max r: the smallest J >= 1 with x <= c_series_x[J], or
// MOM_J when even MOM_J - 1 terms do not reach the bound
__device__ __forceinline__ int series_terms(float x)
{
    int J = 1;
    while (J < MOM_J - 1 && x > c_series_x[J]) ++J;
    return x > c_series_x[J] ? MOM_J : J;
}

struct InvFactorials {
    double v[MOM_J];
    constexpr InvFactorials() : v()
    {
        double f = 1.0;
        for (int j = 0; j < MOM_J; ++j) {
            if (j > 0) f *= j;
            v[j] = 1.0 / f;
        }
    }
};
__device__ constexpr InvFactorials INV_FACT{};

__device__ __forceinline__ void unit_normal_center(const Elem64 &e, double en[3])
{
    double xi, eta;
    domain_center(e.nc, xi, eta);
    enormal(e, xi, eta, en);
    const double nn = 1.0 / norm3(en);
    for (int d = 0; d < 3; ++d) en[d] *= nn;
}

// coefficients c^S_j = S_j / j! at mS[j * SING_THREADS] and, when en is
// given, c^T_j = (j-1) T_j / j! at mT[j * SING_THREADS], j = 0..J, over the np
// points that pts(p, y, W) yields (W = w J / (4 pi)), for J = the terms of
// kmax; returns J (capped at MOM_J - 1) and *rmax = max_p r_p
template <class PointFn>
__device__ int series_moments(int np, PointFn pts, const double x0[3], const double *en, double kmax, double *mS,
                              double *mT, float *rmax)
{
    double r2max = 0.0;
    for (int p = 0; p < np; ++p) {
        double y[3], W;
        pts(p, y, W);
        const double r0 = y[0] - x0[0], r1 = y[1] - x0[1], r2 = y[2] - x0[2];
        r2max = fmax(r2max, r0 * r0 + r1 * r1 + r2 * r2);
    }
    *rmax = (float)sqrt(r2max);
    const int J = min(series_terms((float)kmax * *rmax), MOM_J - 1);
    for (int j = 0; j <= J; ++j) {
        mS[j * SING_THREADS] = 0.0;
        if (en) mT[j * SING_THREADS] = 0.0;
    }
    for (int p = 0; p < np; ++p) {
        double y[3], ws;
        pts(p, y, ws);
        const double r0 = y[0] - x0[0], r1 = y[1] - x0[1], r2 = y[2] - x0[2];
        const double rr = r0 * r0 + r1 * r1 + r2 * r2;
        double pw = 1.0;  // r^{j-1}
        if (en) {
            // nearly singular: the point never coincides with x0
            const double rinv = rsqrt(rr), r = rr * rinv;
            const double wd = ws * ((r0 * en[0] + r1 * en[1] + r2 * en[2]) * rinv);  // W (r.n) / r
            for (int j = 1; j <= J; ++j) {
                mS[j * SING_THREADS] += ws * pw;
                if (j < J) mT[(j + 1) * SING_THREADS] += wd * pw;
                pw *= r;
            }
        } else {
            // self rules may hold the collocation point itself (r = 0, only r^0 survives)
            const double r = sqrt(rr);
            for (int j = 1; j <= J; ++j) {
                mS[j * SING_THREADS] += ws * pw;
                pw *= r;
            }
        }
    }
    for (int j = 1; j <= J; ++j) {
        mS[j * SING_THREADS] *= INV_FACT.v[j];
        if (en) mT[j * SING_THREADS] *= (j - 1) * INV_FACT.v[j];
    }
    return J;
}

// the moments of a triangle's 42-point dynamic rule (table of (y, w J))
__device__ int near_moments(const Elem64 &e, const Pt4 *__restrict__ pts, const double x0[3], double kmax,
                            double *mS, double *mT, float *rmax)
{
    double en[3];
    unit_normal_center(e, en);
    return series_moments(
        42,
        [&](int p, double y[3], double &W) {
            const Pt4 v = pts[p];
            y[0] = v.x;
            y[1] = v.y;
            y[2] = v.z;
            W = v.w * INV_FOUR_PI;
        },
        x0, en, kmax, mS, mT, rmax);
}

// the dynamic sums at wave number k from the coefficients of near_moments
__device__ __forceinline__ void near_series(int J, double k, const double *mS, const double *mT, bool do_s,
                                            bool do_d, Acc &a)
{
    const double u = -k * k;
    const int je = J & ~1, jo = (J & 1) ? J : J - 1;
    if (do_s) {
        double ev = 0.0, od = 0.0;
        for (int j = je; j >= 2; j -= 2) ev = fma(ev, u, mS[j * SING_THREADS]);
        for (int j = jo; j >= 1; j -= 2) od = fma(od, u, mS[j * SING_THREADS]);
        a.sr += u * ev;
        a.si -= k * od;
    }
    if (do_d) {
        double ev = 0.0, od = 0.0;
        for (int j = je; j >= 2; j -= 2) ev = fma(ev, u, mT[j * SING_THREADS]);
        for (int j = jo; j >= 1; j -= 2) od = fma(od, u, mT[j * SING_THREADS]);
        a.dr += u * ev;
        a.di -= k * od;
    }
}

// ------------------------------------------------------------ inverse mapping

// Newton iteration (nihu/core/inverse_mapping.hpp:52-112).  Records the first
// iterate with |f| < 1e-5 (polar scheme) and with |f| < 1e-6 (Telles); both
// come from the same iteration sequence the reference runs separately.
__device__ bool inverse_mapping(const Elem64 &e, const double x0[3], bool need6, double r5[3], double r6[3])
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

__device__ void linearized(const Elem64 &e, double xi0, double eta0, Elem64 &lin)
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
__device__ void near_polar_sum(const Elem64 &e, const Elem64 &lin, int fam, double k, const double x0[3], double xi0,
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
__device__ void near_telles_sum(const Elem64 &e, int fam, double k, const double x0[3], const double im[3], Acc &a)
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

// -------------------------------------------------------------------- self

// (e^{-ikr} - 1) / (4 pi r) over a flat triangle with the 13-point degree-7
// rule, as -ik e^{-ikr/2} sinc(kr/2) / (4 pi)
__device__ void self_tria_dynamic(const Elem64 &e, double k, const double x0[3], Acc &a)
{
    double e1[3], e2[3], nt[3];
    for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
    cross3(e1, e2, nt);
    const double J = norm3(nt);
    double dr = 0.0, di = 0.0;
    for (int p = 0; p < 13; ++p) {
        double xi, eta, w;
        tri_pt(7, p, xi, eta, w);
        double rv[3];
        for (int d = 0; d < 3; ++d) rv[d] = e.c[0][d] + xi * e1[d] + eta * e2[d] - x0[d];
        double r = norm3(rv);
        double s, c;
        sincos_bounded(k * r / 2.0, &s, &c, false);
        double sc = sinc_ref(k * r / 2.0);
        double wj = w * J;
        dr += -k * s * sc * wj;
        di += -k * c * sc * wj;
    }
    a.sr += dr * INV_FOUR_PI;
    a.si += di * INV_FOUR_PI;
}

// the moments of the same 13-point rule (SLP series only)
__device__ int self_tria_moments(const Elem64 &e, const double x0[3], double kmax, double *mS, float *rmax)
{
    double e1[3], e2[3], nt[3];
    for (int d = 0; d < 3; ++d) { e1[d] = e.c[1][d] - e.c[0][d]; e2[d] = e.c[2][d] - e.c[0][d]; }
    cross3(e1, e2, nt);
    const double J = norm3(nt) * INV_FOUR_PI;
    return series_moments(
        13,
        [&](int p, double y[3], double &W) {
            double xi, eta, w;
            tri_pt(7, p, xi, eta, w);
            for (int d = 0; d < 3; ++d) y[d] = e.c[0][d] + xi * e1[d] + eta * e2[d];
            W = w * J;
        },
        x0, nullptr, kmax, mS, nullptr, rmax);
}

__device__ void self_tria(const Elem64 &e, int fam, double k, const double x0[3], Acc &a)
{
    double st = self_static(e, x0);
    double dr = 0.0, di = 0.0;
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
            double r = norm3(rv);
            // (e^{-ikr} - 1)/r = -ik e^{-ikr/2} sinc(kr/2)
            double s, c;
            sincos_bounded(k * r / 2.0, &s, &c, false);
            double sc = sinc_ref(k * r / 2.0);
            double wj = w * J;
            dr += -k * s * sc * wj;
            di += -k * c * sc * wj;
        }
    }
    a.sr += (st + dr) * INV_FOUR_PI;
    a.si += di * INV_FOUR_PI;
    // DLP of a flat triangle over itself is zero
}

__device__ void self_quad(const Elem64 &e, int fam, double k, const double x0[3], bool do_s, bool do_d, Acc &a)
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

// ------------------------------------------------------------------ driver

// BATCH: frequency batch (a.nk > 1), a separate kernel so that the single
// wave number kernel carries none of its code.
template <typename Out, bool BATCH>
__device__ __forceinline__ void singular_pairs(const RegularArgs &a, const NearList &near, int *err)
{
    // frequency batches: per-thread series coefficients (MOM_SMEM bytes, launched only with nk > 1)
    extern __shared__ double s_mom[];
    const int64_t p_begin = near.col_ptr ? near.col_ptr[a.j0] : 0;
    const int64_t p_end = near.col_ptr ? near.col_ptr[a.j1] : 0;
    const int64_t n_near = p_end - p_begin;
    const int64_t n_self = a.same_mesh ? (int64_t)(a.j1 - a.j0) : 0;
    const int64_t total = n_near + n_self;
    const bool do_s = (a.ops & OP_SLP) != 0, do_d = (a.ops & OP_DLP) != 0;
    const int fam = a.family;
    const double k = a.k;
    // nearly singular pairs have r < 1.5 D + (point to centre) <= 3 D_max
    const bool short_series = k * 3.0 * a.trial_size_max <= 0.75;

    // this block's wave numbers [f_lo, f_hi) (gridDim.y chunks of a frequency batch)
    const int f_per = (a.nk + gridDim.y - 1) / gridDim.y;
    const int f_lo = min(a.nk, (int)blockIdx.y * f_per), f_hi = min(a.nk, f_lo + f_per);
    for (int64_t item = (int64_t)blockIdx.x * SING_THREADS + threadIdx.x; item < total;
         item += (int64_t)gridDim.x * SING_THREADS) {
        int i, j;
        bool self;
        if (item < n_near) {
            int64_t p = p_begin + item;
            i = near.rows[p];
            j = near_column(near.col_ptr, a.j0, a.j1, p);
            self = false;
        } else {
            j = a.j0 + (int)(item - n_near);
            i = j;
            self = true;
            if (i >= a.test.n) continue;
        }
        double x0[3] = {a.test.center[3 * (int64_t)i], a.test.center[3 * (int64_t)i + 1],
                        a.test.center[3 * (int64_t)i + 2]};
        Elem64 e;
        load_elem(a.trial, j, e);
        const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
        if (BATCH && e.nc == 3) {
            // frequency batch on a triangle: the k-independent static part and
            // the moments of the dynamic part once, then per wave number the
            // series (or the self term)
            Acc st;
            float rmax = 0.0f;
            double *mS = s_mom + threadIdx.x, *mT = s_mom + MOM_J * SING_THREADS + threadIdx.x;
            const Pt4 *pts = a.trial.dyn42 + 42 * (int64_t)j;
            if (!self) {
                near_static(e, x0, do_s, do_d, st);
                if (fam == FAM_HELMHOLTZ) near_moments(e, pts, x0, a.k_absmax, mS, mT, &rmax);
            } else if (do_s) {
                st.sr = self_static(e, x0) * INV_FOUR_PI;
                if (fam == FAM_HELMHOLTZ) self_tria_moments(e, x0, a.k_absmax, mS, &rmax);
            }
            for (int f = f_lo; f < f_hi; ++f) {
                const double kf = a.ks[f];
                // this wave number's series length (MOM_J: sum the points directly)
                const int Jf = fam == FAM_HELMHOLTZ ? series_terms(fabsf((float)kf) * rmax) : 0;
                Acc acc;
                if (self) {
                    if (do_s) {
                        acc = st;
                        if (fam == FAM_HELMHOLTZ) {
                            if (Jf < MOM_J) near_series(Jf, kf, mS, mT, true, false, acc);
                            else self_tria_dynamic(e, kf, x0, acc);
                        }
                    }
                } else {
                    acc = st;
                    if (fam == FAM_HELMHOLTZ) {
                        if (Jf < MOM_J) near_series(Jf, kf, mS, mT, do_s, do_d, acc);
                        else near_dynamic(e, kf, x0, do_s, do_d, acc, pts, kf * 3.0 * a.trial_size_max <= 0.75);
                    }
                }
                if (do_s) store64(batch_matrix<Out>(a, false, f) + off, acc.sr, acc.si, a.alpha_re, a.alpha_im, a.accumulate);
                if (do_d) store64(batch_matrix<Out>(a, true, f) + off, acc.dr, acc.di, a.alpha_re, a.alpha_im, a.accumulate);
            }
            continue;
        }
        for (int f = f_lo; f < f_hi; ++f) {
            const double kf = a.nk > 1 ? a.ks[f] : k;
            const bool short_f = a.nk > 1 ? kf * 3.0 * a.trial_size_max <= 0.75 : short_series;
            Acc acc;
            bool ok = true;
            if (self) {
                if (e.nc == 3) {
                    if (do_s) self_tria(e, fam, kf, x0, acc);
                } else {
                    self_quad(e, fam, kf, x0, do_s, do_d, acc);
                }
            } else if (e.nc == 3) {
                near_plane(e, fam, kf, x0, do_s, do_d, acc, a.trial.dyn42 + 42 * (int64_t)j, short_f);
            } else {
                const bool telles = fam == FAM_HELMHOLTZ && do_d;
                const bool polar_d = fam == FAM_LAPLACE && do_d;
                double r5[3] = {0, 0, 0}, r6[3] = {0, 0, 0};
                ok = inverse_mapping(e, x0, telles, r5, r6);
                if (ok) {
                    if (do_s || polar_d) {
                        Elem64 lin;
                        linearized(e, r5[0], r5[1], lin);
                        near_polar_sum(e, lin, fam, kf, x0, r5[0], r5[1], do_s, polar_d, acc);
                        near_plane(lin, fam, kf, x0, do_s, polar_d, acc);
                    }
                    if (telles) near_telles_sum(e, fam, kf, x0, r6, acc);
                }
            }
            if (!ok) {
                atomicCAS(err, 0, (int)min(item + 1, (int64_t)0x7fffffff));
                break;
            }
            if (do_s) store64(batch_matrix<Out>(a, false, f) + off, acc.sr, acc.si, a.alpha_re, a.alpha_im, a.accumulate);
            if (do_d) store64(batch_matrix<Out>(a, true, f) + off, acc.dr, acc.di, a.alpha_re, a.alpha_im, a.accumulate);
        }
    }
}

template <typename Out>
__global__ void __launch_bounds__(SING_THREADS) k_singular(RegularArgs a, NearList near, int *err)
{
    singular_pairs<Out, false>(a, near, err);
}

// held to 128 registers (its code alone would take about 166), so that the
// concurrent regular kernel keeps three of its blocks on every SM beside this
// kernel's one; the single wave number kernel comes to 128 by itself, where
// the occupancy hint would only change its schedule
template <typename Out>
__global__ void __launch_bounds__(SING_THREADS, 4) k_singular_batch(RegularArgs a, NearList near, int *err)
{
    singular_pairs<Out, true>(a, near, err);
}

// host values of c_series_x
struct SeriesBounds {
    float x[MOM_J];
    SeriesBounds()
    {
        double lf = 0.0;  // log J!
        for (int J = 0; J < MOM_J; ++J) {
            if (J > 0) lf += std::log((double)J);
            x[J] = J == 0 ? 0.0f : (float)(std::exp((std::log(1e-15) + lf) / (J + 1)) * (1.0 - 1e-5));
        }
    }
};

cudaError_t prepare_singular_batch(cudaStream_t s)
{
    static const SeriesBounds bounds;
    cudaError_t e = cudaMemcpyToSymbolAsync(c_series_x, bounds.x, sizeof(bounds.x), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_singular_batch<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MOM_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_singular_batch<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MOM_SMEM);
    return e;
}

cudaError_t launch_assemble_singular(const RegularArgs &a, const NearList &near, int *err, cudaStream_t s)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one 4-warp block per SM keeps the narrow FP64 pipe busy (a warp-wide
    // FP64 instruction occupies it for many cycles) and leave most of every SM
    // to the concurrently running regular kernel
    int64_t total = (near.col_ptr ? near.nnz : 0) + (a.same_mesh ? (a.j1 - a.j0) : 0);
    int64_t want = (total + SING_THREADS - 1) / SING_THREADS;
    int blocks = (int)max((int64_t)1, min(want, (int64_t)sms));
    // a frequency batch of few pairs: split the wave numbers over gridDim.y so
    // that about one block per SM runs
    dim3 grid(blocks, 1);
    if (a.nk > 1 || a.force_batch) grid.y = (unsigned)max(1, min(a.nk, sms / blocks));
    size_t smem = 0;
    if (a.nk > 1 || a.force_batch) {
        // inside a stream capture the table and the attributes were set beforehand
        // (prepare_singular_batch): a capture records no host-memory copy
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        cudaError_t e = cudaStreamIsCapturing(s, &cap);
        if (e != cudaSuccess) return e;
        if (cap == cudaStreamCaptureStatusNone && (e = prepare_singular_batch(s)) != cudaSuccess) return e;
        smem = MOM_SMEM;
        if (a.dtype == 0) k_singular_batch<float2><<<grid, SING_THREADS, smem, s>>>(a, near, err);
        else k_singular_batch<double2><<<grid, SING_THREADS, smem, s>>>(a, near, err);
    } else {
        if (a.dtype == 0) k_singular<float2><<<blocks, SING_THREADS, 0, s>>>(a, near, err);
        else k_singular<double2><<<blocks, SING_THREADS, 0, s>>>(a, near, err);
    }
    return cudaGetLastError();
}

}  // namespace nihu
