// FP64 singular (self) and nearly singular collocational entries.
//
// One warp evaluates one (test, trial) pair: the quadrature points of every
// scheme are spread over the 32 lanes and the partial sums are reduced with
// warp shuffles, so a pair costs a few points per lane instead of dozens of
// sequential kernel evaluations.  SLP and DLP of a pair share the geometry,
// the inverse mapping and the e^{-ikr} evaluations.
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
#include "geom.cuh"
#include "kernels.h"

namespace nihu {

constexpr int SING_WARPS = 4;

struct Acc {
    double sr = 0, si = 0, dr = 0, di = 0;
};

__device__ __forceinline__ void reduce_acc(Acc &a)
{
    a.sr = warp_sum(a.sr);
    a.si = warp_sum(a.si);
    a.dr = warp_sum(a.dr);
    a.di = warp_sum(a.di);
}

// G(r) and dG/dr of a family; g = e^{-ikr}/(4 pi r)
__device__ __forceinline__ cd green(int fam, double k, double r)
{
    if (fam == FAM_LAPLACE) return {1.0 / r / FOUR_PI, 0.0};
    double s, c;
    sincos(k * r, &s, &c);
    return {c / r / FOUR_PI, -s / r / FOUR_PI};
}

__device__ __forceinline__ cd dgreen(int fam, double k, double r)
{
    if (fam == FAM_LAPLACE) return {-1.0 / (r * r) / FOUR_PI, 0.0};
    double s, c;
    sincos(k * r, &s, &c);
    double kr = k * r;
    double f = 1.0 / (r * r) / FOUR_PI;
    // e^{-ikr} (-ikr - 1) = -(c + kr s) - i (kr c - s)
    return {-(c + kr * s) * f, -(kr * c - s) * f};
}

// kernel value times Jacobian at reference point (xi, eta) of element e seen from x0
__device__ __forceinline__ void kern_on_elem(const Elem64 &e, int fam, double k, const double x0[3], double xi,
                                             double eta, bool do_s, bool do_d, cd &ks, cd &kd)
{
    double y[3], n[3];
    ex(e, xi, eta, y);
    enormal(e, xi, eta, n);
    double J = norm3(n);
    double rv[3] = {y[0] - x0[0], y[1] - x0[1], y[2] - x0[2]};
    double r = norm3(rv);
    if (do_s) ks = cscale(green(fam, k, r), J);
    if (do_d) {
        double rdn = (rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2]) / J / r;
        kd = cscale(dgreen(fam, k, r), rdn * J);
    }
}

// ------------------------------------------------------------------ planar

// rotate the element parallel to the x-y plane (nihu/library/plane_element_helper.hpp:112-126)
__device__ void plane_local(const Elem64 &e, const double x0in[3], double loc[4][3], double x0[3])
{
    double v1[3], v2[3], t0[3], t1[3], t2[3];
    for (int d = 0; d < 3; ++d) { v1[d] = e.c[1][d] - e.c[0][d]; v2[d] = e.c[2][d] - e.c[0][d]; }
    double n1 = norm3(v1);
    for (int d = 0; d < 3; ++d) t0[d] = v1[d] / n1;
    cross3(v1, v2, t2);
    double n2 = norm3(t2);
    for (int d = 0; d < 3; ++d) t2[d] /= n2;
    cross3(t2, t0, t1);
    double n3 = norm3(t1);
    for (int d = 0; d < 3; ++d) t1[d] /= n3;
    for (int a = 0; a < e.nc; ++a) {
        loc[a][0] = dot3(t0, e.c[a]);
        loc[a][1] = dot3(t1, e.c[a]);
        loc[a][2] = dot3(t2, e.c[a]);
    }
    x0[0] = dot3(t0, x0in);
    x0[1] = dot3(t1, x0in);
    x0[2] = dot3(t2, x0in);
}

// side data seen from the projected point: corner angle, foot angle, distance
__device__ __forceinline__ void side_geometry(const double c1[2], const double c2[2], const double p[2], double &th_lim,
                                              double &th0, double &dref, bool guard_short)
{
    double l0 = 1.0, l1 = 0.0;
    double d0 = c2[0] - c1[0], d1 = c2[1] - c1[1];
    double ln = sqrt(d0 * d0 + d1 * d1);
    if (!guard_short || ln > 1e-3) { l0 = d0 / ln; l1 = d1 / ln; }
    double a0 = c1[0] - p[0], a1 = c1[1] - p[1];
    double pr = a0 * l0 + a1 * l1;
    double f0 = a0 - l0 * pr, f1 = a1 - l1 * pr;
    th_lim = atan2(a1, a0);
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

// static (Laplace) nearly singular part over a flat element, lanes 0 .. 6 nc - 1
// (nihu/library/laplace_nearly_singular_integrals.hpp:62-209); adds SLP and DLP
// (real) results to a.sr / a.dr after the warp reduction
__device__ void near_static(const Elem64 &e, const double x0in[3], bool do_s, bool do_d, int lane, Acc &a)
{
    double loc[4][3], x0[3];
    plane_local(e, x0in, loc, x0);
    const double z = x0[2] - loc[0][2];
    double s_sum = 0.0, d_sum = 0.0;
    const int N = e.nc;
    if (lane < 6 * N) {
        int side = lane / 6, q = lane % 6;
        double p[2] = {x0[0], x0[1]};
        double c1[2] = {loc[side][0], loc[side][1]};
        double c2[2] = {loc[(side + 1) % N][0], loc[(side + 1) % N][1]};
        double c3[2] = {loc[(side + 2) % N][0], loc[(side + 2) % N][1]};
        double t1, th0, dref, t2, dummy0, dummy1;
        side_geometry(c1, c2, p, t1, th0, dref, false);
        side_geometry(c2, c3, p, t2, dummy0, dummy1, false);
        wrap_limits(t1, t2);
        double jac = (t2 - t1) / 2.0;
        double xi, w;
        gauss_pt(6, q, xi, w);
        double th = t1 * (1.0 - xi) / 2.0 + t2 * (1.0 + xi) / 2.0;
        double R = dref / cos(th - th0);
        double r = sqrt(R * R + z * z);
        if (do_s) s_sum = (r - fabs(z)) * jac * w;
        if (do_d) d_sum = (1.0 - fabs(z) / r) * jac * w;
    }
    s_sum = warp_sum(s_sum);
    d_sum = warp_sum(d_sum);
    double sg = (0.0 < z) - (z < 0.0);
    a.sr += s_sum / FOUR_PI;
    a.dr += sg * d_sum / FOUR_PI;
}

// dynamic part (K_k - K_0) of the planar nearly singular scheme with the
// degree-14 rule; per-lane partial sums (not reduced)
__device__ void near_dynamic(const Elem64 &e, double k, const double x0[3], bool do_s, bool do_d, int lane, Acc &a)
{
    double en[3];
    {
        double xi, eta;
        domain_center(e.nc, xi, eta);
        enormal(e, xi, eta, en);
        double nn = norm3(en);
        for (int d = 0; d < 3; ++d) en[d] /= nn;
    }
    const int np = e.nc == 3 ? 42 : 64;
    for (int p = lane; p < np; p += 32) {
        double xi, eta, w;
        if (e.nc == 3) tri_pt(14, p, xi, eta, w);
        else {
            double w0, w1;
            gauss_pt(8, p / 8, xi, w0);
            gauss_pt(8, p % 8, eta, w1);
            w = w0 * w1;
        }
        double y[3], n[3];
        ex(e, xi, eta, y);
        enormal(e, xi, eta, n);
        double J = norm3(n);
        double rv[3] = {y[0] - x0[0], y[1] - x0[1], y[2] - x0[2]};
        double r = norm3(rv);
        if (do_s) {
            cd gk = green(FAM_HELMHOLTZ, k, r), g0 = green(FAM_LAPLACE, k, r);
            a.sr += (gk.re - g0.re) * w * J;
            a.si += (gk.im - g0.im) * w * J;
        }
        if (do_d) {
            double rdn = dot3(rv, en) / r;
            cd gk = dgreen(FAM_HELMHOLTZ, k, r), g0 = dgreen(FAM_LAPLACE, k, r);
            a.dr += (gk.re * rdn - g0.re * rdn) * w * J;
            a.di += (gk.im * rdn - g0.im * rdn) * w * J;
        }
    }
}

// full planar constant-element nearly singular integral (reduced into a)
__device__ void near_plane(const Elem64 &e, int fam, double k, const double x0[3], bool do_s, bool do_d, int lane,
                           Acc &a)
{
    Acc dyn;
    if (fam == FAM_HELMHOLTZ) {
        near_dynamic(e, k, x0, do_s, do_d, lane, dyn);
        reduce_acc(dyn);
    }
    Acc st;
    near_static(e, x0, do_s, do_d, lane, st);
    a.sr += st.sr + dyn.sr;
    a.si += dyn.si;
    a.dr += st.dr + dyn.dr;
    a.di += dyn.di;
}

// ------------------------------------------------------------ inverse mapping

// Newton iteration (nihu/core/inverse_mapping.hpp:52-112).  Records the first
// iterate with |f| < 1e-5 (polar scheme) and with |f| < 1e-6 (Telles); both
// come from the same iteration sequence the reference runs separately.
__device__ bool inverse_mapping(const Elem64 &e, const double x0[3], bool need6, double r5[3], double r6[3])
{
    double res[3] = {0.0, 0.0, 0.0};
    bool got5 = false;
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
        double dxe[3] = {0, 0, 0};
        if (e.nc == 4)
            for (int d = 0; d < 3; ++d) dxe[d] = (e.c[0][d] - e.c[1][d] + e.c[2][d] - e.c[3][d]) * 0.25;
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

// polar scheme around (xi0, eta0) with linearized-element subtraction;
// per-lane partial sums of SLP (do_s) and DLP (do_d)
__device__ void near_polar_sum(const Elem64 &e, const Elem64 &lin, int fam, double k, const double x0[3], double xi0,
                               double eta0, bool do_s, bool do_d, int lane, Acc &a)
{
    const int N = e.nc;
    double tl[4], t0[4], dr[4];
    for (int n = 0; n < N; ++n) {
        double c1[2], c2[2], p[2] = {xi0, eta0};
        domain_corner(N, n, c1[0], c1[1]);
        domain_corner(N, (n + 1) % N, c2[0], c2[1]);
        side_geometry(c1, c2, p, tl[n], t0[n], dr[n], true);
    }
    for (int p = lane; p < N * 64; p += 32) {
        int n = p / 64, ia = (p / 8) % 8, ib = p % 8;
        double t1 = tl[n], t2 = tl[(n + 1) % N];
        wrap_limits(t1, t2);
        if (fabs(t2 - t1) < 1e-3) continue;
        double xx, wa, xr, wb;
        gauss_pt(8, ia, xx, wa);
        gauss_pt(8, ib, xr, wb);
        double th = ((1.0 - xx) * t1 + (1.0 + xx) * t2) / 2.0;
        double wth = wa * (t2 - t1) / 2.0;
        double rho_lim = dr[n] / cos(th - t0[n]);
        double rho = (1.0 + xr) * rho_lim / 2.0;
        double wrho = wb * rho_lim / 2.0;
        double xi = xi0 + rho * cos(th), eta = eta0 + rho * sin(th);
        cd fs{0, 0}, fd{0, 0}, ls{0, 0}, ld{0, 0};
        kern_on_elem(e, fam, k, x0, xi, eta, do_s, do_d, fs, fd);
        kern_on_elem(lin, fam, k, x0, xi, eta, do_s, do_d, ls, ld);
        double wt = wth * wrho * rho;
        a.sr += wt * (fs.re - ls.re);
        a.si += wt * (fs.im - ls.im);
        a.dr += wt * (fd.re - ld.re);
        a.di += wt * (fd.im - ld.im);
    }
}

// Telles-transformed 16x16 Gauss rule (DLP only); per-lane partial sums
__device__ void near_telles_sum(const Elem64 &e, int fam, double k, const double x0[3], const double im[3], int lane,
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
    for (int p = lane; p < 256; p += 32) {
        double u[2], wu[2];
        gauss_pt(16, p / 16, u[0], wu[0]);
        gauss_pt(16, p % 16, u[1], wu[1]);
        double w = wu[0] * wu[1], t[2];
        for (int dim = 0; dim < 2; ++dim) {
            double x = u[dim];
            t[dim] = ca[dim] * x * x * x + cb[dim] * x * x + cc[dim] * x + cdd[dim];
            w *= 3.0 * ca[dim] * x * x + 2.0 * cb[dim] * x + cc[dim];
        }
        cd ks{0, 0}, kd{0, 0};
        kern_on_elem(e, fam, k, x0, t[0], t[1], false, true, ks, kd);
        a.dr += kd.re * w;
        a.di += kd.im * w;
    }
}

// -------------------------------------------------------------------- self

// analytic static part of the flat-element 1/r integral from an interior point
// (nihu/library/plane_element_helper.hpp:42-74), lanes 0 .. nc-1
__device__ double self_static(const Elem64 &e, const double x0[3], int lane)
{
    double v = 0.0;
    const int N = e.nc;
    if (lane < N) {
        int i = lane, i1 = (lane + 1) % N;
        double R0[3], R1[3], C[3];
        for (int d = 0; d < 3; ++d) { R0[d] = e.c[i][d] - x0[d]; R1[d] = e.c[i1][d] - x0[d]; C[d] = e.c[i][d] - e.c[i1][d]; }
        double r0 = norm3(R0), r1 = norm3(R1), cn = norm3(C);
        for (int d = 0; d < 3; ++d) { R0[d] /= r0; R1[d] /= r1; C[d] /= cn; }
        double cs = dot3(R0, R1);
        double theta = cs >= 1.0 ? 0.0 : acos(cs);
        double alpha = acos(dot3(R0, C));
        v = r0 * sin(alpha) * log(tan((alpha + theta) / 2.0) / tan(alpha / 2.0));
    }
    return warp_sum(v);
}

__device__ __forceinline__ double sinc_ref(double x)
{
    if (fabs(x) > 1e-3) return sin(x) / x;
    return 1.0 - x * x / 6.0 * (1.0 - x * x / 20.0);
}

__device__ void self_tria(const Elem64 &e, int fam, double k, const double x0[3], int lane, Acc &a)
{
    double st = self_static(e, x0, lane);
    double dr = 0.0, di = 0.0;
    if (fam == FAM_HELMHOLTZ && lane < 13) {
        double xi, eta, w;
        tri_pt(7, lane, xi, eta, w);
        double y[3], n[3];
        ex(e, xi, eta, y);
        enormal(e, xi, eta, n);
        double rv[3] = {y[0] - x0[0], y[1] - x0[1], y[2] - x0[2]};
        double r = norm3(rv);
        // -ik e^{-ikr/2} sinc(kr/2)
        double s, c;
        sincos(k * r / 2.0, &s, &c);
        double sc = sinc_ref(k * r / 2.0);
        double wj = w * norm3(n);
        dr = -k * s * sc * wj;
        di = -k * c * sc * wj;
    }
    dr = warp_sum(dr);
    di = warp_sum(di);
    a.sr += (st + dr) / FOUR_PI;
    a.si += di / FOUR_PI;
    // DLP of a flat triangle over itself is zero
}

__device__ void self_quad(const Elem64 &e, int fam, double k, const double x0[3], bool do_s, bool do_d, int lane,
                          Acc &a)
{
    for (int p = lane; p < 64; p += 32) {
        int d = p / 16, ia = (p % 16) / 4, ib = p % 4;
        double u, wu, v, wv;
        gauss_pt(4, ia, u, wu);
        gauss_pt(4, ib, v, wv);
        double P[4][2];
        P[0][0] = P[1][0] = 0.0;
        P[0][1] = P[1][1] = 0.0;
        domain_corner(4, d, P[2][0], P[2][1]);
        domain_corner(4, (d + 1) % 4, P[3][0], P[3][1]);
        double N[4], dN[4][2];
        shape(4, u, v, N);
        dshape(4, u, v, dN);
        double xi = 0, eta = 0, j00 = 0, j01 = 0, j10 = 0, j11 = 0;
        for (int c = 0; c < 4; ++c) {
            xi += N[c] * P[c][0];
            eta += N[c] * P[c][1];
            j00 += dN[c][0] * P[c][0];
            j01 += dN[c][0] * P[c][1];
            j10 += dN[c][1] * P[c][0];
            j11 += dN[c][1] * P[c][1];
        }
        double wd = wu * wv * (j00 * j11 - j01 * j10);
        cd ks{0, 0}, kd{0, 0};
        kern_on_elem(e, fam, k, x0, xi, eta, do_s, do_d, ks, kd);
        a.sr += ks.re * wd;
        a.si += ks.im * wd;
        a.dr += kd.re * wd;
        a.di += kd.im * wd;
    }
    reduce_acc(a);
}

// ------------------------------------------------------------------ driver

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

template <typename Out>
__global__ void __launch_bounds__(32 * SING_WARPS) k_singular(RegularArgs a, NearList near, int *err)
{
    const int lane = threadIdx.x & 31;
    const int64_t p_begin = near.col_ptr ? near.col_ptr[a.j0] : 0;
    const int64_t p_end = near.col_ptr ? near.col_ptr[a.j1] : 0;
    const int64_t n_near = p_end - p_begin;
    const int64_t n_self = a.same_mesh ? (int64_t)(a.j1 - a.j0) : 0;
    const int64_t total = n_near + n_self;
    const bool do_s = (a.ops & OP_SLP) != 0, do_d = (a.ops & OP_DLP) != 0;
    Out *out_s = reinterpret_cast<Out *>(a.out_s);
    Out *out_d = reinterpret_cast<Out *>(a.out_d);
    const int fam = a.family;
    const double k = a.k;

    for (int64_t item = (int64_t)blockIdx.x * SING_WARPS + (threadIdx.x >> 5); item < total;
         item += (int64_t)gridDim.x * SING_WARPS) {
        int i, j;
        bool self;
        if (item < n_near) {
            int64_t p = p_begin + item;
            i = near.rows[p];
            int lo = a.j0, hi = a.j1 - 1;  // largest j with col_ptr[j] <= p
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (near.col_ptr[mid] <= p) lo = mid;
                else hi = mid - 1;
            }
            j = lo;
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
        Acc acc;
        bool ok = true;
        if (self) {
            if (e.nc == 3) {
                if (do_s) self_tria(e, fam, k, x0, lane, acc);
            } else {
                self_quad(e, fam, k, x0, do_s, do_d, lane, acc);
            }
        } else if (e.nc == 3) {
            near_plane(e, fam, k, x0, do_s, do_d, lane, acc);
        } else {
            const bool telles = fam == FAM_HELMHOLTZ && do_d;
            const bool polar_d = fam == FAM_LAPLACE && do_d;
            double r5[3] = {0, 0, 0}, r6[3] = {0, 0, 0};
            ok = inverse_mapping(e, x0, telles, r5, r6);
            if (ok) {
                Acc part;
                if (do_s || polar_d) {
                    Elem64 lin;
                    linearized(e, r5[0], r5[1], lin);
                    near_polar_sum(e, lin, fam, k, x0, r5[0], r5[1], do_s, polar_d, lane, part);
                    reduce_acc(part);
                    near_plane(lin, fam, k, x0, do_s, polar_d, lane, part);
                }
                if (telles) {
                    Acc tp;
                    near_telles_sum(e, fam, k, x0, r6, lane, tp);
                    reduce_acc(tp);
                    part.dr += tp.dr;
                    part.di += tp.di;
                }
                acc = part;
            }
        }
        if (lane == 0) {
            if (!ok) {
                atomicCAS(err, 0, (int)min(item + 1, (int64_t)0x7fffffff));
                continue;
            }
            const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
            if (do_s) store64(out_s + off, acc.sr, acc.si, a.alpha_re, a.alpha_im, a.accumulate);
            if (do_d) store64(out_d + off, acc.dr, acc.di, a.alpha_re, a.alpha_im, a.accumulate);
        }
    }
}

cudaError_t launch_assemble_singular(const RegularArgs &a, const NearList &near, int *err, cudaStream_t s)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int blocks = sms * 16;
    if (a.dtype == 0) k_singular<float2><<<blocks, 32 * SING_WARPS, 0, s>>>(a, near, err);
    else k_singular<double2><<<blocks, 32 * SING_WARPS, 0, s>>>(a, near, err);
    return cudaGetLastError();
}

}  // namespace nihu
