/*
 * FP64 CPU oracle of NiHu's dense collocational BEM assembly (TEST
 * INFRASTRUCTURE ONLY).  This file is a from-scratch restatement of the
 * reference algorithm, used by the tests as the checker and by bench.py as the
 * timed CPU baseline.  It is never linked into, or called by, the product
 * library.  Every function cites the reference file:line it restates
 * (paths inside the NiHu project).
 *
 * Parity pins: the nearly singular Helmholtz/Laplace SLP element integrals
 * against the reference's golden values
 * (nihu/gtest/test_helmholtz_3d_elem_integrals.cpp:15-36,
 *  nihu/gtest/test_laplace_3d_elem_integrals.cpp:17-37), the analytic
 * pulsating-sphere solution, closed-form Laplace self integrals, and
 * converged brute-force quadrature (see tests/).
 *
 * Conventions (as in the reference):
 *  - time convention e^{+jwt}: G = e^{-ikr}/(4 pi r)
 *    (nihu/library/helmholtz_kernel.hpp:180-186)
 *  - r_vec = y - x, DLP = dG/dr * (r_vec . n_y)/r
 *    (nihu/library/normal_derivative_kernel.hpp:167-180)
 *  - constant elements, collocation at the reference-domain centre
 *    (nihu/core/shapeset.hpp:290-293, nihu/library/lib_domain.cpp:70-71,94)
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../nihu_gb300/csrc/quad_rules.h"

typedef double complex cplx;

#define FAM_HELMHOLTZ 0
#define FAM_LAPLACE 1
#define OP_SLP 1
#define OP_DLP 2
#define OP_DLPT 4
#define OP_HSP 8
#define TRIA_1_ID 32303
#define QUAD_1_ID 32404

static const double PI = 3.14159265358979323846264338327950288;

static const int gauss_off[NIHU_GAUSS_MAX_N] = NIHU_GAUSS_OFFSETS;
static const double gauss_data[NIHU_GAUSS_DATA_LEN] = NIHU_GAUSS_DATA;
static const int tri_npts[15] = NIHU_TRI_NPTS;
static const int tri_off[15] = NIHU_TRI_OFFSETS;
static const double tri_data[NIHU_TRI_DATA_LEN] = NIHU_TRI_DATA;

/* Gauss-Legendre n-point rule (n = degree/2+1,
 * nihu/core/gaussian_quadrature.hpp:136-151) */
static const double *gauss_rule(int n) { return gauss_data + 2 * gauss_off[n - 1]; }

/* ------------------------------------------------------------------ elements */

typedef struct {
    int nc;            /* 3: tria_1, 4: quad_1 */
    double c[4][3];    /* corner coordinates */
    double center[3];  /* x(domain centre), nihu/core/element.hpp:276 */
    double size;       /* mean edge length, nihu/core/element.hpp:280-291 */
} elem_t;

static void shape(int nc, double xi, double eta, double N[4])
{
    if (nc == 3) { /* nihu/library/lib_shape.hpp:159-170 */
        N[0] = 1.0 - xi - eta; N[1] = xi; N[2] = eta; N[3] = 0.0;
    } else {       /* bilinear, corners (-1,-1),(1,-1),(1,1),(-1,1) */
        N[0] = (1.0 - xi) * (1.0 - eta) / 4.0;
        N[1] = (1.0 + xi) * (1.0 - eta) / 4.0;
        N[2] = (1.0 + xi) * (1.0 + eta) / 4.0;
        N[3] = (1.0 - xi) * (1.0 + eta) / 4.0;
    }
}

static void dshape(int nc, double xi, double eta, double dN[4][2])
{
    if (nc == 3) {
        dN[0][0] = -1.0; dN[0][1] = -1.0;
        dN[1][0] = 1.0;  dN[1][1] = 0.0;
        dN[2][0] = 0.0;  dN[2][1] = 1.0;
        dN[3][0] = 0.0;  dN[3][1] = 0.0;
    } else {
        dN[0][0] = -(1.0 - eta) / 4.0; dN[0][1] = -(1.0 - xi) / 4.0;
        dN[1][0] = (1.0 - eta) / 4.0;  dN[1][1] = -(1.0 + xi) / 4.0;
        dN[2][0] = (1.0 + eta) / 4.0;  dN[2][1] = (1.0 + xi) / 4.0;
        dN[3][0] = -(1.0 + eta) / 4.0; dN[3][1] = (1.0 - xi) / 4.0;
    }
}

static void elem_x(const elem_t *e, double xi, double eta, double x[3])
{
    double N[4];
    shape(e->nc, xi, eta, N);
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int a = 0; a < e->nc; ++a) s += N[a] * e->c[a][d];
        x[d] = s;
    }
}

static void elem_dx(const elem_t *e, double xi, double eta, double dxi[3], double deta[3])
{
    double dN[4][2];
    dshape(e->nc, xi, eta, dN);
    for (int d = 0; d < 3; ++d) {
        double s0 = 0.0, s1 = 0.0;
        for (int a = 0; a < e->nc; ++a) { s0 += dN[a][0] * e->c[a][d]; s1 += dN[a][1] * e->c[a][d]; }
        dxi[d] = s0; deta[d] = s1;
    }
}

static void cross(const double a[3], const double b[3], double c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm3(const double a[3]) { return sqrt(dot3(a, a)); }

/* surface normal dx/dxi x dx/deta, its length is the Jacobian
 * (nihu/core/element.hpp:503-515) */
static void elem_normal(const elem_t *e, double xi, double eta, double n[3])
{
    double a[3], b[3];
    elem_dx(e, xi, eta, a, b);
    cross(a, b, n);
}

static void domain_corner(int nc, int i, double *xi, double *eta)
{
    static const double tc[3][2] = {{0, 0}, {1, 0}, {0, 1}};
    static const double qc[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    if (nc == 3) { *xi = tc[i][0]; *eta = tc[i][1]; }
    else { *xi = qc[i][0]; *eta = qc[i][1]; }
}

static void domain_center(int nc, double *xi, double *eta)
{
    if (nc == 3) { *xi = 1.0 / 3.0; *eta = 1.0 / 3.0; }
    else { *xi = 0.0; *eta = 0.0; }
}

/* element constructor: centre and linear size estimate (mean edge length)
 * (nihu/core/element.hpp:271-292) */
static void elem_init(elem_t *e, int nc, const double *coords /* nc x 3 */)
{
    e->nc = nc;
    memset(e->c, 0, sizeof(e->c));
    for (int a = 0; a < nc; ++a)
        for (int d = 0; d < 3; ++d) e->c[a][d] = coords[3 * a + d];
    double xi, eta;
    domain_center(nc, &xi, &eta);
    elem_x(e, xi, eta, e->center);
    double s = 0.0;
    for (int ed = 0; ed < nc; ++ed) {
        double x0[3], x1[3], x0i, x0e, x1i, x1e, dv[3];
        domain_corner(nc, ed, &x0i, &x0e);
        domain_corner(nc, (ed + 1) % nc, &x1i, &x1e);
        elem_x(e, x0i, x0e, x0);
        elem_x(e, x1i, x1e, x1);
        for (int d = 0; d < 3; ++d) dv[d] = x1[d] - x0[d];
        s += norm3(dv);
    }
    e->size = s / nc;
}

/* ------------------------------------------------------------------ kernels */

/* G(r) (nihu/library/helmholtz_kernel.hpp:180-186, laplace_kernel.hpp:137-141) */
static cplx green(int fam, cplx k, double r)
{
    if (fam == FAM_LAPLACE) return 1.0 / r / (4.0 * PI);
    return cexp(-I * (k * r)) / r / (4.0 * PI);
}

/* dG/dr (nihu/library/helmholtz_kernel.hpp:190-195, laplace_kernel.hpp:143-147) */
static cplx dgreen(int fam, cplx k, double r)
{
    if (fam == FAM_LAPLACE) return -1.0 / (r * r) / (4.0 * PI);
    cplx ikr = I * (k * r);
    return cexp(-ikr) / (r * r) / (4.0 * PI) * (-ikr - 1.0);
}

/* SLP kernel G(|y-x|) (nihu/library/normal_derivative_kernel.hpp:131-136) */
static cplx kern_slp(int fam, cplx k, const double x[3], const double y[3])
{
    double rv[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    return green(fam, k, norm3(rv));
}

/* DLP kernel dG/dr (r_vec.n_y)/r, n_y unit
 * (nihu/library/normal_derivative_kernel.hpp:167-175) */
static cplx kern_dlp(int fam, cplx k, const double x[3], const double y[3], const double ny[3])
{
    double rv[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    double r = norm3(rv);
    double rdny = dot3(rv, ny) / r;
    return dgreen(fam, k, r) * rdny;
}

/* DLPt kernel dG/dr (-r_vec.n_x)/r, n_x the unit normal at the collocation point
 * (nihu/library/normal_derivative_kernel.hpp:199-206) */
static cplx kern_dlpt(int fam, cplx k, const double x[3], const double nx[3], const double y[3])
{
    double rv[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    double r = norm3(rv);
    double rdnx = -dot3(rv, nx) / r;
    return dgreen(fam, k, r) * rdnx;
}

/* f[0] = G'' - G'/r, f[1] = G'/r (nihu/library/helmholtz_kernel.hpp:198-205,
 * the Laplace kernel being its k = 0 case) */
static void ddgreen(int fam, cplx k, double r, cplx f[2])
{
    cplx ikr = fam == FAM_LAPLACE ? 0.0 : I * (k * r);
    cplx g = cexp(-ikr) / (r * r * r) / (4.0 * PI);
    f[1] = -g * (1.0 + ikr);
    f[0] = g * (3.0 + ikr * (3.0 + ikr));
}

/* HSP kernel f0 (r.n_x)(r.n_y)-terms - f1 n_x.n_y
 * (nihu/library/normal_derivative_kernel.hpp:242-251) */
static cplx kern_hsp(int fam, cplx k, const double x[3], const double nx[3], const double y[3], const double ny[3])
{
    double rv[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    double r = norm3(rv);
    double rdny = dot3(rv, ny) / r;
    double rdnx = -dot3(rv, nx) / r;
    cplx f[2];
    ddgreen(fam, k, r, f);
    return f[0] * rdnx * rdny - f[1] * dot3(nx, ny);
}

/* nx: unit normal at the collocation point (used by DLPt and HSP only) */
static cplx kern(int fam, int op, cplx k, const double x[3], const double *nx, const double y[3], const double ny[3])
{
    if (op == OP_SLP) return kern_slp(fam, k, x, y);
    if (op == OP_DLP) return kern_dlp(fam, k, x, y, ny);
    if (op == OP_DLPT) return kern_dlpt(fam, k, x, nx, y);
    return kern_hsp(fam, k, x, nx, y, ny);
}

/* ------------------------------------------------------- quadrature degree */

/* distance intervals for accuracy 3 (nihu/library/distance_kernel_intervals.hpp:117-154),
 * evaluated with strict '<' (nihu/tmp/interval.hpp:173-185).  SLP behaves as
 * 1/r in the far field, DLP and DLPt as 1/r^2, HSP as 1/r^3
 * (nihu/library/helmholtz_kernel.hpp:281-306). */
static int interval_degree(int op, double ratio)
{
    if (op == OP_HSP) {
        if (ratio < 10.0 / 10.0) return 9;
        if (ratio < 11.0 / 10.0) return 9;
        if (ratio < 14.0 / 10.0) return 8;
        if (ratio < 19.0 / 10.0) return 6;
        if (ratio < 36.0 / 10.0) return 4;
        if (ratio < 223.0 / 10.0) return 2;
        return 0;
    }
    if (op == OP_SLP) {
        if (ratio < 11.0 / 10.0) return 6;
        if (ratio < 18.0 / 10.0) return 4;
        if (ratio < 91.0 / 10.0) return 2;
        return 0;
    }
    if (ratio < 11.0 / 10.0) return 8;
    if (ratio < 15.0 / 10.0) return 6;
    if (ratio < 28.0 / 10.0) return 4;
    if (ratio < 158.0 / 10.0) return 2;
    return 0;
}

/* field complexity: polynomial order of the constant N-set (0) plus the
 * Jacobian order of the geometry (tria_1: 0, quad_1: 1)
 * (nihu/core/complexity_estimator.hpp:47-62, nihu/library/lib_shape.hpp:134-143,219-228) */
static int field_complexity(int nc) { return nc == 4 ? 1 : 0; }

static double centre_distance(const elem_t *a, const elem_t *b)
{
    double dv[3] = {b->center[0] - a->center[0], b->center[1] - a->center[1], b->center[2] - a->center[2]};
    return norm3(dv);
}

/* -------------------------------------------------------- regular integral */

/* sum_q w_q K(x, y_q) J_q over the trial element with the rule of the given
 * degree (nihu/core/double_integral.hpp:445-467 with the accelerator of :576-585) */
static cplx regular_integral(const elem_t *e, int fam, int op, cplx k, const double x[3], const double *nx,
                             int degree)
{
    cplx sum = 0.0;
    if (e->nc == 3) {
        const double *q = tri_data + 3 * tri_off[degree];
        int np = tri_npts[degree];
        for (int p = 0; p < np; ++p) {
            double y[3], n[3];
            elem_x(e, q[3 * p], q[3 * p + 1], y);
            elem_normal(e, q[3 * p], q[3 * p + 1], n);
            double J = norm3(n);
            double un[3] = {n[0] / J, n[1] / J, n[2] / J};
            sum += kern(fam, op, k, x, nx, y, un) * (J * q[3 * p + 2]);
        }
    } else {
        int ng = degree / 2 + 1;
        const double *g = gauss_rule(ng);
        for (int a = 0; a < ng; ++a)
            for (int b = 0; b < ng; ++b) {
                double xi = g[2 * a], eta = g[2 * b], w = g[2 * a + 1] * g[2 * b + 1];
                double y[3], n[3];
                elem_x(e, xi, eta, y);
                elem_normal(e, xi, eta, n);
                double J = norm3(n);
                double un[3] = {n[0] / J, n[1] / J, n[2] / J};
                sum += kern(fam, op, k, x, nx, y, un) * (J * w);
            }
    }
    return sum;
}

/* ------------------------------------------------- singular self integrals */

/* radii, subtended angles and corner angles seen from an interior point
 * (nihu/library/plane_element_helper.hpp:42-74) */
static void plane_element_helper(const elem_t *e, const double x0[3], double r[4], double theta[4], double alpha[4])
{
    int N = e->nc;
    double R[4][3], C[4][3];
    for (int i = 0; i < N; ++i) {
        for (int d = 0; d < 3; ++d) R[i][d] = e->c[i][d] - x0[d];
        r[i] = norm3(R[i]);
        for (int d = 0; d < 3; ++d) R[i][d] /= r[i];
        for (int d = 0; d < 3; ++d) C[i][d] = e->c[i][d] - e->c[(i + 1) % N][d];
        double cn = norm3(C[i]);
        for (int d = 0; d < 3; ++d) C[i][d] /= cn;
    }
    for (int i = 0; i < N; ++i) {
        double cs = dot3(R[i], R[(i + 1) % N]);
        theta[i] = cs >= 1.0 ? 0.0 : acos(cs);
        alpha[i] = acos(dot3(R[i], C[i]));
    }
}

/* analytic integral of 1/r over a flat element from an interior point, times 4 pi
 * (nihu/library/laplace_singular_integrals.hpp:465-479) */
static double static_self_integral(const elem_t *e, const double x0[3])
{
    double r[4], th[4], al[4], s = 0.0;
    plane_element_helper(e, x0, r, th, al);
    for (int i = 0; i < e->nc; ++i)
        s += r[i] * sin(al[i]) * log(tan((al[i] + th[i]) / 2.0) / tan(al[i] / 2.0));
    return s;
}

/* sinc with the reference's small-argument series (nihu/util/math_functions.hpp:54-61) */
static cplx sinc_ref(cplx x)
{
    if (cabs(x) > 1e-3) return csin(x) / x;
    return 1.0 - x * x / 6.0 * (1.0 - x * x / 20.0);
}

/* constant flat triangle, Helmholtz SLP self term: analytic static part plus
 * the regular dynamic part (e^{-ikr}-1)/r with the degree-7 Dunavant rule
 * (nihu/library/helmholtz_singular_integrals.hpp:703-762) */
static cplx self_tria_slp(const elem_t *e, int fam, cplx k)
{
    double stat = static_self_integral(e, e->center);
    if (fam == FAM_LAPLACE) return stat / (4.0 * PI);
    const double *q = tri_data + 3 * tri_off[7];
    cplx dyn = 0.0;
    for (int p = 0; p < tri_npts[7]; ++p) {
        double y[3], n[3];
        elem_x(e, q[3 * p], q[3 * p + 1], y);
        elem_normal(e, q[3 * p], q[3 * p + 1], n);
        double rv[3] = {y[0] - e->center[0], y[1] - e->center[1], y[2] - e->center[2]};
        double r = norm3(rv);
        cplx dp = -I * k * cexp(-I * k * r / 2.0) * sinc_ref(k * r / 2.0);
        dyn += dp * q[3 * p + 2] * norm3(n);
    }
    return (stat + dyn) / (4.0 * PI);
}

/* quad self term: Duffy-type polar splitting of the reference square into four
 * corner-collapsed quads around the collocation point, each with the 4x4
 * Gauss rule of degree 7 (nihu/core/duffy_quadrature.hpp:82-141,
 * nihu/core/singular_accelerator.hpp:440-448, nihu/core/quadrature.hpp:112-130,
 * evaluated as in nihu/core/double_integral.hpp:474-510) */
static cplx self_quad_duffy(const elem_t *e, int fam, int op, cplx k)
{
    const int ng = 7 / 2 + 1;
    const double *g = gauss_rule(ng);
    double s0, s1;
    domain_center(4, &s0, &s1);
    double x0[3];
    elem_x(e, s0, s1, x0);
    cplx sum = 0.0;
    for (int d = 0; d < 4; ++d) {
        double P[4][2];
        P[0][0] = P[1][0] = s0; P[0][1] = P[1][1] = s1;
        domain_corner(4, d, &P[2][0], &P[2][1]);
        domain_corner(4, (d + 1) % 4, &P[3][0], &P[3][1]);
        for (int a = 0; a < ng; ++a)
            for (int b = 0; b < ng; ++b) {
                double u = g[2 * a], v = g[2 * b], w = g[2 * a + 1] * g[2 * b + 1];
                double N[4], dN[4][2];
                shape(4, u, v, N);
                dshape(4, u, v, dN);
                double xi = 0, eta = 0, j00 = 0, j01 = 0, j10 = 0, j11 = 0;
                for (int c = 0; c < 4; ++c) {
                    xi += N[c] * P[c][0]; eta += N[c] * P[c][1];
                    j00 += dN[c][0] * P[c][0]; j01 += dN[c][0] * P[c][1];
                    j10 += dN[c][1] * P[c][0]; j11 += dN[c][1] * P[c][1];
                }
                double wd = w * (j00 * j11 - j01 * j10);
                double y[3], n[3];
                elem_x(e, xi, eta, y);
                elem_normal(e, xi, eta, n);
                double J = norm3(n);
                double un[3] = {n[0] / J, n[1] / J, n[2] / J};
                sum += kern(fam, op, k, x0, NULL, y, un) * (J * wd);
            }
    }
    return sum;
}

/* the regular remainder (e^{-ikr}(1+ikr) - 1 + (ikr)^2/2) / r^3 of the HSP
 * kernel's expansion, with the reference's series below r = 1e-3
 * (nihu/library/helmholtz_singular_integrals.hpp:768-777) */
static cplx hsp_dynamic(double r, cplx k)
{
    cplx ikr = I * (k * r);
    if (fabs(r) > 1e-3) return (cexp(-ikr) * (1.0 + ikr) - 1.0 + ikr * ikr / 2.0) / r / r / r;
    return -I * k * k * k *
           (1.0 / 3.0 - ikr * (1.0 / 8.0 - ikr * (1.0 / 30.0 - ikr * (1.0 / 144.0 - ikr * (1.0 / 840.0 - ikr / 5760.0)))));
}

/* constant flat triangle, HSP self term: the finite-part static integrals
 * IddG0 = sum (cos(alpha+theta) - cos(alpha)) / (r sin(alpha)) and
 * IG0 (the 1/r integral), sides with theta < 1e-3 skipped, plus the dynamic
 * remainder with the degree-7 Dunavant rule; (IddG0 + k^2/2 IG0 + I_dyn)/(4 pi)
 * (nihu/library/helmholtz_singular_integrals.hpp:764-839) */
static cplx self_tria_hsp(const elem_t *e, int fam, cplx k)
{
    double r[4], th[4], al[4];
    plane_element_helper(e, e->center, r, th, al);
    double IG0 = 0.0, IddG0 = 0.0;
    for (int i = 0; i < e->nc; ++i) {
        if (th[i] < 1e-3) continue;
        IG0 += r[i] * sin(al[i]) * log(tan((al[i] + th[i]) / 2.0) / tan(al[i] / 2.0));
        IddG0 += (cos(al[i] + th[i]) - cos(al[i])) / (r[i] * sin(al[i]));
    }
    if (fam == FAM_LAPLACE) return IddG0 / (4.0 * PI);
    const double *q = tri_data + 3 * tri_off[7];
    cplx dyn = 0.0;
    for (int p = 0; p < tri_npts[7]; ++p) {
        double y[3], n[3];
        elem_x(e, q[3 * p], q[3 * p + 1], y);
        elem_normal(e, q[3 * p], q[3 * p + 1], n);
        double rv[3] = {y[0] - e->center[0], y[1] - e->center[1], y[2] - e->center[2]};
        dyn += hsp_dynamic(norm3(rv), k) * q[3 * p + 2] * norm3(n);
    }
    return (IddG0 + k * k / 2.0 * IG0 + dyn) / (4.0 * PI);
}

/* self-term dispatch (nihu/core/double_integral.hpp:599-639): constant tria
 * SLP and HSP shortcuts, DLP and DLPt = 0 on a flat triangle
 * (nihu/library/normal_derivative_singular_integrals.hpp:13-56), quads by Duffy
 * (SLP and DLP only) */
static cplx self_integral(const elem_t *e, int fam, int op, cplx k)
{
    if (e->nc == 3) {
        if (op == OP_SLP) return self_tria_slp(e, fam, k);
        if (op == OP_HSP) return self_tria_hsp(e, fam, k);
        return 0.0;
    }
    return self_quad_duffy(e, fam, op, k);
}

/* ------------------------------------------------ nearly singular integrals */

/* rotate a flat element parallel to the x-y plane: T = [v1^, (v1 x v2)^ x v1^, (v1 x v2)^]
 * (nihu/library/plane_element_helper.hpp:112-126); the reference solves with
 * T (LU), here T is applied through its transpose (T is orthonormal) */
static void plane_local(const elem_t *e, const double x0in[3], double loc[4][3], double x0[3])
{
    double v1[3], v2[3], t0[3], t1[3], t2[3];
    for (int d = 0; d < 3; ++d) { v1[d] = e->c[1][d] - e->c[0][d]; v2[d] = e->c[2][d] - e->c[0][d]; }
    double n1 = norm3(v1);
    for (int d = 0; d < 3; ++d) t0[d] = v1[d] / n1;
    cross(v1, v2, t2);
    double n2 = norm3(t2);
    for (int d = 0; d < 3; ++d) t2[d] /= n2;
    cross(t2, t0, t1);
    double n3 = norm3(t1);
    for (int d = 0; d < 3; ++d) t1[d] /= n3;
    for (int a = 0; a < e->nc; ++a) {
        loc[a][0] = dot3(t0, e->c[a]); loc[a][1] = dot3(t1, e->c[a]); loc[a][2] = dot3(t2, e->c[a]);
    }
    x0[0] = dot3(t0, x0in); x0[1] = dot3(t1, x0in); x0[2] = dot3(t2, x0in);
}

static int sgn(double v) { return (0.0 < v) - (v < 0.0); }

/* Gauss points per side of the angular integral of the static part: 6 is the
 * reference's line rule of order 10 (nihu/library/laplace_nearly_singular_integrals.hpp:66).
 * Tests raise it to reproduce the reference's golden values, which were made
 * with a converged angular integral (see tests/test_oracle_golden.py). */
static int g_static_gauss = 10 / 2 + 1;

int oracle_set_static_gauss_points(int n)
{
    if (n < 1 || n > NIHU_GAUSS_MAX_N) return 0;
    g_static_gauss = n;
    return 1;
}

/* semi-analytic static part over a flat element seen from x0: radial integral
 * analytic, angular integral with 6-point Gauss per side.
 *   SLP: (1/4pi) sum_sides int (sqrt(R^2+z^2) - |z|) dtheta
 *   DLP: sgn(z)/(4pi) sum_sides int (1 - |z|/sqrt(R^2+z^2)) dtheta
 * (nihu/library/laplace_nearly_singular_integrals.hpp:62-136 and :139-209,
 *  geometry nihu/library/plane_element_helper.hpp:76-99) */
static double static_near(const elem_t *e, const double x0in[3], int op)
{
    double loc[4][3], x0[3];
    int N = e->nc;
    plane_local(e, x0in, loc, x0);
    double th_lim[4], th0[4], dref[4];
    for (int n = 0; n < N; ++n) {
        const double *c1 = loc[n], *c2 = loc[(n + 1) % N];
        double l[2] = {c2[0] - c1[0], c2[1] - c1[1]};
        double ln = sqrt(l[0] * l[0] + l[1] * l[1]);
        l[0] /= ln; l[1] /= ln;
        double d1[2] = {c1[0] - x0[0], c1[1] - x0[1]};
        double pr = d1[0] * l[0] + d1[1] * l[1];
        double d0[2] = {d1[0] - l[0] * pr, d1[1] - l[1] * pr};
        th_lim[n] = atan2(d1[1], d1[0]);
        th0[n] = atan2(d0[1], d0[0]);
        dref[n] = sqrt(d0[0] * d0[0] + d0[1] * d0[1]);
    }
    double z = x0[2] - loc[0][2];
    const double *g = gauss_rule(g_static_gauss);
    double res = 0.0;
    for (int i = 0; i < N; ++i) {
        double t1 = th_lim[i], t2 = th_lim[(i + 1) % N];
        if (fabs(t2 - t1) > PI) {
            if (t2 > t1) t1 += 2.0 * PI; else t2 += 2.0 * PI;
        }
        double jac = (t2 - t1) / 2.0;
        for (int q = 0; q < g_static_gauss; ++q) {
            double xi = g[2 * q], w = g[2 * q + 1];
            double th = t1 * (1.0 - xi) / 2.0 + t2 * (1.0 + xi) / 2.0;
            double R = dref[i] / cos(th - th0[i]);
            double r = sqrt(R * R + z * z);
            if (op == OP_SLP) res += (r - fabs(z)) * jac * w;
            else res += (1.0 - fabs(z) / r) * jac * w;
        }
    }
    if (op == OP_SLP) return res / (4.0 * PI);
    return sgn(z) * res / (4.0 * PI);
}

/* static parts of DLPt and HSP over a flat element seen from x0 with unit
 * normal nx (both expressed in the element's plane frame), per side
 *   DLPt: 6-point Gauss: -nx.r_vec/r + (nx_0 cos t + nx_1 sin t) ln(R + r) - nx_2 sgn(z)
 *   HSP: 21-point Gauss: -R^2/(r^2 z) (-r_vec.nx/r), or -nx_2/R when |z| <= 1e-12
 * with r_vec = (R cos t, R sin t, -z), all over 4 pi
 * (nihu/library/laplace_nearly_singular_integrals.hpp:212-298 and :301-380) */
static double static_near_bm(const elem_t *e, const double x0in[3], const double nxin[3], int op)
{
    double loc[4][3], x0[3], nx[3];
    int N = e->nc;
    plane_local(e, x0in, loc, x0);
    {
        /* the same rotation applied to the normal (plane_local does not translate) */
        double unused[4][3];
        plane_local(e, nxin, unused, nx);
    }
    double th_lim[4], th0[4], dref[4];
    for (int n = 0; n < N; ++n) {
        const double *c1 = loc[n], *c2 = loc[(n + 1) % N];
        double l[2] = {c2[0] - c1[0], c2[1] - c1[1]};
        double ln = sqrt(l[0] * l[0] + l[1] * l[1]);
        l[0] /= ln; l[1] /= ln;
        double d1[2] = {c1[0] - x0[0], c1[1] - x0[1]};
        double pr = d1[0] * l[0] + d1[1] * l[1];
        double d0[2] = {d1[0] - l[0] * pr, d1[1] - l[1] * pr};
        th_lim[n] = atan2(d1[1], d1[0]);
        th0[n] = atan2(d0[1], d0[0]);
        dref[n] = sqrt(d0[0] * d0[0] + d0[1] * d0[1]);
    }
    double z = x0[2] - loc[0][2];
    const int ng = op == OP_HSP ? 40 / 2 + 1 : g_static_gauss;
    const double *g = gauss_rule(ng);
    double res = 0.0;
    for (int i = 0; i < N; ++i) {
        double t1 = th_lim[i], t2 = th_lim[(i + 1) % N];
        if (fabs(t2 - t1) > PI) {
            if (t2 > t1) t1 += 2.0 * PI; else t2 += 2.0 * PI;
        }
        double jac = (t2 - t1) / 2.0;
        for (int q = 0; q < ng; ++q) {
            double xi = g[2 * q], w = g[2 * q + 1];
            double th = t1 * (1.0 - xi) / 2.0 + t2 * (1.0 + xi) / 2.0;
            double R = dref[i] / cos(th - th0[i]);
            double r = sqrt(R * R + z * z);
            double rv[3] = {R * cos(th), R * sin(th), -z};
            double f;
            if (op == OP_DLPT) {
                f = -dot3(nx, rv) / r + (nx[0] * cos(th) + nx[1] * sin(th)) * log(R + r) - nx[2] * sgn(z);
            } else {
                double rdnx = -dot3(rv, nx) / r;
                f = fabs(z) > 1e-12 ? -R * R / (r * r) / z * rdnx : -nx[2] / R;
            }
            res += f * jac * w;
        }
    }
    return res / (4.0 * PI);
}

/* constant flat element, nearly singular: static Laplace part semi-analytic,
 * dynamic part (K_k - K_0) with the degree-14 regular rule (Dunavant 42 points
 * on triangles, 8x8 Gauss on quads)
 * (nihu/library/helmholtz_nearly_singular_integrals.hpp:48-84 SLP, :91-129 DLP) */
static cplx near_plane(const elem_t *e, int fam, int op, cplx k, const double x0[3], const double *nx)
{
    double st = (op == OP_DLPT || op == OP_HSP) ? static_near_bm(e, x0, nx, op) : static_near(e, x0, op);
    if (fam == FAM_LAPLACE) return st;
    double en[3];
    {
        double xi, eta;
        domain_center(e->nc, &xi, &eta);
        elem_normal(e, xi, eta, en);
        double nn = norm3(en);
        for (int d = 0; d < 3; ++d) en[d] /= nn;
    }
    cplx dyn = 0.0;
    if (e->nc == 3) {
        const double *q = tri_data + 3 * tri_off[14];
        for (int p = 0; p < tri_npts[14]; ++p) {
            double y[3], n[3];
            elem_x(e, q[3 * p], q[3 * p + 1], y);
            elem_normal(e, q[3 * p], q[3 * p + 1], n);
            cplx kd = kern(FAM_HELMHOLTZ, op, k, x0, nx, y, en) - kern(FAM_LAPLACE, op, k, x0, nx, y, en);
            dyn += kd * q[3 * p + 2] * norm3(n);
        }
    } else {
        const double *g = gauss_rule(14 / 2 + 1);
        for (int a = 0; a < 8; ++a)
            for (int b = 0; b < 8; ++b) {
                double xi = g[2 * a], eta = g[2 * b], w = g[2 * a + 1] * g[2 * b + 1];
                double y[3], n[3];
                elem_x(e, xi, eta, y);
                elem_normal(e, xi, eta, n);
                cplx kd = kern(FAM_HELMHOLTZ, op, k, x0, nx, y, en) - kern(FAM_LAPLACE, op, k, x0, nx, y, en);
                dyn += kd * w * norm3(n);
            }
    }
    return st + dyn;
}

/* Newton iteration for the image (xi, eta) and the scaled normal offset zeta of
 * a point x0 near a surface element (nihu/core/inverse_mapping.hpp:52-112);
 * returns 1 on convergence */
static int inverse_mapping(const elem_t *e, const double x0[3], double tol, int max_iter, double res[3])
{
    res[0] = res[1] = res[2] = 0.0;
    for (int it = 0; it < max_iter; ++it) {
        double xi = res[0], eta = res[1], zeta = res[2];
        double y[3], dxi[3], deta[3], n[3];
        elem_x(e, xi, eta, y);
        elem_dx(e, xi, eta, dxi, deta);
        cross(dxi, deta, n);
        double sq = sqrt(norm3(n));
        for (int d = 0; d < 3; ++d) n[d] /= sq;
        double f[3];
        for (int d = 0; d < 3; ++d) f[d] = y[d] + n[d] * zeta - x0[d];
        if (norm3(f) < tol) return 1;
        /* second derivatives: only x_{xi eta} is nonzero for the bilinear quad */
        double dxx[3] = {0, 0, 0}, dxe[3] = {0, 0, 0}, dee[3] = {0, 0, 0};
        if (e->nc == 4)
            for (int d = 0; d < 3; ++d) dxe[d] = (e->c[0][d] - e->c[1][d] + e->c[2][d] - e->c[3][d]) / 4.0;
        double t1[3], t2[3], dnxi[3], dneta[3];
        cross(dxx, deta, t1); cross(dxi, dxe, t2);
        for (int d = 0; d < 3; ++d) dnxi[d] = (t1[d] + t2[d]) / sq;
        cross(dxe, deta, t1); cross(dxi, dee, t2);
        for (int d = 0; d < 3; ++d) dneta[d] = (t1[d] + t2[d]) / sq;
        double A[3][3];
        for (int d = 0; d < 3; ++d) {
            A[d][0] = dxi[d] + dnxi[d] * zeta;
            A[d][1] = deta[d] + dneta[d] * zeta;
            A[d][2] = n[d];
        }
        /* solve A s = f by Gaussian elimination with partial pivoting */
        double M[3][4];
        for (int r = 0; r < 3; ++r) { for (int c = 0; c < 3; ++c) M[r][c] = A[r][c]; M[r][3] = f[r]; }
        for (int c = 0; c < 3; ++c) {
            int p = c;
            for (int r = c + 1; r < 3; ++r) if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
            if (p != c) for (int q = 0; q < 4; ++q) { double t = M[c][q]; M[c][q] = M[p][q]; M[p][q] = t; }
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
    return 0;
}

/* linearized element around xi0: corners x(xi0) + dx(xi0)(xi_c - xi0)
 * (nihu/core/element.hpp:418-437) */
static void linearized_elem(const elem_t *e, double xi0, double eta0, elem_t *lin)
{
    double x0[3], dxi[3], deta[3], coords[12];
    elem_x(e, xi0, eta0, x0);
    elem_dx(e, xi0, eta0, dxi, deta);
    for (int a = 0; a < e->nc; ++a) {
        double ci, ce;
        domain_corner(e->nc, a, &ci, &ce);
        for (int d = 0; d < 3; ++d) coords[3 * a + d] = x0[d] + dxi[d] * (ci - xi0) + deta[d] * (ce - eta0);
    }
    elem_init(lin, e->nc, coords);
}

static cplx kern_on_elem(const elem_t *e, int fam, int op, cplx k, const double x0[3], double xi, double eta)
{
    double y[3], n[3];
    elem_x(e, xi, eta, y);
    elem_normal(e, xi, eta, n);
    double J = norm3(n);
    double un[3] = {n[0] / J, n[1] / J, n[2] / J};
    return kern(fam, op, k, x0, NULL, y, un) * J;
}

/* polar quadrature around the image of x0 in the reference domain with the
 * linearized-element integrand subtracted, plus the planar constant-element
 * shortcut on the linearized element; radial and tangential Gauss order 15
 * (8 points) (nihu/library/nearly_singular_collocational.hpp:87-198) */
static int near_polar(const elem_t *e, int fam, int op, cplx k, const double x0[3], cplx *out)
{
    double im[3];
    if (!inverse_mapping(e, x0, 1e-5, 100, im)) return 0;
    double xi0 = im[0], eta0 = im[1];
    elem_t lin;
    linearized_elem(e, xi0, eta0, &lin);
    int N = e->nc;
    double th_lim[4], th0[4], dref[4];
    for (int n = 0; n < N; ++n) {
        double c1[2], c2[2];
        domain_corner(N, n, &c1[0], &c1[1]);
        domain_corner(N, (n + 1) % N, &c2[0], &c2[1]);
        double l[2] = {1.0, 0.0};
        double dl[2] = {c2[0] - c1[0], c2[1] - c1[1]};
        double ln = sqrt(dl[0] * dl[0] + dl[1] * dl[1]);
        if (ln > 1e-3) { l[0] = dl[0] / ln; l[1] = dl[1] / ln; }
        double d1[2] = {c1[0] - xi0, c1[1] - eta0};
        double pr = d1[0] * l[0] + d1[1] * l[1];
        double d0[2] = {d1[0] - l[0] * pr, d1[1] - l[1] * pr};
        th_lim[n] = atan2(d1[1], d1[0]);
        th0[n] = atan2(d0[1], d0[0]);
        dref[n] = sqrt(d0[0] * d0[0] + d0[1] * d0[1]);
    }
    const double *g = gauss_rule(15 / 2 + 1);
    const int ng = 8;
    cplx I0 = 0.0;
    for (int n = 0; n < N; ++n) {
        double t1 = th_lim[n], t2 = th_lim[(n + 1) % N];
        if (fabs(t2 - t1) > PI) {
            if (t2 > t1) t1 += 2.0 * PI; else t2 += 2.0 * PI;
        }
        if (fabs(t2 - t1) < 1e-3) continue;
        for (int a = 0; a < ng; ++a) {
            double xx = g[2 * a];
            double th = ((1.0 - xx) * t1 + (1.0 + xx) * t2) / 2.0;
            double wth = g[2 * a + 1] * (t2 - t1) / 2.0;
            double rho_lim = dref[n] / cos(th - th0[n]);
            for (int b = 0; b < ng; ++b) {
                double rho = (1.0 + g[2 * b]) * rho_lim / 2.0;
                double wrho = g[2 * b + 1] * rho_lim / 2.0;
                double xi = xi0 + rho * cos(th), eta = eta0 + rho * sin(th);
                cplx F = kern_on_elem(e, fam, op, k, x0, xi, eta);
                cplx Fl = kern_on_elem(&lin, fam, op, k, x0, xi, eta);
                I0 += wth * wrho * rho * (F - Fl);
            }
        }
    }
    I0 += near_plane(&lin, fam, op, k, x0, NULL);
    *out = I0;
    return 1;
}

/* Telles (1987) cubic transformation of a tensor Gauss rule towards the image
 * of x0 (nihu/library/telles_1987.hpp:44-113), 16x16 points (order 30)
 * (nihu/library/nearly_singular_collocational_telles.hpp:85-110) */
static int near_telles(const elem_t *e, int fam, int op, cplx k, const double x0[3], cplx *out)
{
    double im[3];
    if (!inverse_mapping(e, x0, 1e-6, 100, im)) return 0;
    double dist = im[2];
    double rbar;
    if (dist < 0.05) rbar = 0.0;
    else if (dist <= 1.3) rbar = 0.85 + 0.24 * log(dist);
    else if (dist <= 3.618) rbar = 0.893 + 0.0832 * log(dist);
    else rbar = 1.0;
    double ca[2], cb[2], cc[2], cd[2];
    for (int dim = 0; dim < 2; ++dim) {
        double eb = im[dim];
        double f = 1.0 + 2.0 * rbar;
        double q = 1.0 / (2.0 * f) * ((eb * (3.0 - 2.0 * rbar) - 2.0 * eb * eb * eb / f) * 1.0 / f - eb);
        double p = 1.0 / (3.0 * f * f) * (4.0 * rbar * (1.0 - rbar) + 3.0 * (1.0 - eb * eb));
        double s = sqrt(q * q + p * p * p);
        double gb = cbrt(-q + s) + cbrt(-q - s) + eb / f;
        double Q = 1.0 + 3.0 * gb * gb;
        ca[dim] = (1.0 - rbar) / Q;
        cb[dim] = -3.0 * (1.0 - rbar) * gb / Q;
        cc[dim] = (3.0 * gb * gb + rbar) / Q;
        cd[dim] = -cb[dim];
    }
    const double *g = gauss_rule(30 / 2 + 1);
    const int ng = 16;
    cplx sum = 0.0;
    for (int a = 0; a < ng; ++a)
        for (int b = 0; b < ng; ++b) {
            double u[2] = {g[2 * a], g[2 * b]};
            double w = g[2 * a + 1] * g[2 * b + 1];
            double t[2];
            for (int dim = 0; dim < 2; ++dim) {
                double x = u[dim];
                t[dim] = ca[dim] * x * x * x + cb[dim] * x * x + cc[dim] * x + cd[dim];
                w *= 3.0 * ca[dim] * x * x + 2.0 * cb[dim] * x + cc[dim];
            }
            sum += kern_on_elem(e, fam, op, k, x0, t[0], t[1]) * w;
        }
    *out = sum;
    return 1;
}

/* nearly singular dispatch (nihu/library/helmholtz_nearly_singular_integrals.hpp:223-408,
 * nihu/library/laplace_nearly_singular_integrals.hpp:399-590): constant triangles
 * use the planar semi-analytic scheme; quads use polar subtraction, except
 * Helmholtz DLP which uses Telles */
static int near_integral(const elem_t *e, int fam, int op, cplx k, const double x0[3], const double *nx, cplx *out)
{
    if (e->nc == 3) { *out = near_plane(e, fam, op, k, x0, nx); return 1; }
    if (fam == FAM_HELMHOLTZ && op == OP_DLP) return near_telles(e, fam, op, k, x0, out);
    return near_polar(e, fam, op, k, x0, out);
}

/* ------------------------------------------------------------ meshes & API */

static char g_err[256];

static int load_elem(const double *nodes, int n_nodes, const int *elems, int cols, int i, elem_t *e)
{
    const int *row = elems + (long)i * cols;
    int nc;
    if (row[0] == TRIA_1_ID) nc = 3;
    else if (row[0] == QUAD_1_ID) nc = 4;
    else { snprintf(g_err, sizeof g_err, "unknown element type id %d", row[0]); return 0; }
    if (cols < 1 + nc) { snprintf(g_err, sizeof g_err, "element row too short"); return 0; }
    double coords[12];
    for (int a = 0; a < nc; ++a) {
        int nd = row[1 + a];
        if (nd < 0 || nd >= n_nodes) { snprintf(g_err, sizeof g_err, "node index out of range"); return 0; }
        for (int d = 0; d < 3; ++d) coords[3 * a + d] = nodes[3 * nd + d];
    }
    elem_init(e, nc, coords);
    return 1;
}

const char *oracle_last_error(void) { return g_err; }

/*
 * One entry: self -> nearly singular -> regular, exactly as
 * nihu/core/double_integral.hpp:543-673.  Returns 0 on error.
 */
static void unit_normal_center(const elem_t *e, double n[3])
{
    double xi, eta;
    domain_center(e->nc, &xi, &eta);
    elem_normal(e, xi, eta, n);
    double nn = norm3(n);
    for (int d = 0; d < 3; ++d) n[d] /= nn;
}

static int entry(const elem_t *te, const elem_t *re, int same_id, int fam, int op, cplx k, cplx *out)
{
    double nx[3];
    if (op == OP_DLPT || op == OP_HSP) {
        if (re->nc != 3) {
            snprintf(g_err, sizeof g_err, "DLPt / HSP: constant triangle trial elements only");
            return 0;
        }
        unit_normal_center(te, nx);
    }
    if (same_id && te->nc == re->nc) { *out = self_integral(re, fam, op, k); return 1; }
    double ratio = centre_distance(te, re) / re->size;
    if (ratio < 1.5) {
        if (!near_integral(re, fam, op, k, te->center, nx, out)) {
            snprintf(g_err, sizeof g_err, "Could not perform inverse mapping");
            return 0;
        }
        return 1;
    }
    int cmax = field_complexity(te->nc) > field_complexity(re->nc) ? field_complexity(te->nc) : field_complexity(re->nc);
    int degree = cmax + interval_degree(op, ratio);
    if (degree > 14) { snprintf(g_err, sizeof g_err, "Too high quadrature degree selected for collocational integration"); return 0; }
    if (re->nc == 3 && tri_npts[degree] == 0) { snprintf(g_err, sizeof g_err, "unsupported dunavant degree"); return 0; }
    *out = regular_integral(re, fam, op, k, te->center, nx, degree);
    return 1;
}

/*
 * Assemble the block rows [row_begin, row_end) x columns [col_begin, col_end)
 * of the operator (fam, op) between a test and a trial mesh into
 * out[(i - row_begin) + (j - col_begin)*ld] (column-major, complex128
 * as interleaved doubles).  out = alpha*op if accumulate == 0, else out +=
 * alpha*op (nihu/core/assembly.hpp:69-76 with block += semantics).
 * same_mesh enables the self terms (nihu/core/integral_transform.hpp:156).
 */
int oracle_assemble(const double *tnodes, int tn_nodes, const int *telems, int tn_elems, int tcols,
                    const double *rnodes, int rn_nodes, const int *relems, int rn_elems, int rcols,
                    int same_mesh, int fam, int op, double k_re, double k_im, double alpha_re, double alpha_im,
                    int row_begin, int row_end, int col_begin, int col_end, double *out, long ld, int accumulate)
{
    const cplx k = k_re + I * k_im;  /* complex for a lossy medium (nihu/library/helmholtz_kernel.hpp:42-54) */
    if (row_begin < 0 || row_end > tn_elems || row_begin > row_end) { snprintf(g_err, sizeof g_err, "bad row range"); return 0; }
    if (col_begin < 0 || col_end > rn_elems || col_begin > col_end) { snprintf(g_err, sizeof g_err, "bad column range"); return 0; }
    cplx alpha = alpha_re + I * alpha_im;
    /* element geometry is built once per mesh, like the reference's mesh
     * construction (nihu/core/mesh.hpp:137-160) */
    elem_t *trial = (elem_t *)malloc(sizeof(elem_t) * (size_t)(rn_elems > 0 ? rn_elems : 1));
    if (!trial) { snprintf(g_err, sizeof g_err, "out of host memory"); return 0; }
    int ok = 1;
    for (int j = 0; j < rn_elems && ok; ++j) ok = load_elem(rnodes, rn_nodes, relems, rcols, j, &trial[j]);
    for (int i = row_begin; i < row_end && ok; ++i) {
        elem_t te;
        if (!(ok = load_elem(tnodes, tn_nodes, telems, tcols, i, &te))) break;
        for (int j = col_begin; j < col_end; ++j) {
            cplx v;
            if (!(ok = entry(&te, &trial[j], same_mesh && i == j, fam, op, k, &v))) break;
            cplx *dst = (cplx *)out + (long)(i - row_begin) + (long)(j - col_begin) * ld;
            if (accumulate) *dst += alpha * v; else *dst = alpha * v;
        }
    }
    free(trial);
    return ok;
}

/*
 * Entries of an explicit pair list (test rows[p], trial cols[p]), p < n,
 * each with the full singular check, as NiHu's FMM near field evaluates them
 * (nihu/fmm/p2p_integral.hpp:87-99 over the index pairs of
 * nihu/fmm/p2p_precompute.hpp:110-180).  out[2p], out[2p+1] = (re, im).
 * Returns 0 on error.
 */
int oracle_assemble_pairs(const double *tnodes, int tn_nodes, const int *telems, int tn_elems, int tcols,
                          const double *rnodes, int rn_nodes, const int *relems, int rn_elems, int rcols,
                          int same_mesh, int fam, int op, double k_re, double k_im, long n, const int *rows,
                          const int *cols, double *out)
{
    const cplx k = k_re + I * k_im;
    for (long p = 0; p < n; ++p) {
        int i = rows[p], j = cols[p];
        if (i < 0 || i >= tn_elems || j < 0 || j >= rn_elems) {
            snprintf(g_err, sizeof g_err, "pair %ld: index out of range", p);
            return 0;
        }
        elem_t te, re;
        if (!load_elem(tnodes, tn_nodes, telems, tcols, i, &te)) return 0;
        if (!load_elem(rnodes, rn_nodes, relems, rcols, j, &re)) return 0;
        cplx v;
        if (!entry(&te, &re, same_mesh && i == j, fam, op, k, &v)) return 0;
        out[2 * p] = creal(v);
        out[2 * p + 1] = cimag(v);
    }
    return 1;
}

/* ------------------------------------------------------------ Galerkin */

/* Regular Galerkin double integral: the rule of the given degree on both
 * elements, every test point against every trial point, constant shape
 * functions (nihu/core/double_integral.hpp:175-202 with the diadic dual
 * accelerator of :300-312) */
static cplx galerkin_regular(const elem_t *te, const elem_t *re, int fam, int op, cplx k, int degree)
{
    double tx[64][3], tw[64], ty[64][3], tn[64][3], rw[64];
    int nt = 0, nr = 0;
    for (int side = 0; side < 2; ++side) {
        const elem_t *e = side == 0 ? te : re;
        int cnt = 0;
        double (*pts)[3] = side == 0 ? tx : ty;
        double *ws = side == 0 ? tw : rw;
        if (e->nc == 3) {
            const double *q = tri_data + 3 * tri_off[degree];
            for (int p = 0; p < tri_npts[degree]; ++p, ++cnt) {
                double n[3];
                elem_x(e, q[3 * p], q[3 * p + 1], pts[cnt]);
                elem_normal(e, q[3 * p], q[3 * p + 1], n);
                double J = norm3(n);
                ws[cnt] = q[3 * p + 2] * J;
                if (side == 1) for (int d = 0; d < 3; ++d) tn[cnt][d] = n[d] / J;
            }
        } else {
            int ng = degree / 2 + 1;
            const double *g = gauss_rule(ng);
            for (int a = 0; a < ng; ++a)
                for (int b = 0; b < ng; ++b, ++cnt) {
                    double n[3];
                    elem_x(e, g[2 * a], g[2 * b], pts[cnt]);
                    elem_normal(e, g[2 * a], g[2 * b], n);
                    double J = norm3(n);
                    ws[cnt] = g[2 * a + 1] * g[2 * b + 1] * J;
                    if (side == 1) for (int d = 0; d < 3; ++d) tn[cnt][d] = n[d] / J;
                }
        }
        if (side == 0) nt = cnt; else nr = cnt;
    }
    cplx sum = 0.0;
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < nr; ++b) sum += tw[a] * kern(fam, op, k, tx[a], NULL, ty[b], tn[b]) * rw[b];
    return sum;
}

/* Singular Galerkin quadrature on a pair of triangles with a common face
 * (match 2), edge (1) or corner (0): the 4D Gauss product on (0,1)^4 with
 * n = 7/2 + 1 = 4 points per direction (the kernels' singular quadrature
 * order 7, nihu/library/helmholtz_kernel.hpp:69-71), split into Duffy-type
 * subdomains in coordinate differences -- 3 (face, symmetric), 6 (edge), 1
 * (corner, symmetric) -- and mapped back to the reference triangle
 * (nihu/core/singular_galerkin_quadrature.hpp:200-420).  Points are stored as
 * (test xi, eta, trial xi, eta, w); a symmetric rule also holds the swapped
 * copy of every point. */
#define GAL_N 4
#define GAL_MAX (6 * GAL_N * GAL_N * GAL_N * GAL_N)
static int g_gal_count[3];
static double g_gal[3][GAL_MAX][5];

static void gal_map(int match, int sub, const double u[4], double *w, double out[4])
{
    double a1, a2, b1, b2, jac;  /* test point (a1, a2), difference (b1, b2) */
    if (match == 2) {
        if (sub == 0) {
            b1 = u[0]; b2 = u[0] * u[1];
            a1 = (1.0 - b1) * u[2]; a2 = a1 * u[3];
            jac = (1.0 - b1) * a1;
        } else if (sub == 1) {
            b1 = u[0] * u[1]; b2 = u[0] * (u[1] - 1.0);
            a1 = (1.0 - b1 + b2) * u[2] - b2; a2 = (a1 + b2) * u[3] - b2;
            jac = (1.0 - b1 + b2) * (a1 + b2);
        } else {
            b1 = u[0] * u[1]; b2 = u[0];
            a1 = (1.0 - b2) * u[2] + b2 - b1; a2 = (a1 - b2 + b1) * u[3];
            jac = (1.0 - b2) * (a1 - b2 + b1);
        }
        *w *= jac * u[0];
    } else if (match == 1) {
        const double p = u[0], q = u[1], r = u[2], s = u[3];
        switch (sub) {
        case 0: b1 = -p * q; b2 = -p * q * r; a1 = (1.0 - p) * s + p; a2 = p * (1.0 - q + q * r); break;
        case 1: b1 = p * q; b2 = p * q * r; a1 = (1.0 - p) * s + p * (1.0 - q); a2 = p * (1.0 - q); break;
        case 2: b1 = -p * q * r; b2 = p * q * (1.0 - r); a1 = (1.0 - p) * s + p; a2 = p * (1.0 - q); break;
        case 3: b1 = p * q * r; b2 = p * q * (r - 1.0); a1 = (1.0 - p) * s + p * (1.0 - q * r); a2 = p * (1.0 - q * r); break;
        case 4: b1 = -p * q * r; b2 = -p * q; a1 = (1.0 - p) * s + p; a2 = p; break;
        default: b1 = p * q * r; b2 = p * q; a1 = (1.0 - p) * s + p * (1.0 - q * r); a2 = p * (1.0 - q); break;
        }
        *w *= q * p * p * (1.0 - p);
    } else {
        a1 = u[0]; a2 = a1 * u[1];
        double e1 = a1 * u[2], e2 = e1 * u[3];
        *w *= u[2] * u[0] * u[0] * u[0];
        b1 = e1 - a1; b2 = e2 - a2;
    }
    /* (a1, a2) and (a1 + b1, a2 + b2) live on 0 <= x2 <= x1 <= 1: shift to the simplex */
    out[0] = a1 - a2; out[1] = a2;
    out[2] = (a1 + b1) - (a2 + b2); out[3] = a2 + b2;
}

static void gal_build(int match)
{
    const double *g = gauss_rule(GAL_N);
    double x[GAL_N], w[GAL_N];
    for (int i = 0; i < GAL_N; ++i) { x[i] = (1.0 + g[2 * i]) / 2.0; w[i] = g[2 * i + 1] / 2.0; }
    const int subs = match == 2 ? 3 : (match == 1 ? 6 : 1);
    const int sym = match != 1;
    int n = 0;
    for (int i1 = 0; i1 < GAL_N; ++i1)
        for (int i2 = 0; i2 < GAL_N; ++i2)
            for (int i3 = 0; i3 < GAL_N; ++i3)
                for (int i4 = 0; i4 < GAL_N; ++i4)
                    for (int sub = 0; sub < subs; ++sub) {
                        double u[4] = {x[i1], x[i2], x[i3], x[i4]}, ww = w[i1] * w[i2] * w[i3] * w[i4], o[4];
                        gal_map(match, sub, u, &ww, o);
                        double *d = g_gal[match][n++];
                        d[0] = o[0]; d[1] = o[1]; d[2] = o[2]; d[3] = o[3]; d[4] = ww;
                        if (sym) {
                            d = g_gal[match][n++];
                            d[0] = o[2]; d[1] = o[3]; d[2] = o[0]; d[3] = o[1]; d[4] = ww;
                        }
                    }
    g_gal_count[match] = n;
}

/* first common node of two triangles in each (cyclic order: the one the
 * common edge starts from), as nihu/core/element.hpp:376-413 */
static int common_nodes(const int *ta, int na, const int *tb, int nb, int *ind1, int *ind2)
{
    int num = 0, s1 = 0, s2 = 0;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            if (ta[i] != tb[j]) continue;
            if (num == 0) { s1 = i; s2 = j; }
            else {
                if (i < s1 || (i == na - 1 && s1 == 0 && num == 1)) s1 = i;
                if (j < s2 || (j == nb - 1 && s2 == 0 && num == 1)) s2 = j;
            }
            ++num;
        }
    *ind1 = s1; *ind2 = s2;
    return num;
}

/* reference-triangle point under a corner rotation: corner k of the rotated
 * triangle is corner perm[k] of the reference one */
static void tri_rotate(const int perm[3], double xi, double eta, double *oxi, double *oeta)
{
    static const double C[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
    double N[3] = {1.0 - xi - eta, xi, eta};
    *oxi = N[0] * C[perm[0]][0] + N[1] * C[perm[1]][0] + N[2] * C[perm[2]][0];
    *oeta = N[0] * C[perm[0]][1] + N[1] * C[perm[1]][1] + N[2] * C[perm[2]][1];
}

/* singular Galerkin integral of a matched triangle pair: the test rule is
 * rotated so that its first common node sits at corner 0, the trial rule so
 * that the common edge runs the opposite way (edge) or its common node sits
 * at corner 0 (corner) (nihu/core/singular_accelerator.hpp:270-310) */
static cplx galerkin_singular(const elem_t *te, const elem_t *re, int fam, int op, cplx k, int match, int ind1,
                              int ind2)
{
    if (!g_gal_count[match]) gal_build(match);
    int pt[3], pr[3];
    for (int q = 0; q < 3; ++q) {
        pt[q] = match == 2 ? q : (ind1 + q) % 3;
        pr[q] = match == 2 ? q : (match == 1 ? (ind2 + 1 + 3 - q) % 3 : (ind2 + q) % 3);
    }
    double nt[3], nr[3];
    elem_normal(te, 0.25, 0.25, nt);
    elem_normal(re, 0.25, 0.25, nr);
    const double Jt = norm3(nt), Jr = norm3(nr);
    double un[3] = {nr[0] / Jr, nr[1] / Jr, nr[2] / Jr};
    cplx sum = 0.0;
    for (int p = 0; p < g_gal_count[match]; ++p) {
        const double *d = g_gal[match][p];
        double a, b, x[3], y[3];
        tri_rotate(pt, d[0], d[1], &a, &b);
        elem_x(te, a, b, x);
        tri_rotate(pr, d[2], d[3], &a, &b);
        elem_x(re, a, b, y);
        sum += d[4] * Jt * kern(fam, op, k, x, NULL, y, un) * Jr;
    }
    return sum;
}

/* Singular Galerkin quadrature on a pair of quads (nihu/core/singular_galerkin_quadrature.hpp:430-600):
 * the coordinate difference mu = eta' - xi (eta' = the trial point after a
 * reflection that puts both elements side by side: none for a face match,
 * (eta_0, -2 - eta_1) for an edge, -2 - eta for a corner) is integrated over
 * Duffy quads (corners 0 and 1 at the singularity; 4 / 6 / 5 of them) with
 * the 4 x 4 Gauss rule, and for each mu the test point xi over the part of
 * [-1, 1]^2 that keeps the trial point inside its square, again 4 x 4 Gauss;
 * both maps bilinear with signed Jacobians (quadrature.hpp:112-127).  A face
 * match is symmetric (each point also with test and trial swapped). */
#define GALQ_MAX (4 * 16 * 16 * 2)
static int g_galq_count[3];
static double g_galq[3][GALQ_MAX][5];

static const double GALQ_FACE[4][4][2] = {{{0, 0}, {0, 0}, {2, -2}, {2, 0}}, {{0, 0}, {0, 0}, {2, 0}, {2, 2}},
                                          {{0, 0}, {0, 0}, {2, 2}, {0, 2}}, {{0, 0}, {0, 0}, {0, 2}, {-2, 2}}};
static const double GALQ_EDGE[6][4][2] = {{{0, 0}, {0, 0}, {-2, 0}, {-2, -2}}, {{0, 0}, {0, 0}, {-2, -2}, {0, -2}},
                                          {{0, 0}, {0, 0}, {0, -2}, {2, -2}},  {{0, 0}, {0, 0}, {2, -2}, {2, 0}},
                                          {{-2, -2}, {-2, -4}, {0, -4}, {0, -2}}, {{0, -2}, {0, -4}, {2, -4}, {2, -2}}};
static const double GALQ_CORNER[5][4][2] = {{{0, 0}, {0, 0}, {-2, 0}, {-2, -2}}, {{0, 0}, {0, 0}, {-2, -2}, {0, -2}},
                                            {{-4, 0}, {-4, -2}, {-2, -2}, {-2, 0}},
                                            {{-4, -2}, {-4, -4}, {-2, -4}, {-2, -2}},
                                            {{-2, -2}, {-2, -4}, {0, -4}, {0, -2}}};

/* bilinear map of (u, v) in [-1,1]^2 onto the quad with corners C: point and signed Jacobian */
static void quad_map(const double C[4][2], double u, double v, double *x, double *y, double *det)
{
    double N[4], dN[4][2];
    shape(4, u, v, N);
    dshape(4, u, v, dN);
    double a = 0, b = 0, j00 = 0, j01 = 0, j10 = 0, j11 = 0;
    for (int c = 0; c < 4; ++c) {
        a += N[c] * C[c][0]; b += N[c] * C[c][1];
        j00 += dN[c][0] * C[c][0]; j01 += dN[c][0] * C[c][1];
        j10 += dN[c][1] * C[c][0]; j11 += dN[c][1] * C[c][1];
    }
    *x = a; *y = b;
    *det = j00 * j11 - j01 * j10;
}

static void reflect(int match, double e0, double e1, double *o0, double *o1)
{
    if (match == 2) { *o0 = e0; *o1 = e1; }
    else if (match == 1) { *o0 = e0; *o1 = -2.0 - e1; }
    else { *o0 = -2.0 - e0; *o1 = -2.0 - e1; }
}

static void galq_build(int match)
{
    const double *g = gauss_rule(GAL_N);
    const int subs = match == 2 ? 4 : (match == 1 ? 6 : 5);
    const double (*tab)[4][2] = match == 2 ? GALQ_FACE : (match == 1 ? GALQ_EDGE : GALQ_CORNER);
    double lo[2], hi[2];
    reflect(match, -1.0, -1.0, &lo[0], &lo[1]);
    reflect(match, 1.0, 1.0, &hi[0], &hi[1]);
    for (int c = 0; c < 2; ++c)
        if (lo[c] > hi[c]) { double t = lo[c]; lo[c] = hi[c]; hi[c] = t; }
    int n = 0;
    for (int d = 0; d < subs; ++d)
        for (int a = 0; a < GAL_N; ++a)
            for (int b = 0; b < GAL_N; ++b) {
                double mu0, mu1, det;
                quad_map(tab[d], g[2 * a], g[2 * b], &mu0, &mu1, &det);
                const double wo = g[2 * a + 1] * g[2 * b + 1] * det;
                /* the test points that keep mu + xi in the reflected trial square */
                double R[4][2];
                double x0 = -mu0 + lo[0], x1 = -mu0 + hi[0], y0 = -mu1 + lo[1], y1 = -mu1 + hi[1];
                x0 = x0 < -1.0 ? -1.0 : (x0 > 1.0 ? 1.0 : x0);
                x1 = x1 < -1.0 ? -1.0 : (x1 > 1.0 ? 1.0 : x1);
                y0 = y0 < -1.0 ? -1.0 : (y0 > 1.0 ? 1.0 : y0);
                y1 = y1 < -1.0 ? -1.0 : (y1 > 1.0 ? 1.0 : y1);
                R[0][0] = x0; R[0][1] = y0; R[1][0] = x1; R[1][1] = y0;
                R[2][0] = x1; R[2][1] = y1; R[3][0] = x0; R[3][1] = y1;
                for (int c = 0; c < GAL_N; ++c)
                    for (int e = 0; e < GAL_N; ++e) {
                        double xi0, xi1, di;
                        quad_map(R, g[2 * c], g[2 * e], &xi0, &xi1, &di);
                        const double w = wo * g[2 * c + 1] * g[2 * e + 1] * di;
                        double et0, et1;
                        reflect(match, mu0 + xi0, mu1 + xi1, &et0, &et1);
                        double *q = g_galq[match][n++];
                        q[0] = xi0; q[1] = xi1; q[2] = et0; q[3] = et1; q[4] = w;
                        if (match == 2) {
                            q = g_galq[match][n++];
                            q[0] = et0; q[1] = et1; q[2] = xi0; q[3] = xi1; q[4] = w;
                        }
                    }
            }
    g_galq_count[match] = n;
}

/* quad point under a corner rotation: corner k of the rotated square is
 * corner perm[k] of (-1,-1), (1,-1), (1,1), (-1,1) */
static void quad_rotate(const int perm[4], double u, double v, double *ou, double *ov)
{
    static const double C[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    double N[4];
    shape(4, u, v, N);
    *ou = 0.0; *ov = 0.0;
    for (int k = 0; k < 4; ++k) { *ou += N[k] * C[perm[k]][0]; *ov += N[k] * C[perm[k]][1]; }
}

/* singular Galerkin integral of a matched quad pair (rotations as for
 * triangles: nihu/core/singular_accelerator.hpp:270-310) */
static cplx galerkin_singular_quad(const elem_t *te, const elem_t *re, int fam, int op, cplx k, int match, int ind1,
                                   int ind2)
{
    if (!g_galq_count[match]) galq_build(match);
    int pt[4], pr[4];
    for (int q = 0; q < 4; ++q) {
        pt[q] = match == 2 ? q : (ind1 + q) % 4;
        pr[q] = match == 2 ? q : (match == 1 ? (ind2 + 1 + 4 - q) % 4 : (ind2 + q) % 4);
    }
    cplx sum = 0.0;
    for (int p = 0; p < g_galq_count[match]; ++p) {
        const double *d = g_galq[match][p];
        double a, b, x[3], y[3], nt[3], nr[3];
        quad_rotate(pt, d[0], d[1], &a, &b);
        elem_x(te, a, b, x);
        elem_normal(te, a, b, nt);
        quad_rotate(pr, d[2], d[3], &a, &b);
        elem_x(re, a, b, y);
        elem_normal(re, a, b, nr);
        const double Jt = norm3(nt), Jr = norm3(nr);
        double un[3] = {nr[0] / Jr, nr[1] / Jr, nr[2] / Jr};
        sum += d[4] * Jt * kern(fam, op, k, x, NULL, y, un) * Jr;
    }
    return sum;
}

/* singular Galerkin integral of a matched triangle-quad pair (corner or
 * edge match; nihu/core/singular_galerkin_quadrature.hpp:624-790).  The
 * reference square of the quad is split into the triangles (0, 1, 2) and
 * (0, 2, 3) of its corners (-1,-1), (1,-1), (1,1), (-1,1); a corner match
 * takes the triangle-triangle corner rule on both, an edge match the edge
 * rule on (0, 1, 2) (which holds the common edge) and the corner rule on
 * (0, 2, 3).  The rule's triangle points go onto the sub-triangle by its
 * linear map (weights times its Jacobian, 4).  A triangle test element with
 * a quad trial element takes the same rule with test and trial swapped
 * (:767-790).  Rotations as for the other pairs
 * (nihu/core/singular_accelerator.hpp:290-320). */
static cplx galerkin_singular_mixed(const elem_t *te, const elem_t *re, int fam, int op, cplx k, int match,
                                    int ind1, int ind2)
{
    static const double Q[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    static const int SUB[2][3] = {{0, 1, 2}, {0, 2, 3}};
    if (!g_gal_count[0]) gal_build(0);
    if (!g_gal_count[1]) gal_build(1);
    const int nt = te->nc, nr = re->nc;
    int pt[4], pr[4];
    for (int q = 0; q < nt; ++q) pt[q] = (ind1 + q) % nt;
    for (int q = 0; q < nr; ++q) pr[q] = match == 1 ? (ind2 + 1 + nr - q) % nr : (ind2 + q) % nr;
    const int quad_is_test = nt == 4;
    cplx sum = 0.0;
    for (int sub = 0; sub < 2; ++sub) {
        const int m = (match == 1 && sub == 0) ? 1 : 0;  /* edge rule on (0, 1, 2) of an edge match */
        for (int p = 0; p < g_gal_count[m]; ++p) {
            const double *d = g_gal[m][p];
            /* the rule's first triangle goes onto the quad's sub-triangle */
            const double N[3] = {1.0 - d[0] - d[1], d[0], d[1]};
            double qu = 0.0, qv = 0.0;
            for (int c = 0; c < 3; ++c) { qu += N[c] * Q[SUB[sub][c]][0]; qv += N[c] * Q[SUB[sub][c]][1]; }
            double tu, tv, ru, rv;
            if (quad_is_test) {
                quad_rotate(pt, qu, qv, &tu, &tv);
                tri_rotate(pr, d[2], d[3], &ru, &rv);
            } else {
                tri_rotate(pt, d[2], d[3], &tu, &tv);
                quad_rotate(pr, qu, qv, &ru, &rv);
            }
            double x[3], y[3], ntv[3], nrv[3];
            elem_x(te, tu, tv, x);
            elem_normal(te, tu, tv, ntv);
            elem_x(re, ru, rv, y);
            elem_normal(re, ru, rv, nrv);
            const double Jt = norm3(ntv), Jr = norm3(nrv);
            double un[3] = {nrv[0] / Jr, nrv[1] / Jr, nrv[2] / Jr};
            sum += 4.0 * d[4] * Jt * kern(fam, op, k, x, NULL, y, un) * Jr;
        }
    }
    return sum;
}

/* the quad rule of a match type for tests: count, then points */
int oracle_galerkin_quad_rule(int match, double *out)
{
    if (match < 0 || match > 2) return 0;
    if (!g_galq_count[match]) galq_build(match);
    if (out)
        for (int p = 0; p < g_galq_count[match]; ++p)
            for (int c = 0; c < 5; ++c) out[5 * p + c] = g_galq[match][p][c];
    return g_galq_count[match];
}

/* One Galerkin entry (nihu/core/double_integral.hpp:318-384): face match for
 * the same element of one mesh, edge / corner match for triangles of one mesh
 * sharing 2 / 1 nodes, otherwise the regular rule of degree C + interval(d/D) */
static int galerkin_entry(const elem_t *te, const elem_t *re, const int *tn, const int *rn, int same_mesh, int same_id,
                          int fam, int op, cplx k, cplx *out)
{
    if (op != OP_SLP && op != OP_DLP) {
        snprintf(g_err, sizeof g_err, "Galerkin: SLP and DLP only");
        return 0;
    }
    int match = -1, ind1 = 0, ind2 = 0;
    if (same_mesh) {
        if (same_id) match = 2;
        else {
            int num = common_nodes(tn, te->nc, rn, re->nc, &ind1, &ind2);
            match = num > 1 ? 1 : (num == 1 ? 0 : -1);
        }
    }
    if (match >= 0) {
        if (te->nc != re->nc) *out = galerkin_singular_mixed(te, re, fam, op, k, match, ind1, ind2);
        else *out = te->nc == 3 ? galerkin_singular(te, re, fam, op, k, match, ind1, ind2)
                                : galerkin_singular_quad(te, re, fam, op, k, match, ind1, ind2);
        return 1;
    }
    double ratio = centre_distance(te, re) / re->size;
    int cmax = field_complexity(te->nc) > field_complexity(re->nc) ? field_complexity(te->nc) : field_complexity(re->nc);
    int degree = cmax + interval_degree(op, ratio);
    if (degree > 14 || (te->nc == 3 && tri_npts[degree] == 0)) {
        snprintf(g_err, sizeof g_err, "unsupported quadrature degree %d", degree);
        return 0;
    }
    *out = galerkin_regular(te, re, fam, op, k, degree);
    return 1;
}

/* Galerkin assembly of rows [row_begin, row_end) x columns [col_begin, col_end)
 * with the conventions of oracle_assemble (nihu/core/assembly.hpp:69-76) */
int oracle_assemble_galerkin(const double *tnodes, int tn_nodes, const int *telems, int tn_elems, int tcols,
                             const double *rnodes, int rn_nodes, const int *relems, int rn_elems, int rcols,
                             int same_mesh, int fam, int op, double k_re, double k_im, double alpha_re,
                             double alpha_im, int row_begin, int row_end, int col_begin, int col_end, double *out,
                             long ld, int accumulate)
{
    const cplx k = k_re + I * k_im;
    if (row_begin < 0 || row_end > tn_elems || row_begin > row_end) { snprintf(g_err, sizeof g_err, "bad row range"); return 0; }
    if (col_begin < 0 || col_end > rn_elems || col_begin > col_end) { snprintf(g_err, sizeof g_err, "bad column range"); return 0; }
    cplx alpha = alpha_re + I * alpha_im;
    for (int i = row_begin; i < row_end; ++i) {
        elem_t te;
        if (!load_elem(tnodes, tn_nodes, telems, tcols, i, &te)) return 0;
        const int *tn = telems + (long)i * tcols + 1;
        for (int j = col_begin; j < col_end; ++j) {
            elem_t re;
            if (!load_elem(rnodes, rn_nodes, relems, rcols, j, &re)) return 0;
            const int *rn = relems + (long)j * rcols + 1;
            cplx v;
            if (!galerkin_entry(&te, &re, tn, rn, same_mesh, same_mesh && i == j, fam, op, k, &v)) return 0;
            cplx *dst = (cplx *)out + (long)(i - row_begin) + (long)(j - col_begin) * ld;
            if (accumulate) *dst += alpha * v; else *dst = alpha * v;
        }
    }
    return 1;
}

/* the singular Galerkin rule of a match type for tests: count, then points
 * (test xi, eta, trial xi, eta, w) */
int oracle_galerkin_rule(int match, double *out)
{
    if (match < 0 || match > 2) return 0;
    if (!g_gal_count[match]) gal_build(match);
    if (out)
        for (int p = 0; p < g_gal_count[match]; ++p)
            for (int c = 0; c < 5; ++c) out[5 * p + c] = g_gal[match][p][c];
    return g_gal_count[match];
}

/* element geometry for tests: centre[3], size, normal at centre[3] (unnormalised) */
int oracle_elem_geometry(const double *coords, int nc, double *out7)
{
    elem_t e;
    elem_init(&e, nc, coords);
    double xi, eta, n[3];
    domain_center(nc, &xi, &eta);
    elem_normal(&e, xi, eta, n);
    out7[0] = e.center[0]; out7[1] = e.center[1]; out7[2] = e.center[2];
    out7[3] = e.size;
    out7[4] = n[0]; out7[5] = n[1]; out7[6] = n[2];
    return 1;
}

/* single element integrals for known-answer tests.  kind: 0 regular (given
 * degree), 1 nearly singular dispatch, 2 self, 3 planar near-singular scheme
 * (constant-plane formula even on quads). out = (re, im). */
int oracle_elem_integral_nx(const double *coords, int nc, const double *x0, const double *nx, int fam, int op,
                            double k_re, double k_im, int kind, int degree, double *out)
{
    const cplx k = k_re + I * k_im;
    elem_t e;
    elem_init(&e, nc, coords);
    cplx v = 0.0;
    if ((op == OP_DLPT || op == OP_HSP) && (!nx || nc != 3)) return 0;
    if (kind == 0) v = regular_integral(&e, fam, op, k, x0, nx, degree);
    else if (kind == 1) { if (!near_integral(&e, fam, op, k, x0, nx, &v)) return 0; }
    else if (kind == 2) v = self_integral(&e, fam, op, k);
    else if (kind == 3) v = near_plane(&e, fam, op, k, x0, nx);
    else return 0;
    out[0] = creal(v); out[1] = cimag(v);
    return 1;
}

/* the same for SLP and DLP (no normal at the collocation point) */
int oracle_elem_integral(const double *coords, int nc, const double *x0, int fam, int op, double k_re,
                         double k_im, int kind, int degree, double *out)
{
    if (op != OP_SLP && op != OP_DLP) return 0;
    return oracle_elem_integral_nx(coords, nc, x0, NULL, fam, op, k_re, k_im, kind, degree, out);
}

/* per-pair quadrature degree of one operator for tests: -1 self, -2 near */
int oracle_degree(const double *tnodes, int tn_nodes, const int *telems, int tn_elems, int tcols,
                  const double *rnodes, int rn_nodes, const int *relems, int rn_elems, int rcols,
                  int same_mesh, int op, int row_begin, int row_end, int *out)
{
    for (int i = row_begin; i < row_end; ++i) {
        elem_t te;
        if (!load_elem(tnodes, tn_nodes, telems, tcols, i, &te)) return 0;
        for (int j = 0; j < rn_elems; ++j) {
            elem_t re;
            if (!load_elem(rnodes, rn_nodes, relems, rcols, j, &re)) return 0;
            int code;
            if (same_mesh && i == j && te.nc == re.nc) code = -1;
            else {
                double ratio = centre_distance(&te, &re) / re.size;
                if (ratio < 1.5) code = -2;
                else {
                    int cmax = field_complexity(te.nc) > field_complexity(re.nc) ? field_complexity(te.nc) : field_complexity(re.nc);
                    code = cmax + interval_degree(op, ratio);
                }
            }
            out[(long)(i - row_begin) * rn_elems + j] = code;
        }
    }
    return 1;
}

/* per-pair classification for tests: level code per (i,j):
 * -1 self, -2 near, else degree(SLP)*16 + degree(DLP) */
int oracle_classify(const double *tnodes, int tn_nodes, const int *telems, int tn_elems, int tcols,
                    const double *rnodes, int rn_nodes, const int *relems, int rn_elems, int rcols,
                    int same_mesh, int row_begin, int row_end, int *out)
{
    for (int i = row_begin; i < row_end; ++i) {
        elem_t te;
        if (!load_elem(tnodes, tn_nodes, telems, tcols, i, &te)) return 0;
        for (int j = 0; j < rn_elems; ++j) {
            elem_t re;
            if (!load_elem(rnodes, rn_nodes, relems, rcols, j, &re)) return 0;
            int code;
            if (same_mesh && i == j && te.nc == re.nc) code = -1;
            else {
                double ratio = centre_distance(&te, &re) / re.size;
                if (ratio < 1.5) code = -2;
                else {
                    int cmax = field_complexity(te.nc) > field_complexity(re.nc) ? field_complexity(te.nc) : field_complexity(re.nc);
                    code = (cmax + interval_degree(OP_SLP, ratio)) * 16 + cmax + interval_degree(OP_DLP, ratio);
                }
            }
            out[(long)(i - row_begin) * rn_elems + j] = code;
        }
    }
    return 1;
}
