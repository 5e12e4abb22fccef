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
#include "singular_schemes.cuh"

namespace nihu {

constexpr int SING_THREADS = 128;
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

// self term of a constant triangle, complex (lossy) wave number: the static
// part as self_tria, the dynamic part in the complex sinc form
// (tria_self_slp_dynamic_ck)
__device__ void self_tria_ck(const Elem64 &e, int fam, cd k, const double x0[3], Acc &a)
{
    const double st = self_static(e, x0);
    cd dyn{0.0, 0.0};
    if (fam == FAM_HELMHOLTZ) dyn = tria_self_slp_dynamic_ck(e, k, x0);
    a.sr += (st + dyn.re) * INV_FOUR_PI;
    a.si += dyn.im * INV_FOUR_PI;
}

// one nearly singular or self pair with a complex (lossy) wave number: the
// FP64 schemes with the complex kernel, in both precision modes
__device__ bool pair_ck(const RegularArgs &a, const Elem64 &e, const double x0[3], bool self, int j, bool do_s,
                        bool do_d, Acc &acc)
{
    const int fam = a.family;
    const cd kc{a.k, a.k_im};
    if (self) {
        if (e.nc == 3) {
            if (do_s) self_tria_ck(e, fam, kc, x0, acc);
        } else {
            self_quad(e, fam, kc, x0, do_s, do_d, acc);
        }
        return true;
    }
    if (e.nc == 3) {
        if (fam == FAM_HELMHOLTZ) near_dynamic_ck(e, kc, x0, do_s, do_d, acc, a.trial.dyn42 + 42 * (int64_t)j);
        near_static(e, x0, do_s, do_d, acc);
        return true;
    }
    const bool telles = fam == FAM_HELMHOLTZ && do_d;
    const bool polar_d = fam == FAM_LAPLACE && do_d;
    double r5[3] = {0, 0, 0}, r6[3] = {0, 0, 0};
    if (!inverse_mapping(e, x0, telles, r5, r6)) return false;
    if (do_s || polar_d) {
        Elem64 lin;
        linearized(e, r5[0], r5[1], lin);
        near_polar_sum(e, lin, fam, kc, x0, r5[0], r5[1], do_s, polar_d, acc);
        if (fam == FAM_HELMHOLTZ) near_dynamic_ck(lin, kc, x0, do_s, polar_d, acc, nullptr);
        near_static(lin, x0, do_s, polar_d, acc);
    }
    if (telles) near_telles_sum(e, fam, kc, x0, r6, acc);
    return true;
}

// ------------------------------------------------------------------ driver

// the SLP entry of item `item` of wave number f: into the matrix, or in
// right-hand-side mode into near_slp (the regular kernel sums the rest)
template <typename Out>
__device__ __forceinline__ void store_slp(const RegularArgs &a, int f, int64_t items, int64_t item, int64_t off,
                                          const Acc &acc)
{
    if (a.near_slp)
        a.near_slp[(int64_t)f * items + item] =
            make_double2(a.alpha_re * acc.sr - a.alpha_im * acc.si, a.alpha_re * acc.si + a.alpha_im * acc.sr);
    else
        store64(batch_matrix<Out>(a, false, f) + off, acc.sr, acc.si, a.alpha_re, a.alpha_im, a.accumulate);
}

// BATCH: frequency batch (a.nk > 1), a separate kernel so that the single
// wave number kernel carries none of its code.
template <typename Out, bool BATCH, bool CK = false>
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
        if constexpr (CK) {
            // complex (lossy) wave number: single wave number only
            Acc acc;
            if (!pair_ck(a, e, x0, self, j, do_s, do_d, acc)) {
                atomicCAS(err, 0, (int)min(item + 1, (int64_t)0x7fffffff));
                break;
            }
            if (do_s) store_slp<Out>(a, 0, total, item, off, acc);
            if (do_d) store64(batch_matrix<Out>(a, true, 0) + off, acc.dr, acc.di, a.alpha_re, a.alpha_im, a.accumulate);
            continue;
        }
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
                if (do_s) store_slp<Out>(a, f, total, item, off, acc);
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
                if (a.precision == 0) {
                    // FP32 regular quadrature: the dynamic part and the static
                    // part's angular point sums in FP32 as well
                    if (fam == FAM_HELMHOLTZ) near_dynamic_f32(e, kf, x0, do_s, do_d, acc);
                    near_static_f32(e, a.trial.frame + 16 * (int64_t)j, x0, do_s, do_d, acc);
                } else {
                    near_plane(e, fam, kf, x0, do_s, do_d, acc, a.trial.dyn42 + 42 * (int64_t)j, short_f);
                }
            } else {
                const bool telles = fam == FAM_HELMHOLTZ && do_d;
                const bool polar_d = fam == FAM_LAPLACE && do_d;
                double r5[3] = {0, 0, 0}, r6[3] = {0, 0, 0};
                ok = inverse_mapping(e, x0, telles, r5, r6);
                if (ok) {
                    if (do_s || polar_d) {
                        Elem64 lin;
                        linearized(e, r5[0], r5[1], lin);
                        if (a.precision == 0) {
                            // FP32 regular quadrature: the schemes' sums in FP32 as well
                            near_polar_sum_f32(e, fam, kf, x0, r5[0], r5[1], do_s, polar_d, acc);
                            if (fam == FAM_HELMHOLTZ) near_dynamic_quad_f32(lin, kf, x0, do_s, polar_d, acc);
                            near_static(lin, x0, do_s, polar_d, acc);
                        } else {
                            near_polar_sum(e, lin, fam, kf, x0, r5[0], r5[1], do_s, polar_d, acc);
                            near_plane(lin, fam, kf, x0, do_s, polar_d, acc);
                        }
                    }
                    if (telles) {
                        if (a.precision == 0) near_telles_sum_f32(e, fam, kf, x0, r6, acc);
                        else near_telles_sum(e, fam, kf, x0, r6, acc);
                    }
                }
            }
            if (!ok) {
                atomicCAS(err, 0, (int)min(item + 1, (int64_t)0x7fffffff));
                break;
            }
            if (do_s) store_slp<Out>(a, f, total, item, off, acc);
            if (do_d) store64(batch_matrix<Out>(a, true, f) + off, acc.dr, acc.di, a.alpha_re, a.alpha_im, a.accumulate);
        }
    }
}

// held to 128 registers so that three blocks of the concurrent regular kernel
// keep every SM beside this kernel's one (it would take 164 by itself, with
// the FP32 dynamic part beside the FP64 schemes, which left room for two)
template <typename Out>
__global__ void __launch_bounds__(SING_THREADS, 4) k_singular(RegularArgs a, NearList near, int *err)
{
    singular_pairs<Out, false>(a, near, err);
}

// complex (lossy) wave number: its own kernel, so the real-k kernel carries none of it
template <typename Out>
__global__ void __launch_bounds__(SING_THREADS, 4) k_singular_ck(RegularArgs a, NearList near, int *err)
{
    singular_pairs<Out, false, true>(a, near, err);
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
    // the whole carveout as shared memory on the SMs this kernel starts on, so
    // that the concurrent regular kernel's blocks (with their shared row sums
    // in right-hand-side mode) still fit beside its block
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_singular_batch<float2>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_singular_batch<double2>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    return e;
}

cudaError_t launch_assemble_singular(const RegularArgs &a, const NearList &near, int *err, cudaStream_t s)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // this kernel needs no shared memory, but the regular kernel's blocks
    // beside it do: the same carveout preference as theirs, so that an SM
    // this kernel starts on is configured for both (set once per device)
    static bool carveout_set[64] = {};
    if (dev >= 0 && dev < 64 && !carveout_set[dev]) {
        cudaError_t e = cudaSuccess;
        const int pct = regular_carveout_percent();
        for (const void *f : {(const void *)k_singular<float2>, (const void *)k_singular<double2>,
                              (const void *)k_singular_ck<float2>, (const void *)k_singular_ck<double2>})
            if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
        if (e != cudaSuccess) return e;
        carveout_set[dev] = true;
    }
    // one 4-warp block per SM keeps the narrow FP64 pipe busy (a warp-wide
    // FP64 instruction occupies it for many cycles) and leave most of every SM
    // to the concurrently running regular kernel
    int64_t total = (near.col_ptr ? near.nnz : 0) + (a.same_mesh ? (a.j1 - a.j0) : 0);
    int64_t want = (total + SING_THREADS - 1) / SING_THREADS;
    // quads: the pairs' FP32 sums need more warps than the FP64 pipe does;
    // up to four blocks per SM once the regular kernel's blocks drain
    const int per_sm = (a.trial.has_quad && a.precision == 0 && a.nk <= 1 && !a.force_batch) ? 4 : 1;
    int blocks = (int)max((int64_t)1, min(want, (int64_t)sms * per_sm));
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
    } else if (a.k_im != 0.0) {
        if (a.dtype == 0) k_singular_ck<float2><<<blocks, SING_THREADS, 0, s>>>(a, near, err);
        else k_singular_ck<double2><<<blocks, SING_THREADS, 0, s>>>(a, near, err);
    } else {
        if (a.dtype == 0) k_singular<float2><<<blocks, SING_THREADS, 0, s>>>(a, near, err);
        else k_singular<double2><<<blocks, SING_THREADS, 0, s>>>(a, near, err);
    }
    return cudaGetLastError();
}

}  // namespace nihu
