// Burton-Miller operators: the transposed double layer (DLPt) and the
// hypersingular operator (HSP) of the Helmholtz and Laplace 3D kernels on
// constant triangle trial elements, alone or fused with SLP and DLP into the
// two Burton-Miller system matrices
//     A = DLP + c HSP,   B = SLP + c DLPt
// (nihu/applications/helmholtz/helmholtz_3d_coll.cpp:60-100; the identity
// terms are added by the caller).
//
// Kernels (r_vec = y - x, n_x the unit normal at the collocation point):
//   DLPt = dG/dr (-r_vec.n_x)/r                  (normal_derivative_kernel.hpp:199-206)
//   HSP  = f0 (-r_vec.n_x/r)(r_vec.n_y/r) - f1 n_x.n_y,
//          f1 = G'/r, f0 = G'' - G'/r            (normal_derivative_kernel.hpp:242-251,
//                                                 helmholtz_kernel.hpp:198-205)
// Regular pairs: the distance-adaptive Dunavant rule of each operator; HSP
// decays like 1/r^3 and so has a fourth level (degree 6, 12 points; 13 points
// of degree 7 when the test element is a quad), whose points are made from
// the trial corners (nihu/library/distance_kernel_intervals.hpp:143-154).
// Nearly singular pairs: semi-analytic static Laplace part over the flat
// element (DLPt 6 and HSP 21 Gauss points per side,
// nihu/library/laplace_nearly_singular_integrals.hpp:212-380) plus the
// dynamic part K_k - K_0 with the 42-point degree-14 rule
// (nihu/library/helmholtz_nearly_singular_integrals.hpp:131-220), summed in
// FP64, or in FP32 when the regular quadrature is FP32.
// Self terms: DLPt = 0 on a flat triangle; HSP from the finite-part integrals
// IddG0 and IG0 plus the 13-point dynamic remainder
// (nihu/library/helmholtz_singular_integrals.hpp:764-839,
//  normal_derivative_singular_integrals.hpp:13-56).
//
// Work layout as in assemble_regular.cu (one thread per test row, 32 trial
// columns per block, coalesced column-major stores) and assemble_singular.cu
// (one FP64 thread per nearly singular or self pair).
#include <algorithm>

#include "classify.cuh"
#include "kernels.h"
#include "planar.cuh"

namespace nihu {

constexpr int BM_THREADS = 256;
constexpr int BM_COLS = 32;
constexpr int BM_SING_THREADS = 128;

// squared distance ratios above which every operator of a pair uses the
// 1-point rule (SLP/DLP/DLPt: 15.8^2; with HSP: 22.3^2), with the FP32 margin
// of the plain regular kernel
constexpr float Q_FAR_BM2 = 249.64f * (1.0f + 1e-4f);
constexpr float Q_FAR_BM3 = 497.29f * (1.0f + 1e-4f);

template <typename R>
struct BmSum {
    R sr = 0, si = 0, dr = 0, di = 0, tr = 0, ti = 0, hr = 0, hi = 0;
};

// one quadrature point of all four kernels sharing r, 1/r and one sincos;
// ws / wd / wt / wh select the operators whose rule holds this point
template <int FAM, bool ALL4, typename R>
__device__ __forceinline__ void eval_bm(R rx, R ry, R rz, R wj, R ny0, R ny1, R ny2, R nx0, R nx1, R nx2, R k, R ws,
                                        R wd, R wt, R wh, BmSum<R> &o)
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
    if constexpr (FAM == FAM_HELMHOLTZ) {
        const R kr = k * (r2 * rinv);
        R s, c;
        if constexpr (sizeof(R) == 4) sincos_2pi(kr * 0.159154943091895335769f, s, c);
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
template <int FAM, typename R>
__device__ __forceinline__ void eval_h(R rx, R ry, R rz, R wj, R ny0, R ny1, R ny2, R nx0, R nx1, R nx2, R k,
                                       BmSum<R> &o)
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
    if constexpr (FAM == FAM_HELMHOLTZ) {
        const R kr = k * (r2 * rinv);
        R s, c;
        if constexpr (sizeof(R) == 4) sincos_2pi(kr * 0.159154943091895335769f, s, c);
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

// out = (c0 v0 + c1 v1) [+ out]
template <typename Out, typename R>
__device__ __forceinline__ void store_bm(Out *p, R r0, R i0, R c0r, R c0i, R r1, R i1, R c1r, R c1i, int accumulate)
{
    const R vr = c0r * r0 - c0i * i0 + c1r * r1 - c1i * i1;
    const R vi = c0r * i0 + c0i * r0 + c1r * i1 + c1i * r1;
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

// Work layout as the plain regular kernel: a thread owns a test row, a block
// 32 trial columns.  Three paths per (warp, column):
//   far    every lane d/D >= 22.3: all operators at the centroid
//   middle every lane d/D >= 15.8: SLP, DLP, DLPt at the centroid, HSP at the
//          centroid or (d/D < 22.3) its 3- or 4-point level
//   general the per-lane levels; a level that only HSP uses evaluates HSP alone
template <typename R, typename Out, int FAM, bool ALL4>
__global__ void __launch_bounds__(BM_THREADS, sizeof(R) == 4 ? 4 : 1) k_regular_bm(BmArgs a)
{
    __shared__ float4 s_hi[BM_COLS], s_lo[BM_COLS], s_p0[BM_COLS];
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    const int i = blockIdx.x * BM_THREADS + threadIdx.x;
    const int jb = a.j0 + blockIdx.y * BM_COLS;
    const int ncols = min(BM_COLS, a.j1 - jb);
    if (threadIdx.x < ncols) {
        s_hi[threadIdx.x] = trial.chi[jb + threadIdx.x];
        s_lo[threadIdx.x] = trial.clo[jb + threadIdx.x];
        s_p0[threadIdx.x] = trial.p0[jb + threadIdx.x];
    }
    __syncthreads();
    // whole warps beyond the last row leave; the lanes of a partial last warp
    // stay (clamped, writes masked) for the warp votes
    if ((i & ~31) >= test.n) return;
    const bool row_ok = i < test.n;
    const int ii = row_ok ? i : test.n - 1;
    const float4 ih = test.chi[ii], il = test.clo[ii];
    const int par = il.w != 0.0f ? 1 : 0;
    const bool do_t = ALL4 || (a.ops & OP_DLPT);
    const bool do_h = ALL4 || (a.ops & OP_HSP);
    const R wt_on = do_t ? R(1) : R(0);
    R k, x0, x1, x2, nx0, nx1, nx2, cr[4], ci[4];
    if constexpr (sizeof(R) == 4) {
        k = a.k32;
        x0 = ih.x + il.x;
        x1 = ih.y + il.y;
        x2 = ih.z + il.z;
        const float4 p = test.p0[ii];
        nx0 = p.y;
        nx1 = p.z;
        nx2 = p.w;
#pragma unroll
        for (int o = 0; o < 4; ++o) { cr[o] = a.cre32[o]; ci[o] = a.cim32[o]; }
    } else {
        k = a.k;
        x0 = test.center[3 * (int64_t)ii];
        x1 = test.center[3 * (int64_t)ii + 1];
        x2 = test.center[3 * (int64_t)ii + 2];
        const double *n = test.pts64 + 8 * ((int64_t)ii * 2 * SLOTS) + 4;  // level-0 point: the centre
        nx0 = n[0];
        nx1 = n[1];
        nx2 = n[2];
#pragma unroll
        for (int o = 0; o < 4; ++o) { cr[o] = a.cre[o]; ci[o] = a.cim[o]; }
    }
    const float q_far = do_h ? Q_FAR_BM3 : Q_FAR_BM2;
    Out *out_a = reinterpret_cast<Out *>(a.out_a);
    Out *out_b = reinterpret_cast<Out *>(a.out_b);

    for (int c = 0; c < ncols; ++c) {
        const int j = jb + c;
        const int64_t base = ((int64_t)j * 2 + par) * SLOTS;
        BmSum<R> o;
        bool done = false;
        // the points of regular level L < 3 of trial element j: f(y - x, w J, n_y)
        auto level_points = [&](int L, float dx, float dy, float dz, auto &&f) {
            const int np = level_npts(3, par, L);
            for (int q = 0; q < np; ++q) {
                const int slot = level_slot0(L) + q;
                if constexpr (sizeof(R) == 4) {
                    const float4 y = __ldg(trial.pts32 + 2 * (base + slot));
                    const float4 n = __ldg(trial.pts32 + 2 * (base + slot) + 1);
                    const bool centre = slot == 0;  // the accurate hi/lo centre difference
                    f(centre ? dx : y.x - x0, centre ? dy : y.y - x1, centre ? dz : y.z - x2, y.w, n.x, n.y, n.z);
                } else {
                    const double *y = trial.pts64 + 8 * (base + slot);
                    f(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6]);
                }
            }
        };
        if constexpr (sizeof(R) == 4) {
            const float4 h = s_hi[c];
            const float fx = h.x - x0, fy = h.y - x1, fz = h.z - x2;
            const float q = (fx * fx + fy * fy + fz * fz) * h.w;
            if (__all_sync(0xffffffffu, q > q_far)) {
                const float4 p = s_p0[c];
                eval_bm<FAM, ALL4, float>(fx, fy, fz, p.x, p.y, p.z, p.w, nx0, nx1, nx2, k, 1.0f, 1.0f, wt_on,
                                          do_h ? 1.0f : 0.0f, o);
                done = true;
            } else if (do_h && __all_sync(0xffffffffu, q > Q_FAR_BM2)) {
                int ls, ld, lh;
                float dx, dy, dz;
                classify_bm(ih, il, s_hi[c], s_lo[c], ii, j, test.center, trial.center, trial.size, a.same_mesh, ls,
                            ld, lh, dx, dy, dz);
                const float4 p = s_p0[c];
                eval_bm<FAM, ALL4, float>(fx, fy, fz, p.x, p.y, p.z, p.w, nx0, nx1, nx2, k, 1.0f, 1.0f, wt_on,
                                          lh == 0 ? 1.0f : 0.0f, o);
                if (lh == 1)
                    level_points(1, dx, dy, dz, [&](R rx, R ry, R rz, R wj, R n0, R n1, R n2) {
                        eval_h<FAM, R>(rx, ry, rz, wj, n0, n1, n2, nx0, nx1, nx2, k, o);
                    });
                done = true;
            }
        }
        if (!done) {
            int ls, ld, lh;
            float dx, dy, dz;
            const int kind = classify_bm(ih, il, s_hi[c], s_lo[c], ii, j, test.center, trial.center, trial.size,
                                         a.same_mesh, ls, ld, lh, dx, dy, dz);
            if (kind != KIND_REGULAR || !row_ok) continue;
            for (int L = 0; L < 3; ++L) {
                const bool bs = ALL4 && ls == L, bd = ALL4 && ld == L;
                const bool bt = do_t && ld == L, bh = do_h && lh == L;
                if (bs || bd || bt) {
                    const R ws = bs ? R(1) : R(0), wd = bd ? R(1) : R(0), wt = bt ? R(1) : R(0), wh = bh ? R(1) : R(0);
                    level_points(L, dx, dy, dz, [&](R rx, R ry, R rz, R wj, R n0, R n1, R n2) {
                        eval_bm<FAM, ALL4, R>(rx, ry, rz, wj, n0, n1, n2, nx0, nx1, nx2, k, ws, wd, wt, wh, o);
                    });
                } else if (bh) {
                    level_points(L, dx, dy, dz, [&](R rx, R ry, R rz, R wj, R n0, R n1, R n2) {
                        eval_h<FAM, R>(rx, ry, rz, wj, n0, n1, n2, nx0, nx1, nx2, k, o);
                    });
                }
            }
            if (do_h && lh == 3) {
                // HSP level 3 (only 1.5 <= d/D < 1.9): degree 6 (par 0) or 7 (par 1)
                // on the flat triangle y = c0 + xi e1 + eta e2
                const double *cc = trial.corners + 12 * (int64_t)j;
                const double *n64 = trial.pts64 + 8 * base + 4;
                double e1[3], e2[3], nt[3];
                for (int d = 0; d < 3; ++d) { e1[d] = cc[3 + d] - cc[d]; e2[d] = cc[6 + d] - cc[d]; }
                cross3(e1, e2, nt);
                const double J = norm3(nt);
                const int np = par ? 13 : 12;
                if constexpr (sizeof(R) == 4) {
                    // y - x = (c_j - x) + (y - c_j): the first part from the hi/lo
                    // centres, the second from the corners relative to the centre
                    const double *cen = trial.center + 3 * (int64_t)j;
                    float b[3], f1[3], f2[3];
                    for (int d = 0; d < 3; ++d) {
                        b[d] = (float)(cc[d] - cen[d]);
                        f1[d] = (float)e1[d];
                        f2[d] = (float)e2[d];
                    }
                    const float Jf = (float)J;
                    const float4 p = s_p0[c];
                    for (int q = 0; q < np; ++q) {
                        const float *t = par ? TRI67.p7[q] : TRI67.p6[q];
                        eval_h<FAM, float>(dx + (b[0] + t[0] * f1[0] + t[1] * f2[0]),
                                           dy + (b[1] + t[0] * f1[1] + t[1] * f2[1]),
                                           dz + (b[2] + t[0] * f1[2] + t[1] * f2[2]), t[2] * Jf, p.y, p.z, p.w, nx0,
                                           nx1, nx2, k, o);
                    }
                } else {
                    for (int q = 0; q < np; ++q) {
                        double xi, eta, w;
                        tri_pt(par ? 7 : 6, q, xi, eta, w);
                        double y[3];
                        for (int d = 0; d < 3; ++d) y[d] = cc[d] + xi * e1[d] + eta * e2[d];
                        eval_h<FAM, double>(y[0] - x0, y[1] - x1, y[2] - x2, w * J, n64[0], n64[1], n64[2], nx0,
                                            nx1, nx2, k, o);
                    }
                }
            }
        }
        if (!row_ok) continue;
        const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
        if constexpr (ALL4) {
            store_bm(out_a + off, o.dr, o.di, cr[1], ci[1], o.hr, o.hi, cr[3], ci[3], a.accumulate);
            store_bm(out_b + off, o.sr, o.si, cr[0], ci[0], o.tr, o.ti, cr[2], ci[2], a.accumulate);
        } else {
            if (do_h) store_bm(out_a + off, o.hr, o.hi, cr[3], ci[3], R(0), R(0), R(0), R(0), a.accumulate);
            if (do_t) store_bm(out_b + off, o.tr, o.ti, cr[2], ci[2], R(0), R(0), R(0), R(0), a.accumulate);
        }
    }
}

template <typename R, typename Out, int FAM>
static void launch_bm_ops(const BmArgs &a, dim3 grid, cudaStream_t s)
{
    if (a.ops == (OP_SLP | OP_DLP | OP_DLPT | OP_HSP)) k_regular_bm<R, Out, FAM, true><<<grid, BM_THREADS, 0, s>>>(a);
    else k_regular_bm<R, Out, FAM, false><<<grid, BM_THREADS, 0, s>>>(a);
}

template <typename R, typename Out>
static void launch_bm_fam(const BmArgs &a, dim3 grid, cudaStream_t s)
{
    if (a.family == FAM_HELMHOLTZ) launch_bm_ops<R, Out, FAM_HELMHOLTZ>(a, grid, s);
    else launch_bm_ops<R, Out, FAM_LAPLACE>(a, grid, s);
}

cudaError_t launch_assemble_regular_bm(const BmArgs &a, cudaStream_t s)
{
    const int ncols = a.j1 - a.j0;
    if (a.test.n == 0 || ncols <= 0) return cudaSuccess;
    dim3 grid((a.test.n + BM_THREADS - 1) / BM_THREADS, (ncols + BM_COLS - 1) / BM_COLS);
    if (a.precision == 0) {
        if (a.dtype == 0) launch_bm_fam<float, float2>(a, grid, s);
        else launch_bm_fam<float, double2>(a, grid, s);
    } else {
        if (a.dtype == 0) launch_bm_fam<double, float2>(a, grid, s);
        else launch_bm_fam<double, double2>(a, grid, s);
    }
    return cudaGetLastError();
}

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
__device__ void near_static4(const Elem64 &e, const double x0[3], const double nxg[3], OpSet ops, Acc4 &a)
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
__device__ void near_dynamic4(const Elem64 &e, double k, const double x0[3], const double nx[3], OpSet ops, Acc4 &a,
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

// The same dynamic parts in FP32 (regular quadrature in FP32): K_k - K_0 is
// smooth and, for a nearly singular pair, of relative size (kr)^2 against the
// FP64 static part, so FP32 point sums keep the entry within a few 1e-7 of
// the FP64 value while taking the narrow FP64 pipe out of 42 points per pair.
// The points are formed in FP32 relative to x0 from the corners.
__device__ void near_dynamic4_f32(const Elem64 &e, double k, const double x0[3], const double nx[3], OpSet ops,
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
__device__ void self_tria4(const Elem64 &e, int fam, double k, const double x0[3], OpSet ops, Acc4 &a)
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

// One FP64 thread per nearly singular or self pair, all operators of the
// launch from one plane frame, one set of side angles and one pass over the
// 42 dynamic points
template <typename Out>
__global__ void __launch_bounds__(BM_SING_THREADS) k_singular_bm(BmArgs a, NearList near)
{
    const int64_t p_begin = near.col_ptr ? near.col_ptr[a.j0] : 0;
    const int64_t p_end = near.col_ptr ? near.col_ptr[a.j1] : 0;
    const int64_t n_near = p_end - p_begin;
    const int64_t n_self = a.same_mesh ? (int64_t)(a.j1 - a.j0) : 0;
    const int64_t total = n_near + n_self;
    const bool all4 = a.ops == (OP_SLP | OP_DLP | OP_DLPT | OP_HSP);
    const OpSet ops{all4, all4, (a.ops & OP_DLPT) != 0, (a.ops & OP_HSP) != 0};
    const int fam = a.family;
    const double k = a.k;
    // nearly singular pairs have r < 1.5 D + (point to centre) <= 3 D_max
    const bool short_series = k * 3.0 * a.trial_size_max <= 0.75;
    Out *out_a = reinterpret_cast<Out *>(a.out_a);
    Out *out_b = reinterpret_cast<Out *>(a.out_b);
    for (int64_t item = (int64_t)blockIdx.x * BM_SING_THREADS + threadIdx.x; item < total;
         item += (int64_t)gridDim.x * BM_SING_THREADS) {
        int i, j;
        bool self;
        if (item < n_near) {
            const int64_t p = p_begin + item;
            i = near.rows[p];
            j = near_column(near.col_ptr, a.j0, a.j1, p);
            self = false;
        } else {
            j = a.j0 + (int)(item - n_near);
            i = j;
            self = true;
            if (i >= a.test.n) continue;
        }
        const double x0[3] = {a.test.center[3 * (int64_t)i], a.test.center[3 * (int64_t)i + 1],
                              a.test.center[3 * (int64_t)i + 2]};
        const double *np = a.test.pts64 + 8 * ((int64_t)i * 2 * SLOTS) + 4;  // unit normal at the centre
        const double nx[3] = {np[0], np[1], np[2]};
        Elem64 e;
        load_elem(a.trial, j, e);
        Acc4 acc;
        if (self) {
            self_tria4(e, fam, k, x0, ops, acc);
        } else {
            if (fam == FAM_HELMHOLTZ) {
                if (a.precision == 0) near_dynamic4_f32(e, k, x0, nx, ops, acc);
                else near_dynamic4(e, k, x0, nx, ops, acc, a.trial.dyn42 + 42 * (int64_t)j, short_series);
            }
            near_static4(e, x0, nx, ops, acc);
        }
        const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
        if (ops.d || ops.h)
            store2(out_a + off, ops.d, acc.dr, acc.di, a.cre[1], a.cim[1], ops.h, acc.hr, acc.hi, a.cre[3], a.cim[3],
                   a.accumulate);
        if (ops.s || ops.t)
            store2(out_b + off, ops.s, acc.sr, acc.si, a.cre[0], a.cim[0], ops.t, acc.tr, acc.ti, a.cre[2], a.cim[2],
                   a.accumulate);
    }
}

cudaError_t launch_assemble_singular_bm(const BmArgs &a, const NearList &near, cudaStream_t s)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t total = (near.col_ptr ? near.nnz : 0) + (a.same_mesh ? (a.j1 - a.j0) : 0);
    if (total == 0) return cudaSuccess;
    // at most two 4-warp blocks per SM (the FP64 pipe is the limit)
    const int64_t want = (total + BM_SING_THREADS - 1) / BM_SING_THREADS;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, 2 * (int64_t)sms));
    if (a.dtype == 0) k_singular_bm<float2><<<blocks, BM_SING_THREADS, 0, s>>>(a, near);
    else k_singular_bm<double2><<<blocks, BM_SING_THREADS, 0, s>>>(a, near);
    return cudaGetLastError();
}

}  // namespace nihu
