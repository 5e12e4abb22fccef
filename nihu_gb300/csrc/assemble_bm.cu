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

#include "bm_schemes.cuh"
#include "classify.cuh"
#include "kernels.h"

namespace nihu {

constexpr int BM_THREADS = 256;
constexpr int BM_COLS = 32;
constexpr int BM_SING_THREADS = 128;

// squared distance ratios above which every operator of a pair uses the
// 1-point rule (SLP/DLP/DLPt: 15.8^2; with HSP: 22.3^2), with the FP32 margin
// of the plain regular kernel
constexpr float Q_FAR_BM2 = 249.64f * (1.0f + 1e-4f);
constexpr float Q_FAR_BM3 = 497.29f * (1.0f + 1e-4f);

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
template <typename R, typename Out, int FAM, bool ALL4, bool CK = false>
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
    R k, ki, x0, x1, x2, nx0, nx1, nx2, cr[4], ci[4];
    if constexpr (sizeof(R) == 4) {
        k = a.k32;
        ki = a.k_im32;
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
        ki = a.k_im;
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
                    // the hi/lo centre difference plus the point's offset from the centre
                    f(dx + y.x, dy + y.y, dz + y.z, y.w, n.x, n.y, n.z);
                } else {
                    const double *y = trial.pts64 + 8 * (base + slot);
                    f(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6]);
                }
            }
        };
        if constexpr (sizeof(R) == 4) {
            const float4 h = s_hi[c], l = s_lo[c];  // hi/lo centre difference (as k_regular)
            const float fx = (h.x - ih.x) + (l.x - il.x), fy = (h.y - ih.y) + (l.y - il.y),
                        fz = (h.z - ih.z) + (l.z - il.z);
            const float q = (fx * fx + fy * fy + fz * fz) * h.w;
            if (__all_sync(0xffffffffu, q > q_far)) {
                const float4 p = s_p0[c];
                eval_bm<FAM, ALL4, float, CK>(fx, fy, fz, p.x, p.y, p.z, p.w, nx0, nx1, nx2, k, 1.0f, 1.0f, wt_on,
                                          do_h ? 1.0f : 0.0f, o, ki);
                done = true;
            } else if (do_h && __all_sync(0xffffffffu, q > Q_FAR_BM2)) {
                int ls, ld, lh;
                float dx, dy, dz;
                classify_bm(ih, il, s_hi[c], s_lo[c], ii, j, test.center, trial.center, trial.size, a.same_mesh, ls,
                            ld, lh, dx, dy, dz);
                const float4 p = s_p0[c];
                eval_bm<FAM, ALL4, float, CK>(fx, fy, fz, p.x, p.y, p.z, p.w, nx0, nx1, nx2, k, 1.0f, 1.0f, wt_on,
                                          lh == 0 ? 1.0f : 0.0f, o, ki);
                if (lh == 1)
                    level_points(1, dx, dy, dz, [&](R rx, R ry, R rz, R wj, R n0, R n1, R n2) {
                        eval_h<FAM, R, CK>(rx, ry, rz, wj, n0, n1, n2, nx0, nx1, nx2, k, o, ki);
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
                        eval_bm<FAM, ALL4, R, CK>(rx, ry, rz, wj, n0, n1, n2, nx0, nx1, nx2, k, ws, wd, wt, wh, o, ki);
                    });
                } else if (bh) {
                    level_points(L, dx, dy, dz, [&](R rx, R ry, R rz, R wj, R n0, R n1, R n2) {
                        eval_h<FAM, R, CK>(rx, ry, rz, wj, n0, n1, n2, nx0, nx1, nx2, k, o, ki);
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
                        eval_h<FAM, float, CK>(dx + (b[0] + t[0] * f1[0] + t[1] * f2[0]),
                                           dy + (b[1] + t[0] * f1[1] + t[1] * f2[1]),
                                           dz + (b[2] + t[0] * f1[2] + t[1] * f2[2]), t[2] * Jf, p.y, p.z, p.w, nx0,
                                           nx1, nx2, k, o, ki);
                    }
                } else {
                    for (int q = 0; q < np; ++q) {
                        double xi, eta, w;
                        tri_pt(par ? 7 : 6, q, xi, eta, w);
                        double y[3];
                        for (int d = 0; d < 3; ++d) y[d] = cc[d] + xi * e1[d] + eta * e2[d];
                        eval_h<FAM, double, CK>(y[0] - x0, y[1] - x1, y[2] - x2, w * J, n64[0], n64[1], n64[2], nx0,
                                            nx1, nx2, k, o, ki);
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
    const bool all4 = a.ops == (OP_SLP | OP_DLP | OP_DLPT | OP_HSP);
    if constexpr (FAM == FAM_HELMHOLTZ) {
        if (a.k_im != 0.0) {  // complex (lossy) wave number: separate instantiations
            if (all4) k_regular_bm<R, Out, FAM, true, true><<<grid, BM_THREADS, 0, s>>>(a);
            else k_regular_bm<R, Out, FAM, false, true><<<grid, BM_THREADS, 0, s>>>(a);
            return;
        }
    }
    if (all4) k_regular_bm<R, Out, FAM, true><<<grid, BM_THREADS, 0, s>>>(a);
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

// One FP64 thread per nearly singular or self pair, all operators of the
// launch from one plane frame, one set of side angles and one pass over the
// 42 dynamic points
// CK: a complex (lossy) wave number, the FP64 complex schemes in both modes
template <typename Out, bool CK>
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
        if constexpr (CK) {
            const cd kc{k, a.k_im};
            if (self) {
                self_tria4_ck(e, fam, kc, x0, ops, acc);
            } else {
                near_dynamic4_ck(e, kc, x0, nx, ops, acc, a.trial.dyn42 + 42 * (int64_t)j);
                near_static4(e, x0, nx, ops, acc);
            }
        } else if (self) {
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
    const bool ck = a.family == FAM_HELMHOLTZ && a.k_im != 0.0;
    if (ck) {
        if (a.dtype == 0) k_singular_bm<float2, true><<<blocks, BM_SING_THREADS, 0, s>>>(a, near);
        else k_singular_bm<double2, true><<<blocks, BM_SING_THREADS, 0, s>>>(a, near);
    } else {
        if (a.dtype == 0) k_singular_bm<float2, false><<<blocks, BM_SING_THREADS, 0, s>>>(a, near);
        else k_singular_bm<double2, false><<<blocks, BM_SING_THREADS, 0, s>>>(a, near);
    }
    return cudaGetLastError();
}

}  // namespace nihu
