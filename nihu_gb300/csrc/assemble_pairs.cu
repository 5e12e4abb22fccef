// Pair-list assembly: the entries of an explicit list of (test i, trial j)
// element pairs, each with the full singular check (self -> nearly singular
// -> regular), for sparse near-field matrices.
//
// Restates the FMM near-field (P2P) evaluation of NiHu:
// nihu/fmm/p2p_integral.hpp:87-99 evaluates double_integral::eval(kernel,
// test element, trial element, singular check) per pair, and
// nihu/fmm/p2p_precompute.hpp:110-180 runs it over the index pairs of the P2P
// interaction list into sparse-matrix triplets; the Burton-Miller FMM solver
// combines the operators as DLP + alpha HSP - I/2 and SLP + alpha DLPt +
// alpha/2 I (nihu/fmm/helmholtz_burton_miller_solver.hpp:170-190).
//
// Two kernels: k_pairs_regular (one thread per pair) classifies every pair
// with the reference's decision (FP32 hi/lo centres, FP64 near a threshold),
// evaluates the regular ones (FP32 or FP64 quadrature) and compacts the
// nearly singular ones (from the front) and the self ones (from the back) of
// a list;
// k_pairs_singular (one FP64 thread per listed pair) evaluates those with the
// schemes of the dense kernels.  Entries go to out_a[p] / out_b[p], p the
// pair's position in the list.
#include <algorithm>

#include "bm_schemes.cuh"
#include "classify.cuh"
#include "kernels.h"
#include "singular_schemes.cuh"

namespace nihu {

constexpr int PAIR_THREADS = 256;
constexpr int PAIR_SING_THREADS = 128;

__device__ __forceinline__ bool pair_valid(const PairArgs &a, int i, int j)
{
    return i >= 0 && i < a.test.n && j >= 0 && j < a.trial.n;
}

template <typename Out, typename V>
__device__ __forceinline__ void store_pair(Out *p, V vr, V vi)
{
    Out o;
    o.x = vr;
    o.y = vi;
    *p = o;
}

// CK: a complex (lossy) wave number (the point kernels' complex form)
template <typename R, typename Out, int FAM, bool CK = false>
__global__ void __launch_bounds__(PAIR_THREADS) k_pairs_regular(PairArgs a)
{
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    const bool do_a = (a.ops & (OP_DLP | OP_HSP)) != 0, do_b = (a.ops & (OP_SLP | OP_DLPT)) != 0;
    Out *out_a = reinterpret_cast<Out *>(a.out_a);
    Out *out_b = reinterpret_cast<Out *>(a.out_b);
    for (int64_t p = (int64_t)blockIdx.x * PAIR_THREADS + threadIdx.x; p < a.n;
         p += (int64_t)gridDim.x * PAIR_THREADS) {
        const int i = a.rows[p], j = a.cols[p];
        if (!pair_valid(a, i, j)) {
            atomicCAS(a.bad, 0, (int)min(p + 1, (int64_t)0x7fffffff));
            continue;
        }
        // the reference's decision (nihu/core/double_integral.hpp:543-639):
        // FP32 from the hi/lo centres, FP64 within 1e-5 of a threshold
        const float4 ih = test.chi[i], il = test.clo[i];
        const float4 jh = trial.chi[j], jl = trial.clo[j];
        int ls, ld, lh;
        float dx, dy, dz;
        const int kind = classify_bm(ih, il, jh, jl, i, j, test.center, trial.center, trial.size, a.same_mesh, ls,
                                     ld, lh, dx, dy, dz);
        if (kind != KIND_REGULAR) {
            // nearly singular pairs from the front, self pairs from the back,
            // so that the FP64 kernel's warps run one scheme
            if (kind == KIND_SELF) a.sing[a.n - 1 - (int64_t)atomicAdd(a.n_sing + 1, 1ULL)] = p;
            else a.sing[atomicAdd(a.n_sing, 1ULL)] = p;
            continue;
        }
        const int par = il.w != 0.0f ? 1 : 0;
        const int tnc = trial.nc[j];
        const bool S = (a.ops & OP_SLP) != 0, D = (a.ops & OP_DLP) != 0;
        const bool T = (a.ops & OP_DLPT) != 0, H = (a.ops & OP_HSP) != 0;
        R k, ki, x0, x1, x2, nx0, nx1, nx2, cr[4], ci[4];
        if constexpr (sizeof(R) == 4) {
            k = a.k32;
            ki = a.k_im32;
            x0 = ih.x + il.x;
            x1 = ih.y + il.y;
            x2 = ih.z + il.z;
            const float4 q = test.p0[i];
            nx0 = q.y;
            nx1 = q.z;
            nx2 = q.w;
#pragma unroll
            for (int o = 0; o < 4; ++o) { cr[o] = a.cre32[o]; ci[o] = a.cim32[o]; }
        } else {
            k = a.k;
            ki = a.k_im;
            x0 = test.center[3 * (int64_t)i];
            x1 = test.center[3 * (int64_t)i + 1];
            x2 = test.center[3 * (int64_t)i + 2];
            const double *n = test.pts64 + 8 * ((int64_t)i * 2 * SLOTS) + 4;
            nx0 = n[0];
            nx1 = n[1];
            nx2 = n[2];
#pragma unroll
            for (int o = 0; o < 4; ++o) { cr[o] = a.cre[o]; ci[o] = a.cim[o]; }
        }
        const int64_t base = ((int64_t)j * 2 + par) * SLOTS;
        BmSum<R> o;
        for (int L = 0; L < 3; ++L) {
            const bool bs = S && ls == L, bd = D && ld == L, bt = T && ld == L, bh = H && lh == L;
            if (!(bs || bd || bt || bh)) continue;
            const R ws = bs ? R(1) : R(0), wd = bd ? R(1) : R(0), wt = bt ? R(1) : R(0), wh = bh ? R(1) : R(0);
            const int np = level_npts(tnc, par, L);
            for (int q = 0; q < np; ++q) {
                const int slot = level_slot0(L) + q;
                if constexpr (sizeof(R) == 4) {
                    const float4 y = __ldg(trial.pts32 + 2 * (base + slot));
                    const float4 n = __ldg(trial.pts32 + 2 * (base + slot) + 1);
                    eval_bm<FAM, true, float, CK>(dx + y.x, dy + y.y, dz + y.z, y.w, n.x, n.y, n.z, nx0, nx1, nx2, k,
                                              ws, wd, wt, wh, o, ki);
                } else {
                    const double *y = trial.pts64 + 8 * (base + slot);
                    eval_bm<FAM, true, double, CK>(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6], nx0, nx1, nx2,
                                               k, ws, wd, wt, wh, o, ki);
                }
            }
        }
        if (H && lh == 3) {
            // HSP level 3 on a triangle: degree 6 (par 0) or 7 (par 1) from the corners
            const double *cc = trial.corners + 12 * (int64_t)j;
            const double *n64 = trial.pts64 + 8 * base + 4;
            double e1[3], e2[3], nt[3];
            for (int d = 0; d < 3; ++d) { e1[d] = cc[3 + d] - cc[d]; e2[d] = cc[6 + d] - cc[d]; }
            cross3(e1, e2, nt);
            const double J = norm3(nt);
            const int np = par ? 13 : 12;
            if constexpr (sizeof(R) == 4) {
                // y - x = (c_j - x) + (y - c_j) as in the dense kernel
                const double *cen = trial.center + 3 * (int64_t)j;
                float b[3], f1[3], f2[3];
                for (int d = 0; d < 3; ++d) {
                    b[d] = (float)(cc[d] - cen[d]);
                    f1[d] = (float)e1[d];
                    f2[d] = (float)e2[d];
                }
                const float Jf = (float)J;
                const float4 pj = trial.p0[j];
                for (int q = 0; q < np; ++q) {
                    const float *t = par ? TRI67.p7[q] : TRI67.p6[q];
                    eval_h<FAM, float, CK>(dx + (b[0] + t[0] * f1[0] + t[1] * f2[0]),
                                       dy + (b[1] + t[0] * f1[1] + t[1] * f2[1]),
                                       dz + (b[2] + t[0] * f1[2] + t[1] * f2[2]), t[2] * Jf, pj.y, pj.z, pj.w, nx0,
                                       nx1, nx2, k, o, ki);
                }
            } else {
                for (int q = 0; q < np; ++q) {
                    double xi, eta, w;
                    tri_pt(par ? 7 : 6, q, xi, eta, w);
                    double y[3];
                    for (int d = 0; d < 3; ++d) y[d] = cc[d] + xi * e1[d] + eta * e2[d];
                    eval_h<FAM, double, CK>(y[0] - x0, y[1] - x1, y[2] - x2, w * J, n64[0], n64[1], n64[2], nx0, nx1,
                                        nx2, k, o, ki);
                }
            }
        }
        // out_a = c1 DLP + c3 HSP, out_b = c0 SLP + c2 DLPt
        if (do_a) {
            const R vr = cr[1] * o.dr - ci[1] * o.di + cr[3] * o.hr - ci[3] * o.hi;
            const R vi = cr[1] * o.di + ci[1] * o.dr + cr[3] * o.hi + ci[3] * o.hr;
            store_pair(out_a + p, vr, vi);
        }
        if (do_b) {
            const R vr = cr[0] * o.sr - ci[0] * o.si + cr[2] * o.tr - ci[2] * o.ti;
            const R vi = cr[0] * o.si + ci[0] * o.sr + cr[2] * o.ti + ci[2] * o.tr;
            store_pair(out_b + p, vr, vi);
        }
    }
}

// CK: a complex (lossy) wave number, the FP64 complex schemes in both modes
template <typename Out, bool CK>
__global__ void __launch_bounds__(PAIR_SING_THREADS) k_pairs_singular(PairArgs a)
{
    const unsigned long long n_near = a.n_sing[0], count = n_near + a.n_sing[1];
    const bool S = (a.ops & OP_SLP) != 0, D = (a.ops & OP_DLP) != 0;
    const bool T = (a.ops & OP_DLPT) != 0, H = (a.ops & OP_HSP) != 0;
    const bool bm_ops = T || H;
    const bool do_a = D || H, do_b = S || T;
    const int fam = a.family;
    const double k = a.k;
    const bool short_series = k * 3.0 * a.trial_size_max <= 0.75;
    Out *out_a = reinterpret_cast<Out *>(a.out_a);
    Out *out_b = reinterpret_cast<Out *>(a.out_b);
    for (unsigned long long t = (unsigned long long)blockIdx.x * PAIR_SING_THREADS + threadIdx.x; t < count;
         t += (unsigned long long)gridDim.x * PAIR_SING_THREADS) {
        const int64_t p = t < n_near ? a.sing[t] : a.sing[a.n - 1 - (int64_t)(t - n_near)];
        const int i = a.rows[p], j = a.cols[p];
        const bool self = a.same_mesh && i == j;
        const double x0[3] = {a.test.center[3 * (int64_t)i], a.test.center[3 * (int64_t)i + 1],
                              a.test.center[3 * (int64_t)i + 2]};
        Elem64 e;
        load_elem(a.trial, j, e);
        Acc4 acc;
        if (e.nc == 3) {
            const double *np = a.test.pts64 + 8 * ((int64_t)i * 2 * SLOTS) + 4;
            const double nx[3] = {np[0], np[1], np[2]};
            const OpSet ops{S, D, T, H};
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
                    // as the dense kernels: FP32 dynamic part only for the
                    // Burton-Miller operators under FP32 regular quadrature
                    if (bm_ops && a.precision == 0) near_dynamic4_f32(e, k, x0, nx, ops, acc);
                    else near_dynamic4(e, k, x0, nx, ops, acc, a.trial.dyn42 + 42 * (int64_t)j, short_series);
                }
                near_static4(e, x0, nx, ops, acc);
            }
        } else {
            // quads (SLP and DLP only): Duffy self term, inverse mapping with
            // polar quadrature (Telles for the Helmholtz DLP) when nearly singular
            Acc q;
            if constexpr (CK) {
                // complex (lossy) wave number: the FP64 schemes with the complex kernel
                const cd kc{k, a.k_im};
                if (self) {
                    self_quad(e, fam, kc, x0, S, D, q);
                } else {
                    const bool telles = fam == FAM_HELMHOLTZ && D;
                    const bool polar_d = fam == FAM_LAPLACE && D;
                    double r5[3] = {0, 0, 0}, r6[3] = {0, 0, 0};
                    if (!inverse_mapping(e, x0, telles, r5, r6)) {
                        atomicCAS(a.err, 0, (int)min(p + 1, (int64_t)0x7fffffff));
                        continue;
                    }
                    if (S || polar_d) {
                        Elem64 lin;
                        linearized(e, r5[0], r5[1], lin);
                        near_polar_sum(e, lin, fam, kc, x0, r5[0], r5[1], S, polar_d, q);
                        if (fam == FAM_HELMHOLTZ) near_dynamic_ck(lin, kc, x0, S, polar_d, q, nullptr);
                        near_static(lin, x0, S, polar_d, q);
                    }
                    if (telles) near_telles_sum(e, fam, kc, x0, r6, q);
                }
            } else if (self) {
                self_quad(e, fam, k, x0, S, D, q);
            } else {
                const bool telles = fam == FAM_HELMHOLTZ && D;
                const bool polar_d = fam == FAM_LAPLACE && D;
                double r5[3] = {0, 0, 0}, r6[3] = {0, 0, 0};
                if (!inverse_mapping(e, x0, telles, r5, r6)) {
                    atomicCAS(a.err, 0, (int)min(p + 1, (int64_t)0x7fffffff));
                    continue;
                }
                if (S || polar_d) {
                    Elem64 lin;
                    linearized(e, r5[0], r5[1], lin);
                    if (a.precision == 0) {
                        // FP32 regular quadrature: the schemes' sums in FP32 as well
                        near_polar_sum_f32(e, fam, k, x0, r5[0], r5[1], S, polar_d, q);
                        if (fam == FAM_HELMHOLTZ) near_dynamic_quad_f32(lin, k, x0, S, polar_d, q);
                        near_static(lin, x0, S, polar_d, q);
                    } else {
                        near_polar_sum(e, lin, fam, k, x0, r5[0], r5[1], S, polar_d, q);
                        near_plane(lin, fam, k, x0, S, polar_d, q);
                    }
                }
                if (telles) {
                    if (a.precision == 0) near_telles_sum_f32(e, fam, k, x0, r6, q);
                    else near_telles_sum(e, fam, k, x0, r6, q);
                }
            }
            acc.sr = q.sr;
            acc.si = q.si;
            acc.dr = q.dr;
            acc.di = q.di;
        }
        if (do_a) {
            double vr = a.cre[1] * acc.dr - a.cim[1] * acc.di + a.cre[3] * acc.hr - a.cim[3] * acc.hi;
            double vi = a.cre[1] * acc.di + a.cim[1] * acc.dr + a.cre[3] * acc.hi + a.cim[3] * acc.hr;
            if (self) { vr += a.id_re[0]; vi += a.id_im[0]; }
            store_pair(out_a + p, vr, vi);
        }
        if (do_b) {
            double vr = a.cre[0] * acc.sr - a.cim[0] * acc.si + a.cre[2] * acc.tr - a.cim[2] * acc.ti;
            double vi = a.cre[0] * acc.si + a.cim[0] * acc.sr + a.cre[2] * acc.ti + a.cim[2] * acc.tr;
            if (self) { vr += a.id_re[1]; vi += a.id_im[1]; }
            store_pair(out_b + p, vr, vi);
        }
    }
}

template <typename R, typename Out>
static void launch_pairs_fam(const PairArgs &a, int blocks, cudaStream_t s)
{
    if (a.family == FAM_HELMHOLTZ) {
        if (a.k_im != 0.0) k_pairs_regular<R, Out, FAM_HELMHOLTZ, true><<<blocks, PAIR_THREADS, 0, s>>>(a);
        else k_pairs_regular<R, Out, FAM_HELMHOLTZ><<<blocks, PAIR_THREADS, 0, s>>>(a);
    } else {
        k_pairs_regular<R, Out, FAM_LAPLACE><<<blocks, PAIR_THREADS, 0, s>>>(a);
    }
}

cudaError_t launch_assemble_pairs(const PairArgs &a, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaMemsetAsync(a.n_sing, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const int64_t want = (a.n + PAIR_THREADS - 1) / PAIR_THREADS;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, 8 * (int64_t)sms));
    if (a.precision == 0) {
        if (a.dtype == 0) launch_pairs_fam<float, float2>(a, blocks, s);
        else launch_pairs_fam<float, double2>(a, blocks, s);
    } else {
        if (a.dtype == 0) launch_pairs_fam<double, float2>(a, blocks, s);
        else launch_pairs_fam<double, double2>(a, blocks, s);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // the singular list's length stays on the device: the kernel reads it
    const int64_t swant = (a.n + PAIR_SING_THREADS - 1) / PAIR_SING_THREADS;
    const int sblocks = (int)std::max<int64_t>(1, std::min<int64_t>(swant, 2 * (int64_t)sms));
    const bool ck = a.family == FAM_HELMHOLTZ && a.k_im != 0.0;
    if (ck) {
        if (a.dtype == 0) k_pairs_singular<float2, true><<<sblocks, PAIR_SING_THREADS, 0, s>>>(a);
        else k_pairs_singular<double2, true><<<sblocks, PAIR_SING_THREADS, 0, s>>>(a);
    } else {
        if (a.dtype == 0) k_pairs_singular<float2, false><<<sblocks, PAIR_SING_THREADS, 0, s>>>(a);
        else k_pairs_singular<double2, false><<<sblocks, PAIR_SING_THREADS, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace nihu
