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
// Two kernels: k_pairs_regular (one thread per pair) classifies every pair in
// FP64 exactly as the reference, evaluates the regular ones (FP32 or FP64
// quadrature) and compacts the self and nearly singular ones into a list;
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

template <typename Out>
__device__ __forceinline__ void store_pair(Out *p, double vr, double vi)
{
    Out o;
    o.x = vr;
    o.y = vi;
    *p = o;
}

template <typename R, typename Out, int FAM>
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
        // the reference's FP64 decision (nihu/core/double_integral.hpp:543-639)
        const double ex = trial.center[3 * (int64_t)j] - test.center[3 * (int64_t)i];
        const double ey = trial.center[3 * (int64_t)j + 1] - test.center[3 * (int64_t)i + 1];
        const double ez = trial.center[3 * (int64_t)j + 2] - test.center[3 * (int64_t)i + 2];
        const int code = (a.same_mesh && i == j) ? -1 : bm_code64(sqrt(ex * ex + ey * ey + ez * ez) / trial.size[j]);
        if (code < 0) {
            const unsigned long long slot = atomicAdd(a.n_sing, 1ULL);
            a.sing[slot] = p;
            continue;
        }
        const int lh = code % 4, ls = code / 12, ld = (code / 4) % 3;
        const float4 ih = test.chi[i], il = test.clo[i];
        const float4 jh = trial.chi[j], jl = trial.clo[j];
        const int par = il.w != 0.0f ? 1 : 0;
        const int tnc = trial.nc[j];
        const bool S = (a.ops & OP_SLP) != 0, D = (a.ops & OP_DLP) != 0;
        const bool T = (a.ops & OP_DLPT) != 0, H = (a.ops & OP_HSP) != 0;
        R k, x0, x1, x2, nx0, nx1, nx2;
        if constexpr (sizeof(R) == 4) {
            k = a.k32;
            x0 = ih.x + il.x;
            x1 = ih.y + il.y;
            x2 = ih.z + il.z;
            const float4 q = test.p0[i];
            nx0 = q.y;
            nx1 = q.z;
            nx2 = q.w;
        } else {
            k = a.k;
            x0 = test.center[3 * (int64_t)i];
            x1 = test.center[3 * (int64_t)i + 1];
            x2 = test.center[3 * (int64_t)i + 2];
            const double *n = test.pts64 + 8 * ((int64_t)i * 2 * SLOTS) + 4;
            nx0 = n[0];
            nx1 = n[1];
            nx2 = n[2];
        }
        // hi/lo-accurate centre difference for the level-0 point
        const float dx = (jh.x - ih.x) + (jl.x - il.x);
        const float dy = (jh.y - ih.y) + (jl.y - il.y);
        const float dz = (jh.z - ih.z) + (jl.z - il.z);
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
                    const bool centre = slot == 0;
                    eval_bm<FAM, true, float>(centre ? dx : y.x - x0, centre ? dy : y.y - x1, centre ? dz : y.z - x2,
                                              y.w, n.x, n.y, n.z, nx0, nx1, nx2, k, ws, wd, wt, wh, o);
                } else {
                    const double *y = trial.pts64 + 8 * (base + slot);
                    eval_bm<FAM, true, double>(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6], nx0, nx1, nx2,
                                               k, ws, wd, wt, wh, o);
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
            for (int q = 0; q < np; ++q) {
                double xi, eta, w;
                tri_pt(par ? 7 : 6, q, xi, eta, w);
                double y[3];
                for (int d = 0; d < 3; ++d) y[d] = cc[d] + xi * e1[d] + eta * e2[d];
                if constexpr (sizeof(R) == 4) {
                    const double *cen = trial.center + 3 * (int64_t)j;
                    eval_h<FAM, float>(dx + (float)(y[0] - cen[0]), dy + (float)(y[1] - cen[1]),
                                       dz + (float)(y[2] - cen[2]), (float)(w * J), (float)n64[0], (float)n64[1],
                                       (float)n64[2], nx0, nx1, nx2, k, o);
                } else {
                    eval_h<FAM, double>(y[0] - x0, y[1] - x1, y[2] - x2, w * J, n64[0], n64[1], n64[2], nx0, nx1, nx2,
                                        k, o);
                }
            }
        }
        // out_a = c1 DLP + c3 HSP, out_b = c0 SLP + c2 DLPt (FP64 scaling of the sums)
        if (do_a) {
            const double vr = a.cre[1] * o.dr - a.cim[1] * o.di + a.cre[3] * o.hr - a.cim[3] * o.hi;
            const double vi = a.cre[1] * o.di + a.cim[1] * o.dr + a.cre[3] * o.hi + a.cim[3] * o.hr;
            store_pair(out_a + p, vr, vi);
        }
        if (do_b) {
            const double vr = a.cre[0] * o.sr - a.cim[0] * o.si + a.cre[2] * o.tr - a.cim[2] * o.ti;
            const double vi = a.cre[0] * o.si + a.cim[0] * o.sr + a.cre[2] * o.ti + a.cim[2] * o.tr;
            store_pair(out_b + p, vr, vi);
        }
    }
}

template <typename Out>
__global__ void __launch_bounds__(PAIR_SING_THREADS) k_pairs_singular(PairArgs a)
{
    const unsigned long long count = *a.n_sing;
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
        const int64_t p = a.sing[t];
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
            if (self) {
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
            if (self) {
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
                    near_polar_sum(e, lin, fam, k, x0, r5[0], r5[1], S, polar_d, q);
                    near_plane(lin, fam, k, x0, S, polar_d, q);
                }
                if (telles) near_telles_sum(e, fam, k, x0, r6, q);
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
    if (a.family == FAM_HELMHOLTZ) k_pairs_regular<R, Out, FAM_HELMHOLTZ><<<blocks, PAIR_THREADS, 0, s>>>(a);
    else k_pairs_regular<R, Out, FAM_LAPLACE><<<blocks, PAIR_THREADS, 0, s>>>(a);
}

cudaError_t launch_assemble_pairs(const PairArgs &a, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaMemsetAsync(a.n_sing, 0, sizeof(unsigned long long), s);
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
    if (a.dtype == 0) k_pairs_singular<float2><<<sblocks, PAIR_SING_THREADS, 0, s>>>(a);
    else k_pairs_singular<double2><<<sblocks, PAIR_SING_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace nihu
