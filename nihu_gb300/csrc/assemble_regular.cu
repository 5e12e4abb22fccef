// Regular (far-field) collocational entries: fused SLP + DLP over all
// (test, trial) element pairs, in FP32 (default) or FP64.
//
// Restates nihu/core/double_integral.hpp:445-467 (sum_q w_q K(x_i, y_q) J_q
// with the accelerator of the selected degree, :557-585) for the Helmholtz and
// Laplace 3D SLP/DLP kernels (nihu/library/helmholtz_kernel.hpp:180-195,
// laplace_kernel.hpp:137-147, normal_derivative_kernel.hpp:131-175).
//
// Work layout: a block owns REG_THREADS consecutive test rows and REG_COLS
// consecutive trial columns.  A thread owns one row; for each column it
// classifies the pair (classify.cuh), evaluates the selected rule(s) and
// writes the entry.  Writes of a warp are 32 consecutive entries of one
// column of the column-major matrix (256 B for complex64), so the dominant
// cost -- storing 2 x 8 bytes per pair -- streams at full HBM width.
// Self and nearly singular pairs are skipped (assemble_singular.cu writes
// them), so every entry is written exactly once.
#include <algorithm>

#include "classify.cuh"
#include "kernels.h"

namespace nihu {

constexpr int REG_THREADS = 256;
constexpr int REG_COLS = 32;

// k-independent part of one quadrature point (frequency batches): the
// distance and the SLP and DLP factors of eval_point
template <typename R>
struct PointGeom {
    R r, gs, fd;
};

template <typename R>
__device__ __forceinline__ PointGeom<R> point_geom(R rx, R ry, R rz, R wj, R nx, R ny, R nz, R ws, R wd)
{
    constexpr R INV4PI = R(1.0 / (4.0 * 3.14159265358979323846));
    R r2 = rx * rx + ry * ry + rz * rz;
    R rinv;
    if constexpr (sizeof(R) == 4) rinv = rsqrtf(r2);
    else rinv = rsqrt(r2);
    R g = wj * rinv * INV4PI;
    R rdn = (rx * nx + ry * ny + rz * nz) * rinv;
    return {r2 * rinv, g * ws, -g * rinv * rdn * wd};
}

// the k-dependent part: the same sums as eval_point
template <int FAM, typename R>
__device__ __forceinline__ void point_freq(const PointGeom<R> &p, R k, R &sr, R &si, R &dr, R &di)
{
    if constexpr (FAM == FAM_HELMHOLTZ) {
        R kr = k * p.r;
        R s, c;
        if constexpr (sizeof(R) == 4) sincos_2pi(kr * 0.159154943091895335769f, s, c);
        else sincos(kr, &s, &c);
        sr += p.gs * c;
        si -= p.gs * s;
        dr += p.fd * (c + kr * s);
        di += p.fd * (kr * c - s);
    } else {
        sr += p.gs;
        dr += p.fd;
    }
}

// wave numbers evaluated together per pass over a pair's points
constexpr int FREQ_TILE = 4;

template <typename Out, typename R>
__device__ __forceinline__ void store_entry(Out *p, R re, R im, R are, R aim, bool unit_alpha, int accumulate)
{
    R vr = re, vi = im;
    if (!unit_alpha) {
        vr = are * re - aim * im;
        vi = are * im + aim * re;
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

// Squared distance ratio above which a pair is certainly regular with the
// 1-point rule for both SLP (x >= 9.1) and DLP (x >= 15.8): 15.8^2 with a
// relative margin far larger than the FP32 error of the plain centre
// difference of a far pair.
constexpr float Q_FAR = 249.64f * (1.0f + 1e-4f);

// BATCH: frequency batch (a.nk > 1), a separate instantiation so that the
// single wave number kernel carries none of its code
template <typename R, typename Out, int FAM, int OPS, bool BATCH>
__global__ void __launch_bounds__(REG_THREADS) k_regular(RegularArgs a)
{
    __shared__ float4 s_hi[REG_COLS], s_lo[REG_COLS], s_p0[REG_COLS];
    __shared__ int s_nc[REG_COLS];
    constexpr bool DO_S = (OPS & OP_SLP) != 0;
    constexpr bool DO_D = (OPS & OP_DLP) != 0;
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    const int i = blockIdx.x * REG_THREADS + threadIdx.x;
    const int jb = a.j0 + blockIdx.y * REG_COLS;
    const int ncols = min(REG_COLS, a.j1 - jb);
    if (threadIdx.x < ncols) {
        s_hi[threadIdx.x] = trial.chi[jb + threadIdx.x];
        s_lo[threadIdx.x] = trial.clo[jb + threadIdx.x];
        s_nc[threadIdx.x] = trial.nc[jb + threadIdx.x];
        s_p0[threadIdx.x] = trial.p0[jb + threadIdx.x];
    }
    __syncthreads();
    // whole warps beyond the last row leave; a partial last warp keeps its
    // out-of-range lanes (clamped to the last row, writes masked) so that
    // warp votes see every lane
    if ((i & ~31) >= test.n) return;
    const bool row_ok = i < test.n;
    const int ii = row_ok ? i : test.n - 1;

    const float4 ih = test.chi[ii], il = test.clo[ii];
    const int par = il.w != 0.0f ? 1 : 0;
    R k, are, aim;
    if constexpr (sizeof(R) == 4) {
        k = a.k32;
        are = a.alpha_re32;
        aim = a.alpha_im32;
    } else {
        k = a.k;
        are = a.alpha_re;
        aim = a.alpha_im;
    }
    const bool unit_alpha = a.unit_alpha != 0;
    const int accumulate = a.accumulate;
    R x0, x1, x2;
    if constexpr (sizeof(R) == 8) {
        x0 = test.center[3 * (int64_t)ii];
        x1 = test.center[3 * (int64_t)ii + 1];
        x2 = test.center[3 * (int64_t)ii + 2];
    } else {
        x0 = ih.x + il.x;
        x1 = ih.y + il.y;
        x2 = ih.z + il.z;
    }
    Out *out_s = reinterpret_cast<Out *>(a.out_s);
    Out *out_d = reinterpret_cast<Out *>(a.out_d);
    // frequency batch: this block's wave numbers [f_lo, f_hi) (gridDim.z chunks)
    const int f_per = (a.nk + gridDim.z - 1) / gridDim.z;
    const int f_lo = min(a.nk, (int)blockIdx.z * f_per), f_hi = min(a.nk, f_lo + f_per);

    for (int c = 0; c < ncols; ++c) {
        const int j = jb + c;
        if constexpr (sizeof(R) == 4) {
            // far-field fast path, taken when every lane of the warp is a far
            // pair: one centroid point for both operators
            const float4 h = s_hi[c];
            const float fx = h.x - x0, fy = h.y - x1, fz = h.z - x2;
            const float q = (fx * fx + fy * fy + fz * fz) * h.w;
            if (__all_sync(0xffffffffu, q > Q_FAR)) {
                const float4 p = s_p0[c];
                const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
                if constexpr (BATCH) {
                    const PointGeom<float> gm = point_geom<float>(fx, fy, fz, p.x, p.y, p.z, p.w, R(DO_S), R(DO_D));
                    for (int f = f_lo; f < f_hi; ++f) {
                        R sr = 0, si = 0, dr = 0, di = 0;
                        point_freq<FAM, float>(gm, a.ks32[f], sr, si, dr, di);
                        if (row_ok) {
                            if (DO_S) store_entry(batch_matrix<Out>(a, false, f) + off, sr, si, are, aim, unit_alpha, accumulate);
                            if (DO_D) store_entry(batch_matrix<Out>(a, true, f) + off, dr, di, are, aim, unit_alpha, accumulate);
                        }
                    }
                } else {
                    R sr = 0, si = 0, dr = 0, di = 0;
                    eval_point<FAM, float>(fx, fy, fz, p.x, p.y, p.z, p.w, k, R(DO_S), R(DO_D), sr, si, dr, di);
                    if (row_ok) {
                        if (DO_S) store_entry(out_s + off, sr, si, are, aim, unit_alpha, accumulate);
                        if (DO_D) store_entry(out_d + off, dr, di, are, aim, unit_alpha, accumulate);
                    }
                }
                continue;
            }
        }
        int ls, ld;
        float dx, dy, dz;
        int kind = classify_pair(ih, il, s_hi[c], s_lo[c], ii, j, test.center, trial.center, trial.size,
                                 a.same_mesh, ls, ld, dx, dy, dz);
        if (kind != KIND_REGULAR || !row_ok) continue;
        if (!DO_S) ls = ld;
        if (!DO_D) ld = ls;
        // one uniform loop over this lane's points: SLP and DLP at the same
        // level share every point; otherwise the SLP points come first
        const int tnc = s_nc[c];
        const int nps = level_npts(tnc, par, ls);
        const int npd = level_npts(tnc, par, ld);
        const int n_eval = ls == ld ? nps : nps + npd;
        const int64_t base = ((int64_t)j * 2 + par) * SLOTS;
        if constexpr (BATCH) {
            // frequency batch: each point's geometry once per tile of wave numbers
            for (int f0 = f_lo; f0 < f_hi; f0 += FREQ_TILE) {
                R kf[FREQ_TILE], sr[FREQ_TILE], si[FREQ_TILE], dr[FREQ_TILE], di[FREQ_TILE];
#pragma unroll
                for (int u = 0; u < FREQ_TILE; ++u) {
                    if constexpr (sizeof(R) == 4) kf[u] = f0 + u < f_hi ? a.ks32[f0 + u] : 0.0f;
                    else kf[u] = f0 + u < f_hi ? a.ks[f0 + u] : 0.0;
                    sr[u] = si[u] = dr[u] = di[u] = 0;
                }
                for (int q = 0; q < n_eval; ++q) {
                    int slot;
                    R ws, wd;
                    if (ls == ld) { slot = level_slot0(ls) + q; ws = R(DO_S); wd = R(DO_D); }
                    else if (q < nps) { slot = level_slot0(ls) + q; ws = R(1); wd = R(0); }
                    else { slot = level_slot0(ld) + q - nps; ws = R(0); wd = R(1); }
                    PointGeom<R> gm;
                    if constexpr (sizeof(R) == 4) {
                        const float4 y = __ldg(trial.pts32 + 2 * (base + slot));
                        const float4 n = __ldg(trial.pts32 + 2 * (base + slot) + 1);
                        const bool centre = slot == 0;
                        gm = point_geom<float>(centre ? dx : y.x - x0, centre ? dy : y.y - x1,
                                               centre ? dz : y.z - x2, y.w, n.x, n.y, n.z, ws, wd);
                    } else {
                        const double *y = trial.pts64 + 8 * (base + slot);
                        gm = point_geom<double>(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6], ws, wd);
                    }
#pragma unroll
                    for (int u = 0; u < FREQ_TILE; ++u) point_freq<FAM, R>(gm, kf[u], sr[u], si[u], dr[u], di[u]);
                }
#pragma unroll
                for (int u = 0; u < FREQ_TILE; ++u) {
                    if (f0 + u >= f_hi) break;
                    const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
                    if (DO_S)
                        store_entry(batch_matrix<Out>(a, false, f0 + u) + off, sr[u], si[u], are, aim, unit_alpha, accumulate);
                    if (DO_D)
                        store_entry(batch_matrix<Out>(a, true, f0 + u) + off, dr[u], di[u], are, aim, unit_alpha, accumulate);
                }
            }
        } else {
            R sr = 0, si = 0, dr = 0, di = 0;
            for (int q = 0; q < n_eval; ++q) {
                int slot;
                R ws, wd;
                if (ls == ld) { slot = level_slot0(ls) + q; ws = R(DO_S); wd = R(DO_D); }
                else if (q < nps) { slot = level_slot0(ls) + q; ws = R(1); wd = R(0); }
                else { slot = level_slot0(ld) + q - nps; ws = R(0); wd = R(1); }
                if constexpr (sizeof(R) == 4) {
                    const float4 y = __ldg(trial.pts32 + 2 * (base + slot));
                    const float4 n = __ldg(trial.pts32 + 2 * (base + slot) + 1);
                    // level-0 point: the trial centre; use the accurate hi/lo difference
                    const bool centre = slot == 0;
                    eval_point<FAM, float>(centre ? dx : y.x - x0, centre ? dy : y.y - x1, centre ? dz : y.z - x2, y.w,
                                           n.x, n.y, n.z, k, ws, wd, sr, si, dr, di);
                } else {
                    const double *y = trial.pts64 + 8 * (base + slot);
                    eval_point<FAM, double>(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6], k, ws, wd, sr,
                                            si, dr, di);
                }
            }
            const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
            if (DO_S) store_entry(out_s + off, sr, si, are, aim, unit_alpha, accumulate);
            if (DO_D) store_entry(out_d + off, dr, di, are, aim, unit_alpha, accumulate);
        }
    }
}

template <typename R, typename Out, int FAM, bool BATCH>
static void launch_ops(const RegularArgs &a, dim3 grid, cudaStream_t s)
{
    if (a.ops == OP_SLP) k_regular<R, Out, FAM, OP_SLP, BATCH><<<grid, REG_THREADS, 0, s>>>(a);
    else if (a.ops == OP_DLP) k_regular<R, Out, FAM, OP_DLP, BATCH><<<grid, REG_THREADS, 0, s>>>(a);
    else k_regular<R, Out, FAM, OP_SLP | OP_DLP, BATCH><<<grid, REG_THREADS, 0, s>>>(a);
}

template <typename R, typename Out>
static void launch_fam(const RegularArgs &a, dim3 grid, cudaStream_t s)
{
    const bool batch = a.nk > 1 || a.force_batch;
    if (a.family == FAM_HELMHOLTZ) {
        if (batch) launch_ops<R, Out, FAM_HELMHOLTZ, true>(a, grid, s);
        else launch_ops<R, Out, FAM_HELMHOLTZ, false>(a, grid, s);
    } else {
        if (batch) launch_ops<R, Out, FAM_LAPLACE, true>(a, grid, s);
        else launch_ops<R, Out, FAM_LAPLACE, false>(a, grid, s);
    }
}

cudaError_t launch_assemble_regular(const RegularArgs &a, cudaStream_t s)
{
    int ncols = a.j1 - a.j0;
    if (a.test.n == 0 || ncols <= 0) return cudaSuccess;
    dim3 grid((a.test.n + REG_THREADS - 1) / REG_THREADS, (ncols + REG_COLS - 1) / REG_COLS);
    if (a.nk > 1 || a.force_batch) {
        // small meshes: split the wave numbers over gridDim.z (at least one tile of
        // FREQ_TILE each) until the grid holds about four blocks per SM
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int64_t xy = (int64_t)grid.x * grid.y;
        const int64_t want = (4 * (int64_t)sms + xy - 1) / xy;
        const int most = (a.nk + FREQ_TILE - 1) / FREQ_TILE;
        grid.z = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, most));
    }
    if (a.precision == 0) {
        if (a.dtype == 0) launch_fam<float, float2>(a, grid, s);
        else launch_fam<float, double2>(a, grid, s);
    } else {
        if (a.dtype == 0) launch_fam<double, float2>(a, grid, s);
        else launch_fam<double, double2>(a, grid, s);
    }
    return cudaGetLastError();
}

}  // namespace nihu
