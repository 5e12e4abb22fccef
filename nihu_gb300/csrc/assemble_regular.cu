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
#include "classify.cuh"
#include "kernels.h"

namespace nihu {

constexpr int REG_THREADS = 256;
constexpr int REG_COLS = 32;

template <int FAM, typename R>
__device__ __forceinline__ void eval_point(R rx, R ry, R rz, R wj, R nx, R ny, R nz, R k, bool do_s, bool do_d,
                                           R &sr, R &si, R &dr, R &di)
{
    constexpr R INV4PI = R(1.0 / (4.0 * 3.14159265358979323846));
    R r2 = rx * rx + ry * ry + rz * rz;
    R rinv;
    if constexpr (sizeof(R) == 4) rinv = rsqrtf(r2);
    else rinv = rsqrt(r2);
    R g = wj * rinv * INV4PI;
    if constexpr (FAM == FAM_HELMHOLTZ) {
        R kr = k * (r2 * rinv);
        R s, c;
        if constexpr (sizeof(R) == 4) sincosf(kr, &s, &c);
        else sincos(kr, &s, &c);
        // e^{-ikr} = c - i s
        if (do_s) { sr += g * c; si -= g * s; }
        if (do_d) {
            // dG/dr (r.n)/r = -(1 + ikr) e^{-ikr} / (4 pi r^2) * (r.n)/r
            R f = -g * rinv * ((rx * nx + ry * ny + rz * nz) * rinv);
            dr += f * (c + kr * s);
            di += f * (kr * c - s);
        }
    } else {
        if (do_s) sr += g;
        if (do_d) dr -= g * rinv * ((rx * nx + ry * ny + rz * nz) * rinv);
    }
}

template <typename Out, typename R>
__device__ __forceinline__ void store_entry(Out *p, R re, R im, double are, double aim, int accumulate)
{
    R vr = R(are) * re - R(aim) * im;
    R vi = R(are) * im + R(aim) * re;
    if (accumulate) {
        Out o = *p;
        o.x += vr;
        o.y += vi;
        *p = o;
    } else {
        Out o;
        o.x = vr;
        o.y = vi;
        *p = o;
    }
}

template <typename R, typename Out, int FAM, int OPS>
__global__ void __launch_bounds__(REG_THREADS) k_regular(RegularArgs a)
{
    __shared__ float4 s_hi[REG_COLS], s_lo[REG_COLS], s_p0[REG_COLS];
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
        s_p0[threadIdx.x] = trial.p0[jb + threadIdx.x];
    }
    __syncthreads();
    if (i >= test.n) return;

    const float4 ih = test.chi[i], il = test.clo[i];
    const int par = il.w != 0.0f ? 1 : 0;
    const R k = R(a.k);
    R xi0, xi1, xi2;
    if constexpr (sizeof(R) == 8) {
        xi0 = test.center[3 * (int64_t)i];
        xi1 = test.center[3 * (int64_t)i + 1];
        xi2 = test.center[3 * (int64_t)i + 2];
    }
    Out *out_s = reinterpret_cast<Out *>(a.out_s);
    Out *out_d = reinterpret_cast<Out *>(a.out_d);

    for (int c = 0; c < ncols; ++c) {
        const int j = jb + c;
        int ls, ld;
        float dx, dy, dz;
        int kind = classify_pair(ih, il, s_hi[c], s_lo[c], i, j, test.center, trial.center, trial.size,
                                 a.same_mesh, ls, ld, dx, dy, dz);
        if (kind != KIND_REGULAR) continue;
        R sr = 0, si = 0, dr = 0, di = 0;
        const int tnc = trial.nc[j];
        if constexpr (sizeof(R) == 4) {
            // FP32: level-0 point is the trial centre; r = c_j - c_i from the hi/lo split
            auto eval_level = [&](int lev, bool es, bool ed) {
                if (lev == 0) {
                    float4 p = s_p0[c];
                    eval_point<FAM, float>(dx, dy, dz, p.x, p.y, p.z, p.w, k, es, ed, sr, si, dr, di);
                    return;
                }
                const int np = level_npts(tnc, par, lev);
                const float4 *pp = trial.pts32 + 2 * (((int64_t)j * 2 + par) * SLOTS + level_slot0(lev));
                const float xx = ih.x + il.x, xy = ih.y + il.y, xz = ih.z + il.z;
                for (int q = 0; q < np; ++q) {
                    float4 y = __ldg(pp + 2 * q), n = __ldg(pp + 2 * q + 1);
                    eval_point<FAM, float>(y.x - xx, y.y - xy, y.z - xz, y.w, n.x, n.y, n.z, k, es, ed, sr, si, dr,
                                           di);
                }
            };
            if (!DO_S || !DO_D || ls == ld) {
                eval_level(DO_S && DO_D ? ls : (DO_S ? ls : ld), DO_S, DO_D);
            } else {
                eval_level(ls, true, false);
                eval_level(ld, false, true);
            }
        } else {
            auto eval_level = [&](int lev, bool es, bool ed) {
                const int np = level_npts(tnc, par, lev);
                const double *pp = trial.pts64 + 8 * (((int64_t)j * 2 + par) * SLOTS + level_slot0(lev));
                for (int q = 0; q < np; ++q) {
                    const double *y = pp + 8 * q;
                    eval_point<FAM, double>(y[0] - xi0, y[1] - xi1, y[2] - xi2, y[3], y[4], y[5], y[6], k, es, ed, sr,
                                            si, dr, di);
                }
            };
            if (!DO_S || !DO_D || ls == ld) {
                eval_level(DO_S && DO_D ? ls : (DO_S ? ls : ld), DO_S, DO_D);
            } else {
                eval_level(ls, true, false);
                eval_level(ld, false, true);
            }
        }
        const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
        if (DO_S) store_entry(out_s + off, sr, si, a.alpha_re, a.alpha_im, a.accumulate);
        if (DO_D) store_entry(out_d + off, dr, di, a.alpha_re, a.alpha_im, a.accumulate);
    }
}

template <typename R, typename Out, int FAM>
static void launch_ops(const RegularArgs &a, dim3 grid, cudaStream_t s)
{
    if (a.ops == OP_SLP) k_regular<R, Out, FAM, OP_SLP><<<grid, REG_THREADS, 0, s>>>(a);
    else if (a.ops == OP_DLP) k_regular<R, Out, FAM, OP_DLP><<<grid, REG_THREADS, 0, s>>>(a);
    else k_regular<R, Out, FAM, OP_SLP | OP_DLP><<<grid, REG_THREADS, 0, s>>>(a);
}

template <typename R, typename Out>
static void launch_fam(const RegularArgs &a, dim3 grid, cudaStream_t s)
{
    if (a.family == FAM_HELMHOLTZ) launch_ops<R, Out, FAM_HELMHOLTZ>(a, grid, s);
    else launch_ops<R, Out, FAM_LAPLACE>(a, grid, s);
}

cudaError_t launch_assemble_regular(const RegularArgs &a, cudaStream_t s)
{
    int ncols = a.j1 - a.j0;
    if (a.test.n == 0 || ncols <= 0) return cudaSuccess;
    dim3 grid((a.test.n + REG_THREADS - 1) / REG_THREADS, (ncols + REG_COLS - 1) / REG_COLS);
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
