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
//
// Right-hand-side mode (frequency batches, RegularArgs::rhs_part): the SLP
// entries are not stored; each thread sums SLP_f(i, j) q_f(j) over its
// block's columns per wave number in shared memory, the block writes one
// partial sum per (wave number, row), and k_rhs_reduce adds the partials and
// the FP64 kernel's nearly singular and self entries in a fixed order.  This
// is b = SLP q of the collocation system without the SLP matrix.
#include <algorithm>
#include <type_traits>

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
        if constexpr (sizeof(R) == 4) sincos_reduced(kr, s, c);
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

// right-hand-side mode: wave numbers per block (the gridDim.z split keeps at
// most this many), which sizes the shared row sums and Neumann data
template <typename R>
__host__ __device__ constexpr int rhs_f_max() { return sizeof(R) == 4 ? 16 : 8; }

// the wave numbers per block a launch uses: RegularArgs::rhs_fmax within the
// cap that keeps the shared memory under 48 KB, else the default
template <typename R>
__host__ __device__ inline int rhs_fmax_of(const RegularArgs &a)
{
    constexpr int cap = sizeof(R) == 4 ? 20 : 10;
    return a.rhs_fmax > 0 ? (a.rhs_fmax < cap ? a.rhs_fmax : cap) : rhs_f_max<R>();
}

template <typename R>
using Cplx = std::conditional_t<sizeof(R) == 4, float2, double2>;

// acc += (sr + i si) q
template <typename R2, typename R>
__device__ __forceinline__ void rhs_add(R2 &acc, const R2 q, R sr, R si)
{
    acc.x += sr * q.x - si * q.y;
    acc.y += sr * q.y + si * q.x;
}

// frequency batches store plain entries (unit scale, no accumulation:
// launch_assemble_regular refuses anything else)
template <typename Out, typename R>
__device__ __forceinline__ void store_plain(Out *p, R re, R im)
{
    Out o;
    o.x = re;
    o.y = im;
    *p = o;
}

// the outputs of a frequency batch from wave number f on: a pointer that
// steps by mat_stride, or (TAB) the device table outs (separate matrices);
// the kernel picks the variant once, outside its wave number loops
template <typename Out, bool TAB>
struct BatchCursor {
    Out *p = nullptr;
    void *const *tab = nullptr;
    int64_t step, off;
    __device__ __forceinline__ BatchCursor(const RegularArgs &a, bool dlp, int f, int64_t off_)
        : step(a.mat_stride), off(off_)
    {
        if constexpr (TAB) {
            tab = a.outs + (dlp ? a.nk : 0) + f;
        } else {
            Out *base = reinterpret_cast<Out *>(dlp ? a.out_d : a.out_s);
            p = base ? base + (int64_t)f * a.mat_stride + off : nullptr;
        }
    }
    __device__ __forceinline__ Out *get() const
    {
        if constexpr (TAB) return reinterpret_cast<Out *>(*tab) + off;
        else return p;
    }
    __device__ __forceinline__ void next()
    {
        if constexpr (TAB) ++tab;
        else p += step;
    }
};

// Squared distance ratio above which a pair is certainly regular with the
// 1-point rule for both SLP (x >= 9.1) and DLP (x >= 15.8): 15.8^2 with a
// relative margin far larger than the FP32 error of the plain centre
// difference of a far pair.
constexpr float Q_FAR = 249.64f * (1.0f + 1e-4f);

// BATCH: frequency batch (a.nk > 1), a separate instantiation so that the
// single wave number kernel carries none of its code
// RHS: right-hand-side mode (BATCH only; the SLP entries go into the row sums)
// PLAIN: unit scale and no accumulation (single wave number, FP32), so the
// stores carry no run-time checks
// CK: a complex (lossy) wave number k + i k_im (single wave number, Helmholtz;
// its own instantiation, so the real-k kernels carry none of it)
template <typename R, typename Out, int FAM, int OPS, bool BATCH, bool RHS = false, bool PLAIN = false,
          bool CK = false>
__global__ void __launch_bounds__(REG_THREADS) k_regular(RegularArgs a)
{
    using R2 = Cplx<R>;
    __shared__ float4 s_hi[REG_COLS], s_lo[REG_COLS], s_p0[REG_COLS];
    __shared__ int s_nc[REG_COLS];
    // RHS: Neumann data [f - f_lo][c], then the row sums [f - f_lo][threadIdx.x]
    extern __shared__ __align__(16) unsigned char s_rhs[];
    R2 *s_q = reinterpret_cast<R2 *>(s_rhs);
    R2 *s_acc = s_q + rhs_fmax_of<R>(a) * REG_COLS;
    constexpr bool DO_S = (OPS & OP_SLP) != 0;
    constexpr bool DO_D = (OPS & OP_DLP) != 0;
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    const int i = blockIdx.x * REG_THREADS + threadIdx.x;
    const int jb = a.j0 + blockIdx.y * REG_COLS;
    const int ncols = min(REG_COLS, a.j1 - jb);
    // frequency batch: this block's wave numbers [f_lo, f_hi) (gridDim.z chunks)
    const int f_per = (a.nk + gridDim.z - 1) / gridDim.z;
    const int f_lo = min(a.nk, (int)blockIdx.z * f_per), f_hi = min(a.nk, f_lo + f_per);
    if (threadIdx.x < ncols) {
        s_hi[threadIdx.x] = trial.chi[jb + threadIdx.x];
        s_lo[threadIdx.x] = trial.clo[jb + threadIdx.x];
        s_nc[threadIdx.x] = trial.nc[jb + threadIdx.x];
        s_p0[threadIdx.x] = trial.p0[jb + threadIdx.x];
    }
    if constexpr (RHS) {
        const int nf = f_hi - f_lo;  // at most rhs_fmax_of (launch_assemble_regular)
        for (int t = threadIdx.x; t < nf * REG_COLS; t += REG_THREADS) {
            const int fl = t / REG_COLS, c = t - fl * REG_COLS;
            R2 v;
            v.x = 0;
            v.y = 0;
            if (c < ncols) {
                const double2 qv = a.rhs_q[(int64_t)(f_lo + fl) * trial.n + jb + c];
                v.x = R(qv.x);
                v.y = R(qv.y);
            }
            s_q[t] = v;
        }
        for (int fl = 0; fl < nf; ++fl) {
            R2 z;
            z.x = 0;
            z.y = 0;
            s_acc[fl * REG_THREADS + threadIdx.x] = z;
        }
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
    R k, are, aim, kim;
    if constexpr (sizeof(R) == 4) {
        kim = a.k_im32;
        k = a.k32;
        are = a.alpha_re32;
        aim = a.alpha_im32;
    } else {
        kim = a.k_im;
        k = a.k;
        are = a.alpha_re;
        aim = a.alpha_im;
    }
    (void)kim;
    // one quadrature point of the single wave number paths
    auto ev = [&](R rx, R ry, R rz, R wj, R nx, R ny, R nz, R ws, R wd, R &sr, R &si, R &dr, R &di) {
        if constexpr (CK) eval_point_ck<R>(rx, ry, rz, wj, nx, ny, nz, k, kim, ws, wd, sr, si, dr, di);
        else eval_point<FAM, R>(rx, ry, rz, wj, nx, ny, nz, k, ws, wd, sr, si, dr, di);
    };
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
    // single wave number: this thread's entries of the current column, one
    // column (ld entries) further per step
    const int64_t ldo = a.ld;
    Out *ps = DO_S && !BATCH ? out_s + (int64_t)(jb - a.j0) * ldo + i : nullptr;
    Out *pd = DO_D && !BATCH ? out_d + (int64_t)(jb - a.j0) * ldo + i : nullptr;
    auto put = [&](Out *p, R re, R im) {
        if constexpr (PLAIN) store_plain(p, re, im);
        else store_entry(p, re, im, are, aim, unit_alpha, accumulate);
    };

    for (int c = 0; c < ncols; ++c, ps += DO_S && !BATCH ? ldo : 0, pd += DO_D && !BATCH ? ldo : 0) {
        const int j = jb + c;
        if constexpr (sizeof(R) == 4) {
            // far-field fast path, taken when every lane of the warp is a far
            // pair: one centroid point for both operators
            // the hi/lo centre difference: FP32 relative accuracy of r, which
            // the DLP's r.n of nearly coplanar far pairs needs
            const float4 h = s_hi[c], l = s_lo[c];
            const float fx = (h.x - ih.x) + (l.x - il.x), fy = (h.y - ih.y) + (l.y - il.y),
                        fz = (h.z - ih.z) + (l.z - il.z);
            const float q = (fx * fx + fy * fy + fz * fz) * h.w;
            if (__all_sync(0xffffffffu, q > Q_FAR)) {
                const float4 p = s_p0[c];
                if constexpr (BATCH) {
                    const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
                    const PointGeom<float> gm = point_geom<float>(fx, fy, fz, p.x, p.y, p.z, p.w, R(DO_S), R(DO_D));
                    auto freqs = [&](auto tab) {
                        constexpr bool TAB = decltype(tab)::value;
                        BatchCursor<Out, TAB> cs(a, false, f_lo, off), cd(a, true, f_lo, off);
                        R2 *acc = s_acc + threadIdx.x;
                        const R2 *qc = s_q + c;
                        const float *kp = a.ks32 + f_lo;
                        for (int f = f_lo; f < f_hi; ++f) {
                            R sr = 0, si = 0, dr = 0, di = 0;
                            point_freq<FAM, float>(gm, *kp++, sr, si, dr, di);
                            if (row_ok) {
                                if constexpr (RHS) rhs_add(*acc, *qc, sr, si);
                                else if (DO_S) store_plain(cs.get(), sr, si);
                                if (DO_D) store_plain(cd.get(), dr, di);
                            }
                            if constexpr (RHS) {
                                acc += REG_THREADS;
                                qc += REG_COLS;
                            } else if (DO_S) {
                                cs.next();
                            }
                            if (DO_D) cd.next();
                        }
                    };
                    if (a.outs) freqs(std::true_type{});
                    else freqs(std::false_type{});
                } else {
                    R sr = 0, si = 0, dr = 0, di = 0;
                    ev(fx, fy, fz, p.x, p.y, p.z, p.w, R(DO_S), R(DO_D), sr, si, dr, di);
                    if (row_ok) {
                        if (DO_S) put(ps, sr, si);
                        if (DO_D) put(pd, dr, di);
                    }
                }
                continue;
            }
        }
        if constexpr (sizeof(R) == 4 && !BATCH && OPS == (OP_SLP | OP_DLP)) {
            // every lane certainly has the 1-point SLP rule (d/D >= 9.1) and a
            // certain DLP level, 0 (d/D >= 15.8) or 1 (below): the general
            // path's points in its order -- the centroid, then for level 1 the
            // DLP-only points -- without its per-lane dispatch.  "Certainly"
            // is classify_pair's FP32 guard band, so the levels are its own.
            const float4 jh = s_hi[c], jl = s_lo[c];
            const float mx = (jh.x - ih.x) + (jl.x - il.x), my = (jh.y - ih.y) + (jl.y - il.y),
                        mz = (jh.z - ih.z) + (jl.z - il.z);
            const float mq = (mx * mx + my * my + mz * mz) * jh.w;
            const float mlo = mq * (1.0f - 1e-5f), mhi = mq * (1.0f + 1e-5f);
            const bool d_far = mlo >= 249.64f;
            if (__all_sync(0xffffffffu, mlo >= 82.81f && (d_far || mhi < 249.64f))) {
                if (row_ok) {
                    const int64_t base = ((int64_t)j * 2 + par) * SLOTS;
                    R sr = 0, si = 0, dr = 0, di = 0;
                    const float4 yc = __ldg(trial.pts32 + 2 * base), nc = __ldg(trial.pts32 + 2 * base + 1);
                    ev(mx, my, mz, yc.w, nc.x, nc.y, nc.z, R(1), d_far ? R(1) : R(0), sr, si, dr, di);
                    if (!d_far) {
                        const int npd = level_npts(s_nc[c], par, 1);
                        for (int q = 0; q < npd; ++q) {
                            const int64_t sl = base + level_slot0(1) + q;
                            const float4 y = __ldg(trial.pts32 + 2 * sl), n = __ldg(trial.pts32 + 2 * sl + 1);
                            ev(mx + y.x, my + y.y, mz + y.z, y.w, n.x, n.y, n.z, R(0), R(1), sr, si, dr, di);
                        }
                    }
                    put(ps, sr, si);
                    put(pd, dr, di);
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
            const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
            auto tiles = [&](auto tab) {
                constexpr bool TAB = decltype(tab)::value;
                BatchCursor<Out, TAB> cs(a, false, f_lo, off), cd(a, true, f_lo, off);
                R2 *acc = s_acc + threadIdx.x;
                const R2 *qc = s_q + c;
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
                            gm = point_geom<float>(dx + y.x, dy + y.y, dz + y.z, y.w, n.x, n.y, n.z, ws, wd);
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
                        if constexpr (RHS) {
                            rhs_add(*acc, *qc, sr[u], si[u]);
                            acc += REG_THREADS;
                            qc += REG_COLS;
                        } else if (DO_S) {
                            store_plain(cs.get(), sr[u], si[u]);
                            cs.next();
                        }
                        if (DO_D) {
                            store_plain(cd.get(), dr[u], di[u]);
                            cd.next();
                        }
                    }
                }
            };
            if (a.outs) tiles(std::true_type{});
            else tiles(std::false_type{});
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
                    // r = (c_j - x) + (y - c_j): the hi/lo centre difference plus the
                    // point's offset from the trial centre
                    ev(dx + y.x, dy + y.y, dz + y.z, y.w, n.x, n.y, n.z, ws, wd, sr, si, dr, di);
                } else {
                    const double *y = trial.pts64 + 8 * (base + slot);
                    ev(y[0] - x0, y[1] - x1, y[2] - x2, y[3], y[4], y[5], y[6], ws, wd, sr, si, dr, di);
                }
            }
            if (DO_S) put(ps, sr, si);
            if (DO_D) put(pd, dr, di);
        }
    }
    if constexpr (RHS) {
        if (row_ok) {
            R2 *part = reinterpret_cast<R2 *>(a.rhs_part);
            for (int f = f_lo; f < f_hi; ++f) {
                R2 v = s_acc[(f - f_lo) * REG_THREADS + threadIdx.x];
                if (!unit_alpha) {
                    const R vr = are * v.x - aim * v.y;
                    v.y = are * v.y + aim * v.x;
                    v.x = vr;
                }
                part[((int64_t)f * gridDim.y + blockIdx.y) * test.n + i] = v;
            }
        }
    }
}

int regular_carveout_percent()
{
    // four blocks of k_regular2 (under 10 KB of shared memory each, plus the
    // 1 KB the runtime reserves per block): the 64 KB configuration
    return 25;
}

// ------------------------------------------------- two rows per thread
// The single wave number FP32 kernel for the common case (SLP and DLP, unit
// scale, no accumulation, complex64 columns that allow 16-byte stores): each
// thread owns two adjacent rows, so that one far vote, one set of shared
// loads and the loop's bookkeeping serve two pairs, and each column takes one
// 16-byte store per matrix for both rows.
//
// A column whose 64 rows of a warp are not all far (about 13% of the warp
// iterations on an icosphere, with some 45 of the 64 pairs not far) is not
// evaluated in that warp: its far rows take the centroid there, certainly
// nearly singular and self pairs are left to the singular kernel, and the
// others are appended to the warp's list in shared memory (one 16-bit code
// per pair: row in the block, column in the block), from the front when their
// levels are certain without the FP64 check (SLP 1 point, DLP level 1: most
// of them) and from the back otherwise.  Every REG2_CHUNK columns the warp
// works through its two lists, one pair per lane, so that a pair's cost is
// its own point count, not the largest one in its warp; warps do not wait
// for one another.  A list holds every pair of a chunk, so it cannot
// overflow, and a block needs under 10 KB of shared memory.  The points,
// levels and their order are those of k_regular (the far path, the
// certain-level path and the general dispatch).
constexpr int REG2_THREADS = 256;
constexpr int REG2_ROWS = 2 * REG2_THREADS;
constexpr int REG2_CHUNK = 8;                  // columns per list flush
constexpr int REG2_WLIST = 64 * REG2_CHUNK;    // every pair of a warp's chunk
static_assert(REG2_ROWS <= 512 && REG_COLS <= 128, "a pair code is row (9 bits) | column << 9 in 16 bits");

// the far rule (the element centroid for both operators) with the weight
// w J / (4 pi) given: e^{-ikr}/(4 pi r) and its DLP counterpart
// -(1 + ikr) e^{-ikr} (r.n) / (4 pi r^3)
template <int FAM>
__device__ __forceinline__ void far_point(float rx, float ry, float rz, float w4, float nx, float ny, float nz,
                                          float k, float &sr, float &si, float &dr, float &di)
{
    const float r2 = rx * rx + ry * ry + rz * rz;
    const float rinv = rsqrtf(r2);
    const float g = w4 * rinv;
    const float rn = rx * nx + ry * ny + rz * nz;
    const float f = -g * (rinv * rinv) * rn;
    if constexpr (FAM == FAM_HELMHOLTZ) {
        const float kr = k * (r2 * rinv);
        float sn, cs;
        sincos_reduced(kr, sn, cs);
        sr = g * cs;
        si = -g * sn;
        dr = f * (cs + kr * sn);
        di = f * (kr * cs - sn);
    } else {
        sr = g;
        si = 0.0f;
        dr = f;
        di = 0.0f;
    }
}

// one pair by the general path of k_regular (classify_pair, the uniform loop
// over the lane's points); false when the pair is not regular
template <int FAM>
__device__ __forceinline__ bool pair_general32(const RegularArgs &a, const float4 ih, const float4 il, int par, int i,
                                               int j, const float4 jh, const float4 jl, int tnc, float k, float &sr,
                                               float &si, float &dr, float &di)
{
    int ls, ld;
    float dx, dy, dz;
    const int kind = classify_pair(ih, il, jh, jl, i, j, a.test.center, a.trial.center, a.trial.size, a.same_mesh,
                                   ls, ld, dx, dy, dz);
    if (kind != KIND_REGULAR) return false;
    const int nps = level_npts(tnc, par, ls);
    const int npd = level_npts(tnc, par, ld);
    const int n_eval = ls == ld ? nps : nps + npd;
    const int64_t base = ((int64_t)j * 2 + par) * SLOTS;
    sr = si = dr = di = 0.0f;
    for (int q = 0; q < n_eval; ++q) {
        int slot;
        float ws, wd;
        if (ls == ld) { slot = level_slot0(ls) + q; ws = 1.0f; wd = 1.0f; }
        else if (q < nps) { slot = level_slot0(ls) + q; ws = 1.0f; wd = 0.0f; }
        else { slot = level_slot0(ld) + q - nps; ws = 0.0f; wd = 1.0f; }
        const float4 y = __ldg(a.trial.pts32 + 2 * (base + slot));
        const float4 n = __ldg(a.trial.pts32 + 2 * (base + slot) + 1);
        eval_point<FAM, float>(dx + y.x, dy + y.y, dz + y.z, y.w, n.x, n.y, n.z, k, ws, wd, sr, si, dr, di);
    }
    return true;
}

// one warp's deferred pairs: certain levels (the centroid for the SLP, the
// level-1 points for the DLP) from the front of its list, the others
// (classify_pair and the pair's own rule) from the back
template <int FAM>
__device__ __forceinline__ void regular2_flush(const RegularArgs &a, const unsigned short *wl, int nA, int nB,
                                               int lane, int ib, int jb, const float4 *s_hi, const float4 *s_lo,
                                               const int *s_nc, float2 *out_s, float2 *out_d, int64_t ldo, float k)
{
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    for (int t = lane; t < nA; t += 32) {
        const int code = wl[t];
        const int i = ib + (code & 511), c = code >> 9, j = jb + c;
        const float4 ih = test.chi[i], il = test.clo[i], h = s_hi[c], l = s_lo[c];
        const int par = il.w != 0.0f ? 1 : 0;
        const float mx = (h.x - ih.x) + (l.x - il.x), my = (h.y - ih.y) + (l.y - il.y),
                    mz = (h.z - ih.z) + (l.z - il.z);
        const int64_t base = ((int64_t)j * 2 + par) * SLOTS;
        float sr = 0, si = 0, dr = 0, di = 0;
        const float4 yc = __ldg(trial.pts32 + 2 * base), nc = __ldg(trial.pts32 + 2 * base + 1);
        eval_point<FAM, float>(mx, my, mz, yc.w, nc.x, nc.y, nc.z, k, 1.0f, 0.0f, sr, si, dr, di);
        const int npd = level_npts(s_nc[c], par, 1);
        for (int q = 0; q < npd; ++q) {
            const int64_t sl = base + level_slot0(1) + q;
            const float4 y = __ldg(trial.pts32 + 2 * sl), n = __ldg(trial.pts32 + 2 * sl + 1);
            eval_point<FAM, float>(mx + y.x, my + y.y, mz + y.z, y.w, n.x, n.y, n.z, k, 0.0f, 1.0f, sr, si, dr, di);
        }
        out_s[(int64_t)c * ldo + i] = make_float2(sr, si);
        out_d[(int64_t)c * ldo + i] = make_float2(dr, di);
    }
    for (int t = lane; t < nB; t += 32) {
        const int code = wl[REG2_WLIST - 1 - t];
        const int i = ib + (code & 511), c = code >> 9, j = jb + c;
        const float4 ih = test.chi[i], il = test.clo[i];
        float sr, si, dr, di;
        if (pair_general32<FAM>(a, ih, il, il.w != 0.0f ? 1 : 0, i, j, s_hi[c], s_lo[c], s_nc[c], k, sr, si, dr, di)) {
            out_s[(int64_t)c * ldo + i] = make_float2(sr, si);
            out_d[(int64_t)c * ldo + i] = make_float2(dr, di);
        }
    }
}

template <int FAM>
// 64 registers: three blocks fit beside the concurrent singular kernel's one
__global__ void __launch_bounds__(REG2_THREADS, 4) k_regular2(RegularArgs a)
{
    constexpr float INV4PI = 0.0795774715459476679f;
    __shared__ float4 s_hi[REG_COLS], s_lo[REG_COLS], s_p0[REG_COLS];
    __shared__ int s_nc[REG_COLS];
    __shared__ unsigned short s_list[REG2_THREADS / 32][REG2_WLIST];
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    const int jb = a.j0 + blockIdx.y * REG_COLS;
    const int ncols = min(REG_COLS, a.j1 - jb);
    const int ib = blockIdx.x * REG2_ROWS;
    if (threadIdx.x < ncols) {
        s_hi[threadIdx.x] = trial.chi[jb + threadIdx.x];
        s_lo[threadIdx.x] = trial.clo[jb + threadIdx.x];
        s_nc[threadIdx.x] = trial.nc[jb + threadIdx.x];
        float4 p = trial.p0[jb + threadIdx.x];
        p.x *= INV4PI;  // the far rule's weight w J / (4 pi)
        s_p0[threadIdx.x] = p;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int i0 = ib + 2 * threadIdx.x;
    // warps wholly beyond the last row have nothing to do; a partial warp
    // keeps its lanes (clamped rows, stores masked) so that the votes see
    // every lane.  No block barrier follows.
    if (i0 - 2 * lane >= test.n) return;
    unsigned short *wl = s_list[threadIdx.x >> 5];
    const float k = a.k32;
    const int64_t ldo = a.ld;
    float2 *const out_s = reinterpret_cast<float2 *>(a.out_s) + (int64_t)(jb - a.j0) * ldo;
    float2 *const out_d = reinterpret_cast<float2 *>(a.out_d) + (int64_t)(jb - a.j0) * ldo;
    const bool ok0 = i0 < test.n, ok1 = i0 + 1 < test.n;
    const int r0 = ok0 ? i0 : test.n - 1, r1 = ok1 ? i0 + 1 : test.n - 1;
    const float4 ih0 = test.chi[r0], il0 = test.clo[r0], ih1 = test.chi[r1], il1 = test.clo[r1];
    const unsigned lt = (1u << lane) - 1u;
    // FULL: every row of the block exists (all blocks but the last row
    // block): the row checks drop out of the column loop
    auto columns = [&](auto full_tag) {
        constexpr bool FULL = decltype(full_tag)::value;
        float2 *ps = out_s + i0, *pd = out_d + i0;
        for (int c0 = 0; c0 < ncols; c0 += REG2_CHUNK) {
            const int c1 = min(ncols, c0 + REG2_CHUNK);
            int nA = 0, nB = 0;  // warp-uniform list lengths
            for (int c = c0; c < c1; ++c, ps += ldo, pd += ldo) {
                const float4 h = s_hi[c], l = s_lo[c];
                // hi/lo centre differences of both rows (FP32 relative accuracy of r)
                const float ax = (h.x - ih0.x) + (l.x - il0.x), ay = (h.y - ih0.y) + (l.y - il0.y),
                            az = (h.z - ih0.z) + (l.z - il0.z);
                const float bx = (h.x - ih1.x) + (l.x - il1.x), by = (h.y - ih1.y) + (l.y - il1.y),
                            bz = (h.z - ih1.z) + (l.z - il1.z);
                const float qa = (ax * ax + ay * ay + az * az) * h.w;
                const float qb = (bx * bx + by * by + bz * bz) * h.w;
                const bool fa = qa > Q_FAR, fb = qb > Q_FAR;
                const float4 p = s_p0[c];
                if (__all_sync(0xffffffffu, fa && fb)) {
                    // far: the centroid for both operators, both rows
                    float sr0, si0, dr0, di0, sr1, si1, dr1, di1;
                    far_point<FAM>(ax, ay, az, p.x, p.y, p.z, p.w, k, sr0, si0, dr0, di0);
                    far_point<FAM>(bx, by, bz, p.x, p.y, p.z, p.w, k, sr1, si1, dr1, di1);
                    if (FULL || ok1) {
                        *reinterpret_cast<float4 *>(ps) = make_float4(sr0, si0, sr1, si1);
                        *reinterpret_cast<float4 *>(pd) = make_float4(dr0, di0, dr1, di1);
                    } else if (ok0) {
                        *ps = make_float2(sr0, si0);
                        *pd = make_float2(dr0, di0);
                    }
                    continue;
                }
                // far rows here; the others deferred to the warp's lists
                if (fa && (FULL || ok0)) {
                    float sr, si, dr, di;
                    far_point<FAM>(ax, ay, az, p.x, p.y, p.z, p.w, k, sr, si, dr, di);
                    ps[0] = make_float2(sr, si);
                    pd[0] = make_float2(dr, di);
                }
                if (fb && (FULL || ok1)) {
                    float sr, si, dr, di;
                    far_point<FAM>(bx, by, bz, p.x, p.y, p.z, p.w, k, sr, si, dr, di);
                    ps[1] = make_float2(sr, si);
                    pd[1] = make_float2(dr, di);
                }
                // the FP32 guard band of classify_pair: outside it the class is the FP64 class
                const float alo = qa * (1.0f - 1e-5f), ahi = qa * (1.0f + 1e-5f);
                const float blo = qb * (1.0f - 1e-5f), bhi = qb * (1.0f + 1e-5f);
                const bool da = (FULL || ok0) && !fa && ahi >= 2.25f, db = (FULL || ok1) && !fb && bhi >= 2.25f;  // not certainly near
                const bool ca = da && alo >= 82.81f && ahi < 249.64f, cb = db && blo >= 82.81f && bhi < 249.64f;
                const unsigned mA0 = __ballot_sync(0xffffffffu, ca), mA1 = __ballot_sync(0xffffffffu, cb);
                const unsigned mB0 = __ballot_sync(0xffffffffu, da && !ca), mB1 = __ballot_sync(0xffffffffu, db && !cb);
                const int nA0 = __popc(mA0), nB0 = __popc(mB0);
                const unsigned short code0 = (unsigned short)((i0 - ib) | (c << 9));
                const unsigned short code1 = (unsigned short)((i0 + 1 - ib) | (c << 9));
                if (ca) wl[nA + __popc(mA0 & lt)] = code0;
                if (cb) wl[nA + nA0 + __popc(mA1 & lt)] = code1;
                if (da && !ca) wl[REG2_WLIST - 1 - (nB + __popc(mB0 & lt))] = code0;
                if (db && !cb) wl[REG2_WLIST - 1 - (nB + nB0 + __popc(mB1 & lt))] = code1;
                nA += nA0 + __popc(mA1);
                nB += nB0 + __popc(mB1);
            }
            if (nA + nB) {  // warp-uniform
                __syncwarp();  // the list entries are visible to the whole warp
                regular2_flush<FAM>(a, wl, nA, nB, lane, ib, jb, s_hi, s_lo, s_nc, out_s, out_d, ldo, k);
                __syncwarp();  // read before the next chunk appends
            }
        }
    };
    if (ib + REG2_ROWS <= test.n) columns(std::true_type{});
    else columns(std::false_type{});
}

// partial sums of the same row added in FP32 before one FP64 addition
constexpr int RHS_GROUP = 8;

template <typename R2>
__global__ void __launch_bounds__(256) k_rhs_reduce(const R2 *__restrict__ part, int n_cb, int n, int64_t items,
                                                    const int64_t *__restrict__ row_ptr, const int2 *__restrict__ row_ent,
                                                    const double2 *__restrict__ near_slp, const double2 *__restrict__ q,
                                                    int qn, double2 *__restrict__ b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= n) return;
    using R = decltype(R2::x);
    double re = 0.0, im = 0.0;
    const R2 *p = part + (int64_t)f * n_cb * n + i;
    for (int cb0 = 0; cb0 < n_cb; cb0 += RHS_GROUP) {
        R gr = 0, gi = 0;
        const int cb1 = min(n_cb, cb0 + RHS_GROUP);
        for (int cb = cb0; cb < cb1; ++cb) {
            const R2 v = p[(int64_t)cb * n];
            gr += v.x;
            gi += v.y;
        }
        re += (double)gr;
        im += (double)gi;
    }
    const double2 *qf = q + (int64_t)f * qn;
    const double2 *sf = near_slp + (int64_t)f * items;
    R nr = 0, ni = 0;
    for (int64_t t = row_ptr[i]; t < row_ptr[i + 1]; ++t) {
        const int2 e = row_ent[t];
        const double2 sv = sf[e.x], qv = qf[e.y];
        const R sr = R(sv.x), si = R(sv.y), qr = R(qv.x), qi = R(qv.y);
        nr += sr * qr - si * qi;
        ni += sr * qi + si * qr;
    }
    b[(int64_t)f * n + i] = make_double2(re + (double)nr, im + (double)ni);
}

template <typename R, typename Out, int FAM, bool BATCH>
static void launch_ops(const RegularArgs &a, dim3 grid, cudaStream_t s)
{
    if constexpr (BATCH) {
        if (a.rhs_part) {
            const size_t smem = sizeof(Cplx<R>) * rhs_fmax_of<R>(a) * (REG_COLS + REG_THREADS);
            k_regular<R, Out, FAM, OP_SLP | OP_DLP, true, true><<<grid, REG_THREADS, smem, s>>>(a);
            return;
        }
    }
    if constexpr (!BATCH && FAM == FAM_HELMHOLTZ) {
        if (a.k_im != 0.0) {
            if (a.ops == OP_SLP) k_regular<R, Out, FAM, OP_SLP, false, false, false, true><<<grid, REG_THREADS, 0, s>>>(a);
            else if (a.ops == OP_DLP)
                k_regular<R, Out, FAM, OP_DLP, false, false, false, true><<<grid, REG_THREADS, 0, s>>>(a);
            else k_regular<R, Out, FAM, OP_SLP | OP_DLP, false, false, false, true><<<grid, REG_THREADS, 0, s>>>(a);
            return;
        }
    }
    if constexpr (!BATCH && sizeof(R) == 4) {
        if (a.unit_alpha && !a.accumulate) {
            if (a.ops == OP_SLP) k_regular<R, Out, FAM, OP_SLP, false, false, true><<<grid, REG_THREADS, 0, s>>>(a);
            else if (a.ops == OP_DLP) k_regular<R, Out, FAM, OP_DLP, false, false, true><<<grid, REG_THREADS, 0, s>>>(a);
            else k_regular<R, Out, FAM, OP_SLP | OP_DLP, false, false, true><<<grid, REG_THREADS, 0, s>>>(a);
            return;
        }
    }
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
        if (a.accumulate || !a.unit_alpha) return cudaErrorInvalidValue;  // batches store plain entries
        grid.z = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, most));
        // right-hand-side mode: at most rhs_f_max wave numbers per block
        if (a.rhs_part) {
            const int fmax = a.precision == 0 ? rhs_fmax_of<float>(a) : rhs_fmax_of<double>(a);
            grid.z = std::max<unsigned>(grid.z, (unsigned)((a.nk + fmax - 1) / fmax));
        }
    }
    if (a.precision == 0 && a.dtype == 0 && a.nk <= 1 && !a.force_batch && a.ops == (OP_SLP | OP_DLP) &&
        a.unit_alpha && !a.accumulate && a.k_im == 0.0 && (a.ld & 1) == 0 &&
        (reinterpret_cast<uintptr_t>(a.out_s) & 15) == 0 && (reinterpret_cast<uintptr_t>(a.out_d) & 15) == 0) {
        // two rows per thread with 16-byte stores
        dim3 g2((a.test.n + REG2_ROWS - 1) / REG2_ROWS, grid.y);
        int dev = 0;
        cudaGetDevice(&dev);
        static bool carveout_set[64] = {};
        if (dev >= 0 && dev < 64 && !carveout_set[dev]) {
            cudaError_t e = cudaFuncSetAttribute(k_regular2<FAM_HELMHOLTZ>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                 regular_carveout_percent());
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_regular2<FAM_LAPLACE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         regular_carveout_percent());
            if (e != cudaSuccess) return e;
            carveout_set[dev] = true;
        }
        if (a.family == FAM_HELMHOLTZ) k_regular2<FAM_HELMHOLTZ><<<g2, REG2_THREADS, 0, s>>>(a);
        else k_regular2<FAM_LAPLACE><<<g2, REG2_THREADS, 0, s>>>(a);
        return cudaGetLastError();
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

size_t rhs_part_bytes(const RegularArgs &a)
{
    const int64_t n_cb = (a.j1 - a.j0 + REG_COLS - 1) / REG_COLS;
    return (a.precision == 0 ? sizeof(float2) : sizeof(double2)) * (size_t)a.nk * n_cb * a.test.n;
}

cudaError_t launch_rhs_reduce(const RegularArgs &a, const NearList &near, double2 *b, cudaStream_t s)
{
    const int n = a.test.n;
    if (n == 0 || a.nk == 0) return cudaSuccess;
    const int n_cb = (a.j1 - a.j0 + REG_COLS - 1) / REG_COLS;
    const int64_t items = near.nnz + (a.same_mesh ? a.trial.n : 0);
    dim3 grid((n + 255) / 256, a.nk);
    if (a.precision == 0)
        k_rhs_reduce<float2><<<grid, 256, 0, s>>>((const float2 *)a.rhs_part, n_cb, n, items, near.row_ptr,
                                                  near.row_ent, a.near_slp, a.rhs_q, a.trial.n, b);
    else
        k_rhs_reduce<double2><<<grid, 256, 0, s>>>((const double2 *)a.rhs_part, n_cb, n, items, near.row_ptr,
                                                   near.row_ent, a.near_slp, a.rhs_q, a.trial.n, b);
    return cudaGetLastError();
}

}  // namespace nihu
