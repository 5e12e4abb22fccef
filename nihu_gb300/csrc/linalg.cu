// Dense linear algebra of the solve: identity shift, streamed complex matvec,
// GMRES building blocks (FP64 Gram-Schmidt) and an FP64 LU factorisation.
#include <algorithm>

#include "kernels.h"
#include "linalg.h"

namespace nihu {

// ------------------------------------------------------------------ identity

template <typename Out>
__global__ void k_add_identity(int n, double are, double aim, Out *out, int64_t ld)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Out v = out[(int64_t)i * ld + i];
    v.x += are;
    v.y += aim;
    out[(int64_t)i * ld + i] = v;
}

cudaError_t launch_add_identity(int n, double are, double aim, int dtype, void *out, int64_t ld, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    int t = 256, b = (n + t - 1) / t;
    if (dtype == 0) k_add_identity<float2><<<b, t, 0, s>>>(n, are, aim, (float2 *)out, ld);
    else k_add_identity<double2><<<b, t, 0, s>>>(n, are, aim, (double2 *)out, ld);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ matvec
//
// y = A x for column-major A (m x n).  HBM-bound: every byte of A is read
// once.  A block owns GEMV_ROWS rows of a column split; each thread owns two
// consecutive rows of a complex64 A (one 16-byte load per column) or one row of
// a complex128 A (one 16-byte load).  The split's x chunk is staged in shared
// memory.  Partial sums (FP32 products accumulated in FP32 over at most
// GEMV_SPLIT_COLS columns) are written per split and added in FP64 by
// k_gemv_reduce, which also applies alpha and beta.

constexpr int GEMV_THREADS = 256;
constexpr int GEMV_XCHUNK = 1024;

__global__ void __launch_bounds__(GEMV_THREADS) k_gemv_c64(const float2 *__restrict__ A, int64_t m, int64_t n,
                                                           int64_t lda, const double2 *__restrict__ x,
                                                           double2 *__restrict__ partial, int cols_per_split,
                                                           int64_t a_stride, const int *__restrict__ active)
{
    __shared__ float2 xs[GEMV_XCHUNK];
    if (active && !active[blockIdx.z]) return;  // converged batch member: its matrix is not read
    // batch member blockIdx.z: its matrix, vector and partial sums
    A += blockIdx.z * a_stride;
    x += blockIdx.z * n;
    partial += (int64_t)blockIdx.z * gridDim.y * m;
    const int64_t row0 = ((int64_t)blockIdx.x * GEMV_THREADS + threadIdx.x) * 2;
    const int64_t j_begin = (int64_t)blockIdx.y * cols_per_split;
    const int64_t j_end = min(n, j_begin + cols_per_split);
    float ar0 = 0.f, ai0 = 0.f, ar1 = 0.f, ai1 = 0.f;
    const bool vec = (lda % 2 == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
    for (int64_t jc = j_begin; jc < j_end; jc += GEMV_XCHUNK) {
        const int len = (int)min((int64_t)GEMV_XCHUNK, j_end - jc);
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += GEMV_THREADS) {
            double2 v = x[jc + t];
            xs[t] = make_float2((float)v.x, (float)v.y);
        }
        __syncthreads();
        if (row0 + 1 < m && vec) {
            const float4 *col = reinterpret_cast<const float4 *>(A + jc * lda + row0);
            const int64_t stride = lda / 2;
            int t = 0;
            for (; t + 8 <= len; t += 8) {
                float4 a[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) a[u] = __ldcs(col + (int64_t)(t + u) * stride);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    float2 xv = xs[t + u];
                    ar0 = fmaf(a[u].x, xv.x, ar0); ar0 = fmaf(-a[u].y, xv.y, ar0);
                    ai0 = fmaf(a[u].x, xv.y, ai0); ai0 = fmaf(a[u].y, xv.x, ai0);
                    ar1 = fmaf(a[u].z, xv.x, ar1); ar1 = fmaf(-a[u].w, xv.y, ar1);
                    ai1 = fmaf(a[u].z, xv.y, ai1); ai1 = fmaf(a[u].w, xv.x, ai1);
                }
            }
            for (; t < len; ++t) {
                float4 av = __ldcs(col + (int64_t)t * stride);
                float2 xv = xs[t];
                ar0 = fmaf(av.x, xv.x, ar0); ar0 = fmaf(-av.y, xv.y, ar0);
                ai0 = fmaf(av.x, xv.y, ai0); ai0 = fmaf(av.y, xv.x, ai0);
                ar1 = fmaf(av.z, xv.x, ar1); ar1 = fmaf(-av.w, xv.y, ar1);
                ai1 = fmaf(av.z, xv.y, ai1); ai1 = fmaf(av.w, xv.x, ai1);
            }
        } else {
            for (int t = 0; t < len; ++t) {
                float2 xv = xs[t];
                if (row0 < m) {
                    float2 av = A[(jc + t) * lda + row0];
                    ar0 = fmaf(av.x, xv.x, ar0); ar0 = fmaf(-av.y, xv.y, ar0);
                    ai0 = fmaf(av.x, xv.y, ai0); ai0 = fmaf(av.y, xv.x, ai0);
                }
                if (row0 + 1 < m) {
                    float2 av = A[(jc + t) * lda + row0 + 1];
                    ar1 = fmaf(av.x, xv.x, ar1); ar1 = fmaf(-av.y, xv.y, ar1);
                    ai1 = fmaf(av.x, xv.y, ai1); ai1 = fmaf(av.y, xv.x, ai1);
                }
            }
        }
    }
    double2 *dst = partial + (int64_t)blockIdx.y * m;
    if (row0 < m) dst[row0] = make_double2(ar0, ai0);
    if (row0 + 1 < m) dst[row0 + 1] = make_double2(ar1, ai1);
}

__global__ void __launch_bounds__(GEMV_THREADS) k_gemv_c128(const double2 *__restrict__ A, int64_t m, int64_t n,
                                                            int64_t lda, const double2 *__restrict__ x,
                                                            double2 *__restrict__ partial, int cols_per_split,
                                                            int64_t a_stride, const int *__restrict__ active)
{
    __shared__ double2 xs[GEMV_XCHUNK];
    if (active && !active[blockIdx.z]) return;
    A += blockIdx.z * a_stride;
    x += blockIdx.z * n;
    partial += (int64_t)blockIdx.z * gridDim.y * m;
    const int64_t row = (int64_t)blockIdx.x * GEMV_THREADS + threadIdx.x;
    const int64_t j_begin = (int64_t)blockIdx.y * cols_per_split;
    const int64_t j_end = min(n, j_begin + cols_per_split);
    double ar = 0.0, ai = 0.0;
    for (int64_t jc = j_begin; jc < j_end; jc += GEMV_XCHUNK) {
        const int len = (int)min((int64_t)GEMV_XCHUNK, j_end - jc);
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += GEMV_THREADS) xs[t] = x[jc + t];
        __syncthreads();
        if (row < m) {
            const double2 *col = A + jc * lda + row;
            int t = 0;
            for (; t + 4 <= len; t += 4) {
                double2 a[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) a[u] = __ldcs(col + (int64_t)(t + u) * lda);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    double2 xv = xs[t + u];
                    ar = fma(a[u].x, xv.x, ar); ar = fma(-a[u].y, xv.y, ar);
                    ai = fma(a[u].x, xv.y, ai); ai = fma(a[u].y, xv.x, ai);
                }
            }
            for (; t < len; ++t) {
                double2 av = col[(int64_t)t * lda];
                double2 xv = xs[t];
                ar = fma(av.x, xv.x, ar); ar = fma(-av.y, xv.y, ar);
                ai = fma(av.x, xv.y, ai); ai = fma(av.y, xv.x, ai);
            }
        }
    }
    if (row < m) partial[(int64_t)blockIdx.y * m + row] = make_double2(ar, ai);
}

// y = alpha * sum_s partial[s] + beta * y  (batch member blockIdx.y)
__global__ void k_gemv_reduce(const double2 *__restrict__ partial, int splits, int64_t m, double2 *y, double are,
                              double aim, double bre, double bim, const int *__restrict__ active)
{
    if (active && !active[blockIdx.y]) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    partial += (int64_t)blockIdx.y * splits * m;
    y += (int64_t)blockIdx.y * m;
    if (i >= m) return;
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < splits; ++s) {
        double2 v = partial[(int64_t)s * m + i];
        sr += v.x;
        si += v.y;
    }
    double2 yo = make_double2(0.0, 0.0);
    if (bre != 0.0 || bim != 0.0) yo = y[i];
    y[i] = make_double2(are * sr - aim * si + bre * yo.x - bim * yo.y, are * si + aim * sr + bre * yo.y + bim * yo.x);
}

int gemv_splits(int64_t m, int64_t n, int dtype)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t rows_per_block = dtype == 0 ? 2 * GEMV_THREADS : GEMV_THREADS;
    int64_t row_blocks = (m + rows_per_block - 1) / rows_per_block;
    int64_t want = (int64_t)sms * 4;
    int64_t splits = (want + row_blocks - 1) / row_blocks;
    // at least 256 columns per split keeps the partial traffic negligible
    splits = min(splits, max((int64_t)1, n / 256));
    return (int)max((int64_t)1, min(splits, (int64_t)1024));
}

cudaError_t launch_gemv_batched(int dtype, const void *A, int64_t m, int64_t n, int64_t lda, int64_t a_stride,
                                int batch, const double2 *x, double2 *y, double are, double aim, double bre,
                                double bim, double2 *partial, int splits, cudaStream_t s, const int *active)
{
    if (m == 0 || batch == 0) return cudaSuccess;
    int cols_per_split = (int)((n + splits - 1) / splits);
    if (n == 0) cols_per_split = 0;
    if (dtype == 0) {
        dim3 grid((unsigned)((m + 2 * GEMV_THREADS - 1) / (2 * GEMV_THREADS)), splits, batch);
        k_gemv_c64<<<grid, GEMV_THREADS, 0, s>>>((const float2 *)A, m, n, lda, x, partial, cols_per_split, a_stride,
                                                  active);
    } else {
        dim3 grid((unsigned)((m + GEMV_THREADS - 1) / GEMV_THREADS), splits, batch);
        k_gemv_c128<<<grid, GEMV_THREADS, 0, s>>>((const double2 *)A, m, n, lda, x, partial, cols_per_split,
                                                   a_stride, active);
    }
    dim3 rgrid((unsigned)((m + 255) / 256), batch);
    k_gemv_reduce<<<rgrid, 256, 0, s>>>(partial, splits, m, y, are, aim, bre, bim, active);
    return cudaGetLastError();
}

cudaError_t launch_gemv(int dtype, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *x, double2 *y,
                        double are, double aim, double bre, double bim, double2 *partial, int splits, cudaStream_t s)
{
    return launch_gemv_batched(dtype, A, m, n, lda, 0, 1, x, y, are, aim, bre, bim, partial, splits, s, nullptr);
}

// out(i, i) += alpha on `batch` matrices spaced `stride` elements apart
template <typename Out>
__global__ void k_add_identity_batched(int n, double are, double aim, Out *out, int64_t ld, int64_t stride)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Out *p = out + blockIdx.y * stride + (int64_t)i * ld + i;
    Out v = *p;
    v.x += are;
    v.y += aim;
    *p = v;
}

cudaError_t launch_add_identity_batched(int n, double are, double aim, int dtype, void *out, int64_t ld, int64_t stride,
                                        int batch, cudaStream_t s)
{
    if (n == 0 || batch == 0) return cudaSuccess;
    dim3 g((n + 255) / 256, batch);
    if (dtype == 0) k_add_identity_batched<float2><<<g, 256, 0, s>>>(n, are, aim, (float2 *)out, ld, stride);
    else k_add_identity_batched<double2><<<g, 256, 0, s>>>(n, are, aim, (double2 *)out, ld, stride);
    return cudaGetLastError();
}

__global__ void k_permute_segments(const double2 *__restrict__ src, double2 *__restrict__ dst,
                                   const int64_t *__restrict__ src_off, const int64_t *__restrict__ dst_off,
                                   const int *__restrict__ len)
{
    const int t = blockIdx.y;
    const int n = len[t];
    const double2 *a = src + src_off[t];
    double2 *b = dst + dst_off[t];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}

cudaError_t launch_permute_segments(const double2 *src, double2 *dst, const int64_t *src_off, const int64_t *dst_off,
                                    const int *len, int count, int max_len, cudaStream_t s)
{
    if (count == 0 || max_len == 0) return cudaSuccess;
    dim3 g((unsigned)std::min(64, (max_len + 255) / 256), count);
    k_permute_segments<<<g, 256, 0, s>>>(src, dst, src_off, dst_off, len);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ GMRES
//
// Classical Gram-Schmidt with one reorthogonalisation (CGS2) on FP64 basis
// vectors V[0..k] (each n complex128, contiguous).  Dot products produce
// per-block partial sums that the host adds (it needs them for the Givens
// rotations anyway).

constexpr int DOT_THREADS = 256;

// partial[(v * gridDim.x + b)] = sum over the block's rows of conj(V[v]) . w
__global__ void __launch_bounds__(DOT_THREADS) k_multidot(const double2 *__restrict__ V, int64_t n, int nv,
                                                           const double2 *__restrict__ w, double2 *partial)
{
    __shared__ double sr[DOT_THREADS / 32], si[DOT_THREADS / 32];
    const int v = blockIdx.y;
    const double2 *vec = V + (int64_t)v * n;
    double ar = 0.0, ai = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * DOT_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * DOT_THREADS) {
        double2 a = vec[i], b = w[i];
        ar += a.x * b.x + a.y * b.y;
        ai += a.x * b.y - a.y * b.x;
    }
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sr[wid] = ar; si[wid] = ai; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0, ti = 0.0;
        for (int k = 0; k < DOT_THREADS / 32; ++k) { tr += sr[k]; ti += si[k]; }
        partial[(int64_t)v * gridDim.x + blockIdx.x] = make_double2(tr, ti);
    }
}

// w -= sum_v V[v] h[v]
__global__ void k_subtract_combo(const double2 *__restrict__ V, int64_t n, int nv, const double2 *__restrict__ h,
                                 double2 *w)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = w[i];
    for (int v = 0; v < nv; ++v) {
        double2 a = V[(int64_t)v * n + i], c = h[v];
        acc.x -= a.x * c.x - a.y * c.y;
        acc.y -= a.x * c.y + a.y * c.x;
    }
    w[i] = acc;
}

// x += sum_v V[v] y[v]
__global__ void k_add_combo(const double2 *__restrict__ V, int64_t n, int nv, const double2 *__restrict__ yv,
                            double2 *x)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = x[i];
    for (int v = 0; v < nv; ++v) {
        double2 a = V[(int64_t)v * n + i], c = yv[v];
        acc.x += a.x * c.x - a.y * c.y;
        acc.y += a.x * c.y + a.y * c.x;
    }
    x[i] = acc;
}

// dst = src * s (real scale)
__global__ void k_scale_copy(const double2 *__restrict__ src, double2 *dst, int64_t n, double s)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 v = src[i];
    dst[i] = make_double2(v.x * s, v.y * s);
}

// dst = a - b
__global__ void k_sub(const double2 *__restrict__ a, const double2 *__restrict__ b, double2 *dst, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 u = a[i], v = b[i];
    dst[i] = make_double2(u.x - v.x, u.y - v.y);
}

int dot_blocks(int64_t n)
{
    int64_t b = (n + DOT_THREADS * 4 - 1) / (DOT_THREADS * 4);
    return (int)max((int64_t)1, min(b, (int64_t)64));
}

cudaError_t launch_multidot(const double2 *V, int64_t n, int nv, const double2 *w, double2 *partial, int blocks,
                            cudaStream_t s)
{
    dim3 grid(blocks, nv);
    k_multidot<<<grid, DOT_THREADS, 0, s>>>(V, n, nv, w, partial);
    return cudaGetLastError();
}

cudaError_t launch_subtract_combo(const double2 *V, int64_t n, int nv, const double2 *h, double2 *w, cudaStream_t s)
{
    k_subtract_combo<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V, n, nv, h, w);
    return cudaGetLastError();
}

cudaError_t launch_add_combo(const double2 *V, int64_t n, int nv, const double2 *y, double2 *x, cudaStream_t s)
{
    k_add_combo<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V, n, nv, y, x);
    return cudaGetLastError();
}

cudaError_t launch_scale_copy(const double2 *src, double2 *dst, int64_t n, double sc, cudaStream_t s)
{
    k_scale_copy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n, sc);
    return cudaGetLastError();
}

cudaError_t launch_sub(const double2 *a, const double2 *b, double2 *dst, int64_t n, cudaStream_t s)
{
    k_sub<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, dst, n);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ LU
//
// Right-looking LU with partial pivoting, FP64 complex, column-major.  Per
// column: pivot search (one block), row swap + scaling, rank-1 update of the
// trailing block.  Then forward/back substitution in single-block kernels.

__device__ __forceinline__ double cabs2(double2 v) { return v.x * v.x + v.y * v.y; }

// step k of the factorisation, one block: the pivot (largest |A[i][k]|, i >= k,
// lowest index on ties), the swap of rows k and piv[k] across all columns, and
// column k below the diagonal divided by the pivot
__global__ void __launch_bounds__(1024) k_lu_pivot_swap_scale(double2 *A, int64_t n, int64_t lda, int k, int *piv,
                                                              int *info)
{
    __shared__ double best[32];
    __shared__ int besti[32];
    __shared__ int pk;
    double bv = -1.0;
    int bi = k;
    for (int64_t i = k + threadIdx.x; i < n; i += blockDim.x) {
        double v = cabs2(A[(int64_t)k * lda + i]);
        if (v > bv) { bv = v; bi = (int)i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { best[wid] = bv; besti[wid] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = (blockDim.x + 31) / 32;
        bv = best[0];
        bi = besti[0];
        for (int w = 1; w < nw; ++w)
            if (best[w] > bv || (best[w] == bv && besti[w] < bi)) { bv = best[w]; bi = besti[w]; }
        piv[k] = bi;
        pk = bi;
        if (bv == 0.0 && *info == 0) *info = k + 1;
    }
    __syncthreads();
    const int p = pk;
    if (p != k)
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            double2 t = A[j * lda + k];
            A[j * lda + k] = A[j * lda + p];
            A[j * lda + p] = t;
        }
    __syncthreads();
    double2 d = A[(int64_t)k * lda + k];
    double den = d.x * d.x + d.y * d.y;
    if (den == 0.0) return;
    double2 inv = make_double2(d.x / den, -d.y / den);
    for (int64_t i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
        double2 v = A[(int64_t)k * lda + i];
        A[(int64_t)k * lda + i] = make_double2(v.x * inv.x - v.y * inv.y, v.x * inv.y + v.y * inv.x);
    }
}

// A[i][j] -= A[i][k] A[k][j] for i, j > k (16 x 16 tiles)
__global__ void k_lu_update(double2 *A, int64_t n, int64_t lda, int k)
{
    int64_t i = k + 1 + (int64_t)blockIdx.x * 16 + threadIdx.x;
    int64_t j = k + 1 + (int64_t)blockIdx.y * 16 + threadIdx.y;
    if (i >= n || j >= n) return;
    double2 l = A[(int64_t)k * lda + i], u = A[j * lda + k];
    double2 v = A[j * lda + i];
    v.x -= l.x * u.x - l.y * u.y;
    v.y -= l.x * u.y + l.y * u.x;
    A[j * lda + i] = v;
}

// x = b permuted, then L y = x (unit lower), U x = y; single block
__global__ void __launch_bounds__(1024) k_lu_solve(const double2 *A, int64_t n, int64_t lda, const int *piv,
                                                    const double2 *b, double2 *x)
{
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int64_t k = 0; k < n; ++k) {
            int p = piv[k];
            if (p != k) { double2 t = x[k]; x[k] = x[p]; x[p] = t; }
        }
    __syncthreads();
    for (int64_t k = 0; k < n; ++k) {
        double2 xk = x[k];
        for (int64_t i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
            double2 l = A[k * lda + i];
            double2 v = x[i];
            v.x -= l.x * xk.x - l.y * xk.y;
            v.y -= l.x * xk.y + l.y * xk.x;
            x[i] = v;
        }
        __syncthreads();
    }
    for (int64_t k = n - 1; k >= 0; --k) {
        if (threadIdx.x == 0) {
            double2 d = A[k * lda + k], v = x[k];
            double den = d.x * d.x + d.y * d.y;
            x[k] = make_double2((v.x * d.x + v.y * d.y) / den, (v.y * d.x - v.x * d.y) / den);
        }
        __syncthreads();
        double2 xk = x[k];
        for (int64_t i = threadIdx.x; i < k; i += blockDim.x) {
            double2 u = A[k * lda + i];
            double2 v = x[i];
            v.x -= u.x * xk.x - u.y * xk.y;
            v.y -= u.x * xk.y + u.y * xk.x;
            x[i] = v;
        }
        __syncthreads();
    }
}

cudaError_t launch_lu_factor(double2 *A, int64_t n, int64_t lda, int *piv, int *info, int64_t *launches,
                             cudaStream_t s)
{
    for (int k = 0; k < n; ++k) {
        k_lu_pivot_swap_scale<<<1, 1024, 0, s>>>(A, n, lda, k, piv, info);
        int64_t rem = n - k - 1;
        if (rem > 0) {
            dim3 grid((unsigned)((rem + 15) / 16), (unsigned)((rem + 15) / 16));
            k_lu_update<<<grid, dim3(16, 16), 0, s>>>(A, n, lda, k);
        }
        *launches += rem > 0 ? 2 : 1;
    }
    return cudaGetLastError();
}

cudaError_t launch_lu_solve(const double2 *A, int64_t n, int64_t lda, const int *piv, const double2 *b, double2 *x,
                            cudaStream_t s)
{
    k_lu_solve<<<1, 1024, 0, s>>>(A, n, lda, piv, b, x);
    return cudaGetLastError();
}

// --------------------------------------------------- mixed-precision LU
//
// Complex LU with partial pivoting in FP32, blocked by LU32_NB columns: each
// panel is factorised by one CTA in shared memory (pivot search, row swap,
// scaling and the panel's rank-1 updates), its row swaps are applied to the
// other columns, the panel's rows of U come from a unit-lower triangular
// solve, and the trailing matrix takes one rank-LU32_NB update.  The FP64
// caller refines the solution with the FP64 matrix (residual b - A x in FP64,
// corrections from these factors), so the FP32 factors set the speed and the
// FP64 residual the accuracy.  Row swaps are applied to every column (the
// factors are those of P A = L U, pivots as LAPACK's getrf records them).

constexpr int LU32_NB = 16;
constexpr int LU32_THREADS = 1024;

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// B (n x n, leading dimension n) = A rounded to complex64
__global__ void k_to_c64(const double2 *__restrict__ A, int64_t lda, int n, float2 *__restrict__ B)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n) return;
    const double2 v = A[(int64_t)j * lda + i];
    B[(int64_t)j * n + i] = make_float2((float)v.x, (float)v.y);
}

// panel [j0, j0 + nb) of the n x n matrix A (leading dimension n), rows j0..n
// in shared memory; piv[j0 + kk] = the global pivot row of column j0 + kk;
// info = 1 + the first column with a zero pivot
__global__ void __launch_bounds__(LU32_THREADS) k_lu32_panel(float2 *A, int n, int j0, int nb, int *piv, int *info)
{
    extern __shared__ float2 P[];  // column c of the panel at P + c * m
    __shared__ float wbest[LU32_THREADS / 32];
    __shared__ int wbi[LU32_THREADS / 32];
    __shared__ int s_p;
    __shared__ float2 s_d, s_dk;  // the pivot and the old diagonal entry of the current column
    const int m = n - j0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float2 *G = A + (int64_t)j0 * n + j0;
    for (int c = 0; c < nb; ++c)
        for (int r = tid; r < m; r += blockDim.x) P[c * m + r] = G[(int64_t)c * n + r];
    __syncthreads();
    for (int kk = 0; kk < nb; ++kk) {
        float2 *col = P + kk * m;
        float bv = -1.0f;
        int bi = kk;
        for (int r = kk + tid; r < m; r += blockDim.x) {
            const float v = col[r].x * col[r].x + col[r].y * col[r].y;
            if (v > bv) {
                bv = v;
                bi = r;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            wbest[warp] = bv;
            wbi[warp] = bi;
        }
        __syncthreads();
        if (warp == 0) {
            bv = wbest[lane];
            bi = wbi[lane];
            for (int o = 16; o > 0; o >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane == 0) {
                s_p = bi;
                s_d = col[bi];
                s_dk = col[kk];
                piv[j0 + kk] = j0 + bi;
                if (!(bv > 0.0f) && *info == 0) *info = j0 + kk + 1;
            }
        }
        __syncthreads();
        // swap rows kk and p (columns other than kk) and, in the same pass,
        // column kk: the pivot to row kk, the rest divided by it
        const int p = s_p;
        const float2 d = s_d, dk = s_dk;
        if (p != kk && tid < nb && tid != kk) {
            const float2 t = P[tid * m + kk];
            P[tid * m + kk] = P[tid * m + p];
            P[tid * m + p] = t;
        }
        const float den = d.x * d.x + d.y * d.y;
        const float2 inv = den > 0.0f ? make_float2(d.x / den, -d.y / den) : make_float2(1.0f, 0.0f);
        for (int r = kk + 1 + tid; r < m; r += blockDim.x) {
            const float2 v = r == p ? dk : col[r];
            col[r] = den > 0.0f ? cmulf(v, inv) : v;
        }
        __syncthreads();
        if (tid == 0) col[kk] = d;
        // rank-1 update of the panel's later columns, one row per thread
        for (int r = kk + 1 + tid; r < m; r += blockDim.x) {
            const float2 l = col[r];
            for (int c = kk + 1; c < nb; ++c) {
                const float2 u = P[c * m + kk];
                float2 v = P[c * m + r];
                v.x -= l.x * u.x - l.y * u.y;
                v.y -= l.x * u.y + l.y * u.x;
                P[c * m + r] = v;
            }
        }
        __syncthreads();
    }
    for (int c = 0; c < nb; ++c)
        for (int r = tid; r < m; r += blockDim.x) G[(int64_t)c * n + r] = P[c * m + r];
}

// the panel's row swaps on every column outside [j0, j0 + nb), in order
__global__ void k_lu32_swap(float2 *A, int n, int j0, int nb, const int *__restrict__ piv)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n || (j >= j0 && j < j0 + nb)) return;
    float2 *col = A + (int64_t)j * n;
    for (int kk = 0; kk < nb; ++kk) {
        const int p = piv[j0 + kk];
        if (p != j0 + kk) {
            const float2 t = col[j0 + kk];
            col[j0 + kk] = col[p];
            col[p] = t;
        }
    }
}

// rows [j0, j0 + nb) of columns j >= j0 + nb: U12 = L11^{-1} A12 (unit lower L11)
__global__ void __launch_bounds__(256) k_lu32_trsm(float2 *A, int n, int j0, int nb)
{
    __shared__ float2 L[LU32_NB][LU32_NB];
    for (int t = threadIdx.x; t < LU32_NB * LU32_NB; t += blockDim.x) {
        const int r = t % LU32_NB, c = t / LU32_NB;
        L[r][c] = (r < nb && c < nb) ? A[(int64_t)(j0 + c) * n + j0 + r] : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    const int j = j0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float2 *col = A + (int64_t)j * n + j0;
    float2 x[LU32_NB];
#pragma unroll
    for (int r = 0; r < LU32_NB; ++r) x[r] = r < nb ? col[r] : make_float2(0.0f, 0.0f);
#pragma unroll
    for (int r = 1; r < LU32_NB; ++r)
#pragma unroll
        for (int q = 0; q < r; ++q) {
            const float2 l = L[r][q];
            x[r].x -= l.x * x[q].x - l.y * x[q].y;
            x[r].y -= l.x * x[q].y + l.y * x[q].x;
        }
#pragma unroll
    for (int r = 0; r < LU32_NB; ++r)
        if (r < nb) col[r] = x[r];
}

// A22 -= L21 U12 on the trailing matrix (rows and columns >= j0 + nb), one
// 64 x 64 tile per 256-thread block, 4 x 4 entries per thread
__global__ void __launch_bounds__(256) k_lu32_update(float2 *A, int n, int j0, int nb)
{
    __shared__ float2 Ls[LU32_NB][64], Us[LU32_NB][64];
    const int base = j0 + nb;
    const int i0 = base + blockIdx.x * 64, c0 = base + blockIdx.y * 64;
    const int tid = threadIdx.x;
    for (int t = tid; t < 64 * LU32_NB; t += 256) {
        const int q = t / 64, ii = t % 64;
        const int i = i0 + ii;
        Ls[q][ii] = (q < nb && i < n) ? A[(int64_t)(j0 + q) * n + i] : make_float2(0.0f, 0.0f);
        const int jj = t / LU32_NB, qq = t % LU32_NB;
        const int c = c0 + jj;
        Us[qq][jj] = (qq < nb && c < n) ? A[(int64_t)c * n + j0 + qq] : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    float2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.0f, 0.0f);
    for (int q = 0; q < nb; ++q) {
        float2 l[4], u[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) l[a] = Ls[q][tx + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) u[b] = Us[q][ty * 4 + b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                acc[a][b].x += l[a].x * u[b].x - l[a].y * u[b].y;
                acc[a][b].y += l[a].x * u[b].y + l[a].y * u[b].x;
            }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int c = c0 + ty * 4 + b;
        if (c >= n) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int i = i0 + tx + 16 * a;
            if (i >= n) continue;
            float2 *p = A + (int64_t)c * n + i;
            float2 v = *p;
            v.x -= acc[a][b].x;
            v.y -= acc[a][b].y;
            *p = v;
        }
    }
}

// d = U^{-1} L^{-1} P r from the FP32 factors (one CTA, the vector in shared
// memory): the pivots in order, then blocks of 32 rows -- warp 0 solves the
// diagonal block, every thread updates the remaining rows
// rows [i_begin, i_end) of y less the block's 32 columns (or bn < 32) of the
// factor times y[b0 ..]: loads issued 8 at a time
__device__ __forceinline__ void lu32_block_update(const float2 *__restrict__ A, int n, float2 *y, int b0, int bn,
                                                  int i_begin, int i_end)
{
    for (int i = i_begin + threadIdx.x; i < i_end; i += blockDim.x) {
        float2 acc = y[i];
        if (bn == 32) {
#pragma unroll 8
            for (int q = 0; q < 32; ++q) {
                const float2 l = A[(int64_t)(b0 + q) * n + i], yq = y[b0 + q];
                acc.x -= l.x * yq.x - l.y * yq.y;
                acc.y -= l.x * yq.y + l.y * yq.x;
            }
        } else {
            for (int q = 0; q < bn; ++q) {
                const float2 l = A[(int64_t)(b0 + q) * n + i], yq = y[b0 + q];
                acc.x -= l.x * yq.x - l.y * yq.y;
                acc.y -= l.x * yq.y + l.y * yq.x;
            }
        }
        y[i] = acc;
    }
}

__global__ void __launch_bounds__(LU32_THREADS) k_lu32_solve(const float2 *__restrict__ A, int n,
                                                             const int *__restrict__ piv, const double2 *__restrict__ r,
                                                             double2 *__restrict__ d)
{
    extern __shared__ float2 y[];
    __shared__ float2 D[32][33];  // the current diagonal block, D[row][col]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < n; i += blockDim.x) y[i] = make_float2((float)r[i].x, (float)r[i].y);
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < n; ++k) {
            const int p = piv[k];
            if (p != k) {
                const float2 t = y[k];
                y[k] = y[p];
                y[p] = t;
            }
        }
    __syncthreads();
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int bn = min(32, n - b0);
        for (int t = tid; t < bn * bn; t += blockDim.x) {
            const int c = t / bn, rr = t - c * bn;
            D[rr][c] = A[(int64_t)(b0 + c) * n + b0 + rr];
        }
        __syncthreads();
        if (warp == 0) {
            float2 v = lane < bn ? y[b0 + lane] : make_float2(0.0f, 0.0f);
            for (int q = 0; q < bn - 1; ++q) {
                const float2 yq = make_float2(__shfl_sync(0xffffffffu, v.x, q), __shfl_sync(0xffffffffu, v.y, q));
                if (lane > q && lane < bn) {
                    const float2 l = D[lane][q];
                    v.x -= l.x * yq.x - l.y * yq.y;
                    v.y -= l.x * yq.y + l.y * yq.x;
                }
            }
            if (lane < bn) y[b0 + lane] = v;
        }
        __syncthreads();
        lu32_block_update(A, n, y, b0, bn, b0 + bn, n);
        __syncthreads();
    }
    for (int b1 = n; b1 > 0; b1 -= 32) {
        const int b0 = max(0, b1 - 32), bn = b1 - b0;
        for (int t = tid; t < bn * bn; t += blockDim.x) {
            const int c = t / bn, rr = t - c * bn;
            D[rr][c] = A[(int64_t)(b0 + c) * n + b0 + rr];
        }
        __syncthreads();
        if (warp == 0) {
            float2 v = lane < bn ? y[b0 + lane] : make_float2(0.0f, 0.0f);
            for (int q = bn - 1; q >= 0; --q) {
                if (lane == q) {
                    const float2 u = D[q][q];
                    const float den = u.x * u.x + u.y * u.y;
                    v = make_float2((v.x * u.x + v.y * u.y) / den, (v.y * u.x - v.x * u.y) / den);
                }
                const float2 yq = make_float2(__shfl_sync(0xffffffffu, v.x, q), __shfl_sync(0xffffffffu, v.y, q));
                if (lane < q) {
                    const float2 u = D[lane][q];
                    v.x -= u.x * yq.x - u.y * yq.y;
                    v.y -= u.x * yq.y + u.y * yq.x;
                }
            }
            if (lane < bn) y[b0 + lane] = v;
        }
        __syncthreads();
        lu32_block_update(A, n, y, b0, bn, 0, b0);
        __syncthreads();
    }
    for (int i = tid; i < n; i += blockDim.x) d[i] = make_double2((double)y[i].x, (double)y[i].y);
}

// x += d; sums[0] = |d|^2, sums[1] = |x|^2 (one block, fixed order)
__global__ void __launch_bounds__(1024) k_lu32_update_x(double2 *x, const double2 *__restrict__ d, int n, double *sums)
{
    __shared__ double sd[32], sx[32];
    double ad = 0.0, ax = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 di = d[i];
        double2 xi = x[i];
        xi.x += di.x;
        xi.y += di.y;
        x[i] = xi;
        ad += di.x * di.x + di.y * di.y;
        ax += xi.x * xi.x + xi.y * xi.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ad += __shfl_xor_sync(0xffffffffu, ad, o);
        ax += __shfl_xor_sync(0xffffffffu, ax, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sd[threadIdx.x >> 5] = ad;
        sx[threadIdx.x >> 5] = ax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double td = 0.0, tx = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
            td += sd[w];
            tx += sx[w];
        }
        sums[0] = td;
        sums[1] = tx;
    }
}

size_t lu32_solve_smem(int n) { return sizeof(float2) * (size_t)n; }

// columns of the panel at j0: as many as LU32_NB and the shared memory allow
static int lu32_panel_cols(int n, int j0, size_t smem_max)
{
    const size_t per_col = sizeof(float2) * (size_t)(n - j0);
    return (int)std::min<size_t>({(size_t)LU32_NB, (size_t)(n - j0), smem_max / per_col});
}

// dynamic shared memory a kernel may take: the per-block limit less its static part
template <typename K>
static size_t dyn_smem_max(K kernel, size_t smem_max)
{
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return smem_max > fa.sharedSizeBytes ? smem_max - fa.sharedSizeBytes : 0;
}

bool lu32_fits(int n, size_t smem_max)
{
    return n >= 1 && n <= 65535 && lu32_panel_cols(n, 0, dyn_smem_max(k_lu32_panel, smem_max)) >= 1 &&
           lu32_solve_smem(n) <= dyn_smem_max(k_lu32_solve, smem_max);
}

cudaError_t lu32_prepare(int n, size_t smem_max, size_t *panel_smem)
{
    if (!lu32_fits(n, smem_max)) return cudaErrorInvalidValue;
    // every panel's shared memory (n - j0 rows x its columns) is within the limit
    *panel_smem = dyn_smem_max(k_lu32_panel, smem_max);
    cudaError_t e = cudaFuncSetAttribute(k_lu32_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*panel_smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_lu32_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lu32_solve_smem(n));
    return e;
}

cudaError_t launch_to_c64(const double2 *A, int64_t lda, int n, float2 *F, cudaStream_t s)
{
    k_to_c64<<<dim3((n + 255) / 256, n), 256, 0, s>>>(A, lda, n, F);
    return cudaGetLastError();
}

cudaError_t launch_lu32_factor(float2 *F, int n, int *piv, int *info, size_t panel_smem, int64_t *launches,
                               cudaStream_t s)
{
    const size_t smem_max = panel_smem;
    for (int j0 = 0, nb; j0 < n; j0 += nb) {
        nb = lu32_panel_cols(n, j0, smem_max);
        k_lu32_panel<<<1, LU32_THREADS, sizeof(float2) * (size_t)(n - j0) * nb, s>>>(F, n, j0, nb, piv, info);
        k_lu32_swap<<<(n + 255) / 256, 256, 0, s>>>(F, n, j0, nb, piv);
        *launches += 2;
        const int rest = n - j0 - nb;
        if (rest > 0) {
            k_lu32_trsm<<<(rest + 255) / 256, 256, 0, s>>>(F, n, j0, nb);
            const unsigned t = (unsigned)((rest + 63) / 64);
            k_lu32_update<<<dim3(t, t), 256, 0, s>>>(F, n, j0, nb);
            *launches += 2;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_lu32_solve(const float2 *F, int n, const int *piv, const double2 *r, double2 *d, cudaStream_t s)
{
    k_lu32_solve<<<1, LU32_THREADS, lu32_solve_smem(n), s>>>(F, n, piv, r, d);
    return cudaGetLastError();
}

cudaError_t launch_lu32_update_x(double2 *x, const double2 *d, int n, double *sums, cudaStream_t s)
{
    k_lu32_update_x<<<1, 1024, 0, s>>>(x, d, n, sums);
    return cudaGetLastError();
}

}  // namespace nihu
