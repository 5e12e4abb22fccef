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

}  // namespace nihu
