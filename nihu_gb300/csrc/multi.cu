// Multiple right-hand sides: complex GEMM on the tensor cores and the
// batched vector kernels of a lockstep multi-RHS GMRES.
//
// A complex64 matrix (column-major, m x n, lda) is, viewed as floats, a real
// 2m x n matrix whose even rows hold Re A and odd rows Im A.  With the
// right-hand sides split into planes Xp = [Re X | Im X] (n x 2 nrhs), ONE real
// GEMM Z = A_r Xp (2m x 2 nrhs) reads A once and yields every real product:
//   Re Y = Z[2i, r] - Z[2i+1, nrhs + r],  Im Y = Z[2i, nrhs + r] + Z[2i+1, r].
// The GEMM runs through cuBLAS (a plain library GEMM) in one of three modes:
// FP32 on the CUDA cores, TF32 tensor cores, or BF16x9 (each FP32 operand
// split into three BF16 parts, nine tensor-core products, FP32 accumulation:
// FP32-accurate at tensor-core speed).
#include <cublas_v2.h>

#include <type_traits>

#include "kernels.h"
#include "linalg.h"

namespace nihu {

// Xp[:, r] = Re X[:, r], Xp[:, nrhs + r] = Im X[:, r] (FP32)
__global__ void k_to_planar(const double2 *__restrict__ X, int64_t n, int64_t ldx, int nrhs, float *__restrict__ Xp)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    if (i >= n) return;
    double2 v = X[(int64_t)r * ldx + i];
    Xp[(int64_t)r * n + i] = (float)v.x;
    Xp[(int64_t)(nrhs + r) * n + i] = (float)v.y;
}

// Y = alpha * (complex product from Z) + beta * Y, FP64 accumulation
__global__ void k_combine(const float *__restrict__ Z, int64_t m, int nrhs, double2 *Y, int64_t ldy, double are,
                          double aim, double bre, double bim)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    if (i >= m) return;
    const int64_t ldz = 2 * m;
    double re = (double)Z[(int64_t)r * ldz + 2 * i] - (double)Z[(int64_t)(nrhs + r) * ldz + 2 * i + 1];
    double im = (double)Z[(int64_t)(nrhs + r) * ldz + 2 * i] + (double)Z[(int64_t)r * ldz + 2 * i + 1];
    double2 y = make_double2(0.0, 0.0);
    if (bre != 0.0 || bim != 0.0) y = Y[(int64_t)r * ldy + i];
    Y[(int64_t)r * ldy + i] = make_double2(are * re - aim * im + bre * y.x - bim * y.y,
                                           are * im + aim * re + bre * y.y + bim * y.x);
}

cublasComputeType_t compute_type(int mode)
{
    if (mode == 1) return CUBLAS_COMPUTE_32F_FAST_TF32;
    if (mode == 2) return CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    return CUBLAS_COMPUTE_32F;
}

cudaError_t launch_gemm_c64(void *cublas, int mode, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *X,
                            int64_t ldx, int nrhs, double2 *Y, int64_t ldy, double are, double aim, double bre,
                            double bim, float *Xp, float *Z, cudaStream_t s, int *cublas_status)
{
    *cublas_status = 0;
    if (m == 0 || nrhs == 0) return cudaSuccess;
    dim3 gx((unsigned)((n + 255) / 256), nrhs);
    if (n > 0) k_to_planar<<<gx, 256, 0, s>>>(X, n, ldx, nrhs, Xp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cublasHandle_t h = (cublasHandle_t)cublas;
    cublasSetStream(h, s);
    const float one = 1.0f, zero = 0.0f;
    cublasStatus_t cs;
    if (n > 0) {
        cs = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)(2 * m), 2 * nrhs, (int)n, &one, A, CUDA_R_32F,
                          (int)(2 * lda), Xp, CUDA_R_32F, (int)n, &zero, Z, CUDA_R_32F, (int)(2 * m),
                          compute_type(mode), CUBLAS_GEMM_DEFAULT);
    } else {
        cs = CUBLAS_STATUS_SUCCESS;
        cudaMemsetAsync(Z, 0, sizeof(float) * 2 * m * 2 * nrhs, s);
    }
    if (cs != CUBLAS_STATUS_SUCCESS) {
        *cublas_status = (int)cs;
        return cudaSuccess;
    }
    dim3 gy((unsigned)((m + 255) / 256), nrhs);
    k_combine<<<gy, 256, 0, s>>>(Z, m, nrhs, Y, ldy, are, aim, bre, bim);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ batched
// Vectors are columns of n x nrhs complex128 blocks (leading dimension n);
// a Krylov basis V is (m + 1) such blocks stored back to back.

constexpr int BT = 256;

// part[((v * nrhs + r) * blocks + b)] = sum over the block's rows of conj(V_v[:, r]) . W[:, r];
// F32: products and the thread's and warp's sums in FP32 (the block's in FP64)
template <bool F32>
__global__ void __launch_bounds__(BT) k_bdot(const double2 *__restrict__ V, const double2 *__restrict__ W, int64_t n,
                                             int nrhs, double2 *part)
{
    __shared__ double sr[BT / 32], si[BT / 32];
    const int v = blockIdx.z, r = blockIdx.y;
    const double2 *a = V + ((int64_t)v * nrhs + r) * n;
    const double2 *b = W + (int64_t)r * n;
    using T = std::conditional_t<F32, float, double>;
    T ar = 0, ai = 0;
    for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n; i += (int64_t)gridDim.x * BT) {
        const double2 x = a[i], y = b[i];
        const T xr = (T)x.x, xi = (T)x.y, yr = (T)y.x, yi = (T)y.y;
        ar += xr * yr + xi * yi;
        ai += xr * yi - xi * yr;
    }
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = ar; si[threadIdx.x >> 5] = ai; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0, ti = 0.0;
        for (int k = 0; k < BT / 32; ++k) { tr += sr[k]; ti += si[k]; }
        part[((int64_t)v * nrhs + r) * gridDim.x + blockIdx.x] = make_double2(tr, ti);
    }
}

// out[v * nrhs + r] = sum_b part[(v * nrhs + r) * blocks + b]
__global__ void k_bdot_reduce(const double2 *__restrict__ part, int count, int blocks, double2 *out)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    double sr = 0.0, si = 0.0;
    for (int b = 0; b < blocks; ++b) {
        double2 p = part[(int64_t)t * blocks + b];
        sr += p.x;
        si += p.y;
    }
    out[t] = make_double2(sr, si);
}

// W[:, r] += sign * sum_{v < nv} V_v[:, r] h[v * nrhs + r]; F32: the sum in FP32
template <bool F32>
__global__ void k_bcombo(const double2 *__restrict__ V, int64_t n, int nrhs, int nv, const double2 *__restrict__ h,
                         double sign, double2 *W)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    if (i >= n) return;
    using T = std::conditional_t<F32, float, double>;
    T sr = 0, si = 0;
    for (int v = 0; v < nv; ++v) {
        const double2 a = V[((int64_t)v * nrhs + r) * n + i], c = h[v * nrhs + r];
        const T ar = (T)a.x, ai = (T)a.y, cr = (T)c.x, ci = (T)c.y;
        sr += ar * cr - ai * ci;
        si += ar * ci + ai * cr;
    }
    double2 acc = W[(int64_t)r * n + i];
    acc.x += sign * (double)sr;
    acc.y += sign * (double)si;
    W[(int64_t)r * n + i] = acc;
}

// dst[:, r] = src[:, r] * s[r]
__global__ void k_bscale(const double2 *__restrict__ src, double2 *dst, int64_t n, const double *__restrict__ s)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    if (i >= n) return;
    double2 v = src[(int64_t)r * n + i];
    double f = s[r];
    dst[(int64_t)r * n + i] = make_double2(v.x * f, v.y * f);
}

// R = B - R (element-wise, count complex values)
__global__ void k_rsub(const double2 *__restrict__ B, double2 *R, size_t count)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double2 b = B[i], r = R[i];
    R[i] = make_double2(b.x - r.x, b.y - r.y);
}

cudaError_t launch_rsub(const double2 *B, double2 *R, size_t count, cudaStream_t s)
{
    if (count == 0) return cudaSuccess;
    k_rsub<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(B, R, count);
    return cudaGetLastError();
}

int bdot_blocks(int64_t n)
{
    int64_t b = (n + BT * 8 - 1) / (BT * 8);
    return (int)max((int64_t)1, min(b, (int64_t)16));
}

cudaError_t launch_bdot(const double2 *V, int nv, const double2 *W, int64_t n, int nrhs, double2 *part, double2 *out,
                        cudaStream_t s, bool fp32)
{
    int blocks = bdot_blocks(n);
    dim3 g(blocks, nrhs, nv);
    if (fp32) k_bdot<true><<<g, BT, 0, s>>>(V, W, n, nrhs, part);
    else k_bdot<false><<<g, BT, 0, s>>>(V, W, n, nrhs, part);
    int count = nv * nrhs;
    k_bdot_reduce<<<(count + 255) / 256, 256, 0, s>>>(part, count, blocks, out);
    return cudaGetLastError();
}

cudaError_t launch_bcombo(const double2 *V, int64_t n, int nrhs, int nv, const double2 *h, double sign, double2 *W,
                          cudaStream_t s, bool fp32)
{
    dim3 g((unsigned)((n + 255) / 256), nrhs);
    if (fp32) k_bcombo<true><<<g, 256, 0, s>>>(V, n, nrhs, nv, h, sign, W);
    else k_bcombo<false><<<g, 256, 0, s>>>(V, n, nrhs, nv, h, sign, W);
    return cudaGetLastError();
}

cudaError_t launch_bscale(const double2 *src, double2 *dst, int64_t n, int nrhs, const double *sc, cudaStream_t s)
{
    dim3 g((unsigned)((n + 255) / 256), nrhs);
    k_bscale<<<g, 256, 0, s>>>(src, dst, n, sc);
    return cudaGetLastError();
}

}  // namespace nihu
