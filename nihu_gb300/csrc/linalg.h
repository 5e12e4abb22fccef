// Internal launchers of the dense linear algebra kernels (linalg.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nihu {

// number of column splits of a matvec (partial buffer holds splits * m complex128)
int gemv_splits(int64_t m, int64_t n, int dtype);
cudaError_t launch_gemv(int dtype, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *x, double2 *y,
                        double are, double aim, double bre, double bim, double2 *partial, int splits, cudaStream_t s);

// batch members b = 0..batch-1: y_b = alpha A_b x_b + beta y_b with
// A_b = A + b * a_stride (elements), x_b = x + b * n, y_b = y + b * m;
// partial holds batch * splits * m complex128; active (device, may be NULL)
// skips members whose flag is 0 (their y is left untouched)
cudaError_t launch_gemv_batched(int dtype, const void *A, int64_t m, int64_t n, int64_t lda, int64_t a_stride,
                                int batch, const double2 *x, double2 *y, double are, double aim, double bre,
                                double bim, double2 *partial, int splits, cudaStream_t s, const int *active);
cudaError_t launch_add_identity_batched(int n, double are, double aim, int dtype, void *out, int64_t ld, int64_t stride,
                                        int batch, cudaStream_t s);
// segment t: dst[dst_off[t] + i] = src[src_off[t] + i] for i < len[t]
// (device tables of count entries; max_len bounds every len[t])
cudaError_t launch_permute_segments(const double2 *src, double2 *dst, const int64_t *src_off, const int64_t *dst_off,
                                    const int *len, int count, int max_len, cudaStream_t s);

int dot_blocks(int64_t n);
cudaError_t launch_multidot(const double2 *V, int64_t n, int nv, const double2 *w, double2 *partial, int blocks,
                            cudaStream_t s);
cudaError_t launch_subtract_combo(const double2 *V, int64_t n, int nv, const double2 *h, double2 *w, cudaStream_t s);
cudaError_t launch_add_combo(const double2 *V, int64_t n, int nv, const double2 *y, double2 *x, cudaStream_t s);
cudaError_t launch_scale_copy(const double2 *src, double2 *dst, int64_t n, double sc, cudaStream_t s);
cudaError_t launch_sub(const double2 *a, const double2 *b, double2 *dst, int64_t n, cudaStream_t s);

cudaError_t launch_lu_factor(double2 *A, int64_t n, int64_t lda, int *piv, int *info, int64_t *launches,
                             cudaStream_t s);
// mixed-precision LU (FP32 factors of the FP64 matrix, refined by the caller):
// whether order n fits the kernels' shared memory (smem_max: the device's
// per-block opt-in limit), and the solve kernel's shared memory
bool lu32_fits(int n, size_t smem_max);
size_t lu32_solve_smem(int n);
// kernel attributes for order n (outside any stream capture); panel_smem
// receives the panel kernel's dynamic shared memory limit
cudaError_t lu32_prepare(int n, size_t smem_max, size_t *panel_smem);
// F (n x n complex64, leading dimension n) = A rounded to complex64
cudaError_t launch_to_c64(const double2 *A, int64_t lda, int n, float2 *F, cudaStream_t s);
// F in place = its FP32 LU factors with partial pivoting (piv as getrf,
// info = 1 + first zero pivot column); stream-capturable
cudaError_t launch_lu32_factor(float2 *F, int n, int *piv, int *info, size_t panel_smem, int64_t *launches,
                               cudaStream_t s);
// d = (P^T L U)^{-1} r with the FP32 factors
cudaError_t launch_lu32_solve(const float2 *F, int n, const int *piv, const double2 *r, double2 *d, cudaStream_t s);
// x += d; sums[0] = |d|^2, sums[1] = |x|^2
cudaError_t launch_lu32_update_x(double2 *x, const double2 *d, int n, double *sums, cudaStream_t s);
cudaError_t launch_lu_solve(const double2 *A, int64_t n, int64_t lda, const int *piv, const double2 *b, double2 *x,
                            cudaStream_t s);

// multi.cu: complex GEMM on a real view of A (cuBLAS), batched vector kernels
cudaError_t launch_gemm_c64(void *cublas, int mode, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *X,
                            int64_t ldx, int nrhs, double2 *Y, int64_t ldy, double are, double aim, double bre,
                            double bim, float *Xp, float *Z, cudaStream_t s, int *cublas_status);
// gemm_tc.cu: the same product on the tcgen05 tensor cores, split BF16 with
// FP32 accumulation (parts = 2: BF16x3, parts = 3: BF16x6, FP32-accurate).
// Needs a 16-byte aligned A with an even lda (TMA on the float view);
// scratch holds gemm_tc_scratch_bytes(); err receives a nonzero code if a
// pipeline wait ran out (the kernel then stops and frees its tensor memory).
bool gemm_tc_supported(const void *A, int64_t lda);
size_t gemm_tc_scratch_bytes(int parts, int64_t m, int64_t n, int64_t nrhs);
cudaError_t launch_gemm_tc(int parts, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *X, int64_t ldx,
                           int64_t nrhs, double2 *Y, int64_t ldy, double are, double aim, double bre, double bim,
                           void *scratch, int *err, cudaStream_t s);
int bdot_blocks(int64_t n);
// fp32: products and partial sums in FP32 on the FP64-stored vectors (the
// inner Arnoldi of a refinement), else FP64
cudaError_t launch_bdot(const double2 *V, int nv, const double2 *W, int64_t n, int nrhs, double2 *part, double2 *out,
                        cudaStream_t s, bool fp32 = false);
cudaError_t launch_bcombo(const double2 *V, int64_t n, int nrhs, int nv, const double2 *h, double sign, double2 *W,
                          cudaStream_t s, bool fp32 = false);
cudaError_t launch_bscale(const double2 *src, double2 *dst, int64_t n, int nrhs, const double *sc, cudaStream_t s);
cudaError_t launch_rsub(const double2 *B, double2 *R, size_t count, cudaStream_t s);

}  // namespace nihu
