// Internal launcher interface between the C ABI layer and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace nihu {

// Column-sorted list of nearly singular (test i, trial j) pairs of a mesh pair:
// pairs[col_ptr[j] .. col_ptr[j+1]) hold the rows i of column j.
struct NearList {
    int n_cols = 0;
    int64_t nnz = 0;
    int64_t *col_ptr = nullptr;  // [n_cols + 1]
    int *rows = nullptr;         // [nnz]
    // row index of the FP64 kernel's items (built on demand): the items of
    // row i at row_ent[row_ptr[i] .. row_ptr[i + 1]), each (item, column),
    // in increasing column order; items are near-list positions, then
    // nnz + j for the self term of column j (same mesh)
    int64_t *row_ptr = nullptr;  // [n_rows + 1]
    int2 *row_ent = nullptr;
};

// mesh.cu -----------------------------------------------------------------
// geometry of n elements from device copies of the node and element arrays;
// bad[0] receives 1 + the first invalid element index (0 if all valid)
// size_max receives the largest element size (as the bits of a positive double)
cudaError_t launch_mesh_geometry(const double *nodes, int64_t n_nodes, const int32_t *elems, int n,
                                 int cols, DevMesh m, int *bad, unsigned long long *size_max, cudaStream_t s);

// classify.cu -------------------------------------------------------------
// nearly singular pair lists over a uniform grid of the test centres; the
// grid lives in a scratch buffer of near_grid_scratch_bytes(test.n) bytes
size_t near_grid_buckets(int n_test);
size_t near_grid_scratch_bytes(int n_test);
// builds the grid in scratch and counts the nearly singular rows of every
// column: counts[j]
cudaError_t launch_near_grid_count(const DevMesh &test, const DevMesh &trial, int same_mesh, void *scratch,
                                   int *counts, cudaStream_t s);
// exclusive scan of counts into col_ptr (n + 1 entries), single block
cudaError_t launch_scan(const int *counts, int n, int64_t *col_ptr, cudaStream_t s);
// with the grid of launch_near_grid_count still in scratch: the rows of
// column j in increasing order to rows[col_ptr[j] ..]; tmp has the size of rows
cudaError_t launch_near_grid_fill(const DevMesh &test, const DevMesh &trial, int same_mesh, void *scratch,
                                  const int64_t *col_ptr, int *tmp, int *rows, cudaStream_t s);
// histogram of pair classes (see nihu_gb_pair_statistics)
cudaError_t launch_pair_stats(const DevMesh &test, const DevMesh &trial, int same_mesh,
                              unsigned long long *counts, cudaStream_t s);

// assemble_regular.cu -----------------------------------------------------
// shared-memory carveout preference (percent) of the two-rows regular kernel
// and of the singular kernel that runs beside it
int regular_carveout_percent();
struct RegularArgs {
    DevMesh test, trial;
    int same_mesh;
    int family, ops;
    double k;
    double alpha_re, alpha_im;
    int precision;  // 0 FP32, 1 FP64
    int dtype;      // 0 c64, 1 c128
    void *out_s, *out_d;  // column j at out + (j - j0) * ld
    int64_t ld;
    int j0, j1;
    int accumulate;
    double trial_size_max;  // largest mean edge length of the trial mesh
    // the same parameters pre-rounded on the host, so the FP32 kernel runs no
    // FP64 instruction (the FP64 pipe belongs to the concurrent singular kernel)
    float k32, alpha_re32, alpha_im32;
    int unit_alpha;
    // imaginary part of a complex (lossy) wave number k + i k_im (single wave
    // number only; 0 for the real wave numbers the fast instantiations take)
    double k_im = 0.0;
    float k_im32 = 0.0f;
    // frequency batch: nk > 1 assembles one matrix per wave number ks[f]
    // (FP64 and FP32 copies on the device) at out + f * mat_stride
    int nk = 1;
    const double *ks = nullptr;
    const float *ks32 = nullptr;
    int64_t mat_stride = 0;
    double k_absmax = 0.0;  // largest |ks[f]| of a frequency batch
    // frequency batch into separate matrices (mat_stride unused): SLP matrix
    // f at outs[f], DLP matrix f at outs[nk + f] (device array of pointers)
    void *const *outs = nullptr;
    // 1: the frequency-batch kernels even for nk = 1, so that an entry is the
    // same whatever the batch it is assembled in
    int force_batch = 0;
    // frequency batch with right-hand sides b_f = SLP_f q_f in place of the SLP
    // matrices (all columns in one launch, j0 = 0): q_f at rhs_q + f * trial.n;
    // the regular kernel leaves per block of REG_COLS columns cb the partial
    // sums rhs_part[(f * n_cb + cb) * test.n + i] (float2 in FP32 mode, double2
    // in FP64) over the block's regular pairs; the FP64 kernel leaves the SLP
    // entry of its item p (NearList row index numbering) in near_slp[f * items + p]
    const double2 *rhs_q = nullptr;
    void *rhs_part = nullptr;
    double2 *near_slp = nullptr;
    // right-hand-side mode: wave numbers per block of the regular kernel
    // (0: the default; at most 20 in FP32 mode, 10 in FP64 mode)
    int rhs_fmax = 0;
};

// matrix f of a frequency batch (dlp: the DLP output)
template <typename Out>
__device__ __forceinline__ Out *batch_matrix(const RegularArgs &a, bool dlp, int f)
{
    if (a.outs) return reinterpret_cast<Out *>(a.outs[(dlp ? a.nk : 0) + f]);
    return reinterpret_cast<Out *>(dlp ? a.out_d : a.out_s) + (int64_t)f * a.mat_stride;
}
cudaError_t launch_assemble_regular(const RegularArgs &a, cudaStream_t s);
// right-hand-side mode: the partial sums per wave number of the regular kernel
size_t rhs_part_bytes(const RegularArgs &a);
// b_f(i) = sum_cb rhs_part_f(cb, i) + sum over row i's items p of
// near_slp_f(p) q_f(column of p), in FP64 and a fixed order
cudaError_t launch_rhs_reduce(const RegularArgs &a, const NearList &near, double2 *b, cudaStream_t s);

// assemble_singular.cu ----------------------------------------------------
// nearly singular pairs of columns [j0, j1) and, for the same mesh, the
// diagonal self terms; err receives a nonzero code if an inverse mapping
// failed to converge (1 + pair index)
cudaError_t launch_assemble_singular(const RegularArgs &a, const NearList &near, int *err, cudaStream_t s);
// the frequency-batch kernel's series table and shared-memory attribute (done
// by launch_assemble_singular itself, except inside a stream capture)
cudaError_t prepare_singular_batch(cudaStream_t s);

// assemble_bm.cu ----------------------------------------------------------
// Burton-Miller operators on constant triangle trial elements.  `ops` is
// OP_DLPT and/or OP_HSP, or all four operators (the fused system):
//   out_a = c[1] DLP + c[3] HSP,  out_b = c[0] SLP + c[2] DLPt
// restricted to the operators in ops (complex coefficients c = cre + i cim).
struct BmArgs {
    DevMesh test, trial;
    int same_mesh = 0;
    int family = 0, ops = 0;
    double k = 0.0;
    float k32 = 0.0f;
    double k_im = 0.0;  // imaginary part of a complex (lossy) wave number
    float k_im32 = 0.0f;
    double cre[4] = {0, 0, 0, 0}, cim[4] = {0, 0, 0, 0};
    float cre32[4] = {0, 0, 0, 0}, cim32[4] = {0, 0, 0, 0};
    int precision = 0;  // regular entries: 0 FP32, 1 FP64
    int dtype = 0;      // 0 c64, 1 c128
    void *out_a = nullptr, *out_b = nullptr;  // column j at out + (j - j0) * ld
    int64_t ld = 0;
    int j0 = 0, j1 = 0;
    int accumulate = 0;
    double trial_size_max = 0.0;
};
// regular pairs of columns [j0, j1) (all operators in ops)
cudaError_t launch_assemble_regular_bm(const BmArgs &a, cudaStream_t s);
// nearly singular pairs and self terms of the operators in ops (FP64)
cudaError_t launch_assemble_singular_bm(const BmArgs &a, const NearList &near, cudaStream_t s);

// assemble_pairs.cu -------------------------------------------------------
// Entries of an explicit pair list (rows[p], cols[p]), p < n, each with the
// full self / nearly singular / regular dispatch:
//   out_a[p] = c[1] DLP + c[3] HSP (+ id[0] on a self pair)
//   out_b[p] = c[0] SLP + c[2] DLPt (+ id[1] on a self pair)
// for the operators in ops.  sing / n_sing: device scratch for the compacted
// nearly singular pairs (from the front, count n_sing[0]) and self pairs
// (from the back, count n_sing[1]) of the n entries; bad receives 1 + the
// first pair with an index out of range, err 1 + the first failed inverse
// mapping.
struct PairArgs {
    DevMesh test, trial;
    int same_mesh = 0;
    int family = 0, ops = 0;
    double k = 0.0;
    float k32 = 0.0f;
    double k_im = 0.0;  // imaginary part of a complex (lossy) wave number
    float k_im32 = 0.0f;
    double cre[4] = {0, 0, 0, 0}, cim[4] = {0, 0, 0, 0};
    float cre32[4] = {0, 0, 0, 0}, cim32[4] = {0, 0, 0, 0};
    double id_re[2] = {0, 0}, id_im[2] = {0, 0};
    int precision = 0, dtype = 0;
    int64_t n = 0;
    const int32_t *rows = nullptr, *cols = nullptr;
    void *out_a = nullptr, *out_b = nullptr;
    int64_t *sing = nullptr;
    unsigned long long *n_sing = nullptr;
    int *bad = nullptr, *err = nullptr;
    double trial_size_max = 0.0;
};
cudaError_t launch_assemble_pairs(const PairArgs &a, cudaStream_t s);

// assemble_galerkin.cu ----------------------------------------------------
// Galerkin SLP / DLP (constant elements) of columns [j0, j1), conventions of
// RegularArgs; extra / n_extra / extra_cap: device list of the pairs beyond
// 1.5 D that share a node, err receives -1 if it overflows
struct GalArgs {
    DevMesh test, trial;
    int same_mesh = 0;
    int family = 0, ops = 0;
    double k = 0.0;
    float k32 = 0.0f;
    double k_im = 0.0;  // imaginary part of a complex (lossy) wave number
    float k_im32 = 0.0f;
    double alpha_re = 1.0, alpha_im = 0.0;
    float alpha_re32 = 1.0f, alpha_im32 = 0.0f;
    int precision = 0, dtype = 0;
    void *out_s = nullptr, *out_d = nullptr;
    int64_t ld = 0;
    int j0 = 0, j1 = 0;
    int accumulate = 0;
    int2 *extra = nullptr;
    unsigned int *n_extra = nullptr;
    int extra_cap = 0;
    int *err = nullptr;
};
// the singular Galerkin rules into device memory (once per device)
cudaError_t prepare_galerkin(cudaStream_t s);
cudaError_t launch_galerkin_regular(const GalArgs &a, cudaStream_t s);
// self pairs and the nearly singular list (extra = 0) or the extra list
// (extra = 1, at most max_items entries)
cudaError_t launch_galerkin_near(const GalArgs &a, const NearList &near, int extra, int64_t max_items, cudaStream_t s);
// out(i, i) += alpha * area_i (the Galerkin identity of constant elements)
cudaError_t launch_add_mass(int n, const double *pts64, double are, double aim, int dtype, void *out, int64_t ld,
                            cudaStream_t s);

// linalg.cu ---------------------------------------------------------------
cudaError_t launch_add_identity(int n, double are, double aim, int dtype, void *out, int64_t ld, cudaStream_t s);

}  // namespace nihu
