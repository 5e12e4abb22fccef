/*
 * nihu_gb300 -- C ABI of the GB300-native dense collocation BEM library.
 *
 * One library context drives one GPU (sm_103a) on one CUDA stream.  All
 * entry points return a status code and never throw; a human-readable message
 * for the last failure is available from nihu_gb_last_error().  Calls are
 * synchronous: when a call returns, its results are complete (device or host).
 *
 * The entry points replace the following reference interfaces (paths inside
 * the NiHu project):
 *   - Res << test_space * Op[trial_space]
 *       nihu/core/weighted_residual.hpp:197-206 -> integral_transform::test_on_into
 *       nihu/core/integral_transform.hpp:181-192 -> assembly::eval_into
 *       nihu/core/assembly.hpp:136-157 (hot loop :69-76, block "+=")
 *     => nihu_gb_assemble()
 *   - create_mesh(nodes, elements, tags...)  nihu/core/mesh.hpp:175-193,285-290
 *     => nihu_gb_mesh_create()
 *   - identity_integral_operator, (alpha * I)[space]
 *       nihu/core/single_integral.hpp:146-180, nihu/core/integral_operator.hpp:215-238
 *     => nihu_gb_add_identity()
 *   - dense matvec inside Eigen::GMRES  nihu/fmm/GMRES.h:57-205
 *     => nihu_gb_matvec(), nihu_gb_gmres()
 *   - colPivHouseholderQr().solve()  nihu/applications/helmholtz/helmholtz_3d_coll.cpp:113
 *     => nihu_gb_lu_solve()
 *
 * Matrices are column-major (Eigen's default), row = test DOF, column = trial
 * DOF, leading dimension ld >= number of rows.  Complex numbers are stored as
 * interleaved (re, im) pairs: complex64 = 2 x float, complex128 = 2 x double.
 */
#ifndef NIHU_GB300_H
#define NIHU_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nihu_gb_status {
    NIHU_GB_OK = 0,
    NIHU_GB_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument / logic errors */
    NIHU_GB_ERR_OUT_OF_RANGE = 2,     /* std::out_of_range (e.g. quadrature degree > 14) */
    NIHU_GB_ERR_RUNTIME = 3,          /* std::runtime_error (e.g. inverse mapping failed) */
    NIHU_GB_ERR_CUDA = 4,             /* CUDA runtime failure */
    NIHU_GB_ERR_OUT_OF_MEMORY = 5,    /* device memory budget exhausted */
    NIHU_GB_ERR_NOT_CONVERGED = 6,    /* iterative solver hit its iteration limit */
    NIHU_GB_ERR_NO_DEVICE = 7         /* no usable CUDA device */
} nihu_gb_status;

/* element type ids (nihu/core/element.hpp:112-118) */
#define NIHU_GB_TRIA_1 32303
#define NIHU_GB_QUAD_1 32404

/* kernel families (nihu/library/helmholtz_kernel.hpp, laplace_kernel.hpp) */
#define NIHU_GB_HELMHOLTZ_3D 0
#define NIHU_GB_LAPLACE_3D 1

/* operator bit mask: SLP = G, DLP = dG/dn_y (nihu/library/normal_derivative_kernel.hpp) */
#define NIHU_GB_SLP 1
#define NIHU_GB_DLP 2
/* Burton-Miller operators: DLPt = dG/dn_x, HSP = d2G/dn_x dn_y
 * (helmholtz_3d_DLPt_kernel / helmholtz_3d_HSP_kernel,
 * nihu/library/helmholtz_kernel.hpp:326-334, laplace_kernel.hpp likewise) */
#define NIHU_GB_DLPT 4
#define NIHU_GB_HSP 8

/* storage type of a matrix or vector */
#define NIHU_GB_C64 0  /* complex64: 2 x float32 */
#define NIHU_GB_C128 1 /* complex128: 2 x float64 */

/* arithmetic of the regular (far-field) quadrature; singular and nearly
 * singular integrals are always evaluated in FP64 */
#define NIHU_GB_REGULAR_FP32 0
#define NIHU_GB_REGULAR_FP64 1

/* where a buffer lives */
#define NIHU_GB_HOST 0
#define NIHU_GB_DEVICE 1

typedef struct nihu_gb_ctx nihu_gb_ctx;
typedef struct nihu_gb_mesh nihu_gb_mesh;
typedef struct nihu_gb_server nihu_gb_server;
typedef struct nihu_gb_sweep_plan nihu_gb_sweep_plan;

/* ------------------------------------------------------------------ context */

/* Create a context on `device`.  `stream` is a cudaStream_t to run on, or NULL
 * for a context-owned stream.  `hbm_budget_bytes` caps the device memory the
 * context allocates (0 = no cap). */
nihu_gb_status nihu_gb_ctx_create(int device, void *stream, size_t hbm_budget_bytes, nihu_gb_ctx **out);
void nihu_gb_ctx_destroy(nihu_gb_ctx *ctx);
/* message of the last failed call on this context ("" if none) */
const char *nihu_gb_last_error(const nihu_gb_ctx *ctx);
/* the cudaStream_t the context launches on */
void *nihu_gb_ctx_stream(const nihu_gb_ctx *ctx);
/* device bytes currently held by the context and its meshes */
size_t nihu_gb_ctx_device_bytes(const nihu_gb_ctx *ctx);
/* number of kernels this context has launched since creation */
int64_t nihu_gb_ctx_launch_count(const nihu_gb_ctx *ctx);

/* Per-phase device timing: with profiling enabled, every kernel phase a call
 * launches is bracketed by CUDA events on the context's stream and its device
 * time is accumulated per phase name ("assemble_regular",
 * "assemble_singular", "near_list", "gemv", ...).  Off by default. */
nihu_gb_status nihu_gb_ctx_set_profiling(nihu_gb_ctx *ctx, int enable);
/* Phase `index` (0-based): name, total device milliseconds and launches.
 * Returns NIHU_GB_ERR_OUT_OF_RANGE past the last phase. */
nihu_gb_status nihu_gb_ctx_profile(const nihu_gb_ctx *ctx, int index, const char **name, double *total_ms,
                                   int64_t *launches);
void nihu_gb_ctx_profile_reset(nihu_gb_ctx *ctx);

/* pinned host memory helpers for fast host<->device transfers */
nihu_gb_status nihu_gb_host_alloc(nihu_gb_ctx *ctx, size_t bytes, void **out);
void nihu_gb_host_free(void *ptr);
/* device memory owned by the caller, charged to the context's budget */
nihu_gb_status nihu_gb_device_alloc(nihu_gb_ctx *ctx, size_t bytes, void **out);
void nihu_gb_device_free(nihu_gb_ctx *ctx, void *ptr);
nihu_gb_status nihu_gb_memcpy(nihu_gb_ctx *ctx, void *dst, int dst_where, const void *src, int src_where, size_t bytes);

/* --------------------------------------------------------------------- mesh */

/* Build a mesh from host arrays (nihu/core/mesh.hpp:175-193):
 *   nodes: n_nodes x 3 doubles, row-major (x, y, z)
 *   elems: n_elems x elem_cols int32, row-major; column 0 is the element type
 *          id (NIHU_GB_TRIA_1 / NIHU_GB_QUAD_1), columns 1.. the corner node
 *          indices (unused trailing columns are ignored).
 * Element ids, and so DOF numbers, follow the row order (nihu/core/mesh.hpp:155).
 * Geometry (centres, sizes, normals, quadrature points) is computed on the GPU
 * and kept on the device until nihu_gb_mesh_destroy(). */
nihu_gb_status nihu_gb_mesh_create(nihu_gb_ctx *ctx, const double *nodes, int64_t n_nodes,
                                   const int32_t *elems, int64_t n_elems, int64_t elem_cols,
                                   nihu_gb_mesh **out);
void nihu_gb_mesh_destroy(nihu_gb_mesh *mesh);
int64_t nihu_gb_mesh_num_elements(const nihu_gb_mesh *mesh);

/* ----------------------------------------------------------------- assembly */

/* Assemble the collocational SLP and/or DLP matrices of a kernel family
 * between a test mesh (rows, Dirac collocation at element centres) and a trial
 * mesh (columns, constant elements):
 *     out_op = alpha * Op            (accumulate == 0)
 *     out_op = out_op + alpha * Op   (accumulate != 0, NiHu's "<<" semantics)
 * `ops` is a bit mask of NIHU_GB_SLP / NIHU_GB_DLP; out_slp / out_dlp may be
 * NULL for operators not requested.  test == trial (same handle) enables the
 * singular self terms, as NiHu's same-mesh check does
 * (nihu/core/integral_transform.hpp:156).  k is the real wave number (ignored
 * for Laplace).  dtype is NIHU_GB_C64 or NIHU_GB_C128; where is NIHU_GB_HOST
 * or NIHU_GB_DEVICE for both outputs.  Host outputs are assembled in column
 * panels whose device-to-host copies overlap the next panel's assembly; pinned
 * host memory (nihu_gb_host_alloc) makes those copies fastest.
 * Replaces: nihu/core/weighted_residual.hpp:197-206, nihu/core/assembly.hpp:136-157,
 * per-pair dispatch nihu/core/double_integral.hpp:543-673. */
nihu_gb_status nihu_gb_assemble(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                int family, int ops, double k, double alpha_re, double alpha_im,
                                int precision, int dtype, void *out_slp, void *out_dlp, int64_t ld,
                                int accumulate, int where);

/* nihu_gb_assemble() for a complex wave number k + i k_im: a lossy medium
 * (k_im < 0 damps e^{-ikr} as e^{k_im r}), as the reference's kernels take a
 * complex WaveNumber type (nihu/library/helmholtz_kernel.hpp:42-54).
 * k_im = 0 is nihu_gb_assemble() itself; a nonzero k_im runs separate kernel
 * instantiations (the nearly singular and self terms in FP64 in both
 * precision modes) and is ignored for the Laplace family. */
nihu_gb_status nihu_gb_assemble_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family,
                                  int ops, double k, double k_im, double alpha_re, double alpha_im, int precision,
                                  int dtype, void *out_slp, void *out_dlp, int64_t ld, int accumulate, int where);

/* out(i, i) += alpha for every element i (collocational identity operator on
 * constant elements, nihu/core/single_integral.hpp:146-180).  The matrix is
 * n x n with n = number of mesh elements. */
nihu_gb_status nihu_gb_add_identity(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, double alpha_re, double alpha_im,
                                    int dtype, void *out, int64_t ld, int where);

/* The Galerkin formalism of the SLP / DLP operators on constant elements,
 * A(i, j) = int_{E_i} int_{E_j} K(x, y), with the conventions of
 * nihu_gb_assemble (test == trial handle = one mesh).  On one mesh, pairs
 * that share the element, an edge or a corner take the singular Galerkin
 * rules of their match type (4 Gauss points per direction of a 4D Duffy-type
 * split: 1536 / 1536 / 512 points on triangles, 2048 / 1536 / 1280 on quads);
 * all other pairs the product of the regular rule of degree C + interval(d/D)
 * on both elements.  A mesh may mix triangles and quads: a triangle-quad
 * match takes the triangle-triangle rules on the quad split into two
 * triangles (singular_galerkin_quadrature.hpp:624-790).
 * Replaces: test_space * Op[trial_space] with a function-space test space
 * (nihu/core/double_integral.hpp:143-384, element_match.hpp:60-90,
 * singular_accelerator.hpp:142-330, singular_galerkin_quadrature.hpp:200-420),
 * e.g. nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:55-57. */
nihu_gb_status nihu_gb_assemble_galerkin(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                         int family, int ops, double k, double alpha_re, double alpha_im,
                                         int precision, int dtype, void *out_slp, void *out_dlp, int64_t ld,
                                         int accumulate, int where);

/* nihu_gb_assemble_galerkin() for a complex wave number k + i k_im (a lossy
 * medium): the regular pairs with the complex point kernel, the singular and
 * nearly singular rules in FP64 with the complex kernel in both modes. */
nihu_gb_status nihu_gb_assemble_galerkin_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                           int family, int ops, double k, double k_im, double alpha_re,
                                           double alpha_im, int precision, int dtype, void *out_slp, void *out_dlp,
                                           int64_t ld, int accumulate, int where);

/* out(i, i) += alpha * area_i: the Galerkin identity operator of constant
 * elements (test_space * I[trial_space], nihu/core/single_integral.hpp:97-140). */
nihu_gb_status nihu_gb_add_mass(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, double alpha_re, double alpha_im,
                                int dtype, void *out, int64_t ld, int where);

/* The Burton-Miller operators DLPt (transposed double layer, kernel
 * dG/dr (-r.n_x)/r) and HSP (hypersingular, d2G/dn_x dn_y) with the same
 * conventions as nihu_gb_assemble: `ops` is a bit mask of NIHU_GB_DLPT /
 * NIHU_GB_HSP, out = alpha * Op (or += with accumulate).  n_x is the unit
 * normal at the collocation point (test element centre).  The trial mesh must
 * hold constant triangles only (the reference's constant-plane singular and
 * nearly singular schemes for these kernels are triangle schemes); quad
 * trial elements give NIHU_GB_ERR_INVALID_ARGUMENT.  Regular pairs take the
 * distance-adaptive rule of each kernel (HSP: 1/r^3 intervals 1.9 / 3.6 /
 * 22.3); nearly singular pairs the semi-analytic static part plus the
 * 42-point dynamic part; self terms DLPt = 0 and the finite-part HSP integral.
 * Replaces: test_space * (alpha * Htop)[trial_space] and
 * test_space * (alpha * Dop)[trial_space] of
 * nihu/applications/helmholtz/helmholtz_3d_coll.cpp:53-56,71,87, dispatched by
 * nihu/core/double_integral.hpp:543-673 to
 * nihu/library/helmholtz_singular_integrals.hpp:764-839 and
 * nihu/library/helmholtz_nearly_singular_integrals.hpp:131-220. */
nihu_gb_status nihu_gb_assemble_bm(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                   int family, int ops, double k, double alpha_re, double alpha_im,
                                   int precision, int dtype, void *out_dlpt, void *out_hsp, int64_t ld,
                                   int accumulate, int where);

/* nihu_gb_assemble_bm() for a complex wave number k + i k_im (a lossy
 * medium, as nihu_gb_assemble_c): the four kernels with e^{-ikr}, 1 + ikr and
 * (ikr)^2 complex, the nearly singular dynamic parts and the HSP self term's
 * remainder in FP64 with the complex kernel.  k_im = 0 is nihu_gb_assemble_bm. */
nihu_gb_status nihu_gb_assemble_bm_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                     int family, int ops, double k, double k_im, double alpha_re, double alpha_im,
                                     int precision, int dtype, void *out_dlpt, void *out_hsp, int64_t ld,
                                     int accumulate, int where);

/* The two Burton-Miller system matrices of one mesh with coupling c
 * (the reference application uses c = -i/k):
 *     A = DLP - 1/2 I + c HSP,   B = SLP + c DLPt + c/2 I
 * assembled in one pass over the element pairs (all four kernels share each
 * quadrature point).  The solve is then A p = B q.
 * Replaces: nihu/applications/helmholtz/helmholtz_3d_coll.cpp:60-100 (BM
 * branch, matrices Gs and Hs). */
nihu_gb_status nihu_gb_assemble_burton_miller(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                              double coupling_re, double coupling_im, int precision, int dtype,
                                              void *out_a, void *out_b, int64_t ld, int where);

/* nihu_gb_assemble_burton_miller() for a complex wave number k + i k_im (the
 * coupling is the caller's, e.g. -i / (k + i k_im)). */
nihu_gb_status nihu_gb_assemble_burton_miller_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                                double k_im, double coupling_re, double coupling_im, int precision,
                                                int dtype, void *out_a, void *out_b, int64_t ld, int where);

/* Entries of an explicit list of element pairs (test rows[p], trial cols[p]),
 * each with the full singular check of the dense path (self, nearly singular
 * d/D < 1.5, regular by the interval tables): the near-field (P2P) matrix of
 * a fast multipole or hierarchical solver, in sparse triplet form.  For every
 * p (row / column indices int32):
 *     out_a[p] = c_DLP DLP + c_HSP HSP (+ ident_a if test == trial and rows[p] == cols[p])
 *     out_b[p] = c_SLP SLP + c_DLPt DLPt (+ ident_b likewise)
 * over the operators in `ops` (mask of NIHU_GB_SLP / DLP / DLPT / HSP).
 * coef = {re, im} x (SLP, DLP, DLPt, HSP) (NULL: all 1); ident = {re, im} x
 * (a, b) (NULL: no identity).  out_a is needed when ops has DLP or HSP, out_b
 * when it has SLP or DLPt (dtype complex64 / complex128, n_pairs values).
 * where: NIHU_GB_HOST (pairs and outputs in host memory) or NIHU_GB_DEVICE.
 * DLPt / HSP need constant triangle trial elements.  An index out of range
 * gives NIHU_GB_ERR_INVALID_ARGUMENT.
 * Replaces: nihu/fmm/p2p_integral.hpp:87-99 evaluated over the P2P list by
 * nihu/fmm/p2p_precompute.hpp:110-180 (the Burton-Miller FMM solver's
 * lhs/rhs near fields, nihu/fmm/helmholtz_burton_miller_solver.hpp:170-190). */
nihu_gb_status nihu_gb_assemble_pairs(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                      int family, int ops, double k, const double *coef, const double *ident,
                                      int precision, int dtype, int64_t n_pairs, const int32_t *rows,
                                      const int32_t *cols, void *out_a, void *out_b, int where);

/* nihu_gb_assemble_pairs() for a complex wave number k + i k_im. */
nihu_gb_status nihu_gb_assemble_pairs_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                        int family, int ops, double k, double k_im, const double *coef,
                                        const double *ident, int precision, int dtype, int64_t n_pairs,
                                        const int32_t *rows, const int32_t *cols, void *out_a, void *out_b, int where);

/* Per-pair quadrature statistics of an assembly (no matrix is written):
 * counts[0] self pairs, counts[1] nearly singular pairs, counts[2 + 3*s + d]
 * regular pairs whose SLP uses level s and DLP level d (levels 0, 1, 2 =
 * 1 point / 3-4 points / 6-9 points). */
nihu_gb_status nihu_gb_pair_statistics(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                       int64_t counts[11]);

/* The nearly singular pair list that the assemblies of (test, trial) use,
 * column-sorted: the rows of trial column j, in increasing order, are
 * rows[col_ptr[j] .. col_ptr[j + 1]).  *nnz receives the length; col_ptr
 * (n_trial + 1 entries) and rows (*nnz entries) are written when not NULL,
 * so a first call with NULL arrays sizes them.  The list is built once per
 * mesh pair and kept in the context.
 * Replaces: the per-pair nearly singular test of the reference's double
 * integral dispatch (nihu/core/double_integral.hpp:543-639 with
 * nihu/library/helmholtz_nearly_singular_integrals.hpp:234-246), which it
 * evaluates for every pair of every assembly. */
nihu_gb_status nihu_gb_near_pairs(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                  int64_t *nnz, int64_t *col_ptr, int32_t *rows);

/* ------------------------------------------------------------- linear algebra */

/* y = alpha * A x + beta * y; A is m x n (dtype_a, column-major, lda), x and
 * y are complex128 vectors.  With dtype_a = NIHU_GB_C64 the products are
 * formed in FP32 and the column-panel partial sums are added in FP64. */
nihu_gb_status nihu_gb_matvec(nihu_gb_ctx *ctx, int dtype_a, const void *A, int64_t m, int64_t n, int64_t lda,
                              const void *x, void *y, double alpha_re, double alpha_im,
                              double beta_re, double beta_im, int where);

/* y = alpha * A x + beta * y like nihu_gb_matvec(), for callers that cannot
 * allocate device memory (hosts that reserve all of it for their own pool,
 * request loops that must never wait on the allocator, plug-in hosts whose
 * memory manager forbids allocations behind their back).  No context is
 * needed and nothing is allocated: the partial sums live in one static device
 * array of NIHU_GB_NOALLOC_PARTIAL_ELEMS complex128 values (16 MiB) that every
 * GPU which loads the library keeps until the process exits.  A, x, y are
 * device pointers on the current device; the work is enqueued on `stream`
 * (a cudaStream_t, NULL = the legacy default stream) and is complete when the
 * stream reaches that point.  m above NIHU_GB_NOALLOC_PARTIAL_ELEMS returns
 * NIHU_GB_ERR_OUT_OF_RANGE.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress), so make it before any stream
 * capture; the address is kept per CUDA context, so the first call after a
 * cudaDeviceReset (which makes a new context) looks it up again and should
 * likewise come before any capture.  All calls share the array and every call overwrites the part it
 * reads, so nothing needs clearing -- but two calls that run on the GPU at the
 * same time (different streams or host threads) race and corrupt each other.
 * This entry point has no counterpart in the reference. */
#define NIHU_GB_NOALLOC_PARTIAL_ELEMS (1 << 20)
nihu_gb_status nihu_gb_matvec_noalloc(int dtype_a, const void *A, int64_t m, int64_t n, int64_t lda, const void *x,
                                      void *y, double alpha_re, double alpha_im, double beta_re, double beta_im,
                                      void *stream);

/* arithmetic of a multi-right-hand-side product (nihu_gb_gemm).  BF16X3 and
 * BF16X6 are this library's own tcgen05 kernel: one pass over A, each FP32
 * value split into BF16 parts (2 or 3) in shared and tensor memory, the part
 * products above the target precision accumulated in FP32 in tensor memory
 * (about 1e-5 and FP32 accuracy).  They need A 16-byte aligned with an even
 * lda; otherwise BF16X3 runs as FP32 and BF16X6 as BF16X9.  FP32, TF32 and
 * BF16X9 are cuBLAS (a plain library GEMM on the same real view). */
#define NIHU_GB_GEMM_FP32 0   /* FP32 on the CUDA cores (cuBLAS) */
#define NIHU_GB_GEMM_TF32 1   /* TF32 tensor cores, FP32 accumulation (cuBLAS) */
#define NIHU_GB_GEMM_BF16X9 2 /* split BF16 (3 parts, 9 products), cuBLAS emulation: FP32-accurate */
#define NIHU_GB_GEMM_BF16X3 3 /* split BF16 (2 parts, 3 products), tcgen05: about 1e-5 */
#define NIHU_GB_GEMM_BF16X6 4 /* split BF16 (3 parts, 6 products), tcgen05: FP32-accurate */

/* Y = alpha * A X + beta * Y for nrhs right-hand sides: A complex64 m x n
 * (lda), X n x nrhs (ldx) and Y m x nrhs (ldy) complex128, column-major.
 * One real GEMM on the float view of A (even rows Re A, odd rows Im A) times
 * the planes [Re X | Im X] reads A once; the complex combination and alpha,
 * beta are applied in FP64.  The multi-RHS product of the reference is
 * Eigen's dense product (nihu/applications/helmholtz/helmholtz_3d_coll.cpp:68-74).
 * All buffers on the device when where = NIHU_GB_DEVICE. */
nihu_gb_status nihu_gb_gemm(nihu_gb_ctx *ctx, int mode, const void *A, int64_t m, int64_t n, int64_t lda,
                            const void *X, int64_t ldx, int64_t nrhs, void *Y, int64_t ldy, double alpha_re,
                            double alpha_im, double beta_re, double beta_im, int where);

/* Solve A X = B for nrhs right-hand sides (A complex64 n x n, B and X
 * complex128 n x nrhs, ld = n) by mixed-precision iterative refinement:
 * each outer step runs one GMRES(restart) cycle on every right-hand side in
 * lockstep (the products A [v_1 .. v_nrhs] are one GEMM of mode inner_mode,
 * normally TF32 tensor cores; FP64 Arnoldi), stops a column when its residual
 * estimate falls by inner_tol, adds the correction to X in FP64 and
 * recomputes the residual B - A X with FP32-accurate products (residual_mode
 * NIHU_GB_GEMM_FP32, NIHU_GB_GEMM_BF16X9 or NIHU_GB_GEMM_BF16X6) combined in
 * FP64.  Stops when
 * every column has |B - A X| <= tol |B|.  X starts from zero.
 * rel_residuals (nrhs doubles) receives the final relative residuals. */
nihu_gb_status nihu_gb_solve_multi(nihu_gb_ctx *ctx, const void *A, int64_t n, int64_t lda, const void *B, void *X,
                                   int64_t nrhs, int inner_mode, int residual_mode, int restart, int max_outer,
                                   double tol, double inner_tol, int *outer_iters, int *inner_iters,
                                   double *rel_residuals, int where);

/* Frequency batch: assemble the operators of one mesh pair for nk wave
 * numbers in one pass.  Every thread classifies its pairs once and evaluates
 * them for all wave numbers; the k-independent static part of the nearly
 * singular triangle integrals is computed once.  Matrix f starts at
 * out + f * mat_stride elements (mat_stride >= ld * trial elements); outputs
 * on the device, overwritten (alpha = 1).  Replaces nk calls of the
 * reference's assembly (nihu/core/assembly.hpp:136-157), one per wave number. */
nihu_gb_status nihu_gb_assemble_sweep(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                      int family, int ops, const double *ks, int nk, int precision, int dtype,
                                      void *out_slp, void *out_dlp, int64_t ld, int64_t mat_stride);

/* Frequency sweep of the exterior CBIE (DLP - I/2) p_f = SLP q_f on one mesh
 * (the plain branch of nihu/applications/helmholtz/helmholtz_3d_coll.cpp:36-120
 * for every wave number): batched assembly (complex64, FP64 singular terms),
 * batched right-hand sides, and one persistent GMRES launch over all wave
 * numbers (nihu_gb_solve_batched; at most restart * max_cycles iterations
 * each).  q is n x q_cols complex128 on the host (q_cols = 1 broadcasts one
 * Neumann datum to every wave number, else q_cols = nk); p receives n x nk
 * complex128.  cycles / iters (may be NULL) receive the largest restart-cycle
 * and iteration counts over the wave numbers; rel_residuals (nk doubles, may
 * be NULL) the final relative residual estimates. */
nihu_gb_status nihu_gb_solve_sweep(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, const double *ks, int nk,
                                   int precision, const void *q, int q_cols, void *p, int restart, int max_cycles,
                                   double tol, int *cycles, int *iters, double *rel_residuals);

/* Solve `count` independent dense systems A_f x_f = b_f of any sizes with
 * restarted GMRES(restart) in ONE persistent kernel launch: each
 * thread-block cluster solves one system at a time (FP32 complex matvec on
 * its share of the rows, FP64 Arnoldi with CGS2, cluster reductions through
 * distributed shared memory) and takes the next system from a device
 * counter, largest first, with no host round trip between Krylov steps.
 * Per system the stopping rules of nihu_gb_gmres apply with x0 = 0
 * (nihu/fmm/GMRES.h:57-205 semantics, one call per system in the reference).
 * A[f] (complex64, column-major, leading dimension lda[f]), b[f] and x[f]
 * (complex128, length n[f]) are device pointers held in host arrays.
 * iters, rel_residuals and converged (count entries each, may be NULL)
 * receive the per-system results; returns NIHU_GB_ERR_NOT_CONVERGED, with
 * every x written, when some system stopped at max_iters. */
nihu_gb_status nihu_gb_solve_batched(nihu_gb_ctx *ctx, int count, const void *const *A, const int64_t *n,
                                     const int64_t *lda, const void *const *b, void *const *x, int restart,
                                     int max_iters, double tol, int *iters, double *rel_residuals, int *converged);

/* Frequency sweep over several meshes of uneven size in one call: instance f
 * solves the CBIE (DLP - I/2) p = SLP q on meshes[mesh_of[f]] at wave number
 * ks[f] (helmholtz_3d_coll.cpp:36-120 once per instance in the reference).
 * Each mesh's instances are assembled in one frequency-batched pass
 * (nihu_gb_assemble_sweep), and all instances are solved by one persistent
 * launch (nihu_gb_solve_batched).  q and p are complex128 host arrays holding
 * the instances' columns back to back in instance order (instance f has
 * the element count of its mesh).  iters, rel_residuals and converged (nk
 * entries, may be NULL) as for nihu_gb_solve_batched. */
nihu_gb_status nihu_gb_solve_sweep_batched(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes,
                                           int family, int nk, const double *ks, const int *mesh_of, int precision,
                                           const void *q, void *p, int restart, int max_iters, double tol, int *iters,
                                           double *rel_residuals, int *converged);

/* Solve A x = b with restarted GMRES(restart) (nihu/fmm/GMRES.h:57-205
 * semantics: stop when |residual estimate| / |b - A x0| < tol).  A is n x n
 * (dtype_a) on the device; b and x are complex128 (x holds the initial guess
 * on entry).  The Arnoldi basis and Givens rotations are FP64; the matvec is
 * FP32 when dtype_a = NIHU_GB_C64.  iters / rel_residual may be NULL.
 * Returns NIHU_GB_ERR_NOT_CONVERGED (with x set to the last iterate) when
 * max_iters is reached first. */
nihu_gb_status nihu_gb_gmres(nihu_gb_ctx *ctx, int dtype_a, const void *A, int64_t n, int64_t lda,
                             const void *b, void *x, int restart, int max_iters, double tol,
                             int *iters, double *rel_residual, int where);

/* Solve A x = b by LU factorisation with partial pivoting (complex128 A,
 * n x n, lda): the FP32 factors of A, refined in FP64 (x += (LU)^{-1}
 * (b - A x) with the FP64 residual) until the correction is at FP64
 * rounding; an FP64 factorisation when the order is beyond the FP32 kernels
 * or the refinement stops converging (then a device A is overwritten by its
 * factors).  A host A is copied to the device and left unchanged. */
nihu_gb_status nihu_gb_lu_solve(nihu_gb_ctx *ctx, void *A, int64_t n, int64_t lda, const void *b, void *x,
                                int where);

/* ------------------------------------------------------- composite solve */

/* Exterior collocation BEM solve of the Helmholtz/Laplace CBIE
 *     (DLP - 1/2 I) p = SLP q
 * on one mesh (nihu/applications/helmholtz/helmholtz_3d_coll.cpp:36-120 with
 * the plain CBIE branch): assembles both matrices (dtype), forms the right-hand
 * side on the device, and solves with GMRES (solver = 0) or LU (solver = 1,
 * requires dtype = NIHU_GB_C128).  q and p are complex128 host vectors of
 * length n.  iters / rel_residual may be NULL. */
nihu_gb_status nihu_gb_solve_cbie(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                  int precision, int dtype, const void *q, void *p, int solver,
                                  int restart, int max_iters, double tol, int *iters, double *rel_residual);

/* nihu_gb_solve_cbie() for a complex wave number k + i k_im (a lossy medium;
 * the assembly of nihu_gb_assemble_c()). */
nihu_gb_status nihu_gb_solve_cbie_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k, double k_im,
                                    int precision, int dtype, const void *q, void *p, int solver, int restart,
                                    int max_iters, double tol, int *iters, double *rel_residual);

/* Burton-Miller exterior solve A p = B q (matrices of
 * nihu_gb_assemble_burton_miller) by GMRES (solver 0) or LU (solver 1,
 * dtype = NIHU_GB_C128); arguments as nihu_gb_solve_cbie.  Free of the
 * fictitious interior resonances of the plain CBIE.
 * Replaces: nihu/applications/helmholtz/helmholtz_3d_coll.cpp:36-120 with BM
 * (KHIE + HSIE) defined. */
nihu_gb_status nihu_gb_solve_burton_miller(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                           double coupling_re, double coupling_im, int precision, int dtype,
                                           const void *q, void *p, int solver, int restart, int max_iters, double tol,
                                           int *iters, double *rel_residual);

/* nihu_gb_solve_burton_miller() for a complex wave number k + i k_im. */
nihu_gb_status nihu_gb_solve_burton_miller_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                             double k_im, double coupling_re, double coupling_im, int precision,
                                             int dtype, const void *q, void *p, int solver, int restart, int max_iters,
                                             double tol, int *iters, double *rel_residual);

/* A frequency sweep over fixed meshes captured once as a CUDA graph and
 * replayed per set of wave numbers (the batched counterpart of running
 * helmholtz_3d_coll.cpp:36-120 once per instance).  nk instances, instance f
 * on meshes[mesh_of[f]]; every run's wave numbers satisfy |k| <= k_max (the
 * series of the nearly singular terms are sized for it).  Creation builds
 * the near-pair lists, allocates every buffer (matrices of all instances,
 * Krylov state, pinned staging) and records: the uploads, each mesh's
 * frequency-batch assembly, identities and right-hand sides, the persistent
 * GMRES(restart) launches over all instances, and the downloads; its launch
 * set-up is chosen by measurement (nihu_gb_sweep_plan_tuning). */
nihu_gb_status nihu_gb_sweep_plan_create(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes, int family,
                                         int nk, const int *mesh_of, double k_max, int precision, int restart,
                                         int max_iters, double tol, nihu_gb_sweep_plan **out);

/* One replay: ks (nk), q and p (complex128 host arrays, the instances'
 * columns back to back in instance order) as for nihu_gb_solve_sweep_batched;
 * iters, rel_residuals, converged (nk entries each) may be NULL.  Returns
 * NIHU_GB_ERR_NOT_CONVERGED, with every p written, when some instance stopped
 * at max_iters. */
nihu_gb_status nihu_gb_sweep_plan_run(nihu_gb_sweep_plan *plan, const double *ks, const void *q, void *p, int *iters,
                                      double *rel_residuals, int *converged);
/* The plan's pinned staging buffers (complex128, the instances' columns back
 * to back in instance order, as q and p of nihu_gb_sweep_plan_run).  A run
 * given these very pointers as q and p reads and writes them in place, with
 * no host copy; they stay valid until nihu_gb_sweep_plan_destroy. */
nihu_gb_status nihu_gb_sweep_plan_host_buffers(nihu_gb_sweep_plan *plan, void **q, void **p);
/* The launch set-up the plan's autotuner measured fastest at creation (each
 * candidate captured and replayed on wave numbers spread over (0.1, 1] k_max
 * with unit Neumann data): CTAs per cluster of the persistent GMRES launch,
 * wave numbers per block of the regular assembly kernel, and that replay's
 * time in ms.  Any pointer may be NULL. */
nihu_gb_status nihu_gb_sweep_plan_tuning(const nihu_gb_sweep_plan *plan, int *cluster, int *freq_per_block,
                                         double *replay_ms);
void nihu_gb_sweep_plan_destroy(nihu_gb_sweep_plan *plan);

/* ------------------------------------------------------------ serving */

/* A serving loop for CBIE solves (DLP - I/2) p = SLP q of requests arriving
 * over time (the reference solves one problem per program run,
 * helmholtz_3d_coll.cpp:36-120; it has no counterpart for the loop itself).
 * Requests wait in a FIFO queue until hbm_budget_bytes holds their matrices
 * (complex64; the SLP matrix is freed once the right-hand side is formed)
 * and Krylov state, and at most max_active requests are admitted at once.
 * Each nihu_gb_server_step admits what fits, assembles the new requests (one
 * frequency batch per mesh), and advances every admitted system by at most
 * `quantum` GMRES(restart) steps (0: to the end) in one persistent launch;
 * matrices, Krylov state and iterates stay on the device between steps, and
 * a request's result does not depend on what else is in flight.  The meshes
 * must outlive the server.  Calls on one server are not thread safe. */
nihu_gb_status nihu_gb_server_create(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes, int family,
                                     int precision, size_t hbm_budget_bytes, int max_active, int restart,
                                     int max_iters, double tol, int quantum, nihu_gb_server **out);
void nihu_gb_server_destroy(nihu_gb_server *server);

/* Map `bytes` of device memory (0 or more than the budget: the budget) into
 * the server's memory pool now, so that admissions inside the serving loop
 * map none: the pool keeps freed memory until the server is destroyed.
 * NIHU_GB_ERR_OUT_OF_MEMORY when the device cannot provide it. */
nihu_gb_status nihu_gb_server_reserve(nihu_gb_server *server, size_t bytes);

/* Queue a request on meshes[mesh] at wave number k with Neumann data q
 * (complex128 host vector of the mesh's element count, copied).  *id
 * receives its number (0, 1, 2, ... in submission order).
 * NIHU_GB_ERR_OUT_OF_MEMORY: the request alone exceeds the budget. */
nihu_gb_status nihu_gb_server_submit(nihu_gb_server *server, int mesh, double k, const void *q, int64_t *id);

/* One round (waits for its GPU work); the counts after it may be NULL. */
nihu_gb_status nihu_gb_server_step(nihu_gb_server *server, int *n_queued, int *n_active, int *n_done);

/* Take the oldest finished request: *id (-1 if none), p (complex128, at
 * least the mesh's element count, `capacity`), GMRES iterations, relative
 * residual estimate and convergence flag (each may be NULL). */
nihu_gb_status nihu_gb_server_take(nihu_gb_server *server, int64_t *id, void *p, int64_t capacity, int *iters,
                                   double *rel_residual, int *converged);

#ifdef __cplusplus
}
#endif

#endif /* NIHU_GB300_H */
