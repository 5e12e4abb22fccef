// Matrix-vector product for callers that cannot allocate device memory.
//
// nihu_gb_matvec() takes its per-column-split partial sums from scratch the
// library allocates.  Some callers cannot let a library call cudaMalloc: hosts
// that reserve all device memory for their own pool up front, real-time
// request loops that must never wait on the allocator, or plug-in hosts whose
// memory manager forbids allocations behind their back.  This entry point
// needs no context and allocates nothing: its scratch is one file-scope
// __device__ array of fixed size that every GPU which loads the library holds
// until the process exits.
#include <mutex>

#include "../../include/nihu_gb300.h"
#include "linalg.h"

namespace {

// 16 MiB of partial sums: m * splits <= NIHU_GB_NOALLOC_PARTIAL_ELEMS
constexpr int64_t PARTIAL_ELEMS = NIHU_GB_NOALLOC_PARTIAL_ELEMS;
static __device__ __align__(256) double2 g_partial[PARTIAL_ELEMS];

// Host code cannot use g_partial's name as an address; the device address is
// looked up once per device (with that device current) and cached.
constexpr int MAX_DEVICES = 64;
double2 *g_partial_addr[MAX_DEVICES] = {};
std::mutex g_setup_mu;

nihu_gb_status partial_address(double2 **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        cudaGetLastError();
        return NIHU_GB_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_partial_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_partial);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return NIHU_GB_ERR_CUDA;
        }
        g_partial_addr[dev] = static_cast<double2 *>(p);
    }
    *out = g_partial_addr[dev];
    return NIHU_GB_OK;
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_matvec_noalloc(int dtype_a, const void *A, int64_t m, int64_t n, int64_t lda,
                                                 const void *x, void *y, double alpha_re, double alpha_im,
                                                 double beta_re, double beta_im, void *stream)
{
    if ((dtype_a != NIHU_GB_C64 && dtype_a != NIHU_GB_C128) || m < 0 || n < 0 || lda < (m > 1 ? m : 1) ||
        (m && (!A || !y)) || (n && !x))
        return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (m > PARTIAL_ELEMS) return NIHU_GB_ERR_OUT_OF_RANGE;  // not even one column split fits
    if (m == 0) return NIHU_GB_OK;
    double2 *partial = nullptr;
    nihu_gb_status st = partial_address(&partial);
    if (st != NIHU_GB_OK) return st;
    int splits = nihu::gemv_splits(m, n, dtype_a);
    const int64_t fit = PARTIAL_ELEMS / m;
    if (splits > fit) splits = (int)fit;
    // every (split, row) partial is written before it is read: nothing needs clearing
    cudaError_t e = nihu::launch_gemv(dtype_a, A, m, n, lda, static_cast<const double2 *>(x), static_cast<double2 *>(y),
                                      alpha_re, alpha_im, beta_re, beta_im, partial, splits,
                                      static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return NIHU_GB_ERR_CUDA;
    }
    return NIHU_GB_OK;
}
