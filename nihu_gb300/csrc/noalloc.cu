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
// looked up (with the device current) once per CUDA context and cached.  The
// cache is keyed by the context's unique id, so that after a cudaDeviceReset
// (or any other teardown of the primary context) the first call on the new
// context looks the address up again instead of launching on a stale one.
constexpr int MAX_DEVICES = 64;
struct PartialAddr {
    unsigned long long ctx_id = 0;
    double2 *addr = nullptr;
};
PartialAddr g_partial_addr[MAX_DEVICES];
std::mutex g_setup_mu;

// the current context's unique id through the driver API (found once through
// the runtime, so the library needs no link against the driver)
using CtxGetCurrentFn = int (*)(void **);
using CtxGetIdFn = int (*)(void *, unsigned long long *);

bool current_context_id(unsigned long long *id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    });
    void *ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

nihu_gb_status partial_address(double2 **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        cudaGetLastError();
        return NIHU_GB_ERR_NO_DEVICE;
    }
    // no context may be current yet (a process whose first CUDA call this is):
    // the symbol lookup below makes the device's primary context current
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    PartialAddr &slot = g_partial_addr[dev];
    if (!slot.addr || !have_id || slot.ctx_id != id) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_partial);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return NIHU_GB_ERR_CUDA;
        }
        if (!have_id) have_id = current_context_id(&id);
        slot.addr = static_cast<double2 *>(p);
        slot.ctx_id = have_id ? id : 0;  // 0: looked up again on the next call
    }
    *out = slot.addr;
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
