// C ABI of the GB300 collocation BEM library (declared in include/nihu_gb300.h).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <queue>
#include <string>
#include <utility>
#include <vector>

#include <cublas_v2.h>

#include "../../include/nihu_gb300.h"
#include "kernels.h"
#include "linalg.h"
#include "solve_persistent.h"

using namespace nihu;

struct nihu_gb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaStream_t aux_stream = nullptr;  // high priority: FP64 singular kernel beside the regular one
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool own_stream = false;
    size_t budget = 0;
    size_t used = 0;
    std::map<void *, size_t> allocs;
    std::string err;
    int64_t launches = 0;
    int *d_flag = nullptr;       // device error flag / small scratch (4 ints)
    void *h_small = nullptr;     // pinned host scratch (64 KB)
    uint64_t next_uid = 1;
    // nearly singular pair lists keyed by (test uid, trial uid)
    std::map<std::pair<uint64_t, uint64_t>, NearList> near;
    // reusable device scratch buffers
    std::map<std::string, std::pair<void *, size_t>> scratch;
    // per-phase device timing
    bool profiling = false;
    std::vector<std::string> phase_names;
    std::map<std::string, std::pair<double, int64_t>> phases;
    std::vector<std::pair<std::string, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> event_pool;
    cublasHandle_t cublas = nullptr;  // created on first multi-RHS product
    // the FP32 LU factorisation of the last order, captured as a CUDA graph
    // (one kernel pair per panel): valid for these buffers
    cudaGraphExec_t lu_exec = nullptr;
    int lu_n = 0;
    int64_t lu_launches = 0;
    void *lu_F = nullptr, *lu_piv = nullptr;
};

struct nihu_gb_mesh {
    nihu_gb_ctx *ctx = nullptr;
    uint64_t uid = 0;
    int64_t n = 0;
    double size_max = 0.0;  // largest element size (mean edge length)
    DevMesh dm;
    std::vector<void *> bufs;
};

namespace {

nihu_gb_status fail(nihu_gb_ctx *ctx, nihu_gb_status st, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    return st;
}

nihu_gb_status cuda_fail(nihu_gb_ctx *ctx, cudaError_t e, const char *where)
{
    std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(ctx, NIHU_GB_ERR_OUT_OF_MEMORY, msg);
    return fail(ctx, NIHU_GB_ERR_CUDA, msg);
}

#define CK(call)                                                 \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

nihu_gb_status dmalloc(nihu_gb_ctx *ctx, size_t bytes, void **out)
{
    *out = nullptr;
    if (bytes == 0) bytes = 16;
    if (ctx->budget && ctx->used + bytes > ctx->budget)
        return fail(ctx, NIHU_GB_ERR_OUT_OF_MEMORY,
                    "device memory budget exhausted (" + std::to_string(ctx->used + bytes) + " > " +
                        std::to_string(ctx->budget) + " bytes)");
    cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, NIHU_GB_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    ctx->allocs[*out] = bytes;
    ctx->used += bytes;
    return NIHU_GB_OK;
}

void dfree(nihu_gb_ctx *ctx, void *p)
{
    if (!p) return;
    auto it = ctx->allocs.find(p);
    if (it != ctx->allocs.end()) {
        ctx->used -= it->second;
        ctx->allocs.erase(it);
    }
    cudaFree(p);
}

// named scratch buffer of at least `bytes`, reused across calls
nihu_gb_status scratch(nihu_gb_ctx *ctx, const char *name, size_t bytes, void **out)
{
    auto it = ctx->scratch.find(name);
    if (it != ctx->scratch.end()) {
        if (it->second.second >= bytes) { *out = it->second.first; return NIHU_GB_OK; }
        dfree(ctx, it->second.first);
        ctx->scratch.erase(it);
    }
    nihu_gb_status st = dmalloc(ctx, bytes, out);
    if (st != NIHU_GB_OK) return st;
    ctx->scratch[name] = {*out, bytes};
    return NIHU_GB_OK;
}

void free_near(nihu_gb_ctx *ctx, NearList &nl)
{
    dfree(ctx, nl.col_ptr);
    dfree(ctx, nl.rows);
    dfree(ctx, nl.row_ptr);
    dfree(ctx, nl.row_ent);
    nl = NearList();
}

cudaEvent_t pool_event(nihu_gb_ctx *ctx)
{
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// bracket a phase with events on a stream (no-op unless profiling)
struct Phase {
    nihu_gb_ctx *ctx;
    const char *name;
    cudaStream_t stream;
    cudaEvent_t a = nullptr;
    Phase(nihu_gb_ctx *c, const char *n, cudaStream_t s = nullptr) : ctx(c), name(n), stream(s ? s : c->stream)
    {
        if (ctx->profiling) {
            a = pool_event(ctx);
            cudaEventRecord(a, stream);
        }
    }
    ~Phase()
    {
        if (a) {
            cudaEvent_t b = pool_event(ctx);
            cudaEventRecord(b, stream);
            ctx->pending.push_back({name, {a, b}});
        }
    }
};

// fold completed phase events into the totals (after a stream sync)
void collect_phases(nihu_gb_ctx *ctx)
{
    for (auto &p : ctx->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.second.second) == cudaSuccess &&
            cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
            auto it = ctx->phases.find(p.first);
            if (it == ctx->phases.end()) {
                ctx->phase_names.push_back(p.first);
                ctx->phases[p.first] = {ms, 1};
            } else {
                it->second.first += ms;
                it->second.second += 1;
            }
        }
        ctx->event_pool.push_back(p.second.first);
        ctx->event_pool.push_back(p.second.second);
    }
    ctx->pending.clear();
}

nihu_gb_status sync(nihu_gb_ctx *ctx)
{
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    if (!ctx->pending.empty()) collect_phases(ctx);
    return NIHU_GB_OK;
}

// build (or fetch) the column-sorted nearly singular pair list of a mesh pair
nihu_gb_status get_near(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, NearList **out)
{
    auto key = std::make_pair(test->uid, trial->uid);
    auto it = ctx->near.find(key);
    if (it != ctx->near.end()) { *out = &it->second; return NIHU_GB_OK; }
    NearList nl;
    nl.n_cols = (int)trial->n;
    int same = test == trial;
    void *counts = nullptr, *colptr = nullptr, *grid = nullptr;
    nihu_gb_status st = dmalloc(ctx, sizeof(int) * (trial->n + 1), &counts);
    if (st) return st;
    st = dmalloc(ctx, sizeof(int64_t) * (trial->n + 1), &colptr);
    if (st) { dfree(ctx, counts); return st; }
    nl.col_ptr = (int64_t *)colptr;
    st = scratch(ctx, "near_grid", near_grid_scratch_bytes((int)test->n), &grid);
    if (st) { dfree(ctx, counts); free_near(ctx, nl); return st; }
    cudaError_t e;
    {
        Phase ph(ctx, "near_list");
        e = launch_near_grid_count(test->dm, trial->dm, same, grid, (int *)counts, ctx->stream);
        if (e == cudaSuccess) e = launch_scan((int *)counts, (int)trial->n, nl.col_ptr, ctx->stream);
    }
    ctx->launches += 5;
    int64_t nnz = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nnz, nl.col_ptr + trial->n, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(ctx, counts);
    if (e != cudaSuccess) { free_near(ctx, nl); return cuda_fail(ctx, e, "nearly singular pair count"); }
    nl.nnz = nnz;
    void *rows = nullptr, *tmp = nullptr;
    st = dmalloc(ctx, sizeof(int) * (nnz > 0 ? nnz : 1), &rows);
    if (st) { free_near(ctx, nl); return st; }
    nl.rows = (int *)rows;
    st = scratch(ctx, "near_grid_rows", sizeof(int) * (nnz > 0 ? nnz : 1), &tmp);
    if (st) { free_near(ctx, nl); return st; }
    {
        Phase ph(ctx, "near_list");
        e = launch_near_grid_fill(test->dm, trial->dm, same, grid, nl.col_ptr, (int *)tmp, nl.rows, ctx->stream);
    }
    ctx->launches += 1;
    if (e != cudaSuccess) { free_near(ctx, nl); return cuda_fail(ctx, e, "nearly singular pair fill"); }
    ctx->near[key] = nl;
    *out = &ctx->near[key];
    return NIHU_GB_OK;
}

// the row index of a near list (NearList::row_ptr / row_ent), built once on
// the host from the column lists: the items of each row in column order
nihu_gb_status near_rows(nihu_gb_ctx *ctx, NearList *nl, bool same_mesh, int64_t n_rows)
{
    if (nl->row_ptr) return NIHU_GB_OK;
    const int64_t nnz = nl->nnz, n_cols = nl->n_cols;
    if (nnz + n_cols > 0x7fffffff) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "near list too long for a row index");
    std::vector<int64_t> cp(n_cols + 1);
    std::vector<int> rows(nnz);
    CK(cudaMemcpyAsync(cp.data(), nl->col_ptr, sizeof(int64_t) * cp.size(), cudaMemcpyDeviceToHost, ctx->stream));
    if (nnz) CK(cudaMemcpyAsync(rows.data(), nl->rows, sizeof(int) * nnz, cudaMemcpyDeviceToHost, ctx->stream));
    nihu_gb_status st = sync(ctx);
    if (st) return st;
    const int64_t n_self = same_mesh ? std::min(n_cols, n_rows) : 0;
    std::vector<int64_t> rp(n_rows + 1, 0);
    for (int64_t p = 0; p < nnz; ++p) {
        if (rows[p] < 0 || rows[p] >= n_rows) return fail(ctx, NIHU_GB_ERR_RUNTIME, "near list row out of range");
        ++rp[rows[p] + 1];
    }
    for (int64_t j = 0; j < n_self; ++j) ++rp[j + 1];
    for (int64_t i = 0; i < n_rows; ++i) rp[i + 1] += rp[i];
    std::vector<int2> ent(std::max<int64_t>(rp[n_rows], 1));
    std::vector<int64_t> fill(rp.begin(), rp.end() - 1);
    for (int64_t j = 0; j < n_cols; ++j) {
        for (int64_t p = cp[j]; p < cp[j + 1]; ++p) ent[fill[rows[p]]++] = make_int2((int)p, (int)j);
        if (j < n_self) ent[fill[j]++] = make_int2((int)(nnz + j), (int)j);
    }
    void *drp = nullptr, *dent = nullptr;
    if ((st = dmalloc(ctx, sizeof(int64_t) * rp.size(), &drp))) return st;
    if ((st = dmalloc(ctx, sizeof(int2) * ent.size(), &dent))) {
        dfree(ctx, drp);
        return st;
    }
    cudaError_t e = cudaMemcpyAsync(drp, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dent, ent.data(), sizeof(int2) * ent.size(), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // the host vectors die here
    if (e != cudaSuccess) {
        dfree(ctx, drp);
        dfree(ctx, dent);
        return cuda_fail(ctx, e, "near list row index");
    }
    nl->row_ptr = (int64_t *)drp;
    nl->row_ent = (int2 *)dent;
    return NIHU_GB_OK;
}

size_t elem_bytes(int dtype) { return dtype == NIHU_GB_C64 ? 8 : 16; }

cudaError_t timed_gemv(nihu_gb_ctx *ctx, int dtype, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *x,
                       double2 *y, double are, double aim, double bre, double bim, double2 *partial, int splits)
{
    Phase ph(ctx, dtype == 0 ? "gemv_c64" : "gemv_c128");
    ctx->launches += 2;
    return launch_gemv(dtype, A, m, n, lda, x, y, are, aim, bre, bim, partial, splits, ctx->stream);
}

bool valid_dtype(int d) { return d == NIHU_GB_C64 || d == NIHU_GB_C128; }
bool valid_where(int w) { return w == NIHU_GB_HOST || w == NIHU_GB_DEVICE; }

// regular + singular kernels for columns [j0, j1) into device buffers whose
// column j starts at out + (j - j0) * ld
// The FP64 singular/nearly singular kernel and the FP32 regular kernel write
// disjoint entries and load different pipes (FP64 vs FMA/XU + HBM stores), so
// they run concurrently: the singular kernel first, on the high-priority
// auxiliary stream with one block per SM, the regular kernel on the main
// stream filling the remaining SM resources; the main stream then joins.
nihu_gb_status assemble_panel(nihu_gb_ctx *ctx, RegularArgs a, NearList *nl)
{
    cudaError_t e = cudaEventRecord(ctx->ev_fork, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_fork, 0);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fork");
    {
        Phase ph(ctx, "assemble_singular", ctx->aux_stream);
        e = launch_assemble_singular(a, *nl, ctx->d_flag, ctx->aux_stream);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "assemble_singular launch");
    if ((e = cudaEventRecord(ctx->ev_join, ctx->aux_stream)) != cudaSuccess) return cuda_fail(ctx, e, "join");
    {
        Phase ph(ctx, "assemble_regular");
        e = launch_assemble_regular(a, ctx->stream);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "assemble_regular launch");
    if ((e = cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0)) != cudaSuccess) return cuda_fail(ctx, e, "join");
    ctx->launches += 2;
    return NIHU_GB_OK;
}

nihu_gb_status check_flag(nihu_gb_ctx *ctx)
{
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    nihu_gb_status st = sync(ctx);
    if (st) return st;
    if (flag) {
        CK(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
        return fail(ctx, NIHU_GB_ERR_RUNTIME, "Could not perform inverse mapping (nearly singular pair " +
                                                  std::to_string(flag - 1) + ")");
    }
    return NIHU_GB_OK;
}

// columns [j0, j1) of up to two outputs into device buffers whose column j
// starts at out + (j - j0) * ld
using PanelFn = std::function<nihu_gb_status(void *o0, void *o1, int64_t ld, int j0, int j1)>;

// host outputs: column panels, double-buffered; the D2H copies on the copy
// stream overlap the next panel's kernels (out0 / out1 may be NULL)
nihu_gb_status assemble_host_panels(nihu_gb_ctx *ctx, int64_t M, int64_t N, int dtype, void *out0, void *out1, int64_t ld,
                                    int accumulate, const PanelFn &fn)
{
    const size_t es = elem_bytes(dtype);
    nihu_gb_status st = NIHU_GB_OK;
    const int nbuf_ops = (out0 ? 1 : 0) + (out1 ? 1 : 0);
    const size_t col_bytes = (size_t)M * es;
    size_t panel_cap = (size_t)256 << 20;  // bytes per buffer
    if (ctx->budget) {
        size_t avail = ctx->budget > ctx->used ? ctx->budget - ctx->used : 0;
        panel_cap = std::min(panel_cap, avail / (2 * nbuf_ops + 1));
    }
    int64_t P = std::max<int64_t>(1, (int64_t)(panel_cap / col_bytes));
    P = std::min<int64_t>(P, N);
    void *buf[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    const char *names[2][2] = {{"panel_s0", "panel_d0"}, {"panel_s1", "panel_d1"}};
    for (int b = 0; b < 2; ++b)
        for (int o = 0; o < 2; ++o) {
            if (!(o == 0 ? out0 : out1)) continue;
            st = scratch(ctx, names[b][o], col_bytes * P, &buf[b][o]);
            if (st) return st;
        }
    cudaEvent_t computed[2], copied[2];
    for (int b = 0; b < 2; ++b) {
        cudaEventCreateWithFlags(&computed[b], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming);
    }
    void *outs[2] = {out0, out1};
    cudaError_t e = cudaSuccess;
    int b = 0;
    bool used[2] = {false, false};
    for (int64_t j0 = 0; j0 < N && e == cudaSuccess && st == NIHU_GB_OK; j0 += P, b ^= 1) {
        const int64_t j1 = std::min(N, j0 + P);
        if (used[b]) e = cudaStreamWaitEvent(ctx->stream, copied[b], 0);
        for (int o = 0; o < 2 && e == cudaSuccess; ++o) {
            if (!buf[b][o] || !accumulate) continue;
            e = cudaMemcpy2DAsync(buf[b][o], col_bytes, (char *)outs[o] + j0 * ld * es, ld * es, col_bytes, j1 - j0,
                                  cudaMemcpyHostToDevice, ctx->stream);
        }
        if (e != cudaSuccess) break;
        st = fn(buf[b][0], buf[b][1], M, (int)j0, (int)j1);
        if (st) break;
        e = cudaEventRecord(computed[b], ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, computed[b], 0);
        for (int o = 0; o < 2 && e == cudaSuccess; ++o) {
            if (!buf[b][o]) continue;
            e = cudaMemcpy2DAsync((char *)outs[o] + j0 * ld * es, ld * es, buf[b][o], col_bytes, col_bytes, j1 - j0,
                                  cudaMemcpyDeviceToHost, ctx->copy_stream);
        }
        if (e == cudaSuccess) e = cudaEventRecord(copied[b], ctx->copy_stream);
        used[b] = true;
    }
    cudaError_t e2 = cudaStreamSynchronize(ctx->copy_stream);
    cudaError_t e3 = cudaStreamSynchronize(ctx->stream);
    for (int q = 0; q < 2; ++q) {
        cudaEventDestroy(computed[q]);
        cudaEventDestroy(copied[q]);
    }
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "panel assembly");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "panel copy");
    if (e3 != cudaSuccess) return cuda_fail(ctx, e3, "panel compute");
    return check_flag(ctx);
}

}  // namespace

extern "C" {

nihu_gb_status nihu_gb_ctx_create(int device, void *stream, size_t hbm_budget_bytes, nihu_gb_ctx **out)
{
    if (!out) return NIHU_GB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return NIHU_GB_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return NIHU_GB_ERR_NO_DEVICE;
    nihu_gb_ctx *ctx = new nihu_gb_ctx();
    ctx->device = device;
    ctx->budget = hbm_budget_bytes;
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return NIHU_GB_ERR_CUDA; }
        ctx->own_stream = true;
    }
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->aux_stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        nihu_gb_ctx_destroy(ctx);
        return NIHU_GB_ERR_CUDA;
    }
    void *flag = nullptr;
    if (dmalloc(ctx, 4 * sizeof(int), &flag) != NIHU_GB_OK) { nihu_gb_ctx_destroy(ctx); return NIHU_GB_ERR_OUT_OF_MEMORY; }
    ctx->d_flag = (int *)flag;
    cudaMemset(ctx->d_flag, 0, 4 * sizeof(int));
    if (cudaMallocHost(&ctx->h_small, 1 << 16) != cudaSuccess) { nihu_gb_ctx_destroy(ctx); return NIHU_GB_ERR_CUDA; }
    *out = ctx;
    return NIHU_GB_OK;
}

void nihu_gb_ctx_destroy(nihu_gb_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &kv : ctx->near) free_near(ctx, kv.second);
    for (auto &kv : ctx->scratch) dfree(ctx, kv.second.first);
    dfree(ctx, ctx->d_flag);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->cublas) cublasDestroy(ctx->cublas);
    if (ctx->lu_exec) cudaGraphExecDestroy(ctx->lu_exec);
    collect_phases(ctx);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->aux_stream) cudaStreamSynchronize(ctx->aux_stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *nihu_gb_last_error(const nihu_gb_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

nihu_gb_status nihu_gb_ctx_set_profiling(nihu_gb_ctx *ctx, int enable)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    ctx->profiling = enable != 0;
    return NIHU_GB_OK;
}

nihu_gb_status nihu_gb_ctx_profile(const nihu_gb_ctx *ctx, int index, const char **name, double *total_ms,
                                   int64_t *launches)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (index < 0 || index >= (int)ctx->phase_names.size()) return NIHU_GB_ERR_OUT_OF_RANGE;
    const std::string &nm = ctx->phase_names[index];
    auto it = ctx->phases.find(nm);
    if (name) *name = nm.c_str();
    if (total_ms) *total_ms = it->second.first;
    if (launches) *launches = it->second.second;
    return NIHU_GB_OK;
}

void nihu_gb_ctx_profile_reset(nihu_gb_ctx *ctx)
{
    if (!ctx) return;
    ctx->phases.clear();
    ctx->phase_names.clear();
}
void *nihu_gb_ctx_stream(const nihu_gb_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }
size_t nihu_gb_ctx_device_bytes(const nihu_gb_ctx *ctx) { return ctx ? ctx->used : 0; }
int64_t nihu_gb_ctx_launch_count(const nihu_gb_ctx *ctx) { return ctx ? ctx->launches : 0; }

nihu_gb_status nihu_gb_host_alloc(nihu_gb_ctx *ctx, size_t bytes, void **out)
{
    if (!ctx || !out) return NIHU_GB_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 16);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMallocHost");
    return NIHU_GB_OK;
}

void nihu_gb_host_free(void *ptr)
{
    if (ptr) cudaFreeHost(ptr);
}

nihu_gb_status nihu_gb_device_alloc(nihu_gb_ctx *ctx, size_t bytes, void **out)
{
    if (!ctx || !out) return NIHU_GB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    return dmalloc(ctx, bytes, out);
}

void nihu_gb_device_free(nihu_gb_ctx *ctx, void *ptr)
{
    if (!ctx || !ptr) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    dfree(ctx, ptr);
}

nihu_gb_status nihu_gb_memcpy(nihu_gb_ctx *ctx, void *dst, int dst_where, const void *src, int src_where, size_t bytes)
{
    if (!ctx || (!dst && bytes) || (!src && bytes) || !valid_where(dst_where) || !valid_where(src_where))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_memcpy: bad argument");
    cudaSetDevice(ctx->device);
    cudaMemcpyKind kind = dst_where == NIHU_GB_DEVICE ? (src_where == NIHU_GB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice)
                                                      : (src_where == NIHU_GB_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
    CK(cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
    return sync(ctx);
}

// ------------------------------------------------------------------ mesh

nihu_gb_status nihu_gb_mesh_create(nihu_gb_ctx *ctx, const double *nodes, int64_t n_nodes, const int32_t *elems,
                                   int64_t n_elems, int64_t elem_cols, nihu_gb_mesh **out)
{
    if (!ctx || !out) return NIHU_GB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_nodes < 0 || n_elems < 0 || (n_nodes && !nodes) || (n_elems && !elems) || elem_cols < 4 ||
        elem_cols > 64 || n_elems > 0x3fffffff)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_mesh_create: bad mesh arrays");
    cudaSetDevice(ctx->device);
    nihu_gb_mesh *m = new nihu_gb_mesh();
    m->ctx = ctx;
    m->uid = ctx->next_uid++;
    m->n = n_elems;
    m->dm.n = (int)n_elems;
    const int64_t n = std::max<int64_t>(n_elems, 1);
    struct Req { void **p; size_t bytes; };
    void *corners, *center, *size, *nc, *chi, *clo, *p0, *pts32, *pts64, *dyn42, *nid, *frame;
    Req reqs[] = {{&corners, sizeof(double) * 12 * n}, {&center, sizeof(double) * 3 * n}, {&size, sizeof(double) * n},
                  {&nc, sizeof(int8_t) * n}, {&chi, sizeof(float4) * n}, {&clo, sizeof(float4) * n},
                  {&p0, sizeof(float4) * n}, {&pts32, sizeof(float4) * 2 * 2 * SLOTS * n},
                  {&pts64, sizeof(double) * 8 * 2 * SLOTS * n}, {&dyn42, sizeof(Pt4) * 42 * n},
                  {&nid, sizeof(int4) * n}, {&frame, sizeof(double) * 16 * n}};
    for (auto &r : reqs) {
        nihu_gb_status st = dmalloc(ctx, r.bytes, r.p);
        if (st) { nihu_gb_mesh_destroy(m); return st; }
        m->bufs.push_back(*r.p);
    }
    m->dm.corners = (double *)corners;
    m->dm.center = (double *)center;
    m->dm.size = (double *)size;
    m->dm.nc = (int8_t *)nc;
    m->dm.chi = (float4 *)chi;
    m->dm.clo = (float4 *)clo;
    m->dm.p0 = (float4 *)p0;
    m->dm.pts32 = (float4 *)pts32;
    m->dm.pts64 = (double *)pts64;
    m->dm.dyn42 = (Pt4 *)dyn42;
    m->dm.nid = (int4 *)nid;
    m->dm.frame = (double *)frame;
    for (int64_t e = 0; e < n_elems; ++e) {
        int32_t t = elems[e * elem_cols];
        if (t == NIHU_GB_TRIA_1) m->dm.has_tria = 1;
        else if (t == NIHU_GB_QUAD_1) m->dm.has_quad = 1;
        else {
            nihu_gb_mesh_destroy(m);
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT,
                        "nihu_gb_mesh_create: unknown element type id " + std::to_string(t) + " in row " + std::to_string(e));
        }
        int nc_e = t == NIHU_GB_TRIA_1 ? 3 : 4;
        for (int a = 0; a < nc_e; ++a) {
            int32_t nd = elems[e * elem_cols + 1 + a];
            if (nd < 0 || nd >= n_nodes) {
                nihu_gb_mesh_destroy(m);
                return fail(ctx, NIHU_GB_ERR_OUT_OF_RANGE,
                            "nihu_gb_mesh_create: node index out of range in element " + std::to_string(e));
            }
        }
    }
    if (n_elems > 0) {
        void *dnodes = nullptr, *delems = nullptr;
        nihu_gb_status st = dmalloc(ctx, sizeof(double) * 3 * std::max<int64_t>(n_nodes, 1), &dnodes);
        if (st) { nihu_gb_mesh_destroy(m); return st; }
        st = dmalloc(ctx, sizeof(int32_t) * n_elems * elem_cols, &delems);
        if (st) { dfree(ctx, dnodes); nihu_gb_mesh_destroy(m); return st; }
        cudaError_t e = cudaMemcpyAsync(dnodes, nodes, sizeof(double) * 3 * n_nodes, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(delems, elems, sizeof(int32_t) * n_elems * elem_cols, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_flag, 0, 4 * sizeof(int), ctx->stream);
        unsigned long long *dmax = (unsigned long long *)(ctx->d_flag + 2);
        if (e == cudaSuccess)
            e = launch_mesh_geometry((const double *)dnodes, n_nodes, (const int32_t *)delems, (int)n_elems,
                                     (int)elem_cols, m->dm, ctx->d_flag, dmax, ctx->stream);
        ctx->launches += 1;
        int bad = 0;
        unsigned long long smax = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&smax, dmax, sizeof(smax), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        dfree(ctx, dnodes);
        dfree(ctx, delems);
        if (e != cudaSuccess) { nihu_gb_mesh_destroy(m); return cuda_fail(ctx, e, "mesh geometry"); }
        std::memcpy(&m->size_max, &smax, sizeof(double));
        cudaMemsetAsync(ctx->d_flag, 0, 4 * sizeof(int), ctx->stream);
        if (bad) {
            nihu_gb_mesh_destroy(m);
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "invalid element " + std::to_string(bad - 1));
        }
    }
    *out = m;
    return NIHU_GB_OK;
}

void nihu_gb_mesh_destroy(nihu_gb_mesh *m)
{
    if (!m) return;
    nihu_gb_ctx *ctx = m->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto it = ctx->near.begin(); it != ctx->near.end();) {
        if (it->first.first == m->uid || it->first.second == m->uid) {
            free_near(ctx, it->second);
            it = ctx->near.erase(it);
        } else {
            ++it;
        }
    }
    for (void *p : m->bufs) dfree(ctx, p);
    delete m;
}

int64_t nihu_gb_mesh_num_elements(const nihu_gb_mesh *m) { return m ? m->n : -1; }

// ---------------------------------------------------------------- assembly

nihu_gb_status nihu_gb_assemble(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family,
                                int ops, double k, double alpha_re, double alpha_im, int precision, int dtype,
                                void *out_slp, void *out_dlp, int64_t ld, int accumulate, int where)
{
    return nihu_gb_assemble_c(ctx, test, trial, family, ops, k, 0.0, alpha_re, alpha_im, precision, dtype, out_slp,
                              out_dlp, ld, accumulate, where);
}

nihu_gb_status nihu_gb_assemble_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family,
                                  int ops, double k, double k_im, double alpha_re, double alpha_im, int precision,
                                  int dtype, void *out_slp, void *out_dlp, int64_t ld, int accumulate, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!test || !trial || test->ctx != ctx || trial->ctx != ctx)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: meshes must belong to the context");
    if (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: unknown kernel family");
    if (ops < 1 || ops > 3) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: ops must be SLP, DLP or both");
    if (((ops & NIHU_GB_SLP) && !out_slp) || ((ops & NIHU_GB_DLP) && !out_dlp))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: missing output buffer");
    if (!valid_dtype(dtype) || !valid_where(where) || (precision != 0 && precision != 1))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: bad dtype, precision or location");
    if (ld < std::max<int64_t>(test->n, 1)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: ld < rows");
    if (!std::isfinite(k) || !std::isfinite(k_im) || !std::isfinite(alpha_re) || !std::isfinite(alpha_im))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble: non-finite wave number or scale");
    if (test->n == 0 || trial->n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    NearList *nl = nullptr;
    nihu_gb_status st = get_near(ctx, test, trial, &nl);
    if (st) return st;

    RegularArgs a;
    a.test = test->dm;
    a.trial = trial->dm;
    a.same_mesh = test == trial;
    a.family = family;
    a.ops = ops;
    a.k = family == NIHU_GB_HELMHOLTZ_3D ? k : 0.0;
    a.k_im = family == NIHU_GB_HELMHOLTZ_3D ? k_im : 0.0;
    a.alpha_re = alpha_re;
    a.alpha_im = alpha_im;
    a.precision = precision;
    a.dtype = dtype;
    a.accumulate = accumulate ? 1 : 0;
    a.trial_size_max = trial->size_max;
    a.k32 = (float)a.k;
    a.k_im32 = (float)a.k_im;
    a.alpha_re32 = (float)alpha_re;
    a.alpha_im32 = (float)alpha_im;
    a.unit_alpha = alpha_re == 1.0 && alpha_im == 0.0;
    const int64_t M = test->n, N = trial->n;

    if (where == NIHU_GB_DEVICE) {
        a.out_s = out_slp;
        a.out_d = out_dlp;
        a.ld = ld;
        a.j0 = 0;
        a.j1 = (int)N;
        st = assemble_panel(ctx, a, nl);
        if (st) return st;
        return check_flag(ctx);
    }

    return assemble_host_panels(ctx, M, N, dtype, (ops & NIHU_GB_SLP) ? out_slp : nullptr,
                                (ops & NIHU_GB_DLP) ? out_dlp : nullptr, ld, accumulate,
                                [&](void *o0, void *o1, int64_t pld, int j0, int j1) {
                                    a.out_s = o0;
                                    a.out_d = o1;
                                    a.ld = pld;
                                    a.j0 = j0;
                                    a.j1 = j1;
                                    return assemble_panel(ctx, a, nl);
                                });
}

}  // extern "C"

namespace {

constexpr int BM_ALL = NIHU_GB_SLP | NIHU_GB_DLP | NIHU_GB_DLPT | NIHU_GB_HSP;

// Burton-Miller operators on one column panel: the FP64 nearly singular and
// self kernel on the auxiliary stream beside the regular kernel (as
// assemble_panel), each evaluating every operator of b.ops
nihu_gb_status assemble_panel_bm(nihu_gb_ctx *ctx, const BmArgs &b, NearList *nl)
{
    cudaError_t e = cudaEventRecord(ctx->ev_fork, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_fork, 0);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fork");
    {
        Phase ph(ctx, "assemble_singular_bm", ctx->aux_stream);
        e = launch_assemble_singular_bm(b, *nl, ctx->aux_stream);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "assemble_singular_bm launch");
    if ((e = cudaEventRecord(ctx->ev_join, ctx->aux_stream)) != cudaSuccess) return cuda_fail(ctx, e, "join");
    {
        Phase ph(ctx, "assemble_regular_bm");
        e = launch_assemble_regular_bm(b, ctx->stream);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "assemble_regular_bm launch");
    if ((e = cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0)) != cudaSuccess) return cuda_fail(ctx, e, "join");
    ctx->launches += 2;
    return NIHU_GB_OK;
}

// checks shared by the Burton-Miller entry points
nihu_gb_status bm_check(nihu_gb_ctx *ctx, const char *fn, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                        int family, double k, int precision, int dtype, int where, int64_t ld)
{
    const std::string f(fn);
    if (!test || !trial || test->ctx != ctx || trial->ctx != ctx)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, f + ": meshes must belong to the context");
    if (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, f + ": unknown kernel family");
    if (!valid_dtype(dtype) || !valid_where(where) || (precision != 0 && precision != 1))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, f + ": bad dtype, precision or location");
    if (ld < std::max<int64_t>(test->n, 1)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, f + ": ld < rows");
    if (!std::isfinite(k)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, f + ": non-finite wave number");
    if (trial->dm.has_quad)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, f + ": DLPt / HSP: constant triangle trial elements only");
    return NIHU_GB_OK;
}

BmArgs bm_args(const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family, int ops, double k, double k_im,
               const double c[8], int precision, int dtype, int accumulate)
{
    BmArgs b;
    b.test = test->dm;
    b.trial = trial->dm;
    b.same_mesh = test == trial;
    b.family = family;
    b.ops = ops;
    b.k = family == NIHU_GB_HELMHOLTZ_3D ? k : 0.0;
    b.k32 = (float)b.k;
    b.k_im = family == NIHU_GB_HELMHOLTZ_3D ? k_im : 0.0;
    b.k_im32 = (float)b.k_im;
    for (int o = 0; o < 4; ++o) {
        b.cre[o] = c[2 * o];
        b.cim[o] = c[2 * o + 1];
        b.cre32[o] = (float)c[2 * o];
        b.cim32[o] = (float)c[2 * o + 1];
    }
    b.precision = precision;
    b.dtype = dtype;
    b.accumulate = accumulate ? 1 : 0;
    b.trial_size_max = trial->size_max;
    return b;
}

// all columns of the operators in b.ops into out_a / out_b (device or host)
nihu_gb_status assemble_bm_all(nihu_gb_ctx *ctx, BmArgs b, NearList *nl, void *out_a, void *out_b, int64_t ld,
                               int where, int64_t M, int64_t N)
{
    if (where == NIHU_GB_DEVICE) {
        b.out_a = out_a;
        b.out_b = out_b;
        b.ld = ld;
        b.j0 = 0;
        b.j1 = (int)N;
        nihu_gb_status st = assemble_panel_bm(ctx, b, nl);
        if (st) return st;
        return check_flag(ctx);
    }
    return assemble_host_panels(ctx, M, N, b.dtype, out_a, out_b, ld, b.accumulate,
                                [&](void *o0, void *o1, int64_t pld, int j0, int j1) {
                                    b.out_a = o0;
                                    b.out_b = o1;
                                    b.ld = pld;
                                    b.j0 = j0;
                                    b.j1 = j1;
                                    return assemble_panel_bm(ctx, b, nl);
                                });
}

}  // namespace

extern "C" {

nihu_gb_status nihu_gb_assemble_bm(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family,
                                   int ops, double k, double alpha_re, double alpha_im, int precision, int dtype,
                                   void *out_dlpt, void *out_hsp, int64_t ld, int accumulate, int where)
{
    return nihu_gb_assemble_bm_c(ctx, test, trial, family, ops, k, 0.0, alpha_re, alpha_im, precision, dtype, out_dlpt,
                                 out_hsp, ld, accumulate, where);
}

nihu_gb_status nihu_gb_assemble_bm_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                     int family, int ops, double k, double k_im, double alpha_re, double alpha_im,
                                     int precision, int dtype, void *out_dlpt, void *out_hsp, int64_t ld,
                                     int accumulate, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    nihu_gb_status st = bm_check(ctx, "nihu_gb_assemble_bm", test, trial, family, k, precision, dtype, where, ld);
    if (st) return st;
    if (!std::isfinite(k_im)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_bm: non-finite wave number");
    if (ops < NIHU_GB_DLPT || (ops & ~(NIHU_GB_DLPT | NIHU_GB_HSP)))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_bm: ops must be DLPt, HSP or both");
    if (((ops & NIHU_GB_DLPT) && !out_dlpt) || ((ops & NIHU_GB_HSP) && !out_hsp))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_bm: missing output buffer");
    if (!std::isfinite(alpha_re) || !std::isfinite(alpha_im))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_bm: non-finite scale");
    if (test->n == 0 || trial->n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    NearList *nl = nullptr;
    if ((st = get_near(ctx, test, trial, &nl))) return st;
    const double c[8] = {0, 0, 0, 0, alpha_re, alpha_im, alpha_re, alpha_im};
    BmArgs b = bm_args(test, trial, family, ops, k, k_im, c, precision, dtype, accumulate);
    return assemble_bm_all(ctx, b, nl, (ops & NIHU_GB_HSP) ? out_hsp : nullptr,
                           (ops & NIHU_GB_DLPT) ? out_dlpt : nullptr, ld, where, test->n, trial->n);
}

nihu_gb_status nihu_gb_assemble_burton_miller(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                              double coupling_re, double coupling_im, int precision, int dtype,
                                              void *out_a, void *out_b, int64_t ld, int where)
{
    return nihu_gb_assemble_burton_miller_c(ctx, mesh, family, k, 0.0, coupling_re, coupling_im, precision, dtype,
                                            out_a, out_b, ld, where);
}

nihu_gb_status nihu_gb_assemble_burton_miller_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                                double k_im, double coupling_re, double coupling_im, int precision,
                                                int dtype, void *out_a, void *out_b, int64_t ld, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    nihu_gb_status st =
        bm_check(ctx, "nihu_gb_assemble_burton_miller", mesh, mesh, family, k, precision, dtype, where, ld);
    if (st) return st;
    if (!std::isfinite(k_im))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_burton_miller: non-finite wave number");
    if (!out_a || !out_b) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_burton_miller: missing output buffer");
    if (!std::isfinite(coupling_re) || !std::isfinite(coupling_im))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_burton_miller: non-finite coupling");
    const int64_t n = mesh->n;
    if (n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    NearList *nl = nullptr;
    if ((st = get_near(ctx, mesh, mesh, &nl))) return st;
    const double c[8] = {1, 0, 1, 0, coupling_re, coupling_im, coupling_re, coupling_im};
    BmArgs b = bm_args(mesh, mesh, family, BM_ALL, k, k_im, c, precision, dtype, 0);
    if (where == NIHU_GB_DEVICE) {
        if ((st = assemble_bm_all(ctx, b, nl, out_a, out_b, ld, where, n, n))) return st;
        // A -= I/2, B += c/2 I (helmholtz_3d_coll.cpp:71-72, 91)
        CK(launch_add_identity((int)n, -0.5, 0.0, dtype, out_a, ld, ctx->stream));
        CK(launch_add_identity((int)n, coupling_re / 2.0, coupling_im / 2.0, dtype, out_b, ld, ctx->stream));
        ctx->launches += 2;
        return sync(ctx);
    }
    if ((st = assemble_bm_all(ctx, b, nl, out_a, out_b, ld, where, n, n))) return st;
    if ((st = nihu_gb_add_identity(ctx, mesh, -0.5, 0.0, dtype, out_a, ld, NIHU_GB_HOST))) return st;
    return nihu_gb_add_identity(ctx, mesh, coupling_re / 2.0, coupling_im / 2.0, dtype, out_b, ld, NIHU_GB_HOST);
}

nihu_gb_status nihu_gb_assemble_pairs(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family,
                                      int ops, double k, const double *coef, const double *ident, int precision,
                                      int dtype, int64_t n_pairs, const int32_t *rows, const int32_t *cols,
                                      void *out_a, void *out_b, int where)
{
    return nihu_gb_assemble_pairs_c(ctx, test, trial, family, ops, k, 0.0, coef, ident, precision, dtype, n_pairs,
                                    rows, cols, out_a, out_b, where);
}

nihu_gb_status nihu_gb_assemble_pairs_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                        int family, int ops, double k, double k_im, const double *coef,
                                        const double *ident, int precision, int dtype, int64_t n_pairs,
                                        const int32_t *rows, const int32_t *cols, void *out_a, void *out_b, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!std::isfinite(k_im)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_pairs: non-finite wave number");
    const char *fn = "nihu_gb_assemble_pairs";
    if (!test || !trial || test->ctx != ctx || trial->ctx != ctx)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, std::string(fn) + ": meshes must belong to the context");
    if (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, std::string(fn) + ": unknown kernel family");
    if (ops < 1 || ops > BM_ALL)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, std::string(fn) + ": ops must be a mask of SLP, DLP, DLPt, HSP");
    const bool need_a = (ops & (NIHU_GB_DLP | NIHU_GB_HSP)) != 0, need_b = (ops & (NIHU_GB_SLP | NIHU_GB_DLPT)) != 0;
    if (n_pairs < 0 || (n_pairs > 0 && (!rows || !cols || (need_a && !out_a) || (need_b && !out_b))))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, std::string(fn) + ": missing pair or output array");
    if (!valid_dtype(dtype) || !valid_where(where) || (precision != 0 && precision != 1) || !std::isfinite(k))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, std::string(fn) + ": bad dtype, precision, location or wave number");
    if ((ops & (NIHU_GB_DLPT | NIHU_GB_HSP)) && trial->dm.has_quad)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, std::string(fn) + ": DLPt / HSP: constant triangle trial elements only");
    if (n_pairs == 0) return NIHU_GB_OK;
    if (where == NIHU_GB_HOST) {
        for (int64_t p = 0; p < n_pairs; ++p)
            if (rows[p] < 0 || rows[p] >= test->n || cols[p] < 0 || cols[p] >= trial->n)
                return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT,
                            std::string(fn) + ": pair " + std::to_string(p) + " has an index out of range");
    }
    cudaSetDevice(ctx->device);
    nihu_gb_status st;
    PairArgs a;
    a.test = test->dm;
    a.trial = trial->dm;
    a.same_mesh = test == trial;
    a.family = family;
    a.ops = ops;
    a.k = family == NIHU_GB_HELMHOLTZ_3D ? k : 0.0;
    a.k32 = (float)a.k;
    a.k_im = family == NIHU_GB_HELMHOLTZ_3D ? k_im : 0.0;
    a.k_im32 = (float)a.k_im;
    for (int o = 0; o < 4; ++o) {
        a.cre[o] = coef ? coef[2 * o] : 1.0;
        a.cim[o] = coef ? coef[2 * o + 1] : 0.0;
        a.cre32[o] = (float)a.cre[o];
        a.cim32[o] = (float)a.cim[o];
    }
    for (int o = 0; o < 2; ++o) {
        a.id_re[o] = ident ? ident[2 * o] : 0.0;
        a.id_im[o] = ident ? ident[2 * o + 1] : 0.0;
    }
    a.precision = precision;
    a.dtype = dtype;
    a.n = n_pairs;
    a.trial_size_max = trial->size_max;
    const size_t es = elem_bytes(dtype);
    void *sing, *flags;
    if ((st = scratch(ctx, "pairs_sing", sizeof(int64_t) * n_pairs, &sing))) return st;
    if ((st = scratch(ctx, "pairs_flags", 32, &flags))) return st;
    a.sing = (int64_t *)sing;
    a.n_sing = (unsigned long long *)flags;
    a.bad = (int *)((char *)flags + 16);
    a.err = ctx->d_flag;
    CK(cudaMemsetAsync(a.bad, 0, sizeof(int), ctx->stream));
    if (where == NIHU_GB_DEVICE) {
        a.rows = rows;
        a.cols = cols;
        a.out_a = need_a ? out_a : nullptr;
        a.out_b = need_b ? out_b : nullptr;
    } else {
        void *dr, *dc, *da = nullptr, *db = nullptr;
        if ((st = scratch(ctx, "pairs_rows", sizeof(int32_t) * n_pairs, &dr))) return st;
        if ((st = scratch(ctx, "pairs_cols", sizeof(int32_t) * n_pairs, &dc))) return st;
        if (need_a && (st = scratch(ctx, "pairs_out_a", es * n_pairs, &da))) return st;
        if (need_b && (st = scratch(ctx, "pairs_out_b", es * n_pairs, &db))) return st;
        CK(cudaMemcpyAsync(dr, rows, sizeof(int32_t) * n_pairs, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(dc, cols, sizeof(int32_t) * n_pairs, cudaMemcpyHostToDevice, ctx->stream));
        a.rows = (const int32_t *)dr;
        a.cols = (const int32_t *)dc;
        a.out_a = da;
        a.out_b = db;
    }
    {
        Phase ph(ctx, "assemble_pairs");
        CK(launch_assemble_pairs(a, ctx->stream));
    }
    ctx->launches += 2;
    if (where == NIHU_GB_HOST) {
        if (need_a) CK(cudaMemcpyAsync(out_a, a.out_a, es * n_pairs, cudaMemcpyDeviceToHost, ctx->stream));
        if (need_b) CK(cudaMemcpyAsync(out_b, a.out_b, es * n_pairs, cudaMemcpyDeviceToHost, ctx->stream));
    }
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, a.bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = check_flag(ctx))) return st;  // synchronises; inverse-mapping failures
    if (bad)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT,
                    std::string(fn) + ": pair " + std::to_string(bad - 1) + " has an index out of range");
    return NIHU_GB_OK;
}

nihu_gb_status nihu_gb_assemble_galerkin(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                         int family, int ops, double k, double alpha_re, double alpha_im, int precision,
                                         int dtype, void *out_slp, void *out_dlp, int64_t ld, int accumulate, int where)
{
    return nihu_gb_assemble_galerkin_c(ctx, test, trial, family, ops, k, 0.0, alpha_re, alpha_im, precision, dtype,
                                       out_slp, out_dlp, ld, accumulate, where);
}

nihu_gb_status nihu_gb_assemble_galerkin_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                           int family, int ops, double k, double k_im, double alpha_re,
                                           double alpha_im, int precision, int dtype, void *out_slp, void *out_dlp,
                                           int64_t ld, int accumulate, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    const std::string fn = "nihu_gb_assemble_galerkin";
    if (!std::isfinite(k_im)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": non-finite wave number");
    if (!test || !trial || test->ctx != ctx || trial->ctx != ctx)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": meshes must belong to the context");
    if (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": unknown kernel family");
    if (ops < 1 || ops > 3) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": ops must be SLP, DLP or both");
    if (((ops & NIHU_GB_SLP) && !out_slp) || ((ops & NIHU_GB_DLP) && !out_dlp))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": missing output buffer");
    if (!valid_dtype(dtype) || !valid_where(where) || (precision != 0 && precision != 1))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": bad dtype, precision or location");
    if (ld < std::max<int64_t>(test->n, 1)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": ld < rows");
    if (!std::isfinite(k) || !std::isfinite(alpha_re) || !std::isfinite(alpha_im))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, fn + ": non-finite wave number or scale");
    const bool same = test == trial;
    if (test->n == 0 || trial->n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    NearList *nl = nullptr;
    nihu_gb_status st = get_near(ctx, test, trial, &nl);
    if (st) return st;
    CK(prepare_galerkin(ctx->stream));
    GalArgs g;
    g.test = test->dm;
    g.trial = trial->dm;
    g.same_mesh = same;
    g.family = family;
    g.ops = ops;
    g.k = family == NIHU_GB_HELMHOLTZ_3D ? k : 0.0;
    g.k32 = (float)g.k;
    g.k_im = family == NIHU_GB_HELMHOLTZ_3D ? k_im : 0.0;
    g.k_im32 = (float)g.k_im;
    g.alpha_re = alpha_re;
    g.alpha_im = alpha_im;
    g.alpha_re32 = (float)alpha_re;
    g.alpha_im32 = (float)alpha_im;
    g.precision = precision;
    g.dtype = dtype;
    g.accumulate = accumulate ? 1 : 0;
    g.extra_cap = (int)std::min<int64_t>(std::max<int64_t>(1024, 8 * trial->n), 1 << 26);
    void *extra, *flags;
    if ((st = scratch(ctx, "gal_extra", sizeof(int2) * g.extra_cap, &extra))) return st;
    if ((st = scratch(ctx, "gal_flags", 16, &flags))) return st;
    g.extra = (int2 *)extra;
    g.n_extra = (unsigned int *)flags;
    g.err = (int *)flags + 1;
    CK(cudaMemsetAsync(g.err, 0, sizeof(int), ctx->stream));
    const int64_t M = test->n, N = trial->n;
    auto panel = [&](void *o0, void *o1, int64_t pld, int j0, int j1) -> nihu_gb_status {
        g.out_s = o0;
        g.out_d = o1;
        g.ld = pld;
        g.j0 = j0;
        g.j1 = j1;
        cudaError_t e = cudaMemsetAsync(g.n_extra, 0, sizeof(unsigned int), ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_fork, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_fork, 0);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "fork");
        {
            Phase ph(ctx, "galerkin_near", ctx->aux_stream);
            e = launch_galerkin_near(g, *nl, 0, nl->nnz + (j1 - j0), ctx->aux_stream);
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "galerkin_near launch");
        if ((e = cudaEventRecord(ctx->ev_join, ctx->aux_stream)) != cudaSuccess) return cuda_fail(ctx, e, "join");
        {
            Phase ph(ctx, "galerkin_regular");
            e = launch_galerkin_regular(g, ctx->stream);
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "galerkin_regular launch");
        if ((e = cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0)) != cudaSuccess) return cuda_fail(ctx, e, "join");
        {
            // pairs beyond 1.5 D sharing a node (none on regular meshes)
            Phase ph(ctx, "galerkin_extra");
            e = launch_galerkin_near(g, *nl, 1, std::min<int64_t>(g.extra_cap, 4 * 1024), ctx->stream);
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "galerkin_extra launch");
        ctx->launches += 3;
        return NIHU_GB_OK;
    };
    if (where == NIHU_GB_DEVICE) {
        if ((st = panel(out_slp, out_dlp, ld, 0, (int)N))) return st;
    } else {
        st = assemble_host_panels(ctx, M, N, dtype, (ops & NIHU_GB_SLP) ? out_slp : nullptr,
                                  (ops & NIHU_GB_DLP) ? out_dlp : nullptr, ld, accumulate, panel);
        if (st) return st;
    }
    int err = 0;
    CK(cudaMemcpyAsync(&err, g.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = check_flag(ctx))) return st;
    if (err)
        return fail(ctx, NIHU_GB_ERR_RUNTIME, fn + ": more node-sharing pairs beyond 1.5 D than the list holds");
    return NIHU_GB_OK;
}

nihu_gb_status nihu_gb_add_mass(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, double alpha_re, double alpha_im, int dtype,
                                void *out, int64_t ld, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!mesh || mesh->ctx != ctx || !out || !valid_dtype(dtype) || !valid_where(where) ||
        ld < std::max<int64_t>(mesh->n, 1))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_add_mass: bad argument");
    const int64_t n = mesh->n;
    if (n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    if (where == NIHU_GB_DEVICE) {
        CK(launch_add_mass((int)n, mesh->dm.pts64, alpha_re, alpha_im, dtype, out, ld, ctx->stream));
        ctx->launches += 1;
        return sync(ctx);
    }
    std::vector<double> w((size_t)n);
    // strided copy of the one-point weights (w J of slot 0, parity 0)
    CK(cudaMemcpy2DAsync(w.data(), sizeof(double), mesh->dm.pts64 + 3, 8 * 2 * SLOTS * sizeof(double), sizeof(double),
                         n, cudaMemcpyDeviceToHost, ctx->stream));
    nihu_gb_status st = sync(ctx);
    if (st) return st;
    for (int64_t i = 0; i < n; ++i) {
        if (dtype == NIHU_GB_C64) {
            float *p = (float *)out + 2 * (i * ld + i);
            p[0] += (float)(alpha_re * w[i]);
            p[1] += (float)(alpha_im * w[i]);
        } else {
            double *p = (double *)out + 2 * (i * ld + i);
            p[0] += alpha_re * w[i];
            p[1] += alpha_im * w[i];
        }
    }
    return NIHU_GB_OK;
}

nihu_gb_status nihu_gb_add_identity(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, double alpha_re, double alpha_im,
                                    int dtype, void *out, int64_t ld, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!mesh || !out || !valid_dtype(dtype) || !valid_where(where) || ld < std::max<int64_t>(mesh->n, 1))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_add_identity: bad argument");
    if (where == NIHU_GB_HOST) {
        const int64_t n = mesh->n;
        for (int64_t i = 0; i < n; ++i) {
            if (dtype == NIHU_GB_C64) {
                float *p = (float *)out + 2 * (i * ld + i);
                p[0] += (float)alpha_re;
                p[1] += (float)alpha_im;
            } else {
                double *p = (double *)out + 2 * (i * ld + i);
                p[0] += alpha_re;
                p[1] += alpha_im;
            }
        }
        return NIHU_GB_OK;
    }
    cudaSetDevice(ctx->device);
    CK(launch_add_identity((int)mesh->n, alpha_re, alpha_im, dtype, out, ld, ctx->stream));
    ctx->launches += 1;
    return sync(ctx);
}

nihu_gb_status nihu_gb_pair_statistics(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                       int64_t counts[11])
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!test || !trial || !counts) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_pair_statistics: bad argument");
    cudaSetDevice(ctx->device);
    void *d = nullptr;
    nihu_gb_status st = scratch(ctx, "stats", sizeof(unsigned long long) * 11, &d);
    if (st) return st;
    CK(cudaMemsetAsync(d, 0, sizeof(unsigned long long) * 11, ctx->stream));
    CK(launch_pair_stats(test->dm, trial->dm, test == trial, (unsigned long long *)d, ctx->stream));
    ctx->launches += 1;
    unsigned long long h[11];
    CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    st = sync(ctx);
    for (int q = 0; q < 11; ++q) counts[q] = (int64_t)h[q];
    return st;
}

nihu_gb_status nihu_gb_near_pairs(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                  int64_t *nnz, int64_t *col_ptr, int32_t *rows)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!test || !trial || !nnz) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_near_pairs: bad argument");
    cudaSetDevice(ctx->device);
    NearList *nl = nullptr;
    nihu_gb_status st = get_near(ctx, test, trial, &nl);
    if (st) return st;
    *nnz = nl->nnz;
    if (col_ptr) CK(cudaMemcpyAsync(col_ptr, nl->col_ptr, sizeof(int64_t) * (trial->n + 1), cudaMemcpyDeviceToHost, ctx->stream));
    if (rows && nl->nnz) CK(cudaMemcpyAsync(rows, nl->rows, sizeof(int32_t) * nl->nnz, cudaMemcpyDeviceToHost, ctx->stream));
    return sync(ctx);
}

// ------------------------------------------------------------------ matvec

nihu_gb_status nihu_gb_matvec(nihu_gb_ctx *ctx, int dtype_a, const void *A, int64_t m, int64_t n, int64_t lda,
                              const void *x, void *y, double alpha_re, double alpha_im, double beta_re, double beta_im,
                              int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!valid_dtype(dtype_a) || !valid_where(where) || m < 0 || n < 0 || lda < std::max<int64_t>(m, 1) ||
        (m && (!A || !y)) || (n && !x))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_matvec: bad argument");
    if (m == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    const size_t es = elem_bytes(dtype_a);
    const void *dA = A;
    const double2 *dx = (const double2 *)x;
    double2 *dy = (double2 *)y;
    nihu_gb_status st;
    if (where == NIHU_GB_HOST) {
        void *pa, *px, *py;
        if ((st = scratch(ctx, "mv_A", es * m * n, &pa))) return st;
        if ((st = scratch(ctx, "mv_x", 16 * std::max<int64_t>(n, 1), &px))) return st;
        if ((st = scratch(ctx, "mv_y", 16 * m, &py))) return st;
        CK(cudaMemcpy2DAsync(pa, es * m, A, es * lda, es * m, n, cudaMemcpyHostToDevice, ctx->stream));
        if (n) CK(cudaMemcpyAsync(px, x, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(py, y, 16 * m, cudaMemcpyHostToDevice, ctx->stream));
        dA = pa;
        dx = (const double2 *)px;
        dy = (double2 *)py;
        lda = m;
    }
    int splits = gemv_splits(m, n, dtype_a);
    void *part;
    if ((st = scratch(ctx, "mv_part", 16 * (size_t)splits * m, &part))) return st;
    CK(timed_gemv(ctx, dtype_a, dA, m, n, lda, dx, dy, alpha_re, alpha_im, beta_re, beta_im, (double2 *)part, splits));
    if (where == NIHU_GB_HOST) CK(cudaMemcpyAsync(y, dy, 16 * m, cudaMemcpyDeviceToHost, ctx->stream));
    return sync(ctx);
}

// ------------------------------------------------------------------ GMRES

namespace {

struct Cplx {
    double re, im;
};

nihu_gb_status gmres_device(nihu_gb_ctx *ctx, int dtype_a, const void *A, int64_t n, int64_t lda, const double2 *b,
                            double2 *x, int restart, int max_iters, double tol, int *iters_out, double *res_out)
{
    typedef std::complex<double> C;
    nihu_gb_status st;
    const int m = restart;
    void *pV, *pw, *pt, *ppart, *pdot, *ph;
    if ((st = scratch(ctx, "gm_V", 16 * (size_t)n * (m + 1), &pV))) return st;
    if ((st = scratch(ctx, "gm_w", 16 * (size_t)n, &pw))) return st;
    if ((st = scratch(ctx, "gm_t", 16 * (size_t)n, &pt))) return st;
    int splits = gemv_splits(n, n, dtype_a);
    if ((st = scratch(ctx, "mv_part", 16 * (size_t)splits * n, &ppart))) return st;
    const int dblocks = dot_blocks(n);
    if ((st = scratch(ctx, "gm_dot", 16 * (size_t)dblocks * (m + 1), &pdot))) return st;
    if ((st = scratch(ctx, "gm_h", 16 * (size_t)(m + 1), &ph))) return st;
    double2 *V = (double2 *)pV, *w = (double2 *)pw, *t = (double2 *)pt, *part = (double2 *)ppart;
    double2 *dot = (double2 *)pdot, *dh = (double2 *)ph;
    Cplx *hsm = (Cplx *)ctx->h_small;  // pinned host scratch, (m + 1) * dblocks <= 4096 entries
    if ((size_t)(m + 1) * dblocks * sizeof(Cplx) > (1 << 16)) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "GMRES restart too large");

    auto norm_of = [&](const double2 *v, double *out) -> nihu_gb_status {
        CK(launch_multidot(v, n, 1, v, dot, dblocks, ctx->stream));
        ctx->launches += 1;
        CK(cudaMemcpyAsync(hsm, dot, 16 * dblocks, cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = sync(ctx))) return st;
        double s = 0;
        for (int q = 0; q < dblocks; ++q) s += hsm[q].re;
        *out = std::sqrt(s);
        return NIHU_GB_OK;
    };
    auto project = [&](int nv, std::vector<C> &h) -> nihu_gb_status {
        // h = V[0..nv)^H w ; w -= V h
        CK(launch_multidot(V, n, nv, w, dot, dblocks, ctx->stream));
        ctx->launches += 1;
        CK(cudaMemcpyAsync(hsm, dot, 16 * (size_t)dblocks * nv, cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = sync(ctx))) return st;
        std::vector<double2> hv(nv);
        for (int v = 0; v < nv; ++v) {
            double sr = 0, si = 0;
            for (int q = 0; q < dblocks; ++q) { sr += hsm[v * dblocks + q].re; si += hsm[v * dblocks + q].im; }
            h[v] += C(sr, si);
            hv[v] = make_double2(sr, si);
        }
        CK(cudaMemcpyAsync(dh, hv.data(), 16 * nv, cudaMemcpyHostToDevice, ctx->stream));
        CK(launch_subtract_combo(V, n, nv, dh, w, ctx->stream));
        ctx->launches += 1;
        return NIHU_GB_OK;
    };

    // r0 = b - A x ; reference normalises by the initial residual norm
    CK(timed_gemv(ctx, dtype_a, A, n, n, lda, x, t, 1.0, 0.0, 0.0, 0.0, part, splits));
    CK(launch_sub(b, t, w, n, ctx->stream));
    ctx->launches += 1;
    double r0norm;
    if ((st = norm_of(w, &r0norm))) return st;
    int iters = 0;
    double rel = 0.0;
    if (r0norm == 0.0) {
        if (iters_out) *iters_out = 0;
        if (res_out) *res_out = 0.0;
        return NIHU_GB_OK;
    }
    double beta = r0norm;
    std::vector<std::vector<C>> H(m + 1, std::vector<C>(m, C(0)));
    std::vector<C> g(m + 1), cs(m), sn(m);
    bool converged = false;
    while (true) {
        CK(launch_scale_copy(w, V, n, 1.0 / beta, ctx->stream));
        ctx->launches += 1;
        std::fill(g.begin(), g.end(), C(0));
        g[0] = beta;
        int kdone = 0;
        bool stop = false;
        for (int k = 0; k < m; ++k) {
            ++iters;
            // w = A v_k
            CK(timed_gemv(ctx, dtype_a, A, n, n, lda, V + (size_t)k * n, w, 1.0, 0.0, 0.0, 0.0, part, splits));
            std::vector<C> h(k + 2, C(0));
            if ((st = project(k + 1, h))) return st;
            if ((st = project(k + 1, h))) return st;  // reorthogonalisation (CGS2)
            double hn;
            if ((st = norm_of(w, &hn))) return st;
            h[k + 1] = hn;
            if (hn > 0.0) {
                CK(launch_scale_copy(w, V + (size_t)(k + 1) * n, n, 1.0 / hn, ctx->stream));
                ctx->launches += 1;
            }
            // apply previous Givens rotations, then a new one
            for (int i = 0; i < k; ++i) {
                C a0 = h[i], a1 = h[i + 1];
                h[i] = std::conj(cs[i]) * a0 + std::conj(sn[i]) * a1;
                h[i + 1] = -sn[i] * a0 + cs[i] * a1;
            }
            double den = std::sqrt(std::norm(h[k]) + std::norm(h[k + 1]));
            if (den == 0.0) { cs[k] = 1.0; sn[k] = 0.0; }
            else { cs[k] = h[k] / den; sn[k] = h[k + 1] / den; }
            C a0 = h[k], a1 = h[k + 1];
            h[k] = std::conj(cs[k]) * a0 + std::conj(sn[k]) * a1;
            h[k + 1] = 0.0;
            C g0 = g[k], g1 = g[k + 1];
            g[k] = std::conj(cs[k]) * g0 + std::conj(sn[k]) * g1;
            g[k + 1] = -sn[k] * g0 + cs[k] * g1;
            for (int i = 0; i <= k; ++i) H[i][k] = h[i];
            kdone = k + 1;
            rel = std::abs(g[k + 1]) / r0norm;
            if (rel < tol || iters >= max_iters || hn == 0.0 || kdone == n) { stop = true; break; }
        }
        // y = H^{-1} g, x += V y
        std::vector<C> yv(kdone);
        for (int i = kdone - 1; i >= 0; --i) {
            C s = g[i];
            for (int j = i + 1; j < kdone; ++j) s -= H[i][j] * yv[j];
            yv[i] = s / H[i][i];
        }
        std::vector<double2> yd(kdone);
        for (int i = 0; i < kdone; ++i) yd[i] = make_double2(yv[i].real(), yv[i].imag());
        CK(cudaMemcpyAsync(dh, yd.data(), 16 * kdone, cudaMemcpyHostToDevice, ctx->stream));
        CK(launch_add_combo(V, n, kdone, dh, x, ctx->stream));
        ctx->launches += 1;
        if (rel < tol) converged = true;
        if (stop) break;
        // restart: w = b - A x
        CK(timed_gemv(ctx, dtype_a, A, n, n, lda, x, t, 1.0, 0.0, 0.0, 0.0, part, splits));
        CK(launch_sub(b, t, w, n, ctx->stream));
        ctx->launches += 1;
        if ((st = norm_of(w, &beta))) return st;
        if (beta == 0.0) { converged = true; rel = 0.0; break; }
    }
    if ((st = sync(ctx))) return st;
    if (iters_out) *iters_out = iters;
    if (res_out) *res_out = rel;
    if (!converged) return fail(ctx, NIHU_GB_ERR_NOT_CONVERGED, "GMRES did not reach the tolerance");
    return NIHU_GB_OK;
}

}  // namespace

nihu_gb_status nihu_gb_gmres(nihu_gb_ctx *ctx, int dtype_a, const void *A, int64_t n, int64_t lda, const void *b,
                             void *x, int restart, int max_iters, double tol, int *iters, double *rel_residual,
                             int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!valid_dtype(dtype_a) || !valid_where(where) || n < 0 || lda < std::max<int64_t>(n, 1) || restart < 1 ||
        restart > 256 || max_iters < 1 || !(tol > 0.0) || (n && (!A || !b || !x)))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_gmres: bad argument");
    if (n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    restart = (int)std::min<int64_t>(restart, n);
    nihu_gb_status st;
    const void *dA = A;
    const double2 *db = (const double2 *)b;
    double2 *dx = (double2 *)x;
    const size_t es = elem_bytes(dtype_a);
    if (where == NIHU_GB_HOST) {
        void *pa, *pb, *px;
        if ((st = scratch(ctx, "mv_A", es * n * n, &pa))) return st;
        if ((st = scratch(ctx, "gm_b", 16 * n, &pb))) return st;
        if ((st = scratch(ctx, "gm_x", 16 * n, &px))) return st;
        CK(cudaMemcpy2DAsync(pa, es * n, A, es * lda, es * n, n, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(pb, b, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(px, x, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
        dA = pa;
        db = (const double2 *)pb;
        dx = (double2 *)px;
        lda = n;
    }
    st = gmres_device(ctx, dtype_a, dA, n, lda, db, dx, restart, max_iters, tol, iters, rel_residual);
    if (where == NIHU_GB_HOST && (st == NIHU_GB_OK || st == NIHU_GB_ERR_NOT_CONVERGED)) {
        std::string keep = ctx->err;
        CK(cudaMemcpyAsync(x, dx, 16 * n, cudaMemcpyDeviceToHost, ctx->stream));
        nihu_gb_status s2 = sync(ctx);
        if (s2) return s2;
        ctx->err = keep;
    }
    return st;
}

// ------------------------------------------------------------------ LU

}  // extern "C"

namespace {

// A x = b (complex128, device) with the FP32 LU factors of A refined in FP64:
// x_0 = 0, then d = (LU)^{-1} r, x += d, r = b - A x (FP64 matvec) until the
// correction is within 64 FP64 roundings of x (|d| <= 64 eps |x|, the
// accuracy of an FP64 factorisation).  *refined = false (and nothing solved)
// when the order is beyond the FP32 kernels' shared memory or the
// corrections stop shrinking (cond(A) near 1 / eps32): the caller then
// factorises in FP64.  A is left unchanged.
nihu_gb_status lu_solve_mixed(nihu_gb_ctx *ctx, const double2 *A, int64_t n, int64_t lda, const double2 *b, double2 *x,
                              bool *refined)
{
    *refined = false;
    int smem_optin = 0;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    if (!lu32_fits((int)n, (size_t)smem_optin)) return NIHU_GB_OK;
    nihu_gb_status st;
    void *pf, *ppiv, *pd, *pr, *psums, *ppart;
    const int splits = gemv_splits(n, n, NIHU_GB_C128);
    if ((st = scratch(ctx, "lu32_F", 8 * (size_t)n * n, &pf))) return st;
    if ((st = scratch(ctx, "lu_piv", sizeof(int) * n, &ppiv))) return st;
    if ((st = scratch(ctx, "lu32_d", 16 * (size_t)n, &pd))) return st;
    if ((st = scratch(ctx, "lu32_r", 16 * (size_t)n, &pr))) return st;
    if ((st = scratch(ctx, "lu32_sums", 2 * sizeof(double), &psums))) return st;
    if ((st = scratch(ctx, "lu32_part", 16 * (size_t)splits * n, &ppart))) return st;
    double2 *d = (double2 *)pd, *r = (double2 *)pr;
    size_t panel_smem = 0;
    CK(lu32_prepare((int)n, (size_t)smem_optin, &panel_smem));
    if (!(ctx->lu_exec && ctx->lu_n == n && ctx->lu_F == pf && ctx->lu_piv == ppiv)) {
        // record the panel sequence once per order and buffers
        if (ctx->lu_exec) cudaGraphExecDestroy(ctx->lu_exec);
        ctx->lu_exec = nullptr;
        cudaGraph_t graph = nullptr;
        int64_t counted = 0;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = launch_lu32_factor((float2 *)pf, (int)n, (int *)ppiv, ctx->d_flag + 1, panel_smem, &counted,
                                           ctx->stream);
        cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->lu_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ctx->lu_exec = nullptr;
            return cuda_fail(ctx, e, "LU graph capture");
        }
        ctx->lu_n = (int)n;
        ctx->lu_F = pf;
        ctx->lu_piv = ppiv;
        ctx->lu_launches = counted;
    }
    CK(cudaMemsetAsync(ctx->d_flag + 1, 0, sizeof(int), ctx->stream));
    {
        Phase ph(ctx, "lu_factor");
        CK(launch_to_c64(A, lda, (int)n, (float2 *)pf, ctx->stream));
        CK(cudaGraphLaunch(ctx->lu_exec, ctx->stream));
        ctx->launches += 1 + ctx->lu_launches;
    }
    int info = 0;
    CK(cudaMemcpyAsync(&info, ctx->d_flag + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = sync(ctx))) return st;
    if (info) return fail(ctx, NIHU_GB_ERR_RUNTIME, "LU: exactly singular matrix (zero pivot in column " + std::to_string(info - 1) + ")");
    Phase ph(ctx, "lu_solve");
    CK(cudaMemsetAsync(x, 0, 16 * (size_t)n, ctx->stream));
    CK(cudaMemcpyAsync(r, b, 16 * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
    double sums[2] = {0.0, 0.0}, prev = 0.0;
    const double eps = 2.220446049250313e-16;
    for (int it = 0; it < 12; ++it) {
        CK(launch_lu32_solve((const float2 *)pf, (int)n, (const int *)ppiv, r, d, ctx->stream));
        CK(launch_lu32_update_x(x, d, (int)n, (double *)psums, ctx->stream));
        CK(cudaMemcpyAsync(r, b, 16 * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(launch_gemv(NIHU_GB_C128, A, n, n, lda, x, r, -1.0, 0.0, 1.0, 0.0, (double2 *)ppart, splits, ctx->stream));
        CK(cudaMemcpyAsync(sums, psums, sizeof(sums), cudaMemcpyDeviceToHost, ctx->stream));
        ctx->launches += 4;
        if ((st = sync(ctx))) return st;
        if (!(sums[1] > 0.0) || sums[0] <= 4096.0 * eps * eps * sums[1]) {
            *refined = true;
            return NIHU_GB_OK;
        }
        if (it > 0 && !(sums[0] < 0.25 * prev)) break;  // no longer converging
        prev = sums[0];
    }
    return NIHU_GB_OK;
}

}  // namespace

extern "C" {

nihu_gb_status nihu_gb_lu_solve(nihu_gb_ctx *ctx, void *A, int64_t n, int64_t lda, const void *b, void *x, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!valid_where(where) || n < 0 || lda < std::max<int64_t>(n, 1) || (n && (!A || !b || !x)) || n > 0x7fffffff)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_lu_solve: bad argument");
    if (n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    nihu_gb_status st;
    double2 *dA = (double2 *)A;
    const double2 *db = (const double2 *)b;
    double2 *dx = (double2 *)x;
    if (where == NIHU_GB_HOST) {
        void *pa, *pb, *px;
        if ((st = scratch(ctx, "lu_A", 16 * n * n, &pa))) return st;
        if ((st = scratch(ctx, "lu_b", 16 * n, &pb))) return st;
        if ((st = scratch(ctx, "lu_x", 16 * n, &px))) return st;
        CK(cudaMemcpy2DAsync(pa, 16 * n, A, 16 * lda, 16 * n, n, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(pb, b, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
        dA = (double2 *)pa;
        db = (const double2 *)pb;
        dx = (double2 *)px;
        lda = n;
    }
    bool refined = false;
    if ((st = lu_solve_mixed(ctx, dA, n, lda, db, dx, &refined))) return st;
    if (refined) {
        if (where == NIHU_GB_HOST) CK(cudaMemcpyAsync(x, dx, 16 * n, cudaMemcpyDeviceToHost, ctx->stream));
        return sync(ctx);
    }
    // FP64 factorisation (beyond the FP32 kernels, or the refinement stalled)
    void *ppiv;
    if ((st = scratch(ctx, "lu_piv", sizeof(int) * n, &ppiv))) return st;
    CK(cudaMemsetAsync(ctx->d_flag + 1, 0, sizeof(int), ctx->stream));
    {
        Phase ph(ctx, "lu_factor_fp64");
        CK(launch_lu_factor(dA, n, lda, (int *)ppiv, ctx->d_flag + 1, &ctx->launches, ctx->stream));
    }
    {
        Phase ph(ctx, "lu_solve_fp64");
        CK(launch_lu_solve(dA, n, lda, (const int *)ppiv, db, dx, ctx->stream));
    }
    ctx->launches += 1;
    int info = 0;
    CK(cudaMemcpyAsync(&info, ctx->d_flag + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    if (where == NIHU_GB_HOST) CK(cudaMemcpyAsync(x, dx, 16 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = sync(ctx))) return st;
    if (info) return fail(ctx, NIHU_GB_ERR_RUNTIME, "LU: exactly singular matrix (zero pivot in column " + std::to_string(info - 1) + ")");
    return NIHU_GB_OK;
}

// --------------------------------------------------------- composite solve

}  // extern "C"

namespace {

// rhs = G q, then solve Hm p = rhs by GMRES (solver 0) or LU (solver 1) and
// copy p to the host (the common tail of the composite solves)
nihu_gb_status solve_tail(nihu_gb_ctx *ctx, int64_t n, int dtype, void *G, void *Hm, void *dq, void *drhs, void *dp,
                          void *p, int solver, int restart, int max_iters, double tol, int *iters, double *rel_residual)
{
    nihu_gb_status st;
    int splits = gemv_splits(n, n, dtype);
    void *part;
    if ((st = scratch(ctx, "mv_part", 16 * (size_t)splits * n, &part))) return st;
    CK(timed_gemv(ctx, dtype, G, n, n, n, (const double2 *)dq, (double2 *)drhs, 1.0, 0.0, 0.0, 0.0, (double2 *)part, splits));
    if (solver == 0) {
        CK(cudaMemsetAsync(dp, 0, 16 * n, ctx->stream));
        st = gmres_device(ctx, dtype, Hm, n, n, (const double2 *)drhs, (double2 *)dp, std::min<int64_t>(restart, n),
                          max_iters, tol, iters, rel_residual);
        if (st && st != NIHU_GB_ERR_NOT_CONVERGED) return st;
    } else {
        bool refined = false;
        if ((st = lu_solve_mixed(ctx, (const double2 *)Hm, n, n, (const double2 *)drhs, (double2 *)dp, &refined)))
            return st;
        if (!refined) {
            void *ppiv;
            if ((st = scratch(ctx, "lu_piv", sizeof(int) * n, &ppiv))) return st;
            CK(cudaMemsetAsync(ctx->d_flag + 1, 0, sizeof(int), ctx->stream));
            CK(launch_lu_factor((double2 *)Hm, n, n, (int *)ppiv, ctx->d_flag + 1, &ctx->launches, ctx->stream));
            CK(launch_lu_solve((const double2 *)Hm, n, n, (const int *)ppiv, (const double2 *)drhs, (double2 *)dp,
                               ctx->stream));
            ctx->launches += 1;
        }
        if (iters) *iters = 1;
        if (rel_residual) *rel_residual = 0.0;
        st = NIHU_GB_OK;
    }
    nihu_gb_status keep = st;
    std::string msg = ctx->err;
    CK(cudaMemcpyAsync(p, dp, 16 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = sync(ctx))) return st;
    ctx->err = msg;
    return keep;
}

}  // namespace

extern "C" {

nihu_gb_status nihu_gb_solve_cbie(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k, int precision,
                                  int dtype, const void *q, void *p, int solver, int restart, int max_iters,
                                  double tol, int *iters, double *rel_residual)
{
    return nihu_gb_solve_cbie_c(ctx, mesh, family, k, 0.0, precision, dtype, q, p, solver, restart, max_iters, tol,
                                iters, rel_residual);
}

nihu_gb_status nihu_gb_solve_cbie_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k, double k_im,
                                    int precision, int dtype, const void *q, void *p, int solver, int restart,
                                    int max_iters, double tol, int *iters, double *rel_residual)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!mesh || !q || !p || (solver != 0 && solver != 1) || (solver == 1 && dtype != NIHU_GB_C128) || !valid_dtype(dtype))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_cbie: bad argument");
    const int64_t n = mesh->n;
    if (n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    const size_t es = elem_bytes(dtype);
    nihu_gb_status st;
    void *G, *Hm, *dq, *drhs, *dp;
    if ((st = scratch(ctx, "cbie_G", es * n * n, &G))) return st;
    if ((st = scratch(ctx, "cbie_H", es * n * n, &Hm))) return st;
    if ((st = scratch(ctx, "cbie_q", 16 * n, &dq))) return st;
    if ((st = scratch(ctx, "cbie_rhs", 16 * n, &drhs))) return st;
    if ((st = scratch(ctx, "cbie_p", 16 * n, &dp))) return st;
    CK(cudaMemcpyAsync(dq, q, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
    st = nihu_gb_assemble_c(ctx, mesh, mesh, family, NIHU_GB_SLP | NIHU_GB_DLP, k, k_im, 1.0, 0.0, precision, dtype, G,
                            Hm, n, 0, NIHU_GB_DEVICE);
    if (st) return st;
    CK(launch_add_identity((int)n, -0.5, 0.0, dtype, Hm, n, ctx->stream));
    ctx->launches += 1;
    return solve_tail(ctx, n, dtype, G, Hm, dq, drhs, dp, p, solver, restart, max_iters, tol, iters, rel_residual);
}

nihu_gb_status nihu_gb_solve_burton_miller(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                           double coupling_re, double coupling_im, int precision, int dtype,
                                           const void *q, void *p, int solver, int restart, int max_iters, double tol,
                                           int *iters, double *rel_residual)
{
    return nihu_gb_solve_burton_miller_c(ctx, mesh, family, k, 0.0, coupling_re, coupling_im, precision, dtype, q, p,
                                         solver, restart, max_iters, tol, iters, rel_residual);
}

nihu_gb_status nihu_gb_solve_burton_miller_c(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, double k,
                                             double k_im, double coupling_re, double coupling_im, int precision,
                                             int dtype, const void *q, void *p, int solver, int restart, int max_iters,
                                             double tol, int *iters, double *rel_residual)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!mesh || !q || !p || (solver != 0 && solver != 1) || (solver == 1 && dtype != NIHU_GB_C128) || !valid_dtype(dtype))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_burton_miller: bad argument");
    const int64_t n = mesh->n;
    if (n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    const size_t es = elem_bytes(dtype);
    nihu_gb_status st;
    void *A, *B, *dq, *drhs, *dp;
    if ((st = scratch(ctx, "cbie_G", es * n * n, &B))) return st;
    if ((st = scratch(ctx, "cbie_H", es * n * n, &A))) return st;
    if ((st = scratch(ctx, "cbie_q", 16 * n, &dq))) return st;
    if ((st = scratch(ctx, "cbie_rhs", 16 * n, &drhs))) return st;
    if ((st = scratch(ctx, "cbie_p", 16 * n, &dp))) return st;
    CK(cudaMemcpyAsync(dq, q, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
    st = nihu_gb_assemble_burton_miller_c(ctx, mesh, family, k, k_im, coupling_re, coupling_im, precision, dtype, A,
                                          B, n, NIHU_GB_DEVICE);
    if (st) return st;
    return solve_tail(ctx, n, dtype, B, A, dq, drhs, dp, p, solver, restart, max_iters, tol, iters, rel_residual);
}

}  // extern "C"

// ------------------------------------------------------- multi-RHS

namespace {

nihu_gb_status ensure_cublas(nihu_gb_ctx *ctx)
{
    if (ctx->cublas) return NIHU_GB_OK;
    if (cublasCreate(&ctx->cublas) != CUBLAS_STATUS_SUCCESS) {
        ctx->cublas = nullptr;
        return fail(ctx, NIHU_GB_ERR_CUDA, "cublasCreate failed");
    }
    return NIHU_GB_OK;
}

// the error word of the tensor-core product (zeroed when first allocated)
nihu_gb_status gemm_tc_err(nihu_gb_ctx *ctx, int **out)
{
    const bool fresh = ctx->scratch.find("gemm_err") == ctx->scratch.end();
    void *p;
    nihu_gb_status st = scratch(ctx, "gemm_err", 256, &p);
    if (st) return st;
    if (fresh) CK(cudaMemsetAsync(p, 0, sizeof(int), ctx->stream));
    *out = (int *)p;
    return NIHU_GB_OK;
}

// after a sync: a nonzero error word means a tensor-core product stopped on
// a pipeline wait that ran out (its result is invalid); the word is cleared
nihu_gb_status gemm_tc_check(nihu_gb_ctx *ctx)
{
    auto it = ctx->scratch.find("gemm_err");
    if (it == ctx->scratch.end()) return NIHU_GB_OK;
    int code = 0;
    CK(cudaMemcpy(&code, it->second.first, sizeof(int), cudaMemcpyDeviceToHost));
    if (!code) return NIHU_GB_OK;
    CK(cudaMemset(it->second.first, 0, sizeof(int)));
    return fail(ctx, NIHU_GB_ERR_CUDA, "tensor-core GEMM stopped: a pipeline wait ran out (code " +
                                           std::to_string(code) + ")");
}

// Y = alpha A X + beta Y on the device (A complex64)
nihu_gb_status gemm_device(nihu_gb_ctx *ctx, int mode, const void *A, int64_t m, int64_t n, int64_t lda,
                           const double2 *X, int64_t ldx, int64_t nrhs, double2 *Y, int64_t ldy, double are, double aim,
                           double bre, double bim)
{
    nihu_gb_status st;
    if (mode == NIHU_GB_GEMM_BF16X3 || mode == NIHU_GB_GEMM_BF16X6) {
        if (gemm_tc_supported(A, lda) && n > 0) {
            const int parts = mode == NIHU_GB_GEMM_BF16X3 ? 2 : 3;
            void *ws;
            int *err;
            if ((st = scratch(ctx, "gemm_tc", gemm_tc_scratch_bytes(parts, m, n, nrhs), &ws))) return st;
            if ((st = gemm_tc_err(ctx, &err))) return st;
            cudaError_t e;
            {
                Phase ph(ctx, parts == 2 ? "gemm_bf16x3" : "gemm_bf16x6");
                e = launch_gemm_tc(parts, A, m, n, lda, X, ldx, nrhs, Y, ldy, are, aim, bre, bim, ws, err,
                                   ctx->stream);
            }
            ctx->launches += 3 * ((nrhs + 63) / 64);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "gemm (tensor cores)");
            return NIHU_GB_OK;
        }
        // the float view of A cannot be tiled by TMA (unaligned A or odd lda):
        // the library GEMM of the same or better accuracy
        mode = mode == NIHU_GB_GEMM_BF16X3 ? NIHU_GB_GEMM_FP32 : NIHU_GB_GEMM_BF16X9;
    }
    if ((st = ensure_cublas(ctx))) return st;
    void *xp, *z;
    if ((st = scratch(ctx, "gemm_xp", sizeof(float) * 2 * std::max<int64_t>(n, 1) * nrhs, &xp))) return st;
    if ((st = scratch(ctx, "gemm_z", sizeof(float) * 4 * m * nrhs, &z))) return st;
    int cs = 0;
    cudaError_t e;
    {
        Phase ph(ctx, mode == NIHU_GB_GEMM_TF32 ? "gemm_tf32" : (mode == NIHU_GB_GEMM_BF16X9 ? "gemm_bf16x9" : "gemm_fp32"));
        e = launch_gemm_c64(ctx->cublas, mode, A, m, n, lda, X, ldx, (int)nrhs, Y, ldy, are, aim, bre, bim, (float *)xp,
                            (float *)z, ctx->stream, &cs);
    }
    ctx->launches += 3;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gemm");
    if (cs) return fail(ctx, NIHU_GB_ERR_CUDA, "cublasGemmEx failed with status " + std::to_string(cs));
    return NIHU_GB_OK;
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_gemm(nihu_gb_ctx *ctx, int mode, const void *A, int64_t m, int64_t n, int64_t lda,
                                       const void *X, int64_t ldx, int64_t nrhs, void *Y, int64_t ldy, double alpha_re,
                                       double alpha_im, double beta_re, double beta_im, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (mode < 0 || mode > NIHU_GB_GEMM_BF16X6 || !valid_where(where) || m < 0 || n < 0 || nrhs < 0 ||
        lda < std::max<int64_t>(m, 1) ||
        ldx < std::max<int64_t>(n, 1) || ldy < std::max<int64_t>(m, 1) || (m && nrhs && (!A || !Y)) ||
        (n && nrhs && !X) || m > 0x3fffffff || n > 0x7fffffff || nrhs > 0x3fffffff)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_gemm: bad argument");
    if (m == 0 || nrhs == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    nihu_gb_status st;
    const void *dA = A;
    const double2 *dX = (const double2 *)X;
    double2 *dY = (double2 *)Y;
    if (where == NIHU_GB_HOST) {
        void *pa, *px, *py;
        if ((st = scratch(ctx, "mv_A", 8 * m * n, &pa))) return st;
        if ((st = scratch(ctx, "gm_X", 16 * std::max<int64_t>(n, 1) * nrhs, &px))) return st;
        if ((st = scratch(ctx, "gm_Y", 16 * m * nrhs, &py))) return st;
        CK(cudaMemcpy2DAsync(pa, 8 * m, A, 8 * lda, 8 * m, n, cudaMemcpyHostToDevice, ctx->stream));
        if (n) CK(cudaMemcpy2DAsync(px, 16 * n, X, 16 * ldx, 16 * n, nrhs, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpy2DAsync(py, 16 * m, Y, 16 * ldy, 16 * m, nrhs, cudaMemcpyHostToDevice, ctx->stream));
        dA = pa;
        dX = (const double2 *)px;
        dY = (double2 *)py;
        lda = m;
        ldx = n;
        ldy = m;
    }
    if ((st = gemm_device(ctx, mode, dA, m, n, lda, dX, ldx, nrhs, dY, ldy, alpha_re, alpha_im, beta_re, beta_im)))
        return st;
    if (where == NIHU_GB_HOST)
        CK(cudaMemcpy2DAsync(Y, 16 * ldy, dY, 16 * m, 16 * m, nrhs, cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = sync(ctx))) return st;
    return gemm_tc_check(ctx);
}

namespace {

// one GMRES(restart) cycle on all right-hand sides in lockstep: D = approx A^{-1} R
// for the columns with active[r]; returns the iterations done
// Y = A X for nrhs columns of length n (leading dimension n); `active`
// (device int per column, may be NULL) marks the columns that still iterate
typedef std::function<nihu_gb_status(const double2 *X, double2 *Y, const int *active)> ApplyFn;

nihu_gb_status gmres_cycle_multi(nihu_gb_ctx *ctx, const ApplyFn &apply, int64_t n, const double2 *R, double2 *D,
                                 int nrhs, const std::vector<char> &active, int restart,
                                 const std::vector<double> &target_rel, int *iters)
{
    typedef std::complex<double> C;
    nihu_gb_status st;
    const int m = restart;
    void *pV, *pW, *ppart, *ph, *psc;
    const int blocks = bdot_blocks(n);
    if ((st = scratch(ctx, "mr_V", 16 * (size_t)n * nrhs * (m + 1), &pV))) return st;
    if ((st = scratch(ctx, "mr_W", 16 * (size_t)n * nrhs, &pW))) return st;
    if ((st = scratch(ctx, "mr_part", 16 * (size_t)(m + 1) * nrhs * blocks, &ppart))) return st;
    if ((st = scratch(ctx, "mr_h", 16 * (size_t)(m + 1) * nrhs, &ph))) return st;
    if ((st = scratch(ctx, "mr_sc", 8 * (size_t)nrhs, &psc))) return st;
    double2 *V = (double2 *)pV, *W = (double2 *)pW, *part = (double2 *)ppart, *hd = (double2 *)ph;
    double *scd = (double *)psc;
    const size_t blk = (size_t)n * nrhs;
    std::vector<double2> hh((size_t)(m + 1) * nrhs);
    std::vector<double> sc(nrhs);

    auto norms = [&](const double2 *X, std::vector<double> &out) -> nihu_gb_status {
        CK(launch_bdot(X, 1, X, n, nrhs, part, hd, ctx->stream));
        ctx->launches += 2;
        CK(cudaMemcpyAsync(hh.data(), hd, 16 * (size_t)nrhs, cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = sync(ctx))) return st;
        for (int r = 0; r < nrhs; ++r) out[r] = std::sqrt(std::max(hh[r].x, 0.0));
        return NIHU_GB_OK;
    };

    std::vector<double> beta(nrhs);
    if ((st = norms(R, beta))) return st;
    std::vector<char> act(nrhs);
    for (int r = 0; r < nrhs; ++r) {
        act[r] = active[r] && beta[r] > 0.0;
        sc[r] = act[r] ? 1.0 / beta[r] : 0.0;
    }
    CK(cudaMemcpyAsync(scd, sc.data(), 8 * (size_t)nrhs, cudaMemcpyHostToDevice, ctx->stream));
    CK(launch_bscale(R, V, n, nrhs, scd, ctx->stream));
    ctx->launches += 1;
    std::vector<std::vector<C>> H(nrhs, std::vector<C>((size_t)(m + 1) * m, C(0)));
    std::vector<std::vector<C>> g(nrhs, std::vector<C>(m + 1, C(0))), cs(nrhs, std::vector<C>(m)), sn(nrhs, std::vector<C>(m));
    std::vector<int> kdone(nrhs, 0);
    std::vector<char> run = act;
    void *pact;
    if ((st = scratch(ctx, "mr_active", sizeof(int) * (size_t)nrhs, &pact))) return st;
    int *dact = (int *)pact;
    std::vector<int> runi(nrhs);
    for (int r = 0; r < nrhs; ++r) g[r][0] = beta[r];
    int k = 0;
    for (; k < m; ++k) {
        bool any = false;
        for (int r = 0; r < nrhs; ++r) any = any || run[r];
        if (!any) break;
        // W = A V_k for every right-hand side still iterating, in one call
        for (int r = 0; r < nrhs; ++r) runi[r] = run[r];
        CK(cudaMemcpyAsync(dact, runi.data(), sizeof(int) * nrhs, cudaMemcpyHostToDevice, ctx->stream));
        if ((st = apply(V + (size_t)k * blk, W, dact))) return st;
        std::vector<std::vector<C>> h(nrhs, std::vector<C>(k + 2, C(0)));
        // CGS2 with FP32 products and sums on the FP64-stored basis: this is the
        // inner solve of a refinement (inner tolerance 1e-3 or so), whose
        // residual the outer loop forms in FP64; the FP64 pipe stays free
        for (int pass = 0; pass < 2; ++pass) {
            CK(launch_bdot(V, k + 1, W, n, nrhs, part, hd, ctx->stream, true));
            CK(cudaMemcpyAsync(hh.data(), hd, 16 * (size_t)(k + 1) * nrhs, cudaMemcpyDeviceToHost, ctx->stream));
            if ((st = sync(ctx))) return st;
            for (int v = 0; v <= k; ++v)
                for (int r = 0; r < nrhs; ++r) h[r][v] += C(hh[(size_t)v * nrhs + r].x, hh[(size_t)v * nrhs + r].y);
            CK(launch_bcombo(V, n, nrhs, k + 1, hd, -1.0, W, ctx->stream, true));
            ctx->launches += 3;
        }
        std::vector<double> hn(nrhs);
        if ((st = norms(W, hn))) return st;
        for (int r = 0; r < nrhs; ++r) sc[r] = (run[r] && hn[r] > 0.0) ? 1.0 / hn[r] : 0.0;
        CK(cudaMemcpyAsync(scd, sc.data(), 8 * (size_t)nrhs, cudaMemcpyHostToDevice, ctx->stream));
        CK(launch_bscale(W, V + (size_t)(k + 1) * blk, n, nrhs, scd, ctx->stream));
        ctx->launches += 1;
        for (int r = 0; r < nrhs; ++r) {
            if (!run[r]) continue;
            std::vector<C> &hr = h[r];
            hr[k + 1] = hn[r];
            for (int i = 0; i < k; ++i) {
                C a0 = hr[i], a1 = hr[i + 1];
                hr[i] = std::conj(cs[r][i]) * a0 + std::conj(sn[r][i]) * a1;
                hr[i + 1] = -sn[r][i] * a0 + cs[r][i] * a1;
            }
            double den = std::sqrt(std::norm(hr[k]) + std::norm(hr[k + 1]));
            if (den == 0.0) { cs[r][k] = 1.0; sn[r][k] = 0.0; }
            else { cs[r][k] = hr[k] / den; sn[r][k] = hr[k + 1] / den; }
            C a0 = hr[k], a1 = hr[k + 1];
            hr[k] = std::conj(cs[r][k]) * a0 + std::conj(sn[r][k]) * a1;
            C g0 = g[r][k], g1 = g[r][k + 1];
            g[r][k] = std::conj(cs[r][k]) * g0 + std::conj(sn[r][k]) * g1;
            g[r][k + 1] = -sn[r][k] * g0 + cs[r][k] * g1;
            for (int i = 0; i <= k; ++i) H[r][(size_t)i * m + k] = hr[i];
            kdone[r] = k + 1;
            if (std::abs(g[r][k + 1]) <= target_rel[r] * beta[r] || hn[r] == 0.0) run[r] = 0;
        }
    }
    *iters = k;
    // y = H^{-1} g per column, D += V y
    std::vector<double2> yd((size_t)m * nrhs, make_double2(0.0, 0.0));
    int kmax = 0;
    for (int r = 0; r < nrhs; ++r) {
        int kd = kdone[r];
        kmax = std::max(kmax, kd);
        std::vector<C> y(kd);
        for (int i = kd - 1; i >= 0; --i) {
            C sum = g[r][i];
            for (int j = i + 1; j < kd; ++j) sum -= H[r][(size_t)i * m + j] * y[j];
            y[i] = sum / H[r][(size_t)i * m + i];
        }
        for (int i = 0; i < kd; ++i) yd[(size_t)i * nrhs + r] = make_double2(y[i].real(), y[i].imag());
    }
    if (kmax > 0) {
        CK(cudaMemcpyAsync(hd, yd.data(), 16 * (size_t)kmax * nrhs, cudaMemcpyHostToDevice, ctx->stream));
        CK(launch_bcombo(V, n, nrhs, kmax, hd, 1.0, D, ctx->stream));
        ctx->launches += 1;
    }
    return sync(ctx);
}

}  // namespace

namespace {

// Restarted lockstep GMRES on nrhs columns with an iterative-refinement outer
// loop: X = 0, R = B; per outer step one GMRES cycle of `inner` on R (columns
// still above tol), X += D, R = B - residual(X).  With inner == residual this
// is plain restarted GMRES; with a low-precision inner product and an accurate
// residual it is mixed-precision iterative refinement.  inner_tol <= 0 runs
// each cycle to the global tolerance.
nihu_gb_status multi_solve_driver(nihu_gb_ctx *ctx, const ApplyFn &inner, const ApplyFn &residual, int64_t n,
                                  const double2 *dB, double2 *dX, int64_t nrhs, int restart, int max_outer, double tol,
                                  double inner_tol, int *outer_iters, int *inner_iters, std::vector<double> &rel)
{
    nihu_gb_status st;
    void *pr, *pd, *pp, *ph;
    const size_t blk = 16 * (size_t)n * nrhs;
    if ((st = scratch(ctx, "ms_R", blk, &pr))) return st;
    if ((st = scratch(ctx, "ms_D", blk, &pd))) return st;
    double2 *dR = (double2 *)pr, *dD = (double2 *)pd;
    const int blocks = bdot_blocks(n);
    if ((st = scratch(ctx, "mr_part", 16 * (size_t)(restart + 1) * nrhs * blocks, &pp))) return st;
    if ((st = scratch(ctx, "mr_h", 16 * (size_t)(restart + 1) * nrhs, &ph))) return st;
    std::vector<double2> hh((size_t)nrhs);
    auto norms = [&](const double2 *Xv, std::vector<double> &out) -> nihu_gb_status {
        CK(launch_bdot(Xv, 1, Xv, n, (int)nrhs, (double2 *)pp, (double2 *)ph, ctx->stream));
        ctx->launches += 2;
        CK(cudaMemcpyAsync(hh.data(), ph, 16 * (size_t)nrhs, cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = sync(ctx))) return st;
        for (int64_t r = 0; r < nrhs; ++r) out[r] = std::sqrt(std::max(hh[r].x, 0.0));
        return NIHU_GB_OK;
    };
    std::vector<double> bn(nrhs), rn(nrhs);
    rel.assign(nrhs, 0.0);
    if ((st = norms(dB, bn))) return st;
    CK(cudaMemsetAsync(dX, 0, blk, ctx->stream));
    CK(cudaMemcpyAsync(dR, dB, blk, cudaMemcpyDeviceToDevice, ctx->stream));
    int outer = 0, inner_total = 0;
    bool converged = false;
    while (true) {
        if ((st = norms(dR, rn))) return st;
        double worst = 0.0;
        std::vector<char> active(nrhs);
        std::vector<double> target(nrhs);
        for (int64_t r = 0; r < nrhs; ++r) {
            rel[r] = bn[r] > 0.0 ? rn[r] / bn[r] : 0.0;
            active[r] = rel[r] > tol;
            worst = std::max(worst, rel[r]);
            // stop a column's cycle at inner_tol of its current residual, or at the global tolerance
            target[r] = inner_tol > 0.0 ? inner_tol : (rn[r] > 0.0 ? tol * bn[r] / rn[r] : 1.0);
        }
        if (worst <= tol) { converged = true; break; }
        if (outer >= max_outer) break;
        ++outer;
        CK(cudaMemsetAsync(dD, 0, blk, ctx->stream));
        int it = 0;
        if ((st = gmres_cycle_multi(ctx, inner, n, dR, dD, (int)nrhs, active, restart, target, &it))) return st;
        inner_total += it;
        std::vector<double2> ones((size_t)nrhs, make_double2(1.0, 0.0));
        CK(cudaMemcpyAsync(ph, ones.data(), 16 * (size_t)nrhs, cudaMemcpyHostToDevice, ctx->stream));
        CK(launch_bcombo(dD, n, (int)nrhs, 1, (const double2 *)ph, 1.0, dX, ctx->stream));
        ctx->launches += 1;
        // R = B - A X
        if ((st = residual(dX, dR, nullptr))) return st;
        CK(launch_rsub(dB, dR, (size_t)n * nrhs, ctx->stream));
        ctx->launches += 1;
    }
    if ((st = sync(ctx))) return st;
    if (outer_iters) *outer_iters = outer;
    if (inner_iters) *inner_iters = inner_total;
    if (!converged) return fail(ctx, NIHU_GB_ERR_NOT_CONVERGED, "lockstep GMRES did not reach the tolerance");
    return NIHU_GB_OK;
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_solve_multi(nihu_gb_ctx *ctx, const void *A, int64_t n, int64_t lda, const void *B,
                                              void *X, int64_t nrhs, int inner_mode, int residual_mode, int restart,
                                              int max_outer, double tol, double inner_tol, int *outer_iters,
                                              int *inner_iters, double *rel_residuals, int where)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (inner_mode < 0 || inner_mode > NIHU_GB_GEMM_BF16X6 ||
        (residual_mode != NIHU_GB_GEMM_FP32 && residual_mode != NIHU_GB_GEMM_BF16X9 &&
         residual_mode != NIHU_GB_GEMM_BF16X6) ||
        !valid_where(where) || n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || restart < 1 || restart > 200 ||
        max_outer < 1 || !(tol > 0.0) || !(inner_tol > 0.0) || (n && nrhs && (!A || !B || !X)) || n > 0x3fffffff ||
        nrhs > 4096)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_multi: bad argument");
    if (n == 0 || nrhs == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    restart = (int)std::min<int64_t>(restart, n);
    nihu_gb_status st;
    const void *dA = A;
    void *pb, *px;
    const size_t blk = 16 * (size_t)n * nrhs;
    if ((st = scratch(ctx, "ms_B", blk, &pb))) return st;
    if ((st = scratch(ctx, "ms_X", blk, &px))) return st;
    double2 *dB = (double2 *)pb, *dX = (double2 *)px;
    if (where == NIHU_GB_HOST) {
        void *pa;
        if ((st = scratch(ctx, "mv_A", 8 * n * n, &pa))) return st;
        CK(cudaMemcpy2DAsync(pa, 8 * n, A, 8 * lda, 8 * n, n, cudaMemcpyHostToDevice, ctx->stream));
        dA = pa;
        lda = n;
        CK(cudaMemcpyAsync(dB, B, blk, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        CK(cudaMemcpyAsync(dB, B, blk, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ApplyFn inner = [&](const double2 *Xv, double2 *Yv, const int *) {
        return gemm_device(ctx, inner_mode, dA, n, n, lda, Xv, n, nrhs, Yv, n, 1.0, 0.0, 0.0, 0.0);
    };
    ApplyFn resid = [&](const double2 *Xv, double2 *Yv, const int *) {
        return gemm_device(ctx, residual_mode, dA, n, n, lda, Xv, n, nrhs, Yv, n, 1.0, 0.0, 0.0, 0.0);
    };
    std::vector<double> rel;
    nihu_gb_status sst = multi_solve_driver(ctx, inner, resid, n, dB, dX, nrhs, restart, max_outer, tol, inner_tol,
                                            outer_iters, inner_iters, rel);
    if (sst && sst != NIHU_GB_ERR_NOT_CONVERGED) return sst;
    std::string msg = ctx->err;
    if (where == NIHU_GB_HOST) CK(cudaMemcpyAsync(X, dX, blk, cudaMemcpyDeviceToHost, ctx->stream));
    else CK(cudaMemcpyAsync(X, dX, blk, cudaMemcpyDeviceToDevice, ctx->stream));
    if ((st = sync(ctx))) return st;
    if ((st = gemm_tc_check(ctx))) return st;
    ctx->err = msg;
    if (rel_residuals)
        for (int64_t r = 0; r < nrhs; ++r) rel_residuals[r] = rel[r];
    return sst;
}

// ------------------------------------------------------- frequency sweep

namespace {

nihu_gb_status upload_ks(nihu_gb_ctx *ctx, const double *ks, int nk, const double **dks, const float **dks32)
{
    nihu_gb_status st;
    void *p64, *p32;
    if ((st = scratch(ctx, "sw_k64", 8 * (size_t)nk, &p64))) return st;
    if ((st = scratch(ctx, "sw_k32", 4 * (size_t)nk, &p32))) return st;
    std::vector<float> k32(ks, ks + nk);
    CK(cudaMemcpyAsync(p64, ks, 8 * (size_t)nk, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(p32, k32.data(), 4 * (size_t)nk, cudaMemcpyHostToDevice, ctx->stream));
    *dks = (const double *)p64;
    *dks32 = (const float *)p32;
    return sync(ctx);  // the host vector dies here
}

}  // namespace

namespace {

// frequency batch of one mesh pair: matrices f at out + f * mat_stride, or
// (outs_dev, nk > 1) at the device pointers outs_dev[f] / outs_dev[nk + f];
// with rhs_b (SLP and DLP, one mesh): b_f = SLP_f q_f at rhs_b + f * n from
// q_f at rhs_q + f * n, and no SLP matrix (out_slp unused)
nihu_gb_status assemble_batch(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial, int family, int ops,
                              const double *ks, int nk, int precision, int dtype, void *out_slp, void *out_dlp,
                              int64_t ld, int64_t mat_stride, void *const *outs_dev, bool force_batch = false,
                              const double2 *rhs_q = nullptr, double2 *rhs_b = nullptr)
{
    nihu_gb_status st;
    NearList *nl = nullptr;
    if ((st = get_near(ctx, test, trial, &nl))) return st;
    RegularArgs a;
    a.test = test->dm;
    a.trial = trial->dm;
    a.same_mesh = test == trial;
    a.family = family;
    a.ops = ops;
    a.k = ks[0];
    a.alpha_re = 1.0;
    a.alpha_im = 0.0;
    a.precision = precision;
    a.dtype = dtype;
    a.accumulate = 0;
    a.trial_size_max = trial->size_max;
    a.k32 = (float)ks[0];
    a.alpha_re32 = 1.0f;
    a.alpha_im32 = 0.0f;
    a.unit_alpha = 1;
    a.out_s = out_slp;
    a.out_d = out_dlp;
    a.ld = ld;
    a.j0 = 0;
    a.j1 = (int)trial->n;
    a.nk = nk;
    for (int f = 0; f < nk; ++f) a.k_absmax = std::max(a.k_absmax, std::fabs(ks[f]));
    a.mat_stride = mat_stride;
    a.force_batch = force_batch;
    a.outs = (nk > 1 || force_batch) ? outs_dev : nullptr;
    if (rhs_b) {
        if ((st = near_rows(ctx, nl, a.same_mesh, test->n))) return st;
        void *rp, *ns;
        const int64_t items = nl->nnz + (a.same_mesh ? trial->n : 0);
        a.force_batch = 1;
        a.out_s = nullptr;
        if ((st = scratch(ctx, "sw_rpart", rhs_part_bytes(a), &rp))) return st;
        if ((st = scratch(ctx, "sw_nslp", 16 * (size_t)std::max<int64_t>(items, 1) * nk, &ns))) return st;
        a.rhs_q = rhs_q;
        a.rhs_part = rp;
        a.near_slp = (double2 *)ns;
    }
    if ((st = upload_ks(ctx, ks, nk, &a.ks, &a.ks32))) return st;
    if ((st = assemble_panel(ctx, a, nl))) return st;
    if (rhs_b) {
        Phase ph(ctx, "rhs_reduce");
        CK(launch_rhs_reduce(a, *nl, rhs_b, ctx->stream));
        ctx->launches += 1;
    }
    return check_flag(ctx);
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_assemble_sweep(nihu_gb_ctx *ctx, const nihu_gb_mesh *test, const nihu_gb_mesh *trial,
                                                 int family, int ops, const double *ks, int nk, int precision,
                                                 int dtype, void *out_slp, void *out_dlp, int64_t ld,
                                                 int64_t mat_stride)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!test || !trial || test->ctx != ctx || trial->ctx != ctx || nk < 1 || !ks || ops < 1 || ops > 3 ||
        ((ops & 1) && !out_slp) || ((ops & 2) && !out_dlp) || !valid_dtype(dtype) || (precision != 0 && precision != 1) ||
        ld < std::max<int64_t>(test->n, 1) || mat_stride < ld * trial->n ||
        (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_sweep: bad argument");
    for (int f = 0; f < nk; ++f)
        if (!std::isfinite(ks[f])) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_assemble_sweep: bad k");
    if (test->n == 0 || trial->n == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    return assemble_batch(ctx, test, trial, family, ops, ks, nk, precision, dtype, out_slp, out_dlp, ld, mat_stride,
                          nullptr);
}

// ------------------------------------------------ persistent batched GMRES

namespace {

struct BatchSystem {
    const void *A;  // complex64, column-major
    int64_t n, lda;
    const double2 *b;
    double2 *x;
    double work;  // processing order: larger first
};

struct PersistentPlan {
    int cluster = 0, clusters = 0, vx_smem = 1;
    size_t smem = 0;
};

// Launch shape of one persistent GMRES launch over systems of the given sizes
// (results do not depend on it): the systems, largest first, go to the
// earliest free of the clusters that run at once; a system of nb 128-row
// blocks keeps min(C, nb) CTAs busy for n^2 / min(C, nb) time units, slowed
// in proportion when more CTAs stream at once than HBM feeds (about 60 GB/s
// per 512-thread CTA).  The matvec input moves from shared memory to a
// global buffer when a cluster size's shared memory cannot hold it.
nihu_gb_status plan_persistent(nihu_gb_ctx *ctx, const std::vector<int64_t> &ns, int m, PersistentPlan *out,
                               int force_cluster = 0)
{
    int smem_optin = 0, mem_khz = 0, bus_bits = 0;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    cudaDeviceGetAttribute(&mem_khz, cudaDevAttrMemoryClockRate, ctx->device);
    cudaDeviceGetAttribute(&bus_bits, cudaDevAttrGlobalMemoryBusWidth, ctx->device);
    const double hbm_gbs = 2.0 * mem_khz * 1e3 * bus_bits / 8.0 / 1e9;
    const double feeding = std::max(8.0, 0.8 * hbm_gbs / 60.0);  // CTAs that saturate HBM
    const int count = (int)ns.size();
    int64_t n_max = 1;
    for (int64_t n : ns) n_max = std::max(n_max, n);
    std::vector<int64_t> by_size(ns);
    std::sort(by_size.begin(), by_size.end(), std::greater<int64_t>());
    PersistentPlan best;
    double best_t = 0.0;
    for (int c : {2, 4, 8, 16, 1}) {
        if (force_cluster && c != force_cluster) continue;
        int vs = 1;
        if (persistent_smem_layout((int)n_max, c, m, 1).total > (size_t)smem_optin) vs = 0;
        if (persistent_smem_layout((int)n_max, c, m, vs).total > (size_t)smem_optin) continue;
        int act = 0;
        size_t sm_bytes = 0;
        if (persistent_gmres_plan((int)n_max, m, c, vs, count, &act, &sm_bytes) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        const double rate = std::min(1.0, feeding / ((double)act * c));
        std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
        for (int q = 0; q < act; ++q) free_at.push(0.0);
        double makespan = 0.0;
        for (int64_t n : by_size) {
            const double nb = (double)((n + 127) / 128);
            double t = free_at.top();
            free_at.pop();
            t += (double)n * (double)n / (std::max(1.0, std::min((double)c, nb)) * rate);
            free_at.push(t);
            makespan = std::max(makespan, t);
        }
        // within 3 %, the later candidate (larger clusters) loses to the earlier
        if (!best.cluster || makespan < 0.97 * best_t) {
            best_t = makespan;
            best.cluster = c;
            best.clusters = act;
            best.vx_smem = vs;
            best.smem = sm_bytes;
        }
    }
    if (!best.cluster)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "batched GMRES: system or restart too large for shared memory");
    CK(persistent_gmres_plan((int)n_max, m, best.cluster, best.vx_smem, count, &best.clusters, &best.smem));
    *out = best;
    return NIHU_GB_OK;
}

// One persistent launch of a plan: its items (indices into the caller's item
// array) in processing order, the largest system and the launch shape
struct PersistentLaunch {
    std::vector<int> order;
    int64_t n_max = 1;
    PersistentPlan plan;
};

// The persistent launches over items of sizes ns, each in order of
// decreasing key: one over all; or, when the shape chosen for the larger
// systems (n >= n_max / 2) leaves SMs idle -- clusters of 8 CTAs fit whole
// GPCs, not every SM -- and smaller systems exist, a second launch of the
// smaller systems in the smallest clusters that hold them, sized to the idle
// SMs and started beside the first as its programmatic dependent
// (launch_persistent_gmres).
nihu_gb_status plan_launches(nihu_gb_ctx *ctx, const std::vector<int64_t> &ns, const std::vector<double> &key, int m,
                             std::vector<PersistentLaunch> *out, int force_cluster = 0)
{
    nihu_gb_status st;
    out->clear();
    const int count = (int)ns.size();
    int64_t n_max = 1;
    for (int64_t n : ns) n_max = std::max(n_max, n);
    auto sorted = [&](std::vector<int> v) {
        std::stable_sort(v.begin(), v.end(), [&](int x, int y) { return key[x] > key[y]; });
        return v;
    };
    std::vector<int> big, small;
    for (int q = 0; q < count; ++q) (2 * ns[q] >= n_max ? big : small).push_back(q);
    if (!small.empty()) {
        PersistentLaunch A, B;
        std::vector<int64_t> nsa;
        for (int q : big) nsa.push_back(ns[q]);
        for (int q : small) B.n_max = std::max(B.n_max, ns[q]);
        if ((st = plan_persistent(ctx, nsa, m, &A.plan, force_cluster))) return st;
        int sms = 0, smem_optin = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
        const int spare = sms - A.plan.cluster * A.plan.clusters;
        // the smallest cluster whose shared memory holds the smaller systems
        for (int c : {1, 2, 4}) {
            if (A.plan.cluster < 4 || spare < c) break;
            const int vs = persistent_smem_layout((int)B.n_max, c, m, 1).total <= (size_t)smem_optin ? 1 : 0;
            if (persistent_smem_layout((int)B.n_max, c, m, vs).total > (size_t)smem_optin) continue;
            int act = 0;
            size_t smem = 0;
            if (persistent_gmres_plan((int)B.n_max, m, c, vs, (int)small.size(), &act, &smem) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            B.plan.cluster = c;
            B.plan.clusters = std::min(act, spare / c);
            B.plan.vx_smem = vs;
            B.plan.smem = smem;
            A.order = sorted(big);
            A.n_max = n_max;
            B.order = sorted(small);
            CK(persistent_gmres_smem_limit(std::max(A.plan.smem, B.plan.smem)));
            out->push_back(A);
            out->push_back(B);
            return NIHU_GB_OK;
        }
    }
    PersistentLaunch one;
    if ((st = plan_persistent(ctx, ns, m, &one.plan, force_cluster))) return st;
    std::vector<int> all(count);
    for (int q = 0; q < count; ++q) all[q] = q;
    one.order = sorted(all);
    one.n_max = n_max;
    out->push_back(one);
    return NIHU_GB_OK;
}

// one persistent launch over the items (states in device memory), in order
// of decreasing `work`; asynchronous on the context stream
nihu_gb_status launch_persistent(nihu_gb_ctx *ctx, std::vector<PersistentItem> &items, const std::vector<double> &work,
                                 int m, int max_iters, int quantum, double tol)
{
    const int count = (int)items.size();
    if (count == 0) return NIHU_GB_OK;
    nihu_gb_status st;
    std::vector<int64_t> ns(count);
    int64_t n_max = 1;
    for (int f = 0; f < count; ++f) {
        ns[f] = items[f].n;
        n_max = std::max<int64_t>(n_max, items[f].n);
    }
    std::vector<PersistentLaunch> launches;
    if ((st = plan_launches(ctx, ns, work, m, &launches))) return st;
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device);
    for (const PersistentLaunch &L : launches)
        for (int q : L.order) {
            PersistentItem &it = items[q];
            it.vec = (it.n % 2 == 0) && (it.lda % 2 == 0) && ((reinterpret_cast<uintptr_t>(it.A) & 15) == 0);
            it.stream = 8.0 * (double)it.n * (double)it.n * std::min<int>((int)L.order.size(), L.plan.clusters) >
                        0.5 * l2;
        }
    void *pitems;
    if ((st = scratch(ctx, "pg_items", sizeof(PersistentItem) * (size_t)count, &pitems))) return st;
    CK(cudaMemcpyAsync(pitems, items.data(), sizeof(PersistentItem) * count, cudaMemcpyHostToDevice, ctx->stream));
    std::vector<PersistentArgs> args;
    std::string name = "persistent_gmres[";  // the launch shapes: clusters x CTAs per cluster
    for (size_t t = 0; t < launches.size(); ++t) {
        const PersistentLaunch &L = launches[t];
        const int cnt = (int)L.order.size();
        const std::string tag = std::to_string(t);
        void *porder, *pcnt, *pvx = nullptr;
        if ((st = scratch(ctx, ("pg_order" + tag).c_str(), sizeof(int) * (size_t)cnt, &porder))) return st;
        if ((st = scratch(ctx, ("pg_counter" + tag).c_str(), sizeof(int), &pcnt))) return st;
        if (!L.plan.vx_smem && (st = scratch(ctx, ("pg_vx" + tag).c_str(), 8 * (size_t)L.plan.clusters * L.n_max, &pvx)))
            return st;
        CK(cudaMemcpyAsync(porder, L.order.data(), sizeof(int) * cnt, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemsetAsync(pcnt, 0, sizeof(int), ctx->stream));
        PersistentArgs a{};
        a.items = (const PersistentItem *)pitems;
        a.order = (const int *)porder;
        a.count = cnt;
        a.n_max = (int)L.n_max;
        a.restart = m;
        a.max_iters = max_iters;
        a.quantum = quantum;
        a.tol = tol;
        a.counter = (int *)pcnt;
        a.vxg = (float2 *)pvx;
        a.wait_primary = t > 0;
        args.push_back(a);
        name += (t ? "+" : "") + std::to_string(L.plan.clusters) + "x" + std::to_string(L.plan.cluster) +
                (L.plan.vx_smem ? "" : ",vx global");
    }
    name += "]";
    {
        Phase ph(ctx, name.c_str());
        for (size_t t = 0; t < launches.size(); ++t)
            CK(launch_persistent_gmres(args[t], launches[t].plan.cluster, launches[t].plan.clusters,
                                       launches[t].plan.smem, ctx->stream, t > 0));
    }
    ctx->launches += (int)launches.size();
    // the host vectors above are read by the copies: wait for them before they go
    return sync(ctx);
}

// one persistent launch solving every system to the end; per-system outputs
// on the host (may be NULL)
nihu_gb_status solve_batched_device(nihu_gb_ctx *ctx, const std::vector<BatchSystem> &sys, int restart, int max_iters,
                                    double tol, int *iters, double *rel, int *converged)
{
    const int count = (int)sys.size();
    if (count == 0) return NIHU_GB_OK;
    nihu_gb_status st;
    int64_t n_max = 1, vtotal = 0;
    for (const BatchSystem &s : sys) {
        n_max = std::max(n_max, s.n);
        vtotal += s.n;
    }
    const int m = (int)std::max<int64_t>(1, std::min<int64_t>(restart, n_max));
    const size_t ss = persistent_small_state(m);
    void *pV, *pS, *pst;
    if ((st = scratch(ctx, "pg_V", 16 * (size_t)vtotal * (m + 1), &pV))) return st;
    if ((st = scratch(ctx, "pg_S", 16 * ss * count, &pS))) return st;
    if ((st = scratch(ctx, "pg_st", sizeof(PersistentState) * (size_t)count, &pst))) return st;
    CK(cudaMemsetAsync(pst, 0, sizeof(PersistentState) * (size_t)count, ctx->stream));  // PG_FRESH
    std::vector<PersistentItem> items(count);
    std::vector<double> work(count);
    int64_t voff = 0;
    for (int f = 0; f < count; ++f) {
        const BatchSystem &s = sys[f];
        PersistentItem &it = items[f];
        it.A = (const float2 *)s.A;
        it.lda = s.lda;
        it.b = s.b;
        it.x = s.x;
        it.V = (double2 *)pV + voff * (m + 1);
        it.S = (double2 *)pS + ss * f;
        it.st = (PersistentState *)pst + f;
        it.n = (int)s.n;
        it.pad = 0;
        voff += s.n;
        work[f] = s.work;
    }
    if ((st = launch_persistent(ctx, items, work, m, max_iters, 0, tol))) return st;
    std::vector<PersistentState> hs(count);
    CK(cudaMemcpyAsync(hs.data(), pst, sizeof(PersistentState) * count, cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = sync(ctx))) return st;
    bool all = true;
    for (int f = 0; f < count; ++f) {
        if (iters) iters[f] = hs[f].iters;
        if (converged) converged[f] = hs[f].converged;
        if (rel) rel[f] = hs[f].rel;
        all = all && hs[f].converged;
    }
    if (!all) return fail(ctx, NIHU_GB_ERR_NOT_CONVERGED, "batched GMRES: some systems did not reach the tolerance");
    return NIHU_GB_OK;
}

// CBIE sweep over several meshes: instance f on meshes[mesh_of[f]] at ks[f];
// q_dev / p_dev hold the instances' columns grouped by mesh (offsets `off`)
nihu_gb_status sweep_solve_impl(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes, int family,
                                int nk, const double *ks, const int *mesh_of, int precision, const double2 *q_dev,
                                double2 *p_dev, const std::vector<int64_t> &off, int restart, int max_iters, double tol,
                                int *iters, double *rel, int *converged)
{
    nihu_gb_status st;
    std::vector<BatchSystem> sys(nk);
    void *pb;
    int64_t total = 0;
    for (int f = 0; f < nk; ++f) total += meshes[mesh_of[f]]->n;
    if ((st = scratch(ctx, "swb_b", 16 * (size_t)total, &pb))) return st;
    double2 *b = (double2 *)pb;
    for (int i = 0; i < n_meshes; ++i) {
        const nihu_gb_mesh *mesh = meshes[i];
        const int64_t n = mesh->n;
        std::vector<int> fs;
        std::vector<double> ki;
        for (int f = 0; f < nk; ++f)
            if (mesh_of[f] == i) {
                fs.push_back(f);
                ki.push_back(ks[f]);
            }
        if (fs.empty() || n == 0) {
            for (int f : fs) sys[f] = BatchSystem{nullptr, 0, 1, nullptr, nullptr, 0.0};
            continue;
        }
        const int cnt = (int)fs.size();
        const int64_t stride = n * n;
        void *H;
        const std::string tag = std::to_string(i);
        if ((st = scratch(ctx, ("swb_H" + tag).c_str(), 8 * (size_t)stride * cnt, &H))) return st;
        // the DLP matrices and b_f = SLP_f q_f (the mesh's instances are
        // contiguous in q_dev / b): no SLP matrix
        const int64_t o = off[fs[0]];
        if ((st = assemble_batch(ctx, mesh, mesh, family, NIHU_GB_SLP | NIHU_GB_DLP, ki.data(), cnt, precision,
                                 NIHU_GB_C64, nullptr, H, n, stride, nullptr, true, q_dev + o, b + o)))
            return st;
        CK(launch_add_identity_batched((int)n, -0.5, 0.0, NIHU_GB_C64, H, n, stride, cnt, ctx->stream));
        ctx->launches += 1;
        for (int j = 0; j < cnt; ++j) {
            const int f = fs[j];
            sys[f] = BatchSystem{(const char *)H + 8 * (size_t)stride * j, n, n, b + off[f], p_dev + off[f],
                                 (double)n * (double)n * (1.0 + ks[f])};
        }
    }
    return solve_batched_device(ctx, sys, restart, max_iters, tol, iters, rel, converged);
}

// device offsets of the instances' columns, grouped by mesh in mesh order
std::vector<int64_t> sweep_offsets(int n_meshes, const nihu_gb_mesh *const *meshes, int nk, const int *mesh_of)
{
    std::vector<int64_t> off(nk);
    int64_t o = 0;
    for (int i = 0; i < n_meshes; ++i)
        for (int f = 0; f < nk; ++f)
            if (mesh_of[f] == i) {
                off[f] = o;
                o += meshes[i]->n;
            }
    return off;
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_solve_batched(nihu_gb_ctx *ctx, int count, const void *const *A, const int64_t *n,
                                                const int64_t *lda, const void *const *b, void *const *x, int restart,
                                                int max_iters, double tol, int *iters, double *rel_residuals,
                                                int *converged)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (count < 0 || (count > 0 && (!A || !n || !lda || !b || !x)) || restart < 1 || restart > 200 || max_iters < 1 ||
        !(tol > 0.0))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_batched: bad argument");
    std::vector<BatchSystem> sys(count);
    for (int f = 0; f < count; ++f) {
        if (n[f] < 0 || n[f] > 0x3fffffff || lda[f] < std::max<int64_t>(n[f], 1) || (n[f] > 0 && (!A[f] || !b[f] || !x[f])))
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_batched: bad system " + std::to_string(f));
        sys[f] = BatchSystem{A[f], n[f], lda[f], (const double2 *)b[f], (double2 *)x[f], (double)n[f] * (double)n[f]};
    }
    if (count == 0) return NIHU_GB_OK;
    cudaSetDevice(ctx->device);
    return solve_batched_device(ctx, sys, restart, max_iters, tol, iters, rel_residuals, converged);
}

extern "C" nihu_gb_status nihu_gb_solve_sweep_batched(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes,
                                                      int family, int nk, const double *ks, const int *mesh_of,
                                                      int precision, const void *q, void *p, int restart, int max_iters,
                                                      double tol, int *iters, double *rel_residuals, int *converged)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (n_meshes < 1 || !meshes || nk < 1 || !ks || !mesh_of || !q || !p || restart < 1 || restart > 200 ||
        max_iters < 1 || !(tol > 0.0) || (precision != 0 && precision != 1) ||
        (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_sweep_batched: bad argument");
    for (int i = 0; i < n_meshes; ++i)
        if (!meshes[i] || meshes[i]->ctx != ctx)
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_sweep_batched: bad mesh");
    for (int f = 0; f < nk; ++f)
        if (mesh_of[f] < 0 || mesh_of[f] >= n_meshes || !std::isfinite(ks[f]))
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_sweep_batched: bad instance");
    cudaSetDevice(ctx->device);
    nihu_gb_status st;
    const std::vector<int64_t> off = sweep_offsets(n_meshes, meshes, nk, mesh_of);
    // user layout: instance columns back to back in instance order; device layout: grouped by mesh
    int64_t total = 0;
    std::vector<int64_t> user(nk);
    for (int f = 0; f < nk; ++f) {
        user[f] = total;
        total += meshes[mesh_of[f]]->n;
    }
    if (total == 0) return NIHU_GB_OK;
    std::vector<double2> hq(total);
    for (int f = 0; f < nk; ++f)
        std::memcpy(hq.data() + off[f], (const double2 *)q + user[f], 16 * (size_t)meshes[mesh_of[f]]->n);
    void *pq, *pp;
    if ((st = scratch(ctx, "swb_q", 16 * (size_t)total, &pq))) return st;
    if ((st = scratch(ctx, "swb_p", 16 * (size_t)total, &pp))) return st;
    CK(cudaMemcpyAsync(pq, hq.data(), 16 * (size_t)total, cudaMemcpyHostToDevice, ctx->stream));
    nihu_gb_status sst = sweep_solve_impl(ctx, n_meshes, meshes, family, nk, ks, mesh_of, precision, (const double2 *)pq,
                                          (double2 *)pp, off, restart, max_iters, tol, iters, rel_residuals, converged);
    if (sst && sst != NIHU_GB_ERR_NOT_CONVERGED) {
        sync(ctx);
        return sst;
    }
    std::string msg = ctx->err;
    CK(cudaMemcpyAsync(hq.data(), pp, 16 * (size_t)total, cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = sync(ctx))) return st;
    for (int f = 0; f < nk; ++f)
        std::memcpy((double2 *)p + user[f], hq.data() + off[f], 16 * (size_t)meshes[mesh_of[f]]->n);
    ctx->err = msg;
    return sst;
}

extern "C" nihu_gb_status nihu_gb_solve_sweep(nihu_gb_ctx *ctx, const nihu_gb_mesh *mesh, int family, const double *ks,
                                              int nk, int precision, const void *q, int q_cols, void *p, int restart,
                                              int max_cycles, double tol, int *cycles, int *iters, double *rel_residuals)
{
    if (!ctx) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (!mesh || nk < 1 || !ks || !q || !p || (q_cols != 1 && q_cols != nk) || restart < 1 || restart > 200 ||
        max_cycles < 1 || !(tol > 0.0))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_solve_sweep: bad argument");
    const int64_t n = mesh->n;
    if (n == 0) return NIHU_GB_OK;
    std::vector<double2> qf((size_t)n * nk);
    for (int f = 0; f < nk; ++f)
        std::memcpy(qf.data() + (size_t)n * f, (const double2 *)q + (q_cols == 1 ? 0 : (size_t)n * f), 16 * (size_t)n);
    std::vector<int> mesh_of(nk, 0), it(nk);
    const nihu_gb_mesh *ms[1] = {mesh};
    const int max_iters = (int)std::min<int64_t>((int64_t)restart * max_cycles, 1 << 30);
    nihu_gb_status st = nihu_gb_solve_sweep_batched(ctx, 1, ms, family, nk, ks, mesh_of.data(), precision, qf.data(), p,
                                                    restart, max_iters, tol, it.data(), rel_residuals, nullptr);
    if (st && st != NIHU_GB_ERR_NOT_CONVERGED) return st;
    int most = 0;
    for (int f = 0; f < nk; ++f) most = std::max(most, it[f]);
    const int r = (int)std::min<int64_t>(restart, n);
    if (cycles) *cycles = (most + r - 1) / r;
    if (iters) *iters = most;
    return st;
}

// ------------------------------------------------------------ serving loop
//
// Continuous batching of CBIE solves (helmholtz_3d_coll.cpp:36-120 once per
// request): requests wait in a FIFO queue until the HBM budget holds their
// matrices and Krylov state; every round admits what fits, assembles the new
// requests (one frequency batch per mesh), forms their right-hand sides,
// advances every admitted system by at most `quantum` GMRES steps in one
// persistent launch, and retires the finished ones.  Matrices, Krylov state
// and iterates stay in device memory between rounds; memory comes from a
// stream-ordered pool, so admission and retirement never synchronise the
// device beyond the one wait per round.

struct nihu_gb_server {
    struct Request {
        int64_t id = 0;
        int mesh = 0;
        double k = 0.0;
        std::vector<double2> q;  // Neumann data until admission; then the result p
        size_t held = 0;         // budget bytes held
        void *H = nullptr, *blk = nullptr;  // DLP matrix; vectors and Krylov state
        double2 *b = nullptr, *x = nullptr, *V = nullptr, *S = nullptr;
        int slot = -1;  // status word in the server's state array
        PersistentState st{};
    };
    nihu_gb_ctx *ctx = nullptr;
    std::vector<const nihu_gb_mesh *> meshes;
    int family = 0, precision = 0, restart = 0, max_iters = 0, quantum = 0;
    double tol = 0.0;
    size_t budget = 0, held = 0;
    cudaMemPool_t pool = nullptr;
    double2 *h_stage = nullptr;  // pinned staging of a round's Neumann data
    size_t h_stage_bytes = 0;
    PersistentState *d_states = nullptr;  // one slot per admitted request
    int n_slots = 0;
    std::vector<int> free_slots;
    std::deque<Request *> queue;
    std::vector<Request *> active;
    std::deque<Request *> done;
    int64_t next_id = 0;
};

namespace {

typedef nihu_gb_server::Request SrvReq;

size_t srv_align(size_t x) { return (x + 255) & ~(size_t)255; }

// device bytes of one request's vectors, basis, small state: [b x | V | S]
size_t srv_block_bytes(int64_t n, int m)
{
    return srv_align(2 * 16 * (size_t)n) + srv_align(16 * (size_t)n * (m + 1)) + srv_align(16 * persistent_small_state(m));
}

void srv_release(nihu_gb_server *sv, SrvReq *r)
{
    cudaStream_t s = sv->ctx->stream;
    if (r->H) cudaFreeAsync(r->H, s);
    if (r->blk) cudaFreeAsync(r->blk, s);
    r->H = r->blk = nullptr;
    if (r->slot >= 0) sv->free_slots.push_back(r->slot);
    r->slot = -1;
    sv->held -= r->held;
    r->held = 0;
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_server_create(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes,
                                                int family, int precision, size_t hbm_budget_bytes, int max_active,
                                                int restart, int max_iters, double tol, int quantum,
                                                nihu_gb_server **out)
{
    if (!ctx || !out) return NIHU_GB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_meshes < 1 || !meshes || (precision != 0 && precision != 1) ||
        (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D) || hbm_budget_bytes == 0 || max_active < 1 ||
        restart < 1 || restart > 200 || max_iters < 1 || !(tol > 0.0) || quantum < 0)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_server_create: bad argument");
    for (int i = 0; i < n_meshes; ++i)
        if (!meshes[i] || meshes[i]->ctx != ctx || meshes[i]->n < 1)
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_server_create: bad mesh");
    cudaSetDevice(ctx->device);
    std::unique_ptr<nihu_gb_server> sv(new nihu_gb_server);
    sv->ctx = ctx;
    sv->meshes.assign(meshes, meshes + n_meshes);
    sv->family = family;
    sv->precision = precision;
    sv->budget = hbm_budget_bytes;
    sv->restart = restart;
    sv->max_iters = max_iters;
    sv->tol = tol;
    sv->quantum = quantum;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    CK(cudaMemPoolCreate(&sv->pool, &props));
    uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next requests
    CK(cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep));

    sv->n_slots = max_active;
    void *p;
    nihu_gb_status st;
    if ((st = dmalloc(ctx, sizeof(PersistentState) * (size_t)max_active, &p))) {
        cudaMemPoolDestroy(sv->pool);
        return st;
    }
    sv->d_states = (PersistentState *)p;
    for (int i = max_active - 1; i >= 0; --i) sv->free_slots.push_back(i);
    *out = sv.release();
    return NIHU_GB_OK;
}

extern "C" void nihu_gb_server_destroy(nihu_gb_server *sv)
{
    if (!sv) return;
    cudaSetDevice(sv->ctx->device);
    for (SrvReq *r : sv->active) srv_release(sv, r);
    cudaStreamSynchronize(sv->ctx->stream);
    for (SrvReq *r : sv->queue) delete r;
    for (SrvReq *r : sv->active) delete r;
    for (SrvReq *r : sv->done) delete r;
    dfree(sv->ctx, sv->d_states);
    if (sv->h_stage) cudaFreeHost(sv->h_stage);
    cudaMemPoolDestroy(sv->pool);
    delete sv;
}

extern "C" nihu_gb_status nihu_gb_server_reserve(nihu_gb_server *sv, size_t bytes)
{
    if (!sv) return NIHU_GB_ERR_INVALID_ARGUMENT;
    nihu_gb_ctx *ctx = sv->ctx;
    if (bytes == 0 || bytes > sv->budget) bytes = sv->budget;
    cudaSetDevice(ctx->device);
    // one allocation of the size, freed at once: the pool keeps the memory
    // (release threshold: all), so later admissions map no new device memory
    void *all = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&all, bytes, sv->pool, ctx->stream);
    if (e == cudaSuccess) e = cudaFreeAsync(all, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(ctx, e, "nihu_gb_server_reserve");
    }
    return NIHU_GB_OK;
}

extern "C" nihu_gb_status nihu_gb_server_submit(nihu_gb_server *sv, int mesh, double k, const void *q, int64_t *id)
{
    if (!sv) return NIHU_GB_ERR_INVALID_ARGUMENT;
    nihu_gb_ctx *ctx = sv->ctx;
    if (mesh < 0 || mesh >= (int)sv->meshes.size() || !std::isfinite(k) || !q)
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_server_submit: bad argument");
    const int64_t n = sv->meshes[mesh]->n;
    const size_t need = 8 * (size_t)n * n + srv_block_bytes(n, sv->restart);
    if (need > sv->budget)
        return fail(ctx, NIHU_GB_ERR_OUT_OF_MEMORY, "nihu_gb_server_submit: request larger than the HBM budget");
    SrvReq *r = new SrvReq;
    r->id = sv->next_id++;
    r->mesh = mesh;
    r->k = k;
    r->q.assign((const double2 *)q, (const double2 *)q + n);
    sv->queue.push_back(r);
    if (id) *id = r->id;
    return NIHU_GB_OK;
}

extern "C" nihu_gb_status nihu_gb_server_step(nihu_gb_server *sv, int *n_queued, int *n_active, int *n_done)
{
    if (!sv) return NIHU_GB_ERR_INVALID_ARGUMENT;
    nihu_gb_ctx *ctx = sv->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    nihu_gb_status st;
    const int m = sv->restart;
    // 1. admission, first come first served, while the budget and the state slots hold
    std::vector<SrvReq *> fresh;
    std::unique_ptr<Phase> ph_admit(new Phase(ctx, "serve_admit"));
    while (!sv->queue.empty() && !sv->free_slots.empty()) {
        SrvReq *r = sv->queue.front();
        const int64_t n = sv->meshes[r->mesh]->n;
        const size_t mat = 8 * (size_t)n * n, blk = srv_block_bytes(n, m);
        if (sv->held + mat + blk > sv->budget) break;
        CK(cudaMallocFromPoolAsync(&r->H, mat, sv->pool, s));
        CK(cudaMallocFromPoolAsync(&r->blk, blk, sv->pool, s));
        r->held = mat + blk;
        sv->held += r->held;
        char *p = (char *)r->blk;
        r->b = (double2 *)p;
        r->x = r->b + n;
        p += srv_align(2 * 16 * (size_t)n);
        r->V = (double2 *)p;
        p += srv_align(16 * (size_t)n * (m + 1));
        r->S = (double2 *)p;
        r->slot = sv->free_slots.back();
        sv->free_slots.pop_back();
        CK(cudaMemsetAsync(sv->d_states + r->slot, 0, sizeof(PersistentState), s));  // PG_FRESH
        sv->queue.pop_front();
        fresh.push_back(r);
    }
    // the round's Neumann data, grouped by mesh, into pinned staging: one
    // upload per mesh group below
    size_t stage = 0;
    for (SrvReq *r : fresh) stage += 16 * (size_t)sv->meshes[r->mesh]->n;
    if (stage > sv->h_stage_bytes) {
        if (sv->h_stage) cudaFreeHost(sv->h_stage);
        sv->h_stage = nullptr;
        sv->h_stage_bytes = 0;
        CK(cudaMallocHost((void **)&sv->h_stage, stage));
        sv->h_stage_bytes = stage;
    }
    ph_admit.reset();
    // 2. assembly of the new requests, one frequency batch per mesh: the DLP
    // matrices and the right-hand sides b = SLP q (no SLP matrix)
    std::vector<std::vector<void *>> tables;  // host sources of the pointer uploads, alive until the round's wait
    double2 *hq = sv->h_stage;
    for (int i = 0; i < (int)sv->meshes.size(); ++i) {
        std::vector<SrvReq *> grp;
        for (SrvReq *r : fresh)
            if (r->mesh == i) grp.push_back(r);
        if (grp.empty()) continue;
        const nihu_gb_mesh *mesh = sv->meshes[i];
        const int64_t n = mesh->n;
        const int nk = (int)grp.size();
        std::vector<double> ks(nk);
        tables.emplace_back(2 * (size_t)nk);
        std::vector<void *> &tab = tables.back();
        void *gq, *gb;  // the group's Neumann data and right-hand sides, back to back
        if ((st = scratch(ctx, "srv_q", 16 * (size_t)n * nk, &gq))) return st;
        if ((st = scratch(ctx, "srv_b", 16 * (size_t)n * nk, &gb))) return st;
        for (int f = 0; f < nk; ++f) {
            ks[f] = grp[f]->k;
            tab[f] = nullptr;
            tab[nk + f] = grp[f]->H;
            std::memcpy(hq + (size_t)f * n, grp[f]->q.data(), 16 * (size_t)n);
        }
        {
            Phase ph(ctx, "serve_q_upload");
            CK(cudaMemcpyAsync(gq, hq, 16 * (size_t)n * nk, cudaMemcpyHostToDevice, s));
        }
        hq += (size_t)n * nk;
        // always the frequency-batch kernels: an entry is then the same whatever else arrived with it
        void *douts = nullptr;
        const std::string name = "srv_outs" + std::to_string(i);
        if ((st = scratch(ctx, name.c_str(), sizeof(void *) * 2 * (size_t)nk, &douts))) return st;
        CK(cudaMemcpyAsync(douts, tab.data(), sizeof(void *) * 2 * (size_t)nk, cudaMemcpyHostToDevice, s));
        if ((st = assemble_batch(ctx, mesh, mesh, sv->family, NIHU_GB_SLP | NIHU_GB_DLP, ks.data(), nk, sv->precision,
                                 NIHU_GB_C64, nullptr, grp[0]->H, n, n * n, (void *const *)douts, true,
                                 (const double2 *)gq, (double2 *)gb)))
            return st;
        Phase ph_rhs(ctx, "serve_identity_rhs");
        for (int f = 0; f < nk; ++f) {
            SrvReq *r = grp[f];
            CK(launch_add_identity((int)n, -0.5, 0.0, NIHU_GB_C64, r->H, n, s));
            CK(cudaMemcpyAsync(r->b, (double2 *)gb + (size_t)f * n, 16 * (size_t)n, cudaMemcpyDeviceToDevice, s));
            ctx->launches += 1;
        }
        sv->active.insert(sv->active.end(), grp.begin(), grp.end());
    }
    // 3. every admitted system advances by at most `quantum` steps
    if (!sv->active.empty()) {
        std::vector<PersistentItem> items(sv->active.size());
        std::vector<double> work(sv->active.size());
        for (size_t t = 0; t < sv->active.size(); ++t) {
            SrvReq *r = sv->active[t];
            const int64_t n = sv->meshes[r->mesh]->n;
            PersistentItem &it = items[t];
            it.A = (const float2 *)r->H;
            it.lda = n;
            it.b = r->b;
            it.x = r->x;
            it.V = r->V;
            it.S = r->S;
            it.st = sv->d_states + r->slot;
            it.n = (int)n;
            it.pad = 0;
            work[t] = (double)n * (double)n;
        }
        if ((st = launch_persistent(ctx, items, work, m, sv->max_iters, sv->quantum, sv->tol))) return st;
    }
    // 4. retire the finished systems
    std::vector<PersistentState> hs(sv->n_slots);
    {
        Phase ph(ctx, "serve_state_read");
        CK(cudaMemcpyAsync(hs.data(), sv->d_states, sizeof(PersistentState) * sv->n_slots, cudaMemcpyDeviceToHost, s));
    }
    if ((st = sync(ctx))) return st;
    std::vector<SrvReq *> still;
    std::vector<SrvReq *> finished;
    for (SrvReq *r : sv->active) {
        r->st = hs[r->slot];
        if (r->st.status == PG_DONE) finished.push_back(r);
        else still.push_back(r);
    }
    {
        Phase ph(ctx, "serve_result_read");
        for (SrvReq *r : finished) {
            const int64_t n = sv->meshes[r->mesh]->n;
            r->q.resize(n);
            CK(cudaMemcpyAsync(r->q.data(), r->x, 16 * (size_t)n, cudaMemcpyDeviceToHost, s));
        }
    }
    if (!finished.empty() && (st = sync(ctx))) return st;
    for (SrvReq *r : finished) {
        srv_release(sv, r);
        sv->done.push_back(r);
    }
    sv->active.swap(still);
    if (n_queued) *n_queued = (int)sv->queue.size();
    if (n_active) *n_active = (int)sv->active.size();
    if (n_done) *n_done = (int)sv->done.size();
    return NIHU_GB_OK;
}

extern "C" nihu_gb_status nihu_gb_server_take(nihu_gb_server *sv, int64_t *id, void *p, int64_t capacity, int *iters,
                                              double *rel_residual, int *converged)
{
    if (!sv || !id) return NIHU_GB_ERR_INVALID_ARGUMENT;
    *id = -1;
    if (sv->done.empty()) return NIHU_GB_OK;
    SrvReq *r = sv->done.front();
    const int64_t n = (int64_t)r->q.size();
    if (!p || capacity < n)
        return fail(sv->ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_server_take: result buffer too small");
    std::memcpy(p, r->q.data(), 16 * (size_t)n);
    *id = r->id;
    if (iters) *iters = r->st.iters;
    if (rel_residual) *rel_residual = r->st.rel;
    if (converged) *converged = r->st.converged;
    sv->done.pop_front();
    delete r;
    return NIHU_GB_OK;
}

// ------------------------------------------------------ sweep plan (graph)
//
// A frequency sweep over fixed meshes, captured once as a CUDA graph: the
// wave-number and Neumann-data uploads, every mesh's frequency-batch
// assembly (the FP64 kernel on the auxiliary stream beside the regular one),
// the identities and right-hand sides, the persistent GMRES launch over all
// systems, and the downloads of the solutions, states and error flag.  Each
// run refills pinned staging buffers and replays the graph: no host work,
// allocation or synchronisation inside.  The staging buffers hold the
// instances in the caller's order (one copy each way); the graph permutes
// them to and from the device's mesh-grouped order, and a caller that writes
// into them directly (nihu_gb_sweep_plan_host_buffers) saves the host copies.

struct nihu_gb_sweep_plan {
    struct Group {
        int mesh = 0;
        std::vector<int> fs;       // instances, in instance order
        int64_t n = 0, first = 0;  // elements; position of the group's first instance
        void *H = nullptr;          // DLP matrices (no SLP matrix: right-hand-side mode)
        void *rpart = nullptr;      // regular kernel's partial sums of b
        double2 *nslp = nullptr;    // FP64 kernel's SLP entries
        NearList *nl = nullptr;
    };
    nihu_gb_ctx *ctx = nullptr;
    std::vector<const nihu_gb_mesh *> meshes;
    std::vector<int> mesh_of;
    std::vector<Group> groups;
    std::vector<int> order_of;       // instance f -> position (groups in mesh order)
    std::vector<int64_t> pos_n;      // position -> elements
    std::vector<int64_t> off, user;  // device (position order) and user (instance order) column offsets
    int family = 0, precision = 0, nk = 0, restart = 0, max_iters = 0;
    double tol = 0.0, kmax = 0.0;
    int64_t total = 0;
    std::vector<void *> dbufs;  // device allocations of the plan
    double *d_ks = nullptr;
    float *d_ks32 = nullptr;
    double2 *d_q = nullptr, *d_b = nullptr, *d_x = nullptr;
    double2 *d_user = nullptr;  // Neumann data in, solutions out, in instance order
    int64_t *d_src = nullptr, *d_dst = nullptr;  // permute tables: instance order -> device order
    int *d_len = nullptr;
    int max_len = 0;
    PersistentState *d_st = nullptr;
    // pinned host staging
    double *h_ks = nullptr;
    float *h_ks32 = nullptr;
    double2 *h_q = nullptr, *h_p = nullptr;
    PersistentState *h_st = nullptr;
    // processing order of each persistent launch, refreshed per run (larger
    // n^2 (1 + |k|) first): launch t's items are launch_items[t], its order
    // h_order[order_off[t] ...] and, uploaded in the graph, d_order[...]
    std::vector<std::vector<int>> launch_items;
    std::vector<int> order_off;
    int *h_order = nullptr, *d_order = nullptr;
    // the systems of the persistent launches (positions), their device copy,
    // and the launch set-up the autotuner chose at creation
    std::vector<PersistentItem> items;
    std::vector<int64_t> ns;
    PersistentItem *d_items = nullptr;
    int rhs_fmax = 0;        // wave numbers per regular block (right-hand-side mode)
    int tuned_cluster = 0;   // CTAs per cluster of the (first) persistent launch
    double tuned_ms = 0.0;   // the chosen set-up's replay time on the representative inputs
    int *h_flag = nullptr;
    std::vector<PersistentArgs> pargs;  // one or two persistent launches (plan_launches)
    std::vector<PersistentPlan> pplans;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // the side chain of the capture (every group but the largest): its main
    // and FP64 streams, their fork / join events, and the split / merge events
    cudaStream_t side = nullptr, side_aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_split = nullptr, ev_merge = nullptr;
};

namespace {

void plan_free(nihu_gb_sweep_plan *pl)
{
    if (!pl) return;
    nihu_gb_ctx *ctx = pl->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    for (cudaStream_t t : {pl->side, pl->side_aux})
        if (t) cudaStreamDestroy(t);
    for (cudaEvent_t ev : {pl->ev_fork, pl->ev_join, pl->ev_split, pl->ev_merge})
        if (ev) cudaEventDestroy(ev);
    for (void *p : pl->dbufs) dfree(ctx, p);
    for (void *h : {(void *)pl->h_ks, (void *)pl->h_ks32, (void *)pl->h_q, (void *)pl->h_p, (void *)pl->h_st, (void *)pl->h_order,
                    (void *)pl->h_flag})
        if (h) cudaFreeHost(h);
    delete pl;
}

nihu_gb_status plan_alloc(nihu_gb_sweep_plan *pl, size_t bytes, void **out)
{
    nihu_gb_status st = dmalloc(pl->ctx, std::max<size_t>(bytes, 16), out);
    if (st == NIHU_GB_OK) pl->dbufs.push_back(*out);
    return st;
}

// record the whole sweep on the context stream into pl->graph and instantiate it
nihu_gb_status plan_capture(nihu_gb_sweep_plan *pl)
{
    nihu_gb_ctx *ctx = pl->ctx;
    cudaStream_t s = ctx->stream;
    const bool prof = ctx->profiling;
    ctx->profiling = false;  // no timing events inside the graph
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    nihu_gb_status st = NIHU_GB_OK;
    auto chk = [&](cudaError_t r) {
        if (r != cudaSuccess && e == cudaSuccess) e = r;
    };
    if (e == cudaSuccess) {
        chk(cudaMemcpyAsync(pl->d_ks, pl->h_ks, 8 * (size_t)pl->nk, cudaMemcpyHostToDevice, s));
        chk(cudaMemcpyAsync(pl->d_ks32, pl->h_ks32, 4 * (size_t)pl->nk, cudaMemcpyHostToDevice, s));
        chk(cudaMemcpyAsync(pl->d_user, pl->h_q, 16 * (size_t)pl->total, cudaMemcpyHostToDevice, s));
        chk(launch_permute_segments(pl->d_user, pl->d_q, pl->d_src, pl->d_dst, pl->d_len, pl->nk, pl->max_len, s));
        // the largest group's assembly on the context's streams; the others on
        // the side chain beside it, where their small, latency-bound kernels
        // fill in around the large ones; the chains meet before the solve
        size_t big = 0;
        for (size_t gi = 0; gi < pl->groups.size(); ++gi) {
            const auto &g = pl->groups[gi], &b = pl->groups[big];
            if ((double)g.n * g.n * g.fs.size() > (double)b.n * b.n * b.fs.size()) big = gi;
        }
        chk(cudaEventRecord(pl->ev_split, s));
        chk(cudaStreamWaitEvent(pl->side, pl->ev_split, 0));
        const cudaStream_t main_s = ctx->stream, main_aux = ctx->aux_stream;
        const cudaEvent_t main_fork = ctx->ev_fork, main_join = ctx->ev_join;
        for (size_t gi = 0; gi < pl->groups.size(); ++gi) {
            if (e != cudaSuccess || st) break;
            auto &g = pl->groups[gi];
            // assemble_panel forks and joins on the context's streams: point them at this group's chain
            const bool on_side = gi != big;
            ctx->stream = on_side ? pl->side : main_s;
            ctx->aux_stream = on_side ? pl->side_aux : main_aux;
            ctx->ev_fork = on_side ? pl->ev_fork : main_fork;
            ctx->ev_join = on_side ? pl->ev_join : main_join;
            const cudaStream_t gs = ctx->stream;
            const int cnt = (int)g.fs.size();
            const nihu_gb_mesh *mesh = pl->meshes[g.mesh];
            RegularArgs a;
            a.test = mesh->dm;
            a.trial = mesh->dm;
            a.same_mesh = 1;
            a.family = pl->family;
            a.ops = NIHU_GB_SLP | NIHU_GB_DLP;
            a.k = pl->kmax;
            a.alpha_re = 1.0;
            a.alpha_im = 0.0;
            a.precision = pl->precision;
            a.dtype = NIHU_GB_C64;
            a.accumulate = 0;
            a.trial_size_max = mesh->size_max;
            a.k32 = (float)pl->kmax;
            a.alpha_re32 = 1.0f;
            a.alpha_im32 = 0.0f;
            a.unit_alpha = 1;
            a.out_s = nullptr;
            a.out_d = g.H;
            a.ld = g.n;
            a.j0 = 0;
            a.j1 = (int)g.n;
            a.nk = cnt;
            a.ks = pl->d_ks + g.first;
            a.ks32 = pl->d_ks32 + g.first;
            a.mat_stride = g.n * g.n;
            a.k_absmax = pl->kmax;
            a.force_batch = 1;
            const int64_t o = pl->off[g.fs[0]];
            a.rhs_q = pl->d_q + o;
            a.rhs_part = g.rpart;
            a.near_slp = g.nslp;
            a.rhs_fmax = pl->rhs_fmax;
            st = assemble_panel(ctx, a, g.nl);
            if (st) break;
            chk(launch_add_identity_batched((int)g.n, -0.5, 0.0, NIHU_GB_C64, g.H, g.n, g.n * g.n, cnt, gs));
            chk(launch_rhs_reduce(a, *g.nl, pl->d_b + o, gs));
        }
        ctx->stream = main_s;
        ctx->aux_stream = main_aux;
        ctx->ev_fork = main_fork;
        ctx->ev_join = main_join;
        chk(cudaEventRecord(pl->ev_merge, pl->side));
        chk(cudaStreamWaitEvent(s, pl->ev_merge, 0));
        chk(cudaMemsetAsync(pl->d_st, 0, sizeof(PersistentState) * (size_t)pl->nk, s));
        for (const PersistentArgs &pa : pl->pargs) chk(cudaMemsetAsync(pa.counter, 0, sizeof(int), s));
        chk(cudaMemcpyAsync(pl->d_order, pl->h_order, sizeof(int) * (size_t)pl->nk, cudaMemcpyHostToDevice, s));
        for (size_t t = 0; t < pl->pargs.size(); ++t)
            chk(launch_persistent_gmres(pl->pargs[t], pl->pplans[t].cluster, pl->pplans[t].clusters, pl->pplans[t].smem,
                                        s, t > 0));
        chk(launch_permute_segments(pl->d_x, pl->d_user, pl->d_dst, pl->d_src, pl->d_len, pl->nk, pl->max_len, s));
        chk(cudaMemcpyAsync(pl->h_p, pl->d_user, 16 * (size_t)pl->total, cudaMemcpyDeviceToHost, s));
        chk(cudaMemcpyAsync(pl->h_st, pl->d_st, sizeof(PersistentState) * (size_t)pl->nk, cudaMemcpyDeviceToHost, s));
        chk(cudaMemcpyAsync(pl->h_flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        chk(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), s));
        cudaGraph_t graph = nullptr;
        chk(cudaStreamEndCapture(s, &graph));  // ends the capture even after an error
        pl->graph = graph;
    }
    ctx->profiling = prof;
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "sweep plan capture");
    CK(cudaGraphInstantiate(&pl->exec, pl->graph, 0));
    return NIHU_GB_OK;
}

}  // namespace

namespace {

// each persistent launch's systems in processing order for the wave numbers
// in h_ks: larger n^2 (1 + |k|) first (iteration counts grow with k)
void plan_set_order(nihu_gb_sweep_plan *pl)
{
    for (size_t t = 0; t < pl->launch_items.size(); ++t) {
        std::vector<int> ord = pl->launch_items[t];
        std::vector<double> key(pl->nk, 0.0);
        for (int q_ : ord) key[q_] = (double)pl->pos_n[q_] * pl->pos_n[q_] * (1.0 + std::fabs(pl->h_ks[q_]));
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return key[x] > key[y]; });
        std::copy(ord.begin(), ord.end(), pl->h_order + pl->order_off[t]);
    }
}

// the persistent launches over the plan's systems (force_cluster: the CTAs
// per cluster of the first launch, 0 = the launch model's choice); the
// systems' device copy, counters and matvec-input buffers follow
nihu_gb_status plan_setup_launches(nihu_gb_sweep_plan *pl, int force_cluster)
{
    nihu_gb_ctx *ctx = pl->ctx;
    nihu_gb_status st;
    pl->launch_items.clear();
    pl->order_off.clear();
    pl->pargs.clear();
    pl->pplans.clear();
    std::vector<PersistentLaunch> launches;
    if ((st = plan_launches(ctx, pl->ns, std::vector<double>(pl->ns.begin(), pl->ns.end()), pl->restart, &launches,
                            force_cluster)))
        return st;
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device);
    std::vector<PersistentItem> items = pl->items;
    for (const PersistentLaunch &L : launches)
        for (int q : L.order) {
            PersistentItem &it = items[q];
            it.vec = (it.n % 2 == 0) && (it.lda % 2 == 0) && ((reinterpret_cast<uintptr_t>(it.A) & 15) == 0);
            it.stream = 8.0 * (double)it.n * (double)it.n * std::min<int>((int)L.order.size(), L.plan.clusters) >
                        0.5 * l2;
        }
    CK(cudaMemcpy(pl->d_items, items.data(), sizeof(PersistentItem) * (size_t)pl->nk, cudaMemcpyHostToDevice));
    for (size_t t = 0, o = 0; t < launches.size(); ++t) {
        const PersistentLaunch &L = launches[t];
        const int cnt = (int)L.order.size();
        pl->launch_items.push_back(L.order);
        pl->order_off.push_back((int)o);
        void *dcnt, *dvx = nullptr;
        if ((st = plan_alloc(pl, sizeof(int), &dcnt))) return st;
        if (!L.plan.vx_smem && (st = plan_alloc(pl, 8 * (size_t)L.plan.clusters * L.n_max, &dvx))) return st;
        PersistentArgs a{};
        a.items = pl->d_items;
        a.order = pl->d_order + o;
        o += cnt;
        a.count = cnt;
        a.n_max = (int)L.n_max;
        a.restart = pl->restart;
        a.max_iters = pl->max_iters;
        a.quantum = 0;
        a.tol = pl->tol;
        a.counter = (int *)dcnt;
        a.vxg = (float2 *)dvx;
        a.wait_primary = t > 0;
        pl->pargs.push_back(a);
        pl->pplans.push_back(L.plan);
    }
    return NIHU_GB_OK;
}

void plan_drop_graph(nihu_gb_sweep_plan *pl)
{
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    pl->exec = nullptr;
    pl->graph = nullptr;
}

// The autotuner: the plan's launch set-up is measured, not modelled.  Each
// candidate -- the persistent launch's CTAs per cluster (the launch model's
// choice, 4, 8, 16) times the wave numbers per regular block (8, 16, 20) -- is
// captured and replayed on representative inputs (wave numbers spread over
// (0.1, 1] k_max, unit Neumann data); the fastest replay's set-up is kept
// and captured for good.
nihu_gb_status plan_autotune(nihu_gb_sweep_plan *pl)
{
    nihu_gb_ctx *ctx = pl->ctx;
    nihu_gb_status st;
    for (int f = 0; f < pl->nk; ++f) {
        const int q_ = pl->order_of[f];
        pl->h_ks[q_] = pl->kmax * (0.1 + 0.9 * (f + 0.5) / pl->nk);
        pl->h_ks32[q_] = (float)pl->h_ks[q_];
    }
    for (int64_t i = 0; i < pl->total; ++i) pl->h_q[i] = make_double2(1.0, 0.0);
    cudaEvent_t t0, t1;
    CK(cudaEventCreate(&t0));
    CK(cudaEventCreate(&t1));
    double best_ms = -1.0;
    int best_c = 0, best_f = 0;
    std::vector<int> seen;
    for (int c : {0, 4, 8, 16}) {
        if (plan_setup_launches(pl, c) != NIHU_GB_OK) {
            cudaGetLastError();
            continue;
        }
        const int shape = pl->pplans[0].cluster;
        if (std::find(seen.begin(), seen.end(), shape) != seen.end()) continue;
        seen.push_back(shape);
        for (int fm : {8, 16, 20}) {
            pl->rhs_fmax = fm;
            plan_drop_graph(pl);
            if (plan_capture(pl) != NIHU_GB_OK) {
                cudaGetLastError();
                continue;
            }
            plan_set_order(pl);
            float ms = 0.0f;
            cudaError_t e = cudaGraphLaunch(pl->exec, ctx->stream);  // warm-up
            if (e == cudaSuccess) e = cudaEventRecord(t0, ctx->stream);
            if (e == cudaSuccess) e = cudaGraphLaunch(pl->exec, ctx->stream);
            if (e == cudaSuccess) e = cudaEventRecord(t1, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
            if (e != cudaSuccess) {
                cudaEventDestroy(t0);
                cudaEventDestroy(t1);
                return cuda_fail(ctx, e, "sweep plan autotuning");
            }
            if (best_ms < 0.0 || ms < best_ms) {
                best_ms = ms;
                best_c = c;
                best_f = fm;
            }
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    plan_drop_graph(pl);
    if (best_ms < 0.0) return fail(ctx, NIHU_GB_ERR_RUNTIME, "sweep plan: no launch set-up could be captured");
    if ((st = plan_setup_launches(pl, best_c))) return st;
    pl->rhs_fmax = best_f;
    pl->tuned_cluster = pl->pplans[0].cluster;
    pl->tuned_ms = best_ms;
    return plan_capture(pl);
}

}  // namespace

extern "C" nihu_gb_status nihu_gb_sweep_plan_create(nihu_gb_ctx *ctx, int n_meshes, const nihu_gb_mesh *const *meshes,
                                                    int family, int nk, const int *mesh_of, double k_max,
                                                    int precision, int restart, int max_iters, double tol,
                                                    nihu_gb_sweep_plan **out)
{
    if (!ctx || !out) return NIHU_GB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_meshes < 1 || !meshes || nk < 1 || !mesh_of || !(k_max > 0.0) || !std::isfinite(k_max) ||
        (precision != 0 && precision != 1) || (family != NIHU_GB_HELMHOLTZ_3D && family != NIHU_GB_LAPLACE_3D) ||
        restart < 1 || restart > 200 || max_iters < 1 || !(tol > 0.0))
        return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_sweep_plan_create: bad argument");
    for (int i = 0; i < n_meshes; ++i)
        if (!meshes[i] || meshes[i]->ctx != ctx || meshes[i]->n < 1)
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_sweep_plan_create: bad mesh");
    for (int f = 0; f < nk; ++f)
        if (mesh_of[f] < 0 || mesh_of[f] >= n_meshes)
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_sweep_plan_create: bad mesh index");
    cudaSetDevice(ctx->device);
    nihu_gb_status st;
    std::unique_ptr<nihu_gb_sweep_plan, void (*)(nihu_gb_sweep_plan *)> pl(new nihu_gb_sweep_plan, plan_free);
    pl->ctx = ctx;
    pl->meshes.assign(meshes, meshes + n_meshes);
    pl->mesh_of.assign(mesh_of, mesh_of + nk);
    pl->family = family;
    pl->precision = precision;
    pl->nk = nk;
    pl->max_iters = max_iters;
    pl->tol = tol;
    pl->kmax = k_max;
    pl->off = sweep_offsets(n_meshes, meshes, nk, mesh_of);
    pl->user.resize(nk);
    pl->order_of.resize(nk);
    int64_t n_max = 1;
    for (int f = 0; f < nk; ++f) {
        pl->user[f] = pl->total;
        pl->total += meshes[mesh_of[f]]->n;
        n_max = std::max<int64_t>(n_max, meshes[mesh_of[f]]->n);
    }
    const int m = (int)std::min<int64_t>(restart, n_max);
    pl->restart = m;
    int pos = 0;
    for (int i = 0; i < n_meshes; ++i) {
        nihu_gb_sweep_plan::Group g;
        g.mesh = i;
        g.n = meshes[i]->n;
        g.first = pos;
        for (int f = 0; f < nk; ++f)
            if (mesh_of[f] == i) {
                g.fs.push_back(f);
                pl->order_of[f] = pos++;
            }
        if (!g.fs.empty()) pl->groups.push_back(g);
    }
    // device buffers
    void *p;
    const size_t ss = persistent_small_state(m);
    if ((st = plan_alloc(pl.get(), 8 * (size_t)nk, &p))) return st;
    pl->d_ks = (double *)p;
    if ((st = plan_alloc(pl.get(), 4 * (size_t)nk, &p))) return st;
    pl->d_ks32 = (float *)p;
    double2 *bufs[4];
    for (int t = 0; t < 4; ++t) {
        if ((st = plan_alloc(pl.get(), 16 * (size_t)pl->total, &p))) return st;
        bufs[t] = (double2 *)p;
    }
    pl->d_q = bufs[0];
    pl->d_b = bufs[1];
    pl->d_x = bufs[2];
    pl->d_user = bufs[3];
    {
        std::vector<int> len(nk);
        for (int f = 0; f < nk; ++f) {
            len[f] = (int)meshes[mesh_of[f]]->n;
            pl->max_len = std::max(pl->max_len, len[f]);
        }
        if ((st = plan_alloc(pl.get(), sizeof(int64_t) * nk, &p))) return st;
        pl->d_src = (int64_t *)p;
        if ((st = plan_alloc(pl.get(), sizeof(int64_t) * nk, &p))) return st;
        pl->d_dst = (int64_t *)p;
        if ((st = plan_alloc(pl.get(), sizeof(int) * nk, &p))) return st;
        pl->d_len = (int *)p;
        CK(cudaMemcpy(pl->d_src, pl->user.data(), sizeof(int64_t) * nk, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(pl->d_dst, pl->off.data(), sizeof(int64_t) * nk, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(pl->d_len, len.data(), sizeof(int) * nk, cudaMemcpyHostToDevice));
    }
    void *dV, *dS, *dst, *ditems, *dorder;
    if ((st = plan_alloc(pl.get(), 16 * (size_t)pl->total * (m + 1), &dV))) return st;
    if ((st = plan_alloc(pl.get(), 16 * ss * nk, &dS))) return st;
    if ((st = plan_alloc(pl.get(), sizeof(PersistentState) * (size_t)nk, &dst))) return st;
    pl->d_st = (PersistentState *)dst;
    for (auto &g : pl->groups) {
        const size_t cnt = g.fs.size();
        if ((st = plan_alloc(pl.get(), 8 * (size_t)g.n * g.n * cnt, &g.H))) return st;
        if ((st = get_near(ctx, meshes[g.mesh], meshes[g.mesh], &g.nl))) return st;
        if ((st = near_rows(ctx, g.nl, true, g.n))) return st;
        RegularArgs ra;
        ra.test = meshes[g.mesh]->dm;
        ra.precision = precision;
        ra.j0 = 0;
        ra.j1 = (int)g.n;
        ra.nk = (int)cnt;
        if ((st = plan_alloc(pl.get(), rhs_part_bytes(ra), &g.rpart))) return st;
        if ((st = plan_alloc(pl.get(), 16 * (size_t)(g.nl->nnz + g.n) * cnt, &p))) return st;
        g.nslp = (double2 *)p;
    }
    // the persistent launches' systems (launch shape: plan_setup_launches)
    pl->items.assign(nk, PersistentItem{});
    pl->ns.assign(nk, 0);
    pl->pos_n.assign(nk, 0);
    for (auto &g : pl->groups)
        for (size_t j = 0; j < g.fs.size(); ++j) {
            const int f = g.fs[j], q = pl->order_of[f];
            pl->pos_n[q] = g.n;
            PersistentItem &it = pl->items[q];
            it.A = (const float2 *)g.H + (size_t)g.n * g.n * j;
            it.lda = g.n;
            it.b = pl->d_b + pl->off[f];
            it.x = pl->d_x + pl->off[f];
            it.V = (double2 *)dV + pl->off[f] * (m + 1);
            it.S = (double2 *)dS + ss * q;
            it.st = pl->d_st + q;
            it.n = (int)g.n;
            it.pad = 0;
            pl->ns[q] = g.n;
        }
    if ((st = plan_alloc(pl.get(), sizeof(PersistentItem) * (size_t)nk, &ditems))) return st;
    pl->d_items = (PersistentItem *)ditems;
    if ((st = plan_alloc(pl.get(), sizeof(int) * (size_t)nk, &dorder))) return st;
    pl->d_order = (int *)dorder;
    CK(cudaMallocHost((void **)&pl->h_order, sizeof(int) * (size_t)nk));
    // pinned staging
    CK(cudaMallocHost((void **)&pl->h_ks, 8 * (size_t)nk));
    CK(cudaMallocHost((void **)&pl->h_ks32, 4 * (size_t)nk));
    CK(cudaMallocHost((void **)&pl->h_q, 16 * (size_t)pl->total));
    CK(cudaMallocHost((void **)&pl->h_p, 16 * (size_t)pl->total));
    CK(cudaMallocHost((void **)&pl->h_st, sizeof(PersistentState) * (size_t)nk));
    CK(cudaMallocHost((void **)&pl->h_flag, sizeof(int)));
    {
        int prio_lo = 0, prio_hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
        CK(cudaStreamCreateWithFlags(&pl->side, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithPriority(&pl->side_aux, cudaStreamNonBlocking, prio_hi));
        for (cudaEvent_t *ev : {&pl->ev_fork, &pl->ev_join, &pl->ev_split, &pl->ev_merge})
            CK(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    }
    CK(prepare_singular_batch(ctx->stream));
    if ((st = sync(ctx))) return st;
    if ((st = plan_autotune(pl.get()))) return st;
    *out = pl.release();
    return NIHU_GB_OK;
}

extern "C" nihu_gb_status nihu_gb_sweep_plan_run(nihu_gb_sweep_plan *pl, const double *ks, const void *q, void *p,
                                                 int *iters, double *rel_residuals, int *converged)
{
    if (!pl) return NIHU_GB_ERR_INVALID_ARGUMENT;
    nihu_gb_ctx *ctx = pl->ctx;
    if (!ks || !q || !p) return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_sweep_plan_run: bad argument");
    for (int f = 0; f < pl->nk; ++f)
        if (!std::isfinite(ks[f]) || std::fabs(ks[f]) > pl->kmax)
            return fail(ctx, NIHU_GB_ERR_INVALID_ARGUMENT, "nihu_gb_sweep_plan_run: wave number beyond the plan's k_max");
    cudaSetDevice(ctx->device);
    for (int f = 0; f < pl->nk; ++f) {
        const int q_ = pl->order_of[f];
        pl->h_ks[q_] = ks[f];
        pl->h_ks32[q_] = (float)ks[f];
    }
    plan_set_order(pl);
    if (q != pl->h_q) std::memcpy(pl->h_q, q, 16 * (size_t)pl->total);
    {
        Phase ph(ctx, "sweep_graph");
        CK(cudaGraphLaunch(pl->exec, ctx->stream));
    }
    ctx->launches += 1;
    nihu_gb_status st;
    if ((st = sync(ctx))) return st;
    if (*pl->h_flag)
        return fail(ctx, NIHU_GB_ERR_RUNTIME, "Could not perform inverse mapping (nearly singular pair " +
                                                  std::to_string(*pl->h_flag - 1) + ")");
    if (p != pl->h_p) std::memcpy(p, pl->h_p, 16 * (size_t)pl->total);
    bool all = true;
    for (int f = 0; f < pl->nk; ++f) {
        const PersistentState &s = pl->h_st[pl->order_of[f]];
        if (iters) iters[f] = s.iters;
        if (rel_residuals) rel_residuals[f] = s.rel;
        if (converged) converged[f] = s.converged;
        all = all && s.converged;
    }
    if (!all) return fail(ctx, NIHU_GB_ERR_NOT_CONVERGED, "sweep plan: some systems did not reach the tolerance");
    return NIHU_GB_OK;
}

extern "C" nihu_gb_status nihu_gb_sweep_plan_host_buffers(nihu_gb_sweep_plan *pl, void **q, void **p)
{
    if (!pl || !q || !p) return NIHU_GB_ERR_INVALID_ARGUMENT;
    *q = pl->h_q;
    *p = pl->h_p;
    return NIHU_GB_OK;
}

extern "C" nihu_gb_status nihu_gb_sweep_plan_tuning(const nihu_gb_sweep_plan *pl, int *cluster, int *freq_per_block,
                                                    double *replay_ms)
{
    if (!pl) return NIHU_GB_ERR_INVALID_ARGUMENT;
    if (cluster) *cluster = pl->tuned_cluster;
    if (freq_per_block) *freq_per_block = pl->rhs_fmax;
    if (replay_ms) *replay_ms = pl->tuned_ms;
    return NIHU_GB_OK;
}

extern "C" void nihu_gb_sweep_plan_destroy(nihu_gb_sweep_plan *pl) { plan_free(pl); }
