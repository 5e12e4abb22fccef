// Nearly singular pair lists (column-sorted) and pair statistics.
#include "classify.cuh"
#include "kernels.h"

namespace nihu {

constexpr int CLS_THREADS = 256;

// one block per trial column: count nearly singular test rows
__global__ void __launch_bounds__(CLS_THREADS) k_near_count(DevMesh test, DevMesh trial, int same_mesh, int *counts)
{
    int j = blockIdx.x;
    float4 jh = trial.chi[j], jl = trial.clo[j];
    int total = 0;
    for (int i0 = 0; i0 < test.n; i0 += CLS_THREADS) {
        int i = i0 + threadIdx.x;
        int pred = 0;
        if (i < test.n) {
            int ls, ld;
            float dx, dy, dz;
            pred = classify_pair(test.chi[i], test.clo[i], jh, jl, i, j, test.center, trial.center, trial.size,
                                 same_mesh, ls, ld, dx, dy, dz) == KIND_NEAR;
        }
        total += __syncthreads_count(pred);
    }
    if (threadIdx.x == 0) counts[j] = total;
}

// single-block exclusive scan of n ints into int64 offsets (n + 1 entries)
__global__ void __launch_bounds__(1024) k_scan(const int *counts, int n, int64_t *out)
{
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < n; base += 1024) {
        int idx = base + threadIdx.x;
        int64_t v = idx < n ? counts[idx] : 0;
        int64_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int64_t t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int64_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        int64_t excl = carry + (wid > 0 ? warp_tot[wid - 1] : 0) + x - v;
        if (idx < n) out[idx] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

// one block per trial column: write the nearly singular rows in increasing order
__global__ void __launch_bounds__(CLS_THREADS) k_near_fill(DevMesh test, DevMesh trial, int same_mesh,
                                                            const int64_t *col_ptr, int *rows)
{
    __shared__ int warp_cnt[CLS_THREADS / 32];
    int j = blockIdx.x;
    float4 jh = trial.chi[j], jl = trial.clo[j];
    int64_t pos = col_ptr[j];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i0 = 0; i0 < test.n; i0 += CLS_THREADS) {
        int i = i0 + threadIdx.x;
        int pred = 0;
        if (i < test.n) {
            int ls, ld;
            float dx, dy, dz;
            pred = classify_pair(test.chi[i], test.clo[i], jh, jl, i, j, test.center, trial.center, trial.size,
                                 same_mesh, ls, ld, dx, dy, dz) == KIND_NEAR;
        }
        unsigned m = __ballot_sync(0xffffffffu, pred);
        if (lane == 0) warp_cnt[wid] = __popc(m);
        __syncthreads();
        int before = 0, tot = 0;
        for (int w = 0; w < CLS_THREADS / 32; ++w) {
            if (w < wid) before += warp_cnt[w];
            tot += warp_cnt[w];
        }
        if (pred) rows[pos + before + __popc(m & ((1u << lane) - 1u))] = i;
        pos += tot;
        __syncthreads();
    }
}

// histogram: [0] self, [1] near, [2 + 3 ls + ld] regular
__global__ void __launch_bounds__(CLS_THREADS) k_pair_stats(DevMesh test, DevMesh trial, int same_mesh,
                                                             unsigned long long *counts)
{
    __shared__ unsigned int h[11];
    if (threadIdx.x < 11) h[threadIdx.x] = 0;
    __syncthreads();
    int j = blockIdx.x;
    float4 jh = trial.chi[j], jl = trial.clo[j];
    for (int i = threadIdx.x; i < test.n; i += CLS_THREADS) {
        int ls, ld;
        float dx, dy, dz;
        int kind = classify_pair(test.chi[i], test.clo[i], jh, jl, i, j, test.center, trial.center, trial.size,
                                 same_mesh, ls, ld, dx, dy, dz);
        int bin = kind == KIND_SELF ? 0 : (kind == KIND_NEAR ? 1 : 2 + 3 * ls + ld);
        atomicAdd(&h[bin], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 11 && h[threadIdx.x]) atomicAdd(&counts[threadIdx.x], (unsigned long long)h[threadIdx.x]);
}

cudaError_t launch_near_count(const DevMesh &test, const DevMesh &trial, int same_mesh, int *counts, cudaStream_t s)
{
    if (trial.n == 0) return cudaSuccess;
    k_near_count<<<trial.n, CLS_THREADS, 0, s>>>(test, trial, same_mesh, counts);
    return cudaGetLastError();
}

cudaError_t launch_scan(const int *counts, int n, int64_t *col_ptr, cudaStream_t s)
{
    k_scan<<<1, 1024, 0, s>>>(counts, n, col_ptr);
    return cudaGetLastError();
}

cudaError_t launch_near_fill(const DevMesh &test, const DevMesh &trial, int same_mesh, const int64_t *col_ptr,
                             int *rows, cudaStream_t s)
{
    if (trial.n == 0) return cudaSuccess;
    k_near_fill<<<trial.n, CLS_THREADS, 0, s>>>(test, trial, same_mesh, col_ptr, rows);
    return cudaGetLastError();
}

cudaError_t launch_pair_stats(const DevMesh &test, const DevMesh &trial, int same_mesh, unsigned long long *counts,
                              cudaStream_t s)
{
    if (trial.n == 0) return cudaSuccess;
    k_pair_stats<<<trial.n, CLS_THREADS, 0, s>>>(test, trial, same_mesh, counts);
    return cudaGetLastError();
}

}  // namespace nihu
