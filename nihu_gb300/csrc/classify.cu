// Nearly singular pair lists (column-sorted) and pair statistics.
#include "classify.cuh"
#include "kernels.h"

#include <algorithm>

namespace nihu {

constexpr int CLS_THREADS = 256;

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

// ------------------------------------------------------------ pair discovery
//
// A pair is nearly singular when |c_i - c_j| < 1.5 D_j (classify_pair), so
// the candidates of trial column j lie within r_j = 1.5 D_j of its centre.
// The test centres are binned into a uniform grid of cell size h = 1.5 x the
// mean trial size, the cells hashed into T = 2^b buckets and the elements
// counting-sorted by bucket; column j then visits the cells its box
// [c_j - r_j, c_j + r_j] covers (27 for a column of mean size) and classifies
// only the elements binned there, instead of all n.  Every candidate goes
// through classify_pair, so the list is the brute-force list: a pair with
// d < 1.5 D_j lies in the box because cell coordinates are a monotone
// function of the centre (floor of x / h, clamped), and r_j carries a
// relative margin far above the FP64 rounding of d.  A column whose box
// covers more cells than a scan of all n rows costs (an element much larger
// than the mean) scans all rows.  Rows come out in increasing order per
// column: each column is rank-sorted by its warp after the fill.

constexpr int GRID_THREADS = 256;
constexpr int GRID_WARPS = GRID_THREADS / 32;

struct GridView {
    const double *inv_h;         // 1 / h, written by k_grid_setup
    int *bucket_count;           // [T]
    int64_t *bucket_start;       // [T + 1]
    int4 *cells;                 // [n_test] (cx, cy, cz, element)
    int4 *sorted;                // [n_test] grouped by bucket
    unsigned mask;               // T - 1
};

__device__ __forceinline__ int cell_coord(double x, double inv_h)
{
    double c = floor(x * inv_h);
    c = fmin(fmax(c, -1073741824.0), 1073741824.0);
    return (int)c;
}

__device__ __forceinline__ unsigned cell_bucket(int x, int y, int z, unsigned mask)
{
    unsigned h = (unsigned)x * 0x9E3779B1u + (unsigned)y * 0x85EBCA77u + (unsigned)z * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 13;
    return h & mask;
}

// one block: h from the mean trial size, summed in a fixed order
__global__ void __launch_bounds__(1024) k_grid_setup(const double *__restrict__ trial_size, int n, double *inv_h)
{
    __shared__ double part[32];
    double s = 0.0;
    for (int j = threadIdx.x; j < n; j += 1024) s += trial_size[j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 32; ++w) t += part[w];
        const double h = 1.5 * t / n;
        *inv_h = h > 0.0 ? 1.0 / h : 0.0;
    }
}

__global__ void __launch_bounds__(GRID_THREADS) k_grid_bin(const double *__restrict__ center, int n, GridView g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ih = *g.inv_h;
    int4 c = make_int4(cell_coord(center[3 * (int64_t)i], ih), cell_coord(center[3 * (int64_t)i + 1], ih),
                       cell_coord(center[3 * (int64_t)i + 2], ih), i);
    g.cells[i] = c;
    atomicAdd(&g.bucket_count[cell_bucket(c.x, c.y, c.z, g.mask)], 1);
}

// bucket_count counts down to 0 while its elements are placed
__global__ void __launch_bounds__(GRID_THREADS) k_grid_place(int n, GridView g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int4 c = g.cells[i];
    unsigned b = cell_bucket(c.x, c.y, c.z, g.mask);
    g.sorted[g.bucket_start[b] + atomicSub(&g.bucket_count[b], 1) - 1] = c;
}

// one warp per trial column.  COUNT: counts[j] = its nearly singular rows.
// FILL: writes them to tmp[col_ptr[j] ..] in visiting order, then in
// increasing order to rows[col_ptr[j] ..].
template <bool FILL>
__global__ void __launch_bounds__(GRID_THREADS) k_near_grid(DevMesh test, DevMesh trial, int same_mesh, GridView g,
                                                            int *counts, const int64_t *col_ptr, int *tmp, int *rows)
{
    const int j = blockIdx.x * GRID_WARPS + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (j >= trial.n) return;  // whole warp
    const unsigned lt = (1u << lane) - 1u;
    const float4 jh = trial.chi[j], jl = trial.clo[j];
    const double ih = *g.inv_h;
    const double cx = trial.center[3 * (int64_t)j], cy = trial.center[3 * (int64_t)j + 1],
                 cz = trial.center[3 * (int64_t)j + 2];
    const double r = 1.5 * trial.size[j] * (1.0 + 1e-6) + 1e-9 * fmax(fabs(cx), fmax(fabs(cy), fabs(cz)));
    const int x0 = cell_coord(cx - r, ih), x1 = cell_coord(cx + r, ih);
    const int y0 = cell_coord(cy - r, ih), y1 = cell_coord(cy + r, ih);
    const int z0 = cell_coord(cz - r, ih), z1 = cell_coord(cz + r, ih);
    const double vol = (double)(x1 - x0 + 1) * (double)(y1 - y0 + 1) * (double)(z1 - z0 + 1);
    const int64_t base = FILL ? col_ptr[j] : 0;
    int found = 0;
    // warp-collective: classify (i, j) where ok, record the nearly singular ones
    auto visit = [&](int i, bool ok) {
        int pred = 0;
        if (ok) {
            int ls, ld;
            float dx, dy, dz;
            pred = classify_pair(test.chi[i], test.clo[i], jh, jl, i, j, test.center, trial.center, trial.size,
                                 same_mesh, ls, ld, dx, dy, dz) == KIND_NEAR;
        }
        const unsigned m = __ballot_sync(0xffffffffu, pred);
        if (FILL && pred) tmp[base + found + __popc(m & lt)] = i;
        found += __popc(m);
    };
    if (ih == 0.0 || vol > 27.0 + test.n / 32) {
        for (int i0 = 0; i0 < test.n; i0 += 32) visit(i0 + lane, i0 + lane < test.n);
    } else {
        for (int z = z0; z <= z1; ++z)
            for (int y = y0; y <= y1; ++y)
                for (int x = x0; x <= x1; ++x) {
                    const unsigned b = cell_bucket(x, y, z, g.mask);
                    const int64_t s = g.bucket_start[b], e = g.bucket_start[b + 1];
                    for (int64_t k0 = s; k0 < e; k0 += 32) {
                        bool ok = false;
                        int i = 0;
                        if (k0 + lane < e) {
                            const int4 c = g.sorted[k0 + lane];
                            ok = c.x == x && c.y == y && c.z == z;  // not another cell of the same bucket
                            i = c.w;
                        }
                        visit(i, ok);
                    }
                }
    }
    if (!FILL) {
        if (lane == 0) counts[j] = found;
        return;
    }
    __syncwarp();  // the warp's tmp writes are visible to all its lanes
    for (int a = lane; a < found; a += 32) {
        const int v = tmp[base + a];
        int rank = 0;
        for (int b = 0; b < found; ++b) rank += tmp[base + b] < v;
        rows[base + rank] = v;
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

size_t near_grid_buckets(int n_test)
{
    size_t T = 256;
    while (T < (size_t)n_test) T <<= 1;
    return T;
}

static size_t round256(size_t b) { return (b + 255) / 256 * 256; }

// scratch layout: inv_h | bucket_count[T] | bucket_start[T + 1] | cells[n] | sorted[n]
size_t near_grid_scratch_bytes(int n_test)
{
    const size_t T = near_grid_buckets(n_test);
    return 256 + round256(4 * T) + round256(8 * (T + 1)) + 2 * 16 * (size_t)std::max(n_test, 1);
}

static GridView grid_view(void *scratch, int n_test)
{
    const size_t T = near_grid_buckets(n_test);
    char *p = (char *)scratch;
    GridView g;
    g.inv_h = (const double *)p;
    g.bucket_count = (int *)(p + 256);
    size_t off = 256 + round256(4 * T);
    g.bucket_start = (int64_t *)(p + off);
    off += round256(8 * (T + 1));
    g.cells = (int4 *)(p + off);
    g.sorted = g.cells + std::max(n_test, 1);
    g.mask = (unsigned)(T - 1);
    return g;
}

cudaError_t launch_near_grid_count(const DevMesh &test, const DevMesh &trial, int same_mesh, void *scratch,
                                   int *counts, cudaStream_t s)
{
    if (trial.n == 0) return cudaSuccess;
    GridView g = grid_view(scratch, test.n);
    cudaError_t e = cudaMemsetAsync(g.bucket_count, 0, sizeof(int) * (g.mask + 1), s);
    if (e != cudaSuccess) return e;
    k_grid_setup<<<1, 1024, 0, s>>>(trial.size, trial.n, (double *)g.inv_h);
    if (test.n > 0) {
        const int blocks = (test.n + GRID_THREADS - 1) / GRID_THREADS;
        k_grid_bin<<<blocks, GRID_THREADS, 0, s>>>(test.center, test.n, g);
        k_scan<<<1, 1024, 0, s>>>(g.bucket_count, (int)(g.mask + 1), g.bucket_start);
        k_grid_place<<<blocks, GRID_THREADS, 0, s>>>(test.n, g);
    } else {
        e = cudaMemsetAsync(g.bucket_start, 0, sizeof(int64_t) * (g.mask + 2), s);
        if (e != cudaSuccess) return e;
    }
    k_near_grid<false><<<(trial.n + GRID_WARPS - 1) / GRID_WARPS, GRID_THREADS, 0, s>>>(test, trial, same_mesh, g,
                                                                                       counts, nullptr, nullptr,
                                                                                       nullptr);
    return cudaGetLastError();
}

cudaError_t launch_scan(const int *counts, int n, int64_t *col_ptr, cudaStream_t s)
{
    k_scan<<<1, 1024, 0, s>>>(counts, n, col_ptr);
    return cudaGetLastError();
}

cudaError_t launch_near_grid_fill(const DevMesh &test, const DevMesh &trial, int same_mesh, void *scratch,
                                  const int64_t *col_ptr, int *tmp, int *rows, cudaStream_t s)
{
    if (trial.n == 0) return cudaSuccess;
    GridView g = grid_view(scratch, test.n);
    k_near_grid<true><<<(trial.n + GRID_WARPS - 1) / GRID_WARPS, GRID_THREADS, 0, s>>>(test, trial, same_mesh, g,
                                                                                      nullptr, col_ptr, tmp, rows);
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
