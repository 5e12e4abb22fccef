// Persistent batched GMRES (solve_persistent.cu): many independent dense
// complex64 systems in one launch, one thread-block cluster per system.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace nihu {

constexpr int PERSISTENT_THREADS = 512;

struct PersistentItem {
    const float2 *A;   // n x n, column-major, leading dimension lda
    int64_t lda;
    const double2 *b;  // right-hand side, n
    double2 *x;        // solution, n
    int n;
    int vec;     // 1: n and lda even and A 16-byte aligned (two rows per 16-byte load)
    int stream;  // 1: matrix read with evict-first loads (larger than a share of L2)
    int pad;
};

struct PersistentArgs {
    const PersistentItem *items;
    const int *order;  // processing order of the items (a permutation)
    int count;
    int n_max;
    int restart;
    int max_iters;
    double tol;
    double2 *V;    // clusters * (restart + 1) * n_max basis vectors
    int *counter;  // zero before the launch
    int *iters;    // per item
    double *rel;   // per item: final relative residual estimate
    int *converged;
};

// dynamic shared memory of one CTA, byte offsets
struct PersistentSmem {
    int blocks;  // most 128-row blocks one CTA owns
    size_t vx, wl, red, hp, hc, hk, H, cs, sn, g, y, total;
};

__host__ __device__ inline size_t persistent_align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline PersistentSmem persistent_smem_layout(int n_max, int cluster, int m)
{
    PersistentSmem s;
    size_t o = 0;
    const int pairs = (n_max + 1) / 2;
    const int nb = (pairs + 63) / 64;  // blocks of 64 row pairs
    s.blocks = (nb + cluster - 1) / cluster;
    const size_t rows = 128 * (size_t)s.blocks;
    s.vx = o;   // matvec input, n_max complex64
    o = persistent_align16(o + 8 * (size_t)n_max);
    s.wl = o;   // own rows of the Krylov vector, complex128
    o = persistent_align16(o + 16 * rows);
    s.red = o;  // slice partials of one matvec tile
    o = persistent_align16(o + 16 * (size_t)PERSISTENT_THREADS);
    s.hp = o;   // three rotating buffers of per-block dot-product partials (read by the other CTAs)
    o = persistent_align16(o + 16 * 3 * (size_t)s.blocks * (m + 2));
    s.hc = o;
    o = persistent_align16(o + 16 * (size_t)(m + 2));
    s.hk = o;
    o = persistent_align16(o + 16 * (size_t)(m + 2));
    s.H = o;    // Hessenberg matrix, column-major (m + 1) x m
    o = persistent_align16(o + 16 * (size_t)(m + 1) * m);
    s.cs = o;
    o = persistent_align16(o + 16 * (size_t)m);
    s.sn = o;
    o = persistent_align16(o + 16 * (size_t)m);
    s.g = o;
    o = persistent_align16(o + 16 * (size_t)(m + 1));
    s.y = o;
    o = persistent_align16(o + 16 * (size_t)m);
    s.total = o;
    return s;
}

// clusters that can run at once (at most count) and the dynamic shared memory per CTA
cudaError_t persistent_gmres_plan(int n_max, int restart, int cluster, int count, int *clusters, size_t *smem);
cudaError_t launch_persistent_gmres(const PersistentArgs &a, int cluster, int clusters, size_t smem, cudaStream_t s);

}  // namespace nihu
