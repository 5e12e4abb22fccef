// Persistent batched GMRES (solve_persistent.cu): many independent dense
// complex64 systems in one launch, one thread-block cluster per system at a
// time, with the whole Krylov state of every system in device memory so that
// a launch may advance each system by a bounded number of steps and a later
// launch resumes it exactly.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace nihu {

constexpr int PERSISTENT_THREADS = 512;

// progress of one system between launches
enum PersistentStatus { PG_FRESH = 0, PG_IN_CYCLE = 1, PG_RESTART = 2, PG_DONE = 3 };

struct PersistentState {
    int status;     // PersistentStatus
    int k;          // PG_IN_CYCLE: Arnoldi steps done in the current cycle
    int iters;      // Arnoldi steps done in total
    int converged;  // PG_DONE: relative residual estimate below tol
    double r0;      // |b|, the reference of the relative residual
    double rel;     // latest relative residual estimate
};

struct PersistentItem {
    const float2 *A;   // n x n, column-major, leading dimension lda
    int64_t lda;
    const double2 *b;  // right-hand side, n
    double2 *x;        // solution, n
    double2 *V;        // Arnoldi basis, (restart + 1) vectors of n
    double2 *S;        // small Krylov state, persistent_small_state(restart) complex128
    PersistentState *st;
    int n;
    int vec;     // 1: n and lda even and A 16-byte aligned (two rows per 16-byte load)
    int stream;  // 1: matrix read with evict-first loads (larger than a share of L2)
    int pad;
};

// H ((m + 1) x m, column-major) | cs (m) | sn (m) | g (m + 1)
__host__ __device__ inline size_t persistent_small_state(int m) { return (size_t)(m + 1) * m + 3 * (size_t)m + 1; }

struct PersistentArgs {
    const PersistentItem *items;
    const int *order;  // processing order of the items (a permutation)
    int count;
    int n_max;
    int restart;
    int max_iters;
    int quantum;   // most Arnoldi steps per system in this launch (<= 0: no bound)
    double tol;
    int *counter;  // zero before the launch
    float2 *vxg;   // NULL: matvec input in shared memory; else clusters * n_max complex64
    // 1: launched as the programmatic dependent of the previous persistent
    // launch of its stream (launch_persistent_gmres, dependent = true); the
    // grid's CTAs end by waiting for that launch to complete, so that work
    // ordered after this launch also follows the other
    int wait_primary = 0;
};

// dynamic shared memory of one CTA, byte offsets
struct PersistentSmem {
    int blocks;  // most 128-row blocks one CTA owns
    size_t vx, wl, red, hp, hc, hk, H, cs, sn, g, y, total;
};

__host__ __device__ inline size_t persistent_align16(size_t x) { return (x + 15) & ~(size_t)15; }

// vx_smem = 0: the matvec input lives in global memory (vxg) instead
__host__ __device__ inline PersistentSmem persistent_smem_layout(int n_max, int cluster, int m, int vx_smem)
{
    PersistentSmem s;
    size_t o = 0;
    const int pairs = (n_max + 1) / 2;
    const int nb = (pairs + 63) / 64;  // blocks of 64 row pairs
    s.blocks = (nb + cluster - 1) / cluster;
    const size_t rows = 128 * (size_t)s.blocks;
    s.vx = o;   // matvec input, n_max complex64
    o = persistent_align16(o + (vx_smem ? 8 * (size_t)n_max : 0));
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
cudaError_t persistent_gmres_plan(int n_max, int restart, int cluster, int vx_smem, int count, int *clusters,
                                  size_t *smem);
// dependent: programmatic dependent launch, started as soon as every CTA of
// the previous persistent launch of the stream is running (on the SMs that
// one leaves free); a.wait_primary must then be 1
cudaError_t launch_persistent_gmres(const PersistentArgs &a, int cluster, int clusters, size_t smem, cudaStream_t s,
                                    bool dependent = false);
// raise the kernel's dynamic shared memory limit to smem bytes (several
// launch shapes in one stream: the largest of them)
cudaError_t persistent_gmres_smem_limit(size_t smem);

}  // namespace nihu
