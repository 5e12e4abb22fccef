// Persistent restarted GMRES over many independent dense complex systems.
//
// One thread-block cluster solves one system at a time and takes the next
// from a device counter when it is done, so systems of uneven size and
// uneven iteration count share one launch and the GPU never waits for the
// host between Krylov steps.  Within a cluster, CTA c owns a contiguous slice
// of the rows: it computes those rows of every matvec (complex64 matrix,
// FP32 products summed per column slice, slices added in FP64) and of every
// Arnoldi vector (FP64 classical Gram-Schmidt with one reorthogonalisation).
// Dot products and norms are formed per fixed block of 128 rows and the
// block partials are added in block order through distributed shared memory,
// so a system's result does not depend on the cluster size or on the other
// systems of the launch.  Each CTA then repeats the small Hessenberg / Givens
// work on those identical values, and every loop decision is read from rank 0
// after a cluster barrier, so all CTAs of a cluster pass the same sequence of
// barriers.
//
// Every system keeps its whole Krylov state in device memory (basis V, the
// Hessenberg matrix, Givens rotations, g, the iterate x and a status word),
// so a launch may advance each system by at most `quantum` Arnoldi steps and
// a later launch resumes it exactly where it stopped: the result is bitwise
// the same however the steps are split over launches and whatever else
// shares them.  This is what a serving loop needs to admit new systems
// between launches.
//
// The stopping rules are those of the single-system solver (capi.cu,
// gmres_device): a relative residual estimate |g_{k+1}| / |b| below tol, the
// iteration cap, a zero Krylov vector or k = n end the solve; a cycle that
// reaches the restart length restarts from the true residual b - A x.
// Every loop is bounded by the iteration cap or the quantum; the only waits
// are hardware cluster barriers, which all CTAs of the cluster reach.

#include <cooperative_groups.h>

#include "common.cuh"
#include "solve_persistent.h"

namespace cg = cooperative_groups;

namespace nihu {
namespace {

constexpr int PT = PERSISTENT_THREADS;
constexpr int PW = PT / 32;
constexpr int TILE = 64;            // row pairs per matvec tile (two warps)
constexpr int SLICES = PT / TILE;   // column slices per tile
constexpr int MV_UNROLL = 16;       // matrix loads in flight per thread

__device__ __forceinline__ void fma_pair(float4 a, float2 x, float &ar0, float &ai0, float &ar1, float &ai1)
{
    ar0 = fmaf(a.x, x.x, ar0);
    ar0 = fmaf(-a.y, x.y, ar0);
    ai0 = fmaf(a.x, x.y, ai0);
    ai0 = fmaf(a.y, x.x, ai0);
    ar1 = fmaf(a.z, x.x, ar1);
    ar1 = fmaf(-a.w, x.y, ar1);
    ai1 = fmaf(a.z, x.y, ai1);
    ai1 = fmaf(a.w, x.x, ai1);
}

__device__ __forceinline__ void fma_one(float2 a, float2 x, float &ar, float &ai)
{
    ar = fmaf(a.x, x.x, ar);
    ar = fmaf(-a.y, x.y, ar);
    ai = fmaf(a.x, x.y, ai);
    ai = fmaf(a.y, x.x, ai);
}

template <bool STREAM>
__device__ __forceinline__ float4 load_a(const float4 *p)
{
    if (STREAM) return __ldcs(p);
    return __ldg(p);
}

// wl[row - ra] = sum_j A[row, j] vx[j] for the rows of pairs [pa, pb); the
// input vector vx is in shared memory, or (VXG) in a global buffer that the
// cluster rewrites every step (read around L1)
template <bool STREAM, bool VXG>
__device__ void matvec_rows(const float2 *__restrict__ A, int64_t lda, int n, int pa, int pb, int ra, bool vec,
                            const float2 *vx, double2 *wl, float4 *red)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s = warp >> 1, half = warp & 1;
    const int js = (int)((int64_t)s * n / SLICES), je = (int)((int64_t)(s + 1) * n / SLICES);
    for (int tb = pa; tb < pb; tb += TILE) {
        const int p = tb + half * 32 + lane;
        float ar0 = 0.f, ai0 = 0.f, ar1 = 0.f, ai1 = 0.f;
        if (p < pb) {
            const int row = 2 * p;
            if (vec) {
                // n even, lda even, A 16-byte aligned: rows (row, row + 1) of a column are one float4
                const float4 *col = reinterpret_cast<const float4 *>(A + (int64_t)js * lda + row);
                const int64_t stride = lda / 2;
                int j = js;
                for (; j + MV_UNROLL <= je; j += MV_UNROLL) {
                    float4 v[MV_UNROLL];
#pragma unroll
                    for (int u = 0; u < MV_UNROLL; ++u) v[u] = load_a<STREAM>(col + (int64_t)(j - js + u) * stride);
#pragma unroll
                    for (int u = 0; u < MV_UNROLL; ++u)
                        fma_pair(v[u], VXG ? __ldcg(vx + j + u) : vx[j + u], ar0, ai0, ar1, ai1);
                }
                for (; j < je; ++j)
                    fma_pair(load_a<STREAM>(col + (int64_t)(j - js) * stride), VXG ? __ldcg(vx + j) : vx[j], ar0, ai0,
                             ar1, ai1);
            } else {
                for (int j = js; j < je; ++j) {
                    const float2 xv = VXG ? __ldcg(vx + j) : vx[j];
                    fma_one(A[(int64_t)j * lda + row], xv, ar0, ai0);
                    if (row + 1 < n) fma_one(A[(int64_t)j * lda + row + 1], xv, ar1, ai1);
                }
            }
        }
        red[s * TILE + half * 32 + lane] = make_float4(ar0, ai0, ar1, ai1);
        __syncthreads();
        if (tid < TILE && tb + tid < pb) {
            double r0 = 0.0, i0 = 0.0, r1 = 0.0, i1 = 0.0;
#pragma unroll
            for (int q = 0; q < SLICES; ++q) {
                const float4 t = red[q * TILE + tid];
                r0 += t.x;
                i0 += t.y;
                r1 += t.z;
                i1 += t.w;
            }
            const int row = 2 * (tb + tid);
            wl[row - ra] = make_double2(r0, i0);
            if (row + 1 < n) wl[row + 1 - ra] = make_double2(r1, i1);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconjmul(double2 a, double2 b)  // conj(a) b
{
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double zabs2(double2 a) { return a.x * a.x + a.y * a.y; }

__global__ void __launch_bounds__(PT, 1) k_persistent_gmres(PersistentArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const int cid = blockIdx.x / C;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m = a.restart;
    const bool vxg = a.vxg != nullptr;
    const PersistentSmem L = persistent_smem_layout(a.n_max, C, m, !vxg);
    extern __shared__ __align__(16) unsigned char sm[];
    float2 *vx = vxg ? a.vxg + (int64_t)cid * a.n_max : reinterpret_cast<float2 *>(sm + L.vx);
    double2 *wl = reinterpret_cast<double2 *>(sm + L.wl);
    float4 *red = reinterpret_cast<float4 *>(sm + L.red);
    double2 *hp = reinterpret_cast<double2 *>(sm + L.hp);
    double2 *hc = reinterpret_cast<double2 *>(sm + L.hc);
    double2 *hk = reinterpret_cast<double2 *>(sm + L.hk);
    double2 *H = reinterpret_cast<double2 *>(sm + L.H);
    double2 *cs = reinterpret_cast<double2 *>(sm + L.cs);
    double2 *sn = reinterpret_cast<double2 *>(sm + L.sn);
    double2 *g = reinterpret_cast<double2 *>(sm + L.g);
    double2 *y = reinterpret_cast<double2 *>(sm + L.y);
    __shared__ int ctl[4];
    __shared__ double2 scal[1];
    const int hstride = L.blocks * (m + 2);  // one partial buffer: [local block][entry]
    const int budget = a.quantum > 0 ? a.quantum : 0x7fffffff;
    int buf = 0, slot = 1;
    int nb = 0;  // row blocks of the current system

    // out[t] = sum over all row blocks, in block order, of entry t of the current partial buffer
    auto cluster_sum = [&](int cnt, double2 *out) {
        const double2 *mine = hp + buf * hstride;
        cl.sync();
        for (int t = tid; t < cnt; t += PT) {
            double sr = 0.0, si = 0.0;
            int c = 0, c0 = 0, c1 = (int)((int64_t)nb / C);
            const double2 *peer = cl.map_shared_rank(mine, 0);
            for (int b = 0; b < nb; ++b) {
                while (b >= c1) {
                    ++c;
                    c0 = c1;
                    c1 = (int)((int64_t)(c + 1) * nb / C);
                    peer = cl.map_shared_rank(mine, c);
                }
                const double2 v = peer[(b - c0) * (m + 2) + t];
                sr += v.x;
                si += v.y;
            }
            out[t] = make_double2(sr, si);
        }
        buf = buf == 2 ? 0 : buf + 1;
        __syncthreads();
    };
    // rank 0's value of `local` (thread 0), after a cluster barrier
    auto decide = [&](int local) -> int {
        if (rank == 0 && tid == 0) ctl[slot] = local;
        cl.sync();
        const int d = *cl.map_shared_rank(&ctl[slot], 0);
        slot = slot == 3 ? 1 : slot + 1;
        return d;
    };

    // a programmatic dependent launch of this stream may start now, on the
    // SMs this grid leaves free (no effect on a plain launch)
    asm volatile("griddepcontrol.launch_dependents;");

    for (;;) {
        if (rank == 0 && tid == 0) ctl[0] = atomicAdd(a.counter, 1);
        cl.sync();
        const int item = *cl.map_shared_rank(&ctl[0], 0);
        cl.sync();
        if (item >= a.count) break;
        const int f = a.order[item];
        const PersistentItem it = a.items[f];
        const int n = it.n;
        const int P = (n + 1) / 2;
        nb = (P + TILE - 1) / TILE;
        const int b0 = (int)((int64_t)rank * nb / C), b1 = (int)((int64_t)(rank + 1) * nb / C), nlb = b1 - b0;
        const int pa = min(P, b0 * TILE), pb = min(P, b1 * TILE);
        const int ra = min(n, 2 * pa), rb = min(n, 2 * pb);
        double2 *V = it.V;  // basis vector v at V + v * n
        const bool vec = it.vec != 0;

        // |w|^2 of the cluster's rows: per-block partials, then the block-ordered sum
        auto cluster_norm2 = [&]() -> double {
            double2 *mine = hp + buf * hstride;
            for (int lb = warp; lb < nlb; lb += PW) {
                double s = 0.0;
                const int i0 = ra + lb * 2 * TILE, i1 = min(rb, i0 + 2 * TILE);
                for (int i = i0 + lane; i < i1; i += 32) s += zabs2(wl[i - ra]);
                s = warp_sum(s);
                if (lane == 0) mine[lb * (m + 2)] = make_double2(s, 0.0);
            }
            cluster_sum(1, scal);
            return scal[0].x;
        };
        // the matvec input: src (complete across the cluster) as complex64
        auto load_vx = [&](const double2 *src) {
            if (vxg) {
                for (int i = ra + tid; i < rb; i += PT) {
                    const double2 v = __ldcg(src + i);
                    vx[i] = make_float2((float)v.x, (float)v.y);
                }
                cl.sync();
            } else {
                for (int j = tid; j < n; j += PT) {
                    const double2 v = __ldcg(src + j);
                    vx[j] = make_float2((float)v.x, (float)v.y);
                }
                __syncthreads();
            }
        };
        auto matvec = [&]() {
            if (it.stream) {
                if (vxg) matvec_rows<true, true>(it.A, it.lda, n, pa, pb, ra, vec, vx, wl, red);
                else matvec_rows<true, false>(it.A, it.lda, n, pa, pb, ra, vec, vx, wl, red);
            } else {
                if (vxg) matvec_rows<false, true>(it.A, it.lda, n, pa, pb, ra, vec, vx, wl, red);
                else matvec_rows<false, false>(it.A, it.lda, n, pa, pb, ra, vec, vx, wl, red);
            }
        };
        // a new cycle from the residual in wl with norm beta: V_0 and g = beta e_1
        auto begin_cycle = [&](double beta) {
            const double ib = 1.0 / beta;
            for (int i = ra + tid; i < rb; i += PT) {
                const double2 w = wl[i - ra];
                V[i] = make_double2(w.x * ib, w.y * ib);
            }
            if (tid == 0) {
                g[0] = make_double2(beta, 0.0);
                for (int i = 1; i <= m; ++i) g[i] = make_double2(0.0, 0.0);
            }
        };
        // wl = b - A x on the own rows
        auto residual = [&]() {
            cl.sync();  // x complete across the cluster
            load_vx(it.x);
            matvec();
            for (int i = ra + tid; i < rb; i += PT) wl[i - ra] = zsub(it.b[i], wl[i - ra]);
            __syncthreads();
        };
        // y = H^{-1} g over kdone steps (upper triangular after the rotations), x += V y on the own rows
        auto update_x = [&](int kdone) {
            if (tid == 0) {
                for (int i = kdone - 1; i >= 0; --i) {
                    double2 s = g[i];
                    for (int j = i + 1; j < kdone; ++j) s = zsub(s, zmul(H[(int64_t)j * (m + 1) + i], y[j]));
                    const double2 dg = H[(int64_t)i * (m + 1) + i];
                    const double q = zabs2(dg);
                    y[i] = make_double2((s.x * dg.x + s.y * dg.y) / q, (s.y * dg.x - s.x * dg.y) / q);
                }
            }
            __syncthreads();
            for (int i = ra + tid; i < rb; i += PT) {
                double2 acc = it.x[i];
                for (int v = 0; v < kdone; ++v) acc = zadd(acc, zmul(__ldcg(V + (int64_t)v * n + i), y[v]));
                it.x[i] = acc;
            }
        };

        // the state left by earlier launches (the same for every CTA of the cluster)
        const PersistentState st = *it.st;
        int status = st.status, k = st.k, iters = st.iters;
        double r0 = st.r0;
        double rel = st.rel;  // meaningful in thread 0
        int steps = 0;
        int finished = 0;  // 1: done in this launch; 2: done with a zero residual
        if (status == PG_FRESH) {
            // x = 0, r = b
            for (int i = ra + tid; i < rb; i += PT) {
                it.x[i] = make_double2(0.0, 0.0);
                wl[i - ra] = it.b[i];
            }
            __syncthreads();
            r0 = sqrt(cluster_norm2());
            if (decide(!(r0 == 0.0)) == 0) {
                finished = 2;
            } else {
                begin_cycle(r0);
                k = 0;
            }
        } else if (status == PG_RESTART) {
            residual();
            const double beta = sqrt(cluster_norm2());
            if (decide(!(beta == 0.0)) == 0) {
                finished = 2;
            } else {
                begin_cycle(beta);
                k = 0;
            }
        } else if (status == PG_IN_CYCLE) {
            const double2 *S = it.S;
            const int hs = (m + 1) * m;
            for (int t = tid; t < hs; t += PT) H[t] = S[t];
            for (int t = tid; t < m; t += PT) {
                cs[t] = S[hs + t];
                sn[t] = S[hs + m + t];
            }
            for (int t = tid; t <= m; t += PT) g[t] = S[hs + 2 * m + t];
            __syncthreads();
        } else {
            finished = 3;  // already done: left as it is
        }

        while (finished == 0) {
            cl.sync();  // V_k complete across the cluster
            load_vx(V + (int64_t)k * n);
            ++iters;
            ++steps;
            matvec();
            if (tid <= k) hk[tid] = make_double2(0.0, 0.0);
            for (int pass = 0; pass < 2; ++pass) {  // CGS2
                double2 *mine = hp + buf * hstride;
                for (int task = warp; task < nlb * (k + 1); task += PW) {
                    const int lb = task / (k + 1), v = task - lb * (k + 1);
                    const double2 *Vv = V + (int64_t)v * n;
                    const int i0 = ra + lb * 2 * TILE, i1 = min(rb, i0 + 2 * TILE);
                    double sr = 0.0, si = 0.0;
                    for (int i = i0 + lane; i < i1; i += 32) {
                        const double2 t = zconjmul(__ldcg(Vv + i), wl[i - ra]);
                        sr += t.x;
                        si += t.y;
                    }
                    sr = warp_sum(sr);
                    si = warp_sum(si);
                    if (lane == 0) mine[lb * (m + 2) + v] = make_double2(sr, si);
                }
                cluster_sum(k + 1, hc);
                if (tid <= k) hk[tid] = zadd(hk[tid], hc[tid]);
                for (int i = ra + tid; i < rb; i += PT) {
                    double2 acc = wl[i - ra];
                    for (int v = 0; v <= k; ++v) acc = zsub(acc, zmul(__ldcg(V + (int64_t)v * n + i), hc[v]));
                    wl[i - ra] = acc;
                }
                __syncthreads();
            }
            const double hn = sqrt(cluster_norm2());
            if (hn > 0.0) {
                const double s = 1.0 / hn;
                double2 *Vn = V + (int64_t)(k + 1) * n;
                for (int i = ra + tid; i < rb; i += PT) {
                    const double2 w = wl[i - ra];
                    Vn[i] = make_double2(w.x * s, w.y * s);
                }
            }
            int local = 0;
            if (tid == 0) {
                // previous rotations, then a new one zeroing the subdiagonal
                double2 *Hk = H + (int64_t)k * (m + 1);
                for (int i = 0; i <= k; ++i) Hk[i] = hk[i];
                Hk[k + 1] = make_double2(hn, 0.0);
                for (int i = 0; i < k; ++i) {
                    const double2 a0 = Hk[i], a1 = Hk[i + 1];
                    Hk[i] = zadd(zconjmul(cs[i], a0), zconjmul(sn[i], a1));
                    Hk[i + 1] = zsub(zmul(cs[i], a1), zmul(sn[i], a0));
                }
                const double2 a0 = Hk[k], a1 = Hk[k + 1];
                const double den = sqrt(zabs2(a0) + zabs2(a1));
                const double2 c = den == 0.0 ? make_double2(1.0, 0.0) : make_double2(a0.x / den, a0.y / den);
                const double2 sv = den == 0.0 ? make_double2(0.0, 0.0) : make_double2(a1.x / den, a1.y / den);
                cs[k] = c;
                sn[k] = sv;
                Hk[k] = zadd(zconjmul(c, a0), zconjmul(sv, a1));
                Hk[k + 1] = make_double2(0.0, 0.0);
                const double2 g0 = g[k], g1 = g[k + 1];
                g[k] = zadd(zconjmul(c, g0), zconjmul(sv, g1));
                g[k + 1] = zsub(zmul(c, g1), zmul(sv, g0));
                rel = sqrt(zabs2(g[k + 1])) / r0;
                const bool stop = rel < a.tol || iters >= a.max_iters || hn == 0.0 || k + 1 == n;
                // 2: stop, 1: end of the cycle, 3: quantum used up inside the cycle, 0: next step
                local = stop ? 2 : (k + 1 == m ? 1 : (steps >= budget ? 3 : 0));
            }
            const int d = decide(local);  // also completes V_{k+1} across the cluster
            if (d == 0) {
                ++k;
                continue;
            }
            if (d == 3) {
                // pause inside the cycle: the small state goes to memory for the next launch
                if (rank == 0) {
                    double2 *S = it.S;
                    const int hs = (m + 1) * m;
                    for (int t = tid; t < (k + 1) * (m + 1); t += PT) S[t] = H[t];
                    for (int t = tid; t <= k; t += PT) {
                        S[hs + t] = cs[t];
                        S[hs + m + t] = sn[t];
                    }
                    for (int t = tid; t <= m; t += PT) S[hs + 2 * m + t] = g[t];
                }
                status = PG_IN_CYCLE;
                ++k;
                break;
            }
            update_x(k + 1);
            if (d == 2) {
                finished = 1;
                break;
            }
            // end of a cycle: restart from the true residual, or leave that to the next launch
            k = 0;
            if (steps >= budget) {
                status = PG_RESTART;
                break;
            }
            residual();
            const double beta = sqrt(cluster_norm2());
            if (decide(!(beta == 0.0)) == 0) {
                finished = 2;
                break;
            }
            begin_cycle(beta);
        }
        if (rank == 0 && tid == 0 && finished != 3) {
            PersistentState o;
            o.status = finished ? PG_DONE : status;
            o.k = k;
            o.iters = iters;
            o.r0 = r0;
            o.rel = finished == 2 ? 0.0 : rel;
            o.converged = finished == 2 ? 1 : (finished == 1 ? (rel < a.tol) : 0);
            *it.st = o;
        }
    }
    // dependent launch: the primary launch runs to completion by itself (it
    // never waits on this grid), so this wait ends when it does
    if (a.wait_primary) asm volatile("griddepcontrol.wait;" ::: "memory");
}

}  // namespace

cudaError_t persistent_gmres_plan(int n_max, int restart, int cluster, int vx_smem, int count, int *clusters,
                                  size_t *smem)
{
    const PersistentSmem L = persistent_smem_layout(n_max, cluster, restart, vx_smem);
    cudaError_t e = cudaFuncSetAttribute(k_persistent_gmres, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
    if (e != cudaSuccess) return e;
    if (cluster > 8) {
        e = cudaFuncSetAttribute(k_persistent_gmres, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(PT);
    cfg.dynamicSmemBytes = L.total;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int active = 0;
    e = cudaOccupancyMaxActiveClusters(&active, k_persistent_gmres, &cfg);
    if (e != cudaSuccess) return e;
    if (active < 1) return cudaErrorInvalidConfiguration;
    *clusters = count < active ? count : active;
    *smem = L.total;
    return cudaSuccess;
}

cudaError_t launch_persistent_gmres(const PersistentArgs &a, int cluster, int clusters, size_t smem, cudaStream_t s,
                                    bool dependent)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = dim3(clusters * cluster);
    cfg.blockDim = dim3(PT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = dependent ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, k_persistent_gmres, a);
}

cudaError_t persistent_gmres_smem_limit(size_t smem)
{
    return cudaFuncSetAttribute(k_persistent_gmres, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace nihu
