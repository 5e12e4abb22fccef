// Multi-right-hand-side product Y = alpha A X + beta Y on the 5th-generation
// tensor cores (tcgen05), split BF16 with FP32 accumulation in tensor memory.
//
// A is complex64 (m x n, column-major, lda): viewed as floats it is a real
// 2m x n matrix (even rows Re A, odd rows Im A).  The right-hand sides become
// planes P = [Re X | Im X] (n x 2 nrhs), so ONE real product Z = A_r P reads A
// once and yields every real product of the complex one:
//   Re Y = Z[2i, r] - Z[2i+1, nrhs + r],  Im Y = Z[2i, nrhs + r] + Z[2i+1, r].
//
// Split BF16: an FP32 value x is written as x = x0 + x1 (+ x2) with each part
// the BF16 rounding of what the previous parts leave.  Two parts hold 16 bits
// of the significand, three hold all 24.  The product keeps the part products
// whose order is above the target precision:
//   BF16x3: A0 P0 + A0 P1 + A1 P0           (about 2^-16 per product)
//   BF16x6: those + A0 P2 + A1 P1 + A2 P0   (FP32-accurate)
// all accumulated in FP32 in tensor memory.
//
// Per CTA (one per SM, persistent over units): a unit is 128 rows of A_r (one
// TMEM lane each) times a contiguous range of K (split-K, so that the units
// balance over the SMs); its FP32 partial goes to a workspace and a second
// kernel adds the partials of each row in a fixed order in FP64, forms the
// complex combination and applies alpha and beta.
//
//   warp 8      TMA producer of A: FP32 tiles of A_r (128 rows x 64 K, 32 KB)
//               into a 3-stage ring, with an L2 prefetch of the tile eight
//               tiles ahead (the ring holds too few bytes to cover the DRAM
//               latency at full bandwidth; the prefetch covers it in L2)
//   warp 10     TMA producer of P: the BF16 parts of 64 K of P (K-major,
//               128-byte swizzle) into a 4-stage (BF16x6: 2-stage) ring
//   warps 4-7   converters: thread t reads row t of the FP32 tile from shared
//               memory, splits it into BF16 parts and stores them into tensor
//               memory (row t = lane t), where the MMA reads A from
//   warp 9      MMA issuer (one thread) and TMEM allocator: per 16 K, one
//               tcgen05.mma (M 128, N = 2 nrhs padded to 16, K 16) per part
//               product into a double-buffered FP32 accumulator
//   warps 0-3   epilogue: adds each accumulator chain (1024 K) into a running
//               FP32 sum per row in registers, then writes the unit's partial
//               to the workspace
//
// Every wait is on an mbarrier with a time limit; a wait that runs out sets
// the error word, tells the other roles to stop, and the CTA still waits for
// its own copies and MMAs in flight and frees its tensor memory before it
// returns.  The host reads the error word after the product.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "linalg.h"

namespace nihu {
namespace {

constexpr int TC_BM = 128;                   // rows of A_r per unit (TMEM lanes)
constexpr int TC_BK = 64;                    // K per stage
constexpr int TC_MAXN = 128;                 // 2 nrhs padded to 16, per pass
constexpr int TC_THREADS = 352;              // 11 warps, roles above
constexpr int A_STAGE_BYTES = TC_BK * TC_BM * 4;       // 32 KB FP32 tile
constexpr int X_PART_BYTES = TC_MAXN * TC_BK * 2;      // 16 KB BF16 part tile
constexpr int TMEM_COLS = 512;
constexpr int ACC_COLS = 128;                // one accumulator (N <= 128 FP32 columns)
constexpr int A_TMEM0 = 2 * ACC_COLS;        // A parts after the two accumulators
constexpr int A_PART_COLS = TC_BK / 2;       // 64 BF16 per row = 32 columns
constexpr int PREFETCH_TILES = 8;            // L2 prefetch distance of the A tiles
constexpr long long WAIT_LIMIT = 4000000000LL;  // clock64 cycles (about 2 s)
// K tiles per accumulator chain: the tensor cores round the FP32 accumulator
// once per MMA, so a unit's K range is summed as chains of at most 1024 K
// drained into an FP32 running sum by the epilogue (a few more roundings
// instead of thousands in one chain)
constexpr int CHAIN_TILES = 16;

// the error word's codes
constexpr int ERR_WAIT_TMA = 1, ERR_WAIT_CONVERT = 2, ERR_WAIT_MMA = 3, ERR_WAIT_EPILOGUE = 4;

struct TcArgs {
    int rb_count;     // units of 128 rows of A_r
    int kt_count;     // K tiles of 64
    int splits;       // split-K factor S (<= kt_count)
    int units;        // rb_count * splits
    int npad;         // 2 nrhs padded to 16 (<= 128)
    int64_t ws_rows;  // rb_count * 128
    float *ws;        // [S][npad][ws_rows]
    int *err;         // error word (0 = ok)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the completion of the phase with the given parity.  Returns false
// when another role has stopped the CTA or after WAIT_LIMIT cycles (then it
// stops the CTA and records `code`).
__device__ __noinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *stop, int *err, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*stop) return false;
        if (clock64() - t0 > WAIT_LIMIT) {
            *stop = 1;
            atomicCAS(err, 0, code);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], "
        "[%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// bring a tile into L2 ahead of its load (no shared memory, no completion)
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap *map, int x, int y)
{
    asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[tmem] * B[smem]^T, kind::f16 (BF16 in, FP32 accumulate)
__device__ __forceinline__ void mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrives on `bar` once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
        "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}

__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// 16 FP32 columns of this warp's 32 lanes; the wait is tied to the registers
// so that no use of them moves above it
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 B apart (rows of 64 BF16 = 128 B)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;             // leading-dimension offset (unused: K fits the swizzle row)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride between 8-row groups
    d |= (uint64_t)1 << 46;             // descriptor version of tcgen05
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// x = x0 + x1 + x2 in BF16 (each part the rounding of what the others leave)
__device__ __forceinline__ void split3(float x, float &r1, float &r2, __nv_bfloat16 &p0, __nv_bfloat16 &p1,
                                       __nv_bfloat16 &p2)
{
    p0 = __float2bfloat16_rn(x);
    r1 = x - __bfloat162float(p0);
    p1 = __float2bfloat16_rn(r1);
    r2 = r1 - __bfloat162float(p1);
    p2 = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

template <int SA>
struct Products;
template <>
struct Products<2> {  // BF16x3
    static constexpr int N = 3;
    __device__ static constexpr int a(int p) { return p == 2 ? 1 : 0; }
    __device__ static constexpr int x(int p) { return p == 1 ? 1 : 0; }
};
template <>
struct Products<3> {  // BF16x6
    static constexpr int N = 6;
    __device__ static constexpr int a(int p) { return p == 2 || p == 4 ? 1 : (p == 5 ? 2 : 0); }
    __device__ static constexpr int x(int p) { return p == 1 || p == 4 ? 1 : (p == 3 ? 2 : 0); }
};

template <int SA>
__host__ __device__ constexpr int a_stages() { return 3; }
template <int SA>
__host__ __device__ constexpr int x_stages() { return SA == 2 ? 4 : 2; }
// A-part buffers in tensor memory (SA x 32 columns each, after the two
// accumulators): 4 for BF16x3 (the converters may run three tiles ahead of
// the MMAs), 2 for BF16x6 (what the 512 columns leave)
template <int SA>
__host__ __device__ constexpr int t_bufs() { return SA == 2 ? 4 : 2; }
static_assert(A_TMEM0 + t_bufs<2>() * 2 * A_PART_COLS <= TMEM_COLS, "TMEM columns");
static_assert(A_TMEM0 + t_bufs<3>() * 3 * A_PART_COLS <= TMEM_COLS, "TMEM columns");

template <int SA>
constexpr size_t smem_bytes()
{
    return 1024 + (size_t)a_stages<SA>() * A_STAGE_BYTES + (size_t)x_stages<SA>() * SA * X_PART_BYTES + 256;
}
static_assert(smem_bytes<2>() <= 232448 && smem_bytes<3>() <= 232448, "shared memory per CTA");

// the K range [kt0, kt1) of unit u (split s of row block rb).  Row blocks
// vary fastest, so CTAs that run at the same time read neighbouring row
// blocks of the same columns: one column's segments of 512 B from many CTAs
// form long contiguous runs in DRAM.
struct Unit {
    int rb, s, kt0, kt1;
    __device__ __forceinline__ Unit(int u, int RB, int S, int KT)
    {
        s = u / RB;
        rb = u - s * RB;
        kt0 = (int)((int64_t)s * KT / S);
        kt1 = (int)((int64_t)(s + 1) * KT / S);
    }
};

// SA: BF16 parts of A and of P (2: BF16x3, 3: BF16x6)
template <int SA>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_gemm_split_bf16(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmX, TcArgs a)
{
    constexpr int NSA = a_stages<SA>();
    constexpr int X_STAGES = x_stages<SA>();
    constexpr int NTB = t_bufs<SA>();
    using PR = Products<SA>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    float *sA = reinterpret_cast<float *>(base);
    unsigned char *sX = base + NSA * A_STAGE_BYTES;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sX + X_STAGES * SA * X_PART_BYTES);
    uint64_t *a_full = bars;                  // [NSA] TMA -> converters
    uint64_t *a_empty = a_full + NSA;         // [NSA] converters -> TMA
    uint64_t *x_full = a_empty + NSA;         // [X_STAGES] TMA -> MMA
    uint64_t *x_empty = x_full + X_STAGES;    // [X_STAGES] MMA -> TMA
    uint64_t *t_full = x_empty + X_STAGES;    // [NTB] converters -> MMA (A parts in TMEM)
    uint64_t *t_empty = t_full + NTB;         // [NTB] MMA -> converters
    uint64_t *c_full = t_empty + NTB;         // [2] MMA -> epilogue (accumulator chain)
    uint64_t *c_empty = c_full + 2;           // [2] epilogue -> MMA
    uint64_t *mma_done = c_empty + 2;         // [1] all MMAs of this CTA completed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    volatile int *stop = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSA; ++s) {
            mbar_init(&a_full[s], 1);
            mbar_init(&a_empty[s], 128);
        }
        for (int s = 0; s < X_STAGES; ++s) {
            mbar_init(&x_full[s], 1);
            mbar_init(&x_empty[s], 1);
        }
        for (int s = 0; s < NTB; ++s) {
            mbar_init(&t_full[s], 128);
            mbar_init(&t_empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&c_full[s], 1);
            mbar_init(&c_empty[s], 128);
        }
        mbar_init(mma_done, 1);
        *stop = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 9) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tmem_slot;
    const int S = a.splits, KT = a.kt_count;

    if (warp == 8) {
        // ---------------- TMA producer of A (and its L2 prefetch)
        if (lane == 0) {
            uint32_t ia = 0;
            bool ok = true;
            // the prefetch cursor runs PREFETCH_TILES tiles ahead through this
            // CTA's sequence of units
            int pu = blockIdx.x, pkt = 0;
            Unit pn(pu < a.units ? pu : 0, a.rb_count, S, KT);
            pkt = pn.kt0;
            auto prefetch_next = [&]() {
                if (pu >= a.units) return;
                tma_prefetch_2d(&tmA, pn.rb * TC_BM, pkt * TC_BK);
                if (++pkt >= pn.kt1) {
                    pu += gridDim.x;
                    if (pu < a.units) {
                        pn = Unit(pu, a.rb_count, S, KT);
                        pkt = pn.kt0;
                    }
                }
            };
            for (int p = 0; p < PREFETCH_TILES; ++p) prefetch_next();
            for (int u = blockIdx.x; ok && u < a.units; u += gridDim.x) {
                const Unit un(u, a.rb_count, S, KT);
                for (int kt = un.kt0; kt < un.kt1; ++kt) {
                    const uint32_t st = ia % NSA, ph = (ia / NSA) & 1;
                    if (!(ok = mbar_wait(&a_empty[st], ph ^ 1, stop, a.err, ERR_WAIT_TMA))) break;
                    mbar_expect_tx(&a_full[st], A_STAGE_BYTES);
                    tma_load_2d(sA + (size_t)st * (A_STAGE_BYTES / 4), &tmA, &a_full[st], un.rb * TC_BM, kt * TC_BK);
                    prefetch_next();
                    ++ia;
                }
            }
            if (!ok) {
                // stopped: let the copies already issued land before the CTA
                // exits (a copy always completes; the wait only bounds it)
                volatile int dummy = 0;
                for (uint32_t t = ia > (uint32_t)NSA ? ia - NSA : 0; t < ia; ++t)
                    mbar_wait(&a_full[t % NSA], (t / NSA) & 1, &dummy, a.err, ERR_WAIT_TMA);
            }
        }
    } else if (warp == 10) {
        // ---------------- TMA producer of the P parts
        if (lane == 0) {
            uint32_t ix = 0;
            bool ok = true;
            const uint32_t x_bytes = (uint32_t)SA * a.npad * TC_BK * 2;
            for (int u = blockIdx.x; ok && u < a.units; u += gridDim.x) {
                const Unit un(u, a.rb_count, S, KT);
                for (int kt = un.kt0; kt < un.kt1; ++kt) {
                    const uint32_t xs = ix % X_STAGES, xph = (ix / X_STAGES) & 1;
                    if (!(ok = mbar_wait(&x_empty[xs], xph ^ 1, stop, a.err, ERR_WAIT_TMA))) break;
                    mbar_expect_tx(&x_full[xs], x_bytes);
#pragma unroll
                    for (int p = 0; p < SA; ++p)
                        tma_load_2d(sX + (size_t)(xs * SA + p) * X_PART_BYTES, &tmX, &x_full[xs], kt * TC_BK,
                                    p * a.npad);
                    ++ix;
                }
            }
            if (!ok) {
                volatile int dummy = 0;
                for (uint32_t t = ix > (uint32_t)X_STAGES ? ix - X_STAGES : 0; t < ix; ++t)
                    mbar_wait(&x_full[t % X_STAGES], (t / X_STAGES) & 1, &dummy, a.err, ERR_WAIT_TMA);
            }
        }
    } else if (warp >= 4 && warp < 8) {
        // ---------------- converters: row t of the FP32 tile -> BF16 parts in TMEM lane t
        const int t = threadIdx.x - 128;
        const uint32_t lane_base = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
        uint32_t ia = 0, it = 0;
        bool ok = true;
        for (int u = blockIdx.x; ok && u < a.units; u += gridDim.x) {
            const Unit un(u, a.rb_count, S, KT);
            for (int kt = un.kt0; kt < un.kt1; ++kt) {
                const uint32_t st = ia % NSA, ph = (ia / NSA) & 1;
                if (!(ok = mbar_wait(&a_full[st], ph, stop, a.err, ERR_WAIT_CONVERT))) break;
                const uint32_t tb = it % NTB, tph = (it / NTB) & 1;
                if (!(ok = mbar_wait(&t_empty[tb], tph ^ 1, stop, a.err, ERR_WAIT_CONVERT))) break;
                tc_fence_after();
                const float *src = sA + (size_t)st * (A_STAGE_BYTES / 4) + t;
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    uint32_t w0[16], w1[16], w2[16];
                    float x[32];
#pragma unroll
                    for (int c = 0; c < 32; ++c) x[c] = src[(half * 32 + c) * TC_BM];
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        // K elements k and k + 1 in one word (k in the low half), each
                        // part the BF16 rounding of what the previous parts leave
                        const __nv_bfloat162 h0 = __floats2bfloat162_rn(x[2 * c], x[2 * c + 1]);
                        const float2 f0 = __bfloat1622float2(h0);
                        const float e0 = x[2 * c] - f0.x, e1 = x[2 * c + 1] - f0.y;
                        const __nv_bfloat162 h1 = __floats2bfloat162_rn(e0, e1);
                        w0[c] = bf2_bits(h0);
                        w1[c] = bf2_bits(h1);
                        if constexpr (SA == 3) {
                            const float2 f1 = __bfloat1622float2(h1);
                            w2[c] = bf2_bits(__floats2bfloat162_rn(e0 - f1.x, e1 - f1.y));
                        }
                    }
                    const uint32_t col = A_TMEM0 + (tb * SA) * A_PART_COLS + half * 16;
                    tmem_st16(lane_base + col, w0);
                    tmem_st16(lane_base + col + A_PART_COLS, w1);
                    if constexpr (SA == 3) tmem_st16(lane_base + col + 2 * A_PART_COLS, w2);
                }
                tmem_st_wait();
                mbar_arrive(&a_empty[st]);  // this thread's reads of the FP32 tile are done
                tc_fence_before();
                mbar_arrive(&t_full[tb]);
                ++ia;
                ++it;
            }
        }
    } else if (warp == 9) {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(TC_BM, a.npad);
            uint32_t it = 0, ic = 0;
            bool ok = true;
            for (int u = blockIdx.x; ok && u < a.units; u += gridDim.x) {
                const Unit un(u, a.rb_count, S, KT);
                for (int c0 = un.kt0; ok && c0 < un.kt1; c0 += CHAIN_TILES) {
                    // one accumulator chain: at most CHAIN_TILES K tiles
                    const uint32_t cb = ic & 1, cph = (ic >> 1) & 1;
                    if (!(ok = mbar_wait(&c_empty[cb], cph ^ 1, stop, a.err, ERR_WAIT_MMA))) break;
                    tc_fence_after();
                    const uint32_t d_tmem = tbase + cb * ACC_COLS;
                    uint32_t acc = 0;
                    const int c1 = min(un.kt1, c0 + CHAIN_TILES);
                    for (int kt = c0; kt < c1; ++kt) {
                        const uint32_t tb = it % NTB, tph = (it / NTB) & 1;
                        if (!(ok = mbar_wait(&t_full[tb], tph, stop, a.err, ERR_WAIT_MMA))) break;
                        const uint32_t xs = it % X_STAGES, xph = (it / X_STAGES) & 1;
                        if (!(ok = mbar_wait(&x_full[xs], xph, stop, a.err, ERR_WAIT_MMA))) break;
                        tc_fence_after();
                        const uint32_t a_tmem = tbase + A_TMEM0 + tb * SA * A_PART_COLS;
                        const uint32_t x_smem = smem_u32(sX + (size_t)xs * SA * X_PART_BYTES);
#pragma unroll
                        for (int ks = 0; ks < TC_BK / 16; ++ks) {
#pragma unroll
                            for (int p = 0; p < PR::N; ++p) {
                                const uint64_t bdesc = sw128_desc(x_smem + PR::x(p) * X_PART_BYTES + ks * 32);
                                mma_ts(d_tmem, a_tmem + PR::a(p) * A_PART_COLS + ks * 8, bdesc, idesc, acc);
                                acc = 1;
                            }
                        }
                        mma_commit(&t_empty[tb]);  // the A parts' columns are free once these complete
                        mma_commit(&x_empty[xs]);  // and so is the P stage
                        ++it;
                    }
                    if (!ok) break;
                    mma_commit(&c_full[cb]);
                    ++ic;
                }
            }
            // every MMA of this CTA completes before its tensor memory is freed
            mma_commit(mma_done);
            volatile int dummy = 0;
            mbar_wait(mma_done, 0, &dummy, a.err, ERR_WAIT_MMA);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: chains -> running sum -> workspace [s][column][row]
        const int t = threadIdx.x;
        const uint32_t lane_base = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
        uint32_t ic = 0;
        bool ok = true;
        for (int u = blockIdx.x; ok && u < a.units; u += gridDim.x) {
            const Unit un(u, a.rb_count, S, KT);
            // the unit's sum over its accumulator chains, column c of this row
            float run[TC_MAXN];
#pragma unroll
            for (int c = 0; c < TC_MAXN; ++c) run[c] = 0.0f;
            for (int c0 = un.kt0; c0 < un.kt1; c0 += CHAIN_TILES) {
                const uint32_t cb = ic & 1, cph = (ic >> 1) & 1;
                if (!(ok = mbar_wait(&c_full[cb], cph, stop, a.err, ERR_WAIT_EPILOGUE))) break;
                tc_fence_after();
#pragma unroll
                for (int ch = 0; ch < TC_MAXN / 16; ++ch) {
                    if (ch * 16 < a.npad) {
                        uint32_t r[16];
                        tmem_ld16(lane_base + cb * ACC_COLS + ch * 16, r);
#pragma unroll
                        for (int c = 0; c < 16; ++c) run[ch * 16 + c] += __uint_as_float(r[c]);
                    }
                }
                tc_fence_before();
                mbar_arrive(&c_empty[cb]);
                ++ic;
            }
            if (!ok) break;
            float *dst = a.ws + (size_t)un.s * a.npad * a.ws_rows + (int64_t)un.rb * TC_BM + t;
#pragma unroll
            for (int c = 0; c < TC_MAXN; ++c)
                if (c < a.npad) dst[(int64_t)c * a.ws_rows] = run[c];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 9) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS)
                     : "memory");
    }
}

// P parts: planes[p][c][k] (BF16, K contiguous, padded with zeros), column c
// of P = [Re X | Im X] (c < 2 nrhs)
__global__ void k_split_planes(const double2 *__restrict__ X, int64_t n, int64_t ldx, int nrhs, int npad,
                               int64_t kpad, int parts, __nv_bfloat16 *__restrict__ planes)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (k >= kpad) return;
    float x = 0.0f;
    if (k < n && c < 2 * nrhs) {
        const double2 v = X[(int64_t)(c < nrhs ? c : c - nrhs) * ldx + k];
        x = (float)(c < nrhs ? v.x : v.y);
    }
    float r1, r2;
    __nv_bfloat16 p0, p1, p2;
    split3(x, r1, r2, p0, p1, p2);
    const int64_t plane = (int64_t)npad * kpad;
    planes[(int64_t)c * kpad + k] = p0;
    planes[plane + (int64_t)c * kpad + k] = p1;
    if (parts == 3) planes[2 * plane + (int64_t)c * kpad + k] = p2;
}

// Y[i, r] = alpha (complex combination of Z) + beta Y[i, r], Z = sum over the
// split-K partials (FP64, in partial order)
__global__ void k_gemm_combine(const float *__restrict__ ws, int splits, int npad, int64_t ws_rows, int64_t m,
                               int nrhs, double2 *Y, int64_t ldy, double are, double aim, double bre, double bim)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (i >= m) return;
    double zr_e = 0.0, zr_o = 0.0, zi_e = 0.0, zi_o = 0.0;  // Z[2i|2i+1, r | nrhs + r]
    for (int s = 0; s < splits; ++s) {
        const float *w = ws + (size_t)s * npad * ws_rows;
        const float2 a = *reinterpret_cast<const float2 *>(w + (int64_t)r * ws_rows + 2 * i);
        const float2 b = *reinterpret_cast<const float2 *>(w + (int64_t)(nrhs + r) * ws_rows + 2 * i);
        zr_e += a.x;
        zr_o += a.y;
        zi_e += b.x;
        zi_o += b.y;
    }
    const double re = zr_e - zi_o, im = zi_e + zr_o;
    double2 y = make_double2(0.0, 0.0);
    if (bre != 0.0 || bim != 0.0) y = Y[(int64_t)r * ldy + i];
    Y[(int64_t)r * ldy + i] =
        make_double2(are * re - aim * im + bre * y.x - bim * y.y, are * im + aim * re + bre * y.y + bim * y.x);
}

// cuTensorMapEncodeTiled, found through the runtime (no link against the driver)
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(f);
        cudaGetLastError();
    });
    return fn;
}

int sm_count()
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// split-K factor: the smallest that puts at least 97% of the last wave to work
// (units / (waves * CTAs)), at most 16 and at most the K tiles
int choose_splits(int rb_count, int kt_count, int ctas)
{
    int best = 1;
    double best_eff = 0.0;
    for (int s = 1; s <= std::min(16, kt_count); ++s) {
        const int64_t units = (int64_t)rb_count * s;
        const int64_t waves = (units + ctas - 1) / ctas;
        const double eff = (double)units / (double)(waves * ctas);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = s;
        }
        if (eff >= 0.97) return s;
    }
    return best;
}

struct Plan {
    int npad, rb_count, kt_count, splits, ctas;
    int64_t kpad;
};

Plan make_plan(int64_t m, int64_t n, int nrhs_pass)
{
    Plan p;
    p.npad = (2 * nrhs_pass + 15) / 16 * 16;
    p.rb_count = (int)((2 * m + TC_BM - 1) / TC_BM);
    p.kt_count = (int)((n + TC_BK - 1) / TC_BK);
    p.kpad = (int64_t)p.kt_count * TC_BK;
    const int sms = sm_count();
    p.splits = choose_splits(p.rb_count, p.kt_count, sms);
    p.ctas = (int)std::min<int64_t>((int64_t)p.rb_count * p.splits, sms);
    return p;
}

}  // namespace

bool gemm_tc_supported(const void *A, int64_t lda)
{
    // TMA on the float view: 16-byte aligned base and column stride (8 lda bytes)
    return encode_tiled() != nullptr && (reinterpret_cast<uintptr_t>(A) & 15) == 0 && (lda & 1) == 0;
}

size_t gemm_tc_scratch_bytes(int parts, int64_t m, int64_t n, int64_t nrhs)
{
    if (m == 0 || n == 0 || nrhs == 0) return 256;
    const int pass = (int)std::min<int64_t>(nrhs, TC_MAXN / 2);
    const Plan p = make_plan(m, n, pass);
    const size_t planes = (size_t)parts * p.npad * p.kpad * 2;
    const size_t ws = (size_t)p.splits * p.npad * p.rb_count * TC_BM * 4;
    return 256 + ((planes + 255) & ~(size_t)255) + ws;
}

cudaError_t launch_gemm_tc(int parts, const void *A, int64_t m, int64_t n, int64_t lda, const double2 *X, int64_t ldx,
                           int64_t nrhs, double2 *Y, int64_t ldy, double are, double aim, double bre, double bim,
                           void *scratch, int *err, cudaStream_t s)
{
    if (m == 0 || nrhs == 0) return cudaSuccess;
    if ((parts != 2 && parts != 3) || !gemm_tc_supported(A, lda) || n == 0 || 2 * m > 0x7fffffff)
        return cudaErrorInvalidValue;
    EncodeTiledFn enc = encode_tiled();
    {
        cudaError_t e = parts == 2
                            ? cudaFuncSetAttribute(k_gemm_split_bf16<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem_bytes<2>())
                            : cudaFuncSetAttribute(k_gemm_split_bf16<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem_bytes<3>());
        if (e != cudaSuccess) return e;
    }
    // A_r: 2m rows (contiguous) x n columns of FP32, tiles of 128 rows x 64 K
    CUtensorMap tmA;
    {
        const cuuint64_t dims[2] = {(cuuint64_t)(2 * m), (cuuint64_t)n};
        const cuuint64_t strides[1] = {(cuuint64_t)(8 * lda)};
        const cuuint32_t box[2] = {TC_BM, TC_BK};
        const cuuint32_t estr[2] = {1, 1};
        if (enc(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(A), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    const int pass_max = TC_MAXN / 2;
    for (int64_t r0 = 0; r0 < nrhs; r0 += pass_max) {
        const int pass = (int)std::min<int64_t>(pass_max, nrhs - r0);
        const Plan p = make_plan(m, n, pass);
        __nv_bfloat16 *planes = reinterpret_cast<__nv_bfloat16 *>(static_cast<char *>(scratch) + 256);
        const size_t planes_bytes = ((size_t)parts * p.npad * p.kpad * 2 + 255) & ~(size_t)255;
        float *ws = reinterpret_cast<float *>(static_cast<char *>(scratch) + 256 + planes_bytes);
        dim3 gs((unsigned)((p.kpad + 255) / 256), p.npad);
        k_split_planes<<<gs, 256, 0, s>>>(X + r0 * ldx, n, ldx, pass, p.npad, p.kpad, parts, planes);
        // P parts: parts * npad rows of kpad BF16 (K contiguous), tiles of 64 K x npad rows
        CUtensorMap tmX;
        {
            const cuuint64_t dims[2] = {(cuuint64_t)p.kpad, (cuuint64_t)parts * p.npad};
            const cuuint64_t strides[1] = {(cuuint64_t)(2 * p.kpad)};
            const cuuint32_t box[2] = {TC_BK, (cuuint32_t)p.npad};
            const cuuint32_t estr[2] = {1, 1};
            if (enc(&tmX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, planes, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return cudaErrorInvalidValue;
        }
        TcArgs ta;
        ta.rb_count = p.rb_count;
        ta.kt_count = p.kt_count;
        ta.splits = p.splits;
        ta.units = p.rb_count * p.splits;
        ta.npad = p.npad;
        ta.ws_rows = (int64_t)p.rb_count * TC_BM;
        ta.ws = ws;
        ta.err = err;
        if (parts == 2) k_gemm_split_bf16<2><<<p.ctas, TC_THREADS, smem_bytes<2>(), s>>>(tmA, tmX, ta);
        else k_gemm_split_bf16<3><<<p.ctas, TC_THREADS, smem_bytes<3>(), s>>>(tmA, tmX, ta);
        dim3 gc((unsigned)((m + 255) / 256), pass);
        k_gemm_combine<<<gc, 256, 0, s>>>(ws, p.splits, p.npad, ta.ws_rows, m, pass, Y + r0 * ldy, ldy, are, aim,
                                          bre, bim);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace nihu
