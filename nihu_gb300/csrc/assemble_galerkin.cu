// Galerkin formalism of the SLP and DLP operators on constant elements:
//   A(i, j) = int_{E_i} int_{E_j} K(x, y) dS_y dS_x
// (nihu/core/double_integral.hpp:143-384, the "general" formalism).
//
// Dispatch, as the reference: on one mesh an element pair that shares the
// element (face), two nodes (edge) or one node (corner) takes the singular
// Galerkin rule of its match type (nihu/core/element_match.hpp:60-90,
// nihu/core/singular_accelerator.hpp:220-310); every other pair takes the
// product of the regular rule of degree C + interval(d/D) on both elements
// (complexity_estimator.hpp:69-75, the dual accelerator of
// double_integral.hpp:300-312).  The singular rules are the 4D Gauss products
// (4 points per direction: the kernels' singular quadrature order 7) split
// into Duffy-type subdomains in coordinate differences
// (nihu/core/singular_galerkin_quadrature.hpp:200-420): face 3 subdomains
// (symmetric, 1536 points), edge 6 (1536), corner 1 (symmetric, 512).
//
// Work layout: k_galerkin_regular (FP32 default / FP64) owns the pairs at
// d/D >= 1.5 exactly as the collocation kernel does, with the test element's
// points in the same rule as the trial element's (a far pair is the
// collocation entry times the test element's area); k_galerkin_near (one warp
// per pair, lanes over the rule's points) owns the self pairs, the nearly
// singular list (d/D < 1.5: matched pairs, and unmatched ones with the
// degree-6/8 product rules) and the rare pairs beyond 1.5 D that still share
// a node (collected by the regular kernel).  The near kernel follows the
// regular quadrature's precision: FP64, or FP32 with r_vec formed from
// vectors relative to the common node (matched pairs) or to the element
// centres (unmatched pairs), which keeps FP32 relative accuracy as r -> 0.
#include <algorithm>
#include <mutex>
#include <vector>

#include "classify.cuh"
#include "kernels.h"
#include "singular_schemes.cuh"

namespace nihu {

constexpr int GAL_THREADS = 256;
constexpr int GAL_COLS = 32;
constexpr int GAL_WARPS = 4;
constexpr int GAL_GAUSS = 4;  // points per direction of the singular rules
constexpr int GAL_PER_DIM4 = GAL_GAUSS * GAL_GAUSS * GAL_GAUSS * GAL_GAUSS;
// points of the corner (0), edge (1) and face (2) rules
__host__ __device__ constexpr int gal_npts(int match) { return (match == 0 ? 2 : 6) * GAL_PER_DIM4; }
constexpr int GAL_TOTAL = gal_npts(0) + gal_npts(1) + gal_npts(2);

// the singular rules, (test xi, eta, trial xi, eta, w) per point: corner
// points first, then edge, then face; and in FP32 (test xi, eta, trial xi,
// eta, w, trial xi - test xi, trial eta - test eta, 0), the differences formed
// in FP64
__device__ double g_gal_rule[GAL_TOTAL * 5];

// the quad-quad rules (corner 1280, edge 1536, face 2048 points), the same layout
__host__ __device__ constexpr int galq_npts(int match) { return match == 0 ? 1280 : (match == 1 ? 1536 : 2048); }
__host__ __device__ constexpr int galq_offset(int match)
{
    return match == 0 ? 0 : (match == 1 ? galq_npts(0) : galq_npts(0) + galq_npts(1));
}
constexpr int GALQ_TOTAL = galq_npts(0) + galq_npts(1) + galq_npts(2);
__device__ double g_galq_rule[GALQ_TOTAL * 5];
__device__ __align__(16) float g_gal_rule32[GAL_TOTAL * 8];

__host__ __device__ constexpr int gal_offset(int match)
{
    return match == 0 ? 0 : (match == 1 ? gal_npts(0) : gal_npts(0) + gal_npts(1));
}

// one point of the 4D cube mapped into a subdomain of the match type: test
// point (a1, a2) and trial point (a1 + b1, a2 + b2) on 0 <= x2 <= x1 <= 1,
// weight times the subdomain Jacobian
static void gal_subdomain(int match, int sub, const double u[4], double &w, double out[4])
{
    double a1, a2, b1, b2;
    if (match == 2) {
        double jac;
        if (sub == 0) {
            b1 = u[0];
            b2 = u[0] * u[1];
            a1 = (1.0 - b1) * u[2];
            a2 = a1 * u[3];
            jac = (1.0 - b1) * a1;
        } else if (sub == 1) {
            b1 = u[0] * u[1];
            b2 = u[0] * (u[1] - 1.0);
            a1 = (1.0 - b1 + b2) * u[2] - b2;
            a2 = (a1 + b2) * u[3] - b2;
            jac = (1.0 - b1 + b2) * (a1 + b2);
        } else {
            b1 = u[0] * u[1];
            b2 = u[0];
            a1 = (1.0 - b2) * u[2] + b2 - b1;
            a2 = (a1 - b2 + b1) * u[3];
            jac = (1.0 - b2) * (a1 - b2 + b1);
        }
        w *= jac * u[0];
    } else if (match == 1) {
        const double p = u[0], q = u[1], r = u[2], s = u[3];
        switch (sub) {
        case 0: b1 = -p * q; b2 = -p * q * r; a1 = (1.0 - p) * s + p; a2 = p * (1.0 - q + q * r); break;
        case 1: b1 = p * q; b2 = p * q * r; a1 = (1.0 - p) * s + p * (1.0 - q); a2 = p * (1.0 - q); break;
        case 2: b1 = -p * q * r; b2 = p * q * (1.0 - r); a1 = (1.0 - p) * s + p; a2 = p * (1.0 - q); break;
        case 3: b1 = p * q * r; b2 = p * q * (r - 1.0); a1 = (1.0 - p) * s + p * (1.0 - q * r); a2 = p * (1.0 - q * r); break;
        case 4: b1 = -p * q * r; b2 = -p * q; a1 = (1.0 - p) * s + p; a2 = p; break;
        default: b1 = p * q * r; b2 = p * q; a1 = (1.0 - p) * s + p * (1.0 - q * r); a2 = p * (1.0 - q); break;
        }
        w *= q * p * p * (1.0 - p);
    } else {
        a1 = u[0];
        a2 = a1 * u[1];
        const double e1 = a1 * u[2], e2 = e1 * u[3];
        w *= u[2] * u[0] * u[0] * u[0];
        b1 = e1 - a1;
        b2 = e2 - a2;
    }
    out[0] = a1 - a2;
    out[1] = a2;
    out[2] = (a1 + b1) - (a2 + b2);
    out[3] = a2 + b2;
}

// every Dunavant rule in FP32, (xi, eta, w) per point at the offsets of quad_rules.h
struct TriF32 {
    float v[NIHU_TRI_DATA_LEN];
    constexpr TriF32() : v()
    {
        constexpr double d[NIHU_TRI_DATA_LEN] = NIHU_TRI_DATA;
        for (int q = 0; q < NIHU_TRI_DATA_LEN; ++q) v[q] = (float)d[q];
    }
};
__device__ constexpr TriF32 TRI_F32{};

// host generation of the three rules (the Gauss nodes come from the device
// tables' source, quad_rules.h)
static std::vector<double> gal_rules()
{
    static const double gdata[NIHU_GAUSS_DATA_LEN] = NIHU_GAUSS_DATA;
    static const int goff[NIHU_GAUSS_MAX_N] = NIHU_GAUSS_OFFSETS;
    double x[GAL_GAUSS], wt[GAL_GAUSS];
    for (int i = 0; i < GAL_GAUSS; ++i) {
        x[i] = (1.0 + gdata[2 * (goff[GAL_GAUSS - 1] + i)]) / 2.0;
        wt[i] = gdata[2 * (goff[GAL_GAUSS - 1] + i) + 1] / 2.0;
    }
    std::vector<double> out((size_t)GAL_TOTAL * 5);
    for (int match = 0; match < 3; ++match) {
        const int subs = match == 2 ? 3 : (match == 1 ? 6 : 1);
        const bool sym = match != 1;
        double *d = out.data() + 5 * (size_t)gal_offset(match);
        for (int i1 = 0; i1 < GAL_GAUSS; ++i1)
            for (int i2 = 0; i2 < GAL_GAUSS; ++i2)
                for (int i3 = 0; i3 < GAL_GAUSS; ++i3)
                    for (int i4 = 0; i4 < GAL_GAUSS; ++i4)
                        for (int sub = 0; sub < subs; ++sub) {
                            const double u[4] = {x[i1], x[i2], x[i3], x[i4]};
                            double w = wt[i1] * wt[i2] * wt[i3] * wt[i4], o[4];
                            gal_subdomain(match, sub, u, w, o);
                            d[0] = o[0]; d[1] = o[1]; d[2] = o[2]; d[3] = o[3]; d[4] = w;
                            d += 5;
                            if (sym) {
                                d[0] = o[2]; d[1] = o[3]; d[2] = o[0]; d[3] = o[1]; d[4] = w;
                                d += 5;
                            }
                        }
    }
    return out;
}

// Duffy quads of the coordinate difference mu for the quad-quad rules
// (nihu/library/lib_singular_galerkin_quadrature.cpp)
static const double QF[4][4][2] = {{{0, 0}, {0, 0}, {2, -2}, {2, 0}}, {{0, 0}, {0, 0}, {2, 0}, {2, 2}},
                                   {{0, 0}, {0, 0}, {2, 2}, {0, 2}}, {{0, 0}, {0, 0}, {0, 2}, {-2, 2}}};
static const double QE[6][4][2] = {{{0, 0}, {0, 0}, {-2, 0}, {-2, -2}}, {{0, 0}, {0, 0}, {-2, -2}, {0, -2}},
                                   {{0, 0}, {0, 0}, {0, -2}, {2, -2}},  {{0, 0}, {0, 0}, {2, -2}, {2, 0}},
                                   {{-2, -2}, {-2, -4}, {0, -4}, {0, -2}}, {{0, -2}, {0, -4}, {2, -4}, {2, -2}}};
static const double QC[5][4][2] = {{{0, 0}, {0, 0}, {-2, 0}, {-2, -2}}, {{0, 0}, {0, 0}, {-2, -2}, {0, -2}},
                                   {{-4, 0}, {-4, -2}, {-2, -2}, {-2, 0}}, {{-4, -2}, {-4, -4}, {-2, -4}, {-2, -2}},
                                   {{-2, -2}, {-2, -4}, {0, -4}, {0, -2}}};

// bilinear map of (u, v) in [-1,1]^2 onto the quad with corners C, signed Jacobian
static void quad_corner_map(const double C[4][2], double u, double v, double &x, double &y, double &det)
{
    const double N[4] = {(1 - u) * (1 - v) / 4, (1 + u) * (1 - v) / 4, (1 + u) * (1 + v) / 4, (1 - u) * (1 + v) / 4};
    const double du[4] = {-(1 - v) / 4, (1 - v) / 4, (1 + v) / 4, -(1 + v) / 4};
    const double dv[4] = {-(1 - u) / 4, -(1 + u) / 4, (1 + u) / 4, (1 - u) / 4};
    double j00 = 0, j01 = 0, j10 = 0, j11 = 0;
    x = y = 0;
    for (int c = 0; c < 4; ++c) {
        x += N[c] * C[c][0];
        y += N[c] * C[c][1];
        j00 += du[c] * C[c][0];
        j01 += du[c] * C[c][1];
        j10 += dv[c] * C[c][0];
        j11 += dv[c] * C[c][1];
    }
    det = j00 * j11 - j01 * j10;
}

// the trial point's reflection that sets the two squares side by side:
// none (face), (eta_0, -2 - eta_1) (edge), -2 - eta (corner)
static void quad_reflect(int match, double e0, double e1, double &o0, double &o1)
{
    o0 = match == 0 ? -2.0 - e0 : e0;
    o1 = match == 2 ? e1 : -2.0 - e1;
}

static std::vector<double> galq_rules()
{
    static const double gdata[NIHU_GAUSS_DATA_LEN] = NIHU_GAUSS_DATA;
    static const int goff[NIHU_GAUSS_MAX_N] = NIHU_GAUSS_OFFSETS;
    const double *g = gdata + 2 * goff[GAL_GAUSS - 1];
    std::vector<double> out((size_t)GALQ_TOTAL * 5);
    for (int match = 0; match < 3; ++match) {
        const int subs = match == 2 ? 4 : (match == 1 ? 6 : 5);
        const double (*tab)[4][2] = match == 2 ? QF : (match == 1 ? QE : QC);
        double lo[2], hi[2];
        quad_reflect(match, -1.0, -1.0, lo[0], lo[1]);
        quad_reflect(match, 1.0, 1.0, hi[0], hi[1]);
        for (int c = 0; c < 2; ++c)
            if (lo[c] > hi[c]) std::swap(lo[c], hi[c]);
        double *d = out.data() + 5 * (size_t)galq_offset(match);
        for (int sd = 0; sd < subs; ++sd)
            for (int a = 0; a < GAL_GAUSS; ++a)
                for (int b = 0; b < GAL_GAUSS; ++b) {
                    double mu0, mu1, det;
                    quad_corner_map(tab[sd], g[2 * a], g[2 * b], mu0, mu1, det);
                    const double wo = g[2 * a + 1] * g[2 * b + 1] * det;
                    auto clip = [](double v) { return std::min(1.0, std::max(-1.0, v)); };
                    const double x0 = clip(lo[0] - mu0), x1 = clip(hi[0] - mu0);
                    const double y0 = clip(lo[1] - mu1), y1 = clip(hi[1] - mu1);
                    const double R[4][2] = {{x0, y0}, {x1, y0}, {x1, y1}, {x0, y1}};
                    for (int c = 0; c < GAL_GAUSS; ++c)
                        for (int e = 0; e < GAL_GAUSS; ++e) {
                            double xi0, xi1, di;
                            quad_corner_map(R, g[2 * c], g[2 * e], xi0, xi1, di);
                            const double w = wo * g[2 * c + 1] * g[2 * e + 1] * di;
                            double et0, et1;
                            quad_reflect(match, mu0 + xi0, mu1 + xi1, et0, et1);
                            d[0] = xi0; d[1] = xi1; d[2] = et0; d[3] = et1; d[4] = w;
                            d += 5;
                            if (match == 2) {
                                d[0] = et0; d[1] = et1; d[2] = xi0; d[3] = xi1; d[4] = w;
                                d += 5;
                            }
                        }
                }
    }
    return out;
}

cudaError_t prepare_galerkin(cudaStream_t s)
{
    static std::mutex mu;
    static std::vector<int> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() > dev && done[dev]) return cudaSuccess;
    static const std::vector<double> rules = gal_rules();
    static const std::vector<float> rules32 = [] {
        std::vector<float> f((size_t)GAL_TOTAL * 8, 0.0f);
        for (size_t p = 0; p < (size_t)GAL_TOTAL; ++p) {
            const double *q = rules.data() + 5 * p;
            for (int c = 0; c < 5; ++c) f[8 * p + c] = (float)q[c];
            f[8 * p + 5] = (float)(q[2] - q[0]);
            f[8 * p + 6] = (float)(q[3] - q[1]);
        }
        return f;
    }();
    e = cudaMemcpyToSymbolAsync(g_gal_rule, rules.data(), rules.size() * sizeof(double), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbolAsync(g_gal_rule32, rules32.data(), rules32.size() * sizeof(float), 0,
                                    cudaMemcpyHostToDevice, s);
    static const std::vector<double> qrules = galq_rules();
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbolAsync(g_galq_rule, qrules.data(), qrules.size() * sizeof(double), 0,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    done[dev] = 1;
    return cudaSuccess;
}

// number of common corner nodes of two elements and, for triangles, the first
// common node of each in cyclic order (nihu/core/element.hpp:376-413)
__device__ __forceinline__ int common_nodes(int4 a, int na, int4 b, int nb, int &ind1, int &ind2)
{
    const int A[4] = {a.x, a.y, a.z, a.w}, B[4] = {b.x, b.y, b.z, b.w};
    int num = 0, s1 = 0, s2 = 0;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            if (A[i] != B[j]) continue;
            if (num == 0) {
                s1 = i;
                s2 = j;
            } else {
                if (i < s1 || (i == na - 1 && s1 == 0 && num == 1)) s1 = i;
                if (j < s2 || (j == nb - 1 && s2 == 0 && num == 1)) s2 = j;
            }
            ++num;
        }
    ind1 = s1;
    ind2 = s2;
    return num;
}

// PLAIN: unit scale and no accumulation (FP32): stores without run-time checks;
// CK: a complex (lossy) wave number (eval_point_ck)
template <typename R, typename Out, int FAM, int OPS, bool PLAIN = false, bool CK = false>
__global__ void __launch_bounds__(GAL_THREADS) k_galerkin_regular(GalArgs a)
{
    __shared__ float4 s_hi[GAL_COLS], s_lo[GAL_COLS], s_p0[GAL_COLS];
    __shared__ int4 s_nid[GAL_COLS];
    __shared__ int s_nc[GAL_COLS];
    constexpr bool DO_S = (OPS & OP_SLP) != 0;
    constexpr bool DO_D = (OPS & OP_DLP) != 0;
    const DevMesh &test = a.test;
    const DevMesh &trial = a.trial;
    const int i = blockIdx.x * GAL_THREADS + threadIdx.x;
    const int jb = a.j0 + blockIdx.y * GAL_COLS;
    const int ncols = min(GAL_COLS, a.j1 - jb);
    if (threadIdx.x < ncols) {
        const int j = jb + threadIdx.x;
        s_hi[threadIdx.x] = trial.chi[j];
        s_lo[threadIdx.x] = trial.clo[j];
        s_p0[threadIdx.x] = trial.p0[j];
        s_nid[threadIdx.x] = trial.nid[j];
        s_nc[threadIdx.x] = trial.nc[j];
    }
    __syncthreads();
    if ((i & ~31) >= test.n) return;
    const bool row_ok = i < test.n;
    const int ii = row_ok ? i : test.n - 1;
    const float4 ih = test.chi[ii], il = test.clo[ii];
    const int4 inid = test.nid[ii];
    const int inc = test.nc[ii];
    const float area_i = test.p0[ii].x;  // w J of the one-point rule: the element's area
    R k, ki, are, aim, x0, x1, x2;
    if constexpr (sizeof(R) == 4) {
        k = a.k32;
        ki = a.k_im32;
        are = a.alpha_re32;
        aim = a.alpha_im32;
        x0 = ih.x + il.x;
        x1 = ih.y + il.y;
        x2 = ih.z + il.z;
    } else {
        k = a.k;
        ki = a.k_im;
        are = a.alpha_re;
        aim = a.alpha_im;
        x0 = test.center[3 * (int64_t)ii];
        x1 = test.center[3 * (int64_t)ii + 1];
        x2 = test.center[3 * (int64_t)ii + 2];
    }
    Out *out_s = reinterpret_cast<Out *>(a.out_s);
    Out *out_d = reinterpret_cast<Out *>(a.out_d);
    // this thread's entries of the current column, one column (ld entries) further per step
    const int64_t ldo = a.ld;
    Out *ps = DO_S ? out_s + (int64_t)(jb - a.j0) * ldo + i : nullptr;
    Out *pd = DO_D ? out_d + (int64_t)(jb - a.j0) * ldo + i : nullptr;
    for (int c = 0; c < ncols; ++c, ps += DO_S ? ldo : 0, pd += DO_D ? ldo : 0) {
        const int j = jb + c;
        int ind1, ind2;
        // elements can share a node only when their centres are closer than
        // the sum of their centre-to-corner distances (< 2 D each): compare
        // node ids only then
        const float4 hj = s_hi[c];
        const float ex0 = hj.x - ih.x, ex1 = hj.y - ih.y, ex2 = hj.z - ih.z;
        const float reach = 2.0f * (rsqrtf(ih.w) + rsqrtf(hj.w));
        const bool may_share = a.same_mesh && ex0 * ex0 + ex1 * ex1 + ex2 * ex2 <= 1.01f * reach * reach;
        const int shared = may_share ? common_nodes(inid, inc, s_nid[c], s_nc[c], ind1, ind2) : 0;
        R sr = 0, si = 0, dr = 0, di = 0;
        bool done = false;
        if constexpr (sizeof(R) == 4) {
            // far field: both one-point rules, the centroid kernel times both areas
            const float4 h = s_hi[c], l = s_lo[c];  // hi/lo centre difference (as k_regular)
            const float fx = (h.x - ih.x) + (l.x - il.x), fy = (h.y - ih.y) + (l.y - il.y),
                        fz = (h.z - ih.z) + (l.z - il.z);
            const float q = (fx * fx + fy * fy + fz * fz) * h.w;
            if (__all_sync(0xffffffffu, q > 249.64f * (1.0f + 1e-4f) && shared == 0)) {
                const float4 p = s_p0[c];
                if constexpr (CK)
                    eval_point_ck<float>(fx, fy, fz, p.x, p.y, p.z, p.w, k, ki, DO_S ? area_i : 0.0f,
                                         DO_D ? area_i : 0.0f, sr, si, dr, di);
                else
                    eval_point<FAM, float>(fx, fy, fz, p.x, p.y, p.z, p.w, k, DO_S ? area_i : 0.0f,
                                           DO_D ? area_i : 0.0f, sr, si, dr, di);
                done = true;
            }
        }
        if (!done) {
            int ls, ld;
            float dx, dy, dz;
            const int kind = classify_pair(ih, il, s_hi[c], s_lo[c], ii, j, test.center, trial.center, trial.size,
                                           a.same_mesh, ls, ld, dx, dy, dz);
            if (kind != KIND_REGULAR || !row_ok) continue;  // self and d/D < 1.5: the FP64 kernel
            if (shared > 0) {
                // a node shared beyond 1.5 D (strongly graded mesh): singular rule
                const unsigned slot = atomicAdd(a.n_extra, 1u);
                if (slot < (unsigned)a.extra_cap) a.extra[slot] = make_int2(i, j);
                else atomicCAS(a.err, 0, -1);
                continue;
            }
            if (!DO_S) ls = ld;
            if (!DO_D) ld = ls;
            // the rule of degree C + 2 l on both elements: C = max complexity
            const int cmax = (il.w != 0.0f || s_lo[c].w != 0.0f) ? 1 : 0;
            const int64_t bi = ((int64_t)ii * 2 + cmax) * SLOTS, bj = ((int64_t)j * 2 + cmax) * SLOTS;
            for (int pass = 0; pass < 2; ++pass) {
                const int L = pass == 0 ? ls : ld;
                if (pass == 1 && ld == ls) break;
                const R ws = (DO_S && ls == L) ? R(1) : R(0), wd = (DO_D && ld == L) ? R(1) : R(0);
                const int npi = level_npts(inc, cmax, L), npj = level_npts(s_nc[c], cmax, L);
                for (int p = 0; p < npi; ++p) {
                    const int sp = level_slot0(L) + p;
                    R xp0, xp1, xp2, wp;
                    if constexpr (sizeof(R) == 4) {
                        const float4 y = __ldg(test.pts32 + 2 * (bi + sp));
                        xp0 = y.x;
                        xp1 = y.y;
                        xp2 = y.z;
                        wp = y.w;
                    } else {
                        const double *y = test.pts64 + 8 * (bi + sp);
                        xp0 = y[0];
                        xp1 = y[1];
                        xp2 = y[2];
                        wp = y[3];
                    }
                    for (int q = 0; q < npj; ++q) {
                        const int sq = level_slot0(L) + q;
                        if constexpr (sizeof(R) == 4) {
                            const float4 y = __ldg(trial.pts32 + 2 * (bj + sq));
                            const float4 n = __ldg(trial.pts32 + 2 * (bj + sq) + 1);
                            // r = (c_j - c_i) + (y - c_j) - (x_p - c_i): the hi/lo centre
                            // difference and the points' offsets from their centres
                            if constexpr (CK)
                                eval_point_ck<float>(dx + (y.x - xp0), dy + (y.y - xp1), dz + (y.z - xp2), y.w, n.x,
                                                     n.y, n.z, k, ki, ws * wp, wd * wp, sr, si, dr, di);
                            else
                                eval_point<FAM, float>(dx + (y.x - xp0), dy + (y.y - xp1), dz + (y.z - xp2), y.w, n.x,
                                                       n.y, n.z, k, ws * wp, wd * wp, sr, si, dr, di);
                        } else {
                            const double *y = trial.pts64 + 8 * (bj + sq);
                            if constexpr (CK)
                                eval_point_ck<double>(y[0] - xp0, y[1] - xp1, y[2] - xp2, y[3], y[4], y[5], y[6], k, ki,
                                                      ws * wp, wd * wp, sr, si, dr, di);
                            else
                                eval_point<FAM, double>(y[0] - xp0, y[1] - xp1, y[2] - xp2, y[3], y[4], y[5], y[6], k,
                                                        ws * wp, wd * wp, sr, si, dr, di);
                        }
                    }
                }
            }
        }
        if (!row_ok) continue;
        auto store = [&](Out *p, R re, R im) {
            Out o;
            if constexpr (PLAIN) {
                o.x = re;
                o.y = im;
            } else {
                const R vr = are * re - aim * im, vi = are * im + aim * re;
                if (a.accumulate) {
                    o = *p;
                    o.x += vr;
                    o.y += vi;
                } else {
                    o.x = vr;
                    o.y = vi;
                }
            }
            *p = o;
        };
        if (DO_S) store(ps, sr, si);
        if (DO_D) store(pd, dr, di);
    }
}

// point p of the product rule of a given degree on an element: reference
// coordinates and weight (Dunavant on triangles, Gauss tensor on quads)
__device__ __forceinline__ void product_point(int nc, int degree, int p, double &xi, double &eta, double &w)
{
    if (nc == 3) {
        tri_pt(degree, p, xi, eta, w);
    } else {
        const int ng = degree / 2 + 1;
        double w0, w1;
        gauss_pt(ng, p / ng, xi, w0);
        gauss_pt(ng, p % ng, eta, w1);
        w = w0 * w1;
    }
}

__device__ __forceinline__ int product_npts(int nc, int degree)
{
    if (nc == 3) return g_tri_npts[degree];
    const int ng = degree / 2 + 1;
    return ng * ng;
}

// reference point under a corner rotation of the triangle: corner k of the
// rotated triangle is corner perm[k] of (0,0), (1,0), (0,1)
__device__ __forceinline__ void tri_rotate(const int perm[3], double xi, double eta, double &oxi, double &oeta)
{
    const double N[3] = {1.0 - xi - eta, xi, eta};
    oxi = 0.0;
    oeta = 0.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        oxi += perm[q] == 1 ? N[q] : 0.0;
        oeta += perm[q] == 2 ? N[q] : 0.0;
    }
}

// reference point of the square under a corner rotation: corner k of the
// rotated square is corner perm[k] of (-1,-1), (1,-1), (1,1), (-1,1)
__device__ __forceinline__ void quad_rotate(const int perm[4], double u, double v, double &ou, double &ov)
{
    const double N[4] = {(1 - u) * (1 - v) / 4, (1 + u) * (1 - v) / 4, (1 + u) * (1 + v) / 4, (1 - u) * (1 + v) / 4};
    ou = 0.0;
    ov = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = perm[q];
        ou += (c == 1 || c == 2) ? N[q] : -N[q];
        ov += (c >= 2) ? N[q] : -N[q];
    }
}

// The self pairs, the nearly singular list of columns [j0, j1) (extra = 0)
// or the extra list (extra = 1): one warp per pair
// CK: a complex (lossy) wave number: the FP64 rules with the complex kernel in both modes
template <typename Out, bool CK>
__global__ void __launch_bounds__(GAL_WARPS * 32) k_galerkin_near(GalArgs a, NearList near, int extra)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int64_t n_near = 0, p_begin = 0, total = 0;
    if (extra) {
        total = min((int64_t)*a.n_extra, (int64_t)a.extra_cap);
    } else {
        p_begin = near.col_ptr ? near.col_ptr[a.j0] : 0;
        n_near = (near.col_ptr ? near.col_ptr[a.j1] : 0) - p_begin;
        total = n_near + (a.same_mesh ? (int64_t)(a.j1 - a.j0) : 0);
    }
    const bool do_s = (a.ops & OP_SLP) != 0, do_d = (a.ops & OP_DLP) != 0;
    const int fam = a.family;
    const double k = a.k;
    const cd kc{a.k, a.k_im};
    // kernel values at one point pair: the real or the complex wave number
    auto kp = [&](const double *x, const double *y, const double *n, double J, bool s_, bool d_, cd &ks, cd &kd) {
        if constexpr (CK) kern_point(fam, kc, x, y, n, J, s_, d_, ks, kd);
        else kern_point(fam, k, x, y, n, J, s_, d_, ks, kd);
    };
    Out *out_s = reinterpret_cast<Out *>(a.out_s);
    Out *out_d = reinterpret_cast<Out *>(a.out_d);
    for (int64_t item = warp; item < total; item += nwarps) {
        int i, j;
        if (extra) {
            const int2 e = a.extra[item];
            i = e.x;
            j = e.y;
        } else if (item < n_near) {
            const int64_t p = p_begin + item;
            i = near.rows[p];
            j = near_column(near.col_ptr, a.j0, a.j1, p);
        } else {
            j = a.j0 + (int)(item - n_near);
            i = j;
            if (i >= a.test.n) continue;
        }
        Elem64 te, re;
        load_elem(a.test, i, te);
        load_elem(a.trial, j, re);
        int match = -1, ind1 = 0, ind2 = 0;
        if (a.same_mesh) {
            if (i == j) match = 2;
            else {
                const int num = common_nodes(a.test.nid[i], te.nc, a.trial.nid[j], re.nc, ind1, ind2);
                match = num > 1 ? 1 : (num == 1 ? 0 : -1);
            }
        }
        double sr = 0, si = 0, dr = 0, di = 0;
        if (match >= 0 && te.nc != re.nc) {
            // triangle-quad match, corner or edge (FP64 in both modes;
            // nihu/core/singular_galerkin_quadrature.hpp:624-790): the quad's
            // reference square split into the triangles (0, 1, 2) and (0, 2, 3)
            // of its rotated corners, the triangle-triangle corner rule on both
            // (corner match) or the edge rule on (0, 1, 2) and the corner rule on
            // (0, 2, 3) (edge match); the rule's first triangle on the quad half
            // by its linear map (Jacobian 4), its second on the triangle.  The
            // rotations are those of the other pairs.
            const int ntc = te.nc, nrc = re.nc;
            int pt[4], pr[4];
            for (int q = 0; q < ntc; ++q) pt[q] = (ind1 + q) % ntc;
            for (int q = 0; q < nrc; ++q) pr[q] = match == 1 ? (ind2 + 1 + nrc - q) % nrc : (ind2 + q) % nrc;
            const bool quad_test = ntc == 4;
            const int m_first = match == 1 ? 1 : 0;
            const int na = gal_npts(m_first), total_p = na + gal_npts(0);
            for (int p = lane; p < total_p; p += 32) {
                const int sub = p < na ? 0 : 1;
                const double *q = g_gal_rule + 5 * (size_t)(sub == 0 ? gal_offset(m_first) + p : gal_offset(0) + p - na);
                const double N0 = 1.0 - q[0] - q[1], N1 = q[0], N2 = q[1];
                // half (0, 1, 2): (-1,-1), (1,-1), (1,1); half (0, 2, 3): (-1,-1), (1,1), (-1,1)
                const double qu = sub == 0 ? -N0 + N1 + N2 : -N0 + N1 - N2;
                const double qv = sub == 0 ? -N0 - N1 + N2 : -N0 + N1 + N2;
                double tu, tv, ru, rv;
                if (quad_test) {
                    quad_rotate(pt, qu, qv, tu, tv);
                    tri_rotate(pr, q[2], q[3], ru, rv);
                } else {
                    tri_rotate(pt, q[2], q[3], tu, tv);
                    quad_rotate(pr, qu, qv, ru, rv);
                }
                double x[3], y[3], ntv[3], nrv[3];
                ex(te, tu, tv, x);
                enormal(te, tu, tv, ntv);
                ex(re, ru, rv, y);
                enormal(re, ru, rv, nrv);
                cd ks{0, 0}, kd{0, 0};
                kp(x, y, nrv, norm3(nrv), do_s, do_d, ks, kd);
                const double w = 4.0 * q[4] * norm3(ntv);
                sr += ks.re * w;
                si += ks.im * w;
                dr += kd.re * w;
                di += kd.im * w;
            }
        } else if (match >= 0 && te.nc == 4) {
            // matched quads (FP64, both precisions): points by the bilinear
            // maps, Jacobians and normals per point
            int pt[4], pr[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                pt[q] = match == 2 ? q : (ind1 + q) % 4;
                pr[q] = match == 2 ? q : (match == 1 ? (ind2 + 1 + 4 - q) % 4 : (ind2 + q) % 4);
            }
            const double *rule = g_galq_rule + 5 * (size_t)galq_offset(match);
            const int np = galq_npts(match);
            for (int p = lane; p < np; p += 32) {
                const double *q = rule + 5 * p;
                double u, v, x[3], y[3], nt3[3], nr3[3];
                quad_rotate(pt, q[0], q[1], u, v);
                ex(te, u, v, x);
                enormal(te, u, v, nt3);
                quad_rotate(pr, q[2], q[3], u, v);
                ex(re, u, v, y);
                enormal(re, u, v, nr3);
                cd ks{0, 0}, kd{0, 0};
                kp(x, y, nr3, norm3(nr3), do_s, do_d, ks, kd);
                const double w = q[4] * norm3(nt3);
                sr += ks.re * w;
                si += ks.im * w;
                dr += kd.re * w;
                di += kd.im * w;
            }
        } else if (match >= 0 && a.precision == 0 && !CK) {
            // FP32 regular quadrature: the matched pair's rule in FP32 too.  Both
            // rotated triangles start at the common node P, so r_vec = y - x is
            // formed from P-relative edge vectors and the rule's FP64-formed
            // coordinate differences, keeping FP32 relative accuracy as r -> 0
            int pt[3], pr[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                pt[q] = match == 2 ? q : (ind1 + q) % 3;
                pr[q] = match == 2 ? q : (match == 1 ? (ind2 + 1 + 3 - q) % 3 : (ind2 + q) % 3);
            }
            // corners relative to the test element's corner 0 in FP32 (the
            // differences in FP64); the rest of the set-up in FP32, so the
            // warp's lanes do not repeat FP64 work on the narrow FP64 pipe
            float tc[3][3], rc[3][3];
#pragma unroll
            for (int q = 0; q < 3; ++q)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    tc[q][d] = (float)(te.c[q][d] - te.c[0][d]);
                    rc[q][d] = (float)(re.c[q][d] - te.c[0][d]);
                }
            auto pick = [](const float (&c)[3][3], int idx, int d) {
                return idx == 0 ? c[0][d] : (idx == 1 ? c[1][d] : c[2][d]);
            };
            float at[3], bt[3], ar[3], br[3], nrm[3], ntv[3], nrv[3], e1[3], e2[3], f1[3], f2[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                at[d] = pick(tc, pt[1], d) - pick(tc, pt[0], d);
                bt[d] = pick(tc, pt[2], d) - pick(tc, pt[0], d);
                ar[d] = pick(rc, pr[1], d) - pick(rc, pr[0], d);
                br[d] = pick(rc, pr[2], d) - pick(rc, pr[0], d);
                e1[d] = tc[1][d] - tc[0][d];
                e2[d] = tc[2][d] - tc[0][d];
                f1[d] = rc[1][d] - rc[0][d];  // the trial element's own orientation
                f2[d] = rc[2][d] - rc[0][d];
            }
            ntv[0] = e1[1] * e2[2] - e1[2] * e2[1];
            ntv[1] = e1[2] * e2[0] - e1[0] * e2[2];
            ntv[2] = e1[0] * e2[1] - e1[1] * e2[0];
            nrv[0] = f1[1] * f2[2] - f1[2] * f2[1];
            nrv[1] = f1[2] * f2[0] - f1[0] * f2[2];
            nrv[2] = f1[0] * f2[1] - f1[1] * f2[0];
            const float Jtf = sqrtf(ntv[0] * ntv[0] + ntv[1] * ntv[1] + ntv[2] * ntv[2]);
            const float Jrf = sqrtf(nrv[0] * nrv[0] + nrv[1] * nrv[1] + nrv[2] * nrv[2]);
#pragma unroll
            for (int d = 0; d < 3; ++d) nrm[d] = nrv[d] / Jrf;
            const float wscale = Jtf * Jrf * (float)(1.0 / FOUR_PI);
            const float kf = (float)k;
            const float *rule = g_gal_rule32 + 8 * (size_t)gal_offset(match);
            const int np = gal_npts(match);
            float fsr = 0, fsi = 0, fdr = 0, fdi = 0;
            for (int p = lane; p < np; p += 32) {
                const float4 q0 = *reinterpret_cast<const float4 *>(rule + 8 * p);
                const float4 q1 = *reinterpret_cast<const float4 *>(rule + 8 * p + 4);
                // q0 = (xi1, xi2, eta1, eta2), q1 = (w, eta1 - xi1, eta2 - xi2, 0)
                float rv[3];
                for (int d = 0; d < 3; ++d) {
                    if (match == 2) rv[d] = q1.y * at[d] + q1.z * bt[d];
                    else if (match == 1) rv[d] = q1.y * at[d] + q0.w * br[d] - q0.y * bt[d];
                    else rv[d] = q0.z * ar[d] + q0.w * br[d] - q0.x * at[d] - q0.y * bt[d];
                }
                const float r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
                const float rinv = rsqrtf(r2);
                const float g = q1.x * wscale * rinv;  // w Jt Jr / (4 pi r)
                float sn = 0.0f, cs = 1.0f, kr = 0.0f;
                if (fam == FAM_HELMHOLTZ) {
                    kr = kf * (r2 * rinv);
                    sincosf(kr, &sn, &cs);
                }
                fsr += g * cs;
                fsi -= g * sn;
                const float f = -g * rinv * (rv[0] * nrm[0] + rv[1] * nrm[1] + rv[2] * nrm[2]) * rinv;
                fdr += f * (cs + kr * sn);
                fdi += f * (kr * cs - sn);
            }
            sr = fsr;
            si = fsi;
            dr = do_d ? fdr : 0.0f;
            di = do_d ? fdi : 0.0f;
        } else if (match >= 0) {
            // matched triangles: flat elements
            int pt[3], pr[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                pt[q] = match == 2 ? q : (ind1 + q) % 3;
                pr[q] = match == 2 ? q : (match == 1 ? (ind2 + 1 + 3 - q) % 3 : (ind2 + q) % 3);
            }
            double t1[3], t2[3], r1[3], r2[3], nt[3], nr[3];
            for (int d = 0; d < 3; ++d) {
                t1[d] = te.c[1][d] - te.c[0][d];
                t2[d] = te.c[2][d] - te.c[0][d];
                r1[d] = re.c[1][d] - re.c[0][d];
                r2[d] = re.c[2][d] - re.c[0][d];
            }
            cross3(t1, t2, nt);
            cross3(r1, r2, nr);
            const double Jt = norm3(nt), Jr = norm3(nr);
            const double *rule = g_gal_rule + 5 * (size_t)gal_offset(match);
            const int np = gal_npts(match);
            for (int p = lane; p < np; p += 32) {
                const double *q = rule + 5 * p;
                double u, v, x[3], y[3];
                tri_rotate(pt, q[0], q[1], u, v);
                for (int d = 0; d < 3; ++d) x[d] = te.c[0][d] + u * t1[d] + v * t2[d];
                tri_rotate(pr, q[2], q[3], u, v);
                for (int d = 0; d < 3; ++d) y[d] = re.c[0][d] + u * r1[d] + v * r2[d];
                cd ks{0, 0}, kd{0, 0};
                kp(x, y, nr, Jr, do_s, do_d, ks, kd);
                const double w = q[4] * Jt;
                sr += ks.re * w;
                si += ks.im * w;
                dr += kd.re * w;
                di += kd.im * w;
            }
        } else if (a.precision == 0 && te.nc == 3 && re.nc == 3 && !CK) {
            // unmatched close triangles under FP32 regular quadrature: the same
            // product rules in FP32, points relative to the element centres
            // (r_vec = (c_j - c_i) + (y - c_j) - (x - c_i), the first term
            // formed in FP64); the degree decision in FP32 with the FP64 guard
            // band of the classification
            double dcd[3];
            for (int d = 0; d < 3; ++d) dcd[d] = a.trial.center[3 * (int64_t)j + d] - a.test.center[3 * (int64_t)i + d];
            float c0[3];
            for (int d = 0; d < 3; ++d) c0[d] = (float)dcd[d];
            const float size_j = (float)a.trial.size[j];
            const float ratio = sqrtf(c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2]) / size_j;
            int deg_s, deg_d;
            {
                const double rx = (fabsf(ratio - 1.1f) < 1e-4f || fabsf(ratio - 1.5f) < 1e-4f || fabsf(ratio - 1.8f) < 1e-4f)
                                      ? norm3(dcd) / a.trial.size[j]
                                      : (double)ratio;
                deg_s = rx < 11.0 / 10.0 ? 6 : (rx < T_S1 ? 4 : (rx < T_S0 ? 2 : 0));
                deg_d = rx < 11.0 / 10.0 ? 8 : (rx < T_NEAR ? 6 : (rx < T_D1 ? 4 : (rx < T_D0 ? 2 : 0)));
            }
            float ti0[3], ti1[3], ti2[3], tj0[3], tj1[3], tj2[3], nrm[3], nt[3], nr[3];
            for (int d = 0; d < 3; ++d) {
                ti0[d] = (float)(te.c[0][d] - a.test.center[3 * (int64_t)i + d]);
                ti1[d] = (float)(te.c[1][d] - te.c[0][d]);
                ti2[d] = (float)(te.c[2][d] - te.c[0][d]);
                tj0[d] = (float)(re.c[0][d] - a.trial.center[3 * (int64_t)j + d]);
                tj1[d] = (float)(re.c[1][d] - re.c[0][d]);
                tj2[d] = (float)(re.c[2][d] - re.c[0][d]);
            }
            nt[0] = ti1[1] * ti2[2] - ti1[2] * ti2[1];
            nt[1] = ti1[2] * ti2[0] - ti1[0] * ti2[2];
            nt[2] = ti1[0] * ti2[1] - ti1[1] * ti2[0];
            nr[0] = tj1[1] * tj2[2] - tj1[2] * tj2[1];
            nr[1] = tj1[2] * tj2[0] - tj1[0] * tj2[2];
            nr[2] = tj1[0] * tj2[1] - tj1[1] * tj2[0];
            const float Jt = sqrtf(nt[0] * nt[0] + nt[1] * nt[1] + nt[2] * nt[2]);
            const float Jr = sqrtf(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
            for (int d = 0; d < 3; ++d) nrm[d] = nr[d] / Jr;
            const float kf = (float)k, wscale = Jt * Jr * (float)(1.0 / FOUR_PI);
            const bool one_pass = !do_s || !do_d || deg_s == deg_d;
            float fsr = 0, fsi = 0, fdr = 0, fdi = 0;
            for (int pass = 0; pass < (one_pass ? 1 : 2); ++pass) {
                const bool use_s = one_pass ? do_s : pass == 0;
                const bool use_d = one_pass ? do_d : pass == 1;
                const int deg = use_s ? deg_s : deg_d;
                const int npt = g_tri_npts[deg];
                const float *rule = TRI_F32.v + 3 * g_tri_off[deg];
                for (int p = lane; p < npt * npt; p += 32) {
                    const float *qa = rule + 3 * (p / npt), *qb = rule + 3 * (p % npt);
                    const float fxa = qa[0], fea = qa[1], wa = qa[2], fxb = qb[0], feb = qb[1], wb = qb[2];
                    float rv[3];
                    for (int d = 0; d < 3; ++d)
                        rv[d] = c0[d] + (tj0[d] + fxb * tj1[d] + feb * tj2[d]) - (ti0[d] + fxa * ti1[d] + fea * ti2[d]);
                    const float r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
                    const float rinv = rsqrtf(r2);
                    const float g = wa * wb * wscale * rinv;
                    float sn = 0.0f, cs = 1.0f, kr = 0.0f;
                    if (fam == FAM_HELMHOLTZ) {
                        kr = kf * (r2 * rinv);
                        sincosf(kr, &sn, &cs);
                    }
                    if (use_s) {
                        fsr += g * cs;
                        fsi -= g * sn;
                    }
                    if (use_d) {
                        const float f = -g * rinv * (rv[0] * nrm[0] + rv[1] * nrm[1] + rv[2] * nrm[2]) * rinv;
                        fdr += f * (cs + kr * sn);
                        fdi += f * (kr * cs - sn);
                    }
                }
            }
            sr = fsr;
            si = fsi;
            dr = fdr;
            di = fdi;
        } else {
            // unmatched close pair: product of the degree C + interval(d/D)
            // rules (up to degree 8 + 1), the SLP and DLP degrees apart
            double dc[3];
            for (int d = 0; d < 3; ++d) dc[d] = a.trial.center[3 * (int64_t)j + d] - a.test.center[3 * (int64_t)i + d];
            const double ratio = norm3(dc) / a.trial.size[j];
            const int cmax = (te.nc == 4 || re.nc == 4) ? 1 : 0;
            const int deg_s = cmax + (ratio < 11.0 / 10.0 ? 6 : (ratio < T_S1 ? 4 : (ratio < T_S0 ? 2 : 0)));
            const int deg_d =
                cmax + (ratio < 11.0 / 10.0 ? 8 : (ratio < T_NEAR ? 6 : (ratio < T_D1 ? 4 : (ratio < T_D0 ? 2 : 0))));
            const bool shared_pass = !do_s || !do_d || deg_s == deg_d;
            for (int pass = 0; pass < (shared_pass ? 1 : 2); ++pass) {
                const bool use_s = shared_pass ? do_s : pass == 0;
                const bool use_d = shared_pass ? do_d : pass == 1;
                const int deg = use_s ? deg_s : deg_d;
                const int npt = product_npts(te.nc, deg), npr = product_npts(re.nc, deg);
                for (int p = lane; p < npt * npr; p += 32) {
                    double xi, eta, wt, xr, er, wr;
                    product_point(te.nc, deg, p / npr, xi, eta, wt);
                    product_point(re.nc, deg, p % npr, xr, er, wr);
                    double x[3], y[3], n[3], nx[3];
                    ex(te, xi, eta, x);
                    enormal(te, xi, eta, nx);
                    ex(re, xr, er, y);
                    enormal(re, xr, er, n);
                    cd ks{0, 0}, kd{0, 0};
                    kp(x, y, n, norm3(n), use_s, use_d, ks, kd);
                    const double w = wt * norm3(nx) * wr;
                    if (use_s) {
                        sr += ks.re * w;
                        si += ks.im * w;
                    }
                    if (use_d) {
                        dr += kd.re * w;
                        di += kd.im * w;
                    }
                }
            }
        }
        sr = warp_sum(sr);
        si = warp_sum(si);
        dr = warp_sum(dr);
        di = warp_sum(di);
        if (lane == 0) {
            const int64_t off = (int64_t)(j - a.j0) * a.ld + i;
            if (do_s) store64(out_s + off, sr, si, a.alpha_re, a.alpha_im, a.accumulate);
            if (do_d) store64(out_d + off, dr, di, a.alpha_re, a.alpha_im, a.accumulate);
        }
    }
}

template <typename R, typename Out, int FAM>
static void launch_gal_ops(const GalArgs &a, dim3 grid, cudaStream_t s)
{
    if constexpr (FAM == FAM_HELMHOLTZ) {
        if (a.k_im != 0.0) {  // complex (lossy) wave number: separate instantiations
            if (a.ops == OP_SLP) k_galerkin_regular<R, Out, FAM, OP_SLP, false, true><<<grid, GAL_THREADS, 0, s>>>(a);
            else if (a.ops == OP_DLP) k_galerkin_regular<R, Out, FAM, OP_DLP, false, true><<<grid, GAL_THREADS, 0, s>>>(a);
            else k_galerkin_regular<R, Out, FAM, OP_SLP | OP_DLP, false, true><<<grid, GAL_THREADS, 0, s>>>(a);
            return;
        }
    }
    if constexpr (sizeof(R) == 4) {
        if (a.alpha_re == 1.0 && a.alpha_im == 0.0 && !a.accumulate) {
            if (a.ops == OP_SLP) k_galerkin_regular<R, Out, FAM, OP_SLP, true><<<grid, GAL_THREADS, 0, s>>>(a);
            else if (a.ops == OP_DLP) k_galerkin_regular<R, Out, FAM, OP_DLP, true><<<grid, GAL_THREADS, 0, s>>>(a);
            else k_galerkin_regular<R, Out, FAM, OP_SLP | OP_DLP, true><<<grid, GAL_THREADS, 0, s>>>(a);
            return;
        }
    }
    if (a.ops == OP_SLP) k_galerkin_regular<R, Out, FAM, OP_SLP><<<grid, GAL_THREADS, 0, s>>>(a);
    else if (a.ops == OP_DLP) k_galerkin_regular<R, Out, FAM, OP_DLP><<<grid, GAL_THREADS, 0, s>>>(a);
    else k_galerkin_regular<R, Out, FAM, OP_SLP | OP_DLP><<<grid, GAL_THREADS, 0, s>>>(a);
}

template <typename R, typename Out>
static void launch_gal_fam(const GalArgs &a, dim3 grid, cudaStream_t s)
{
    if (a.family == FAM_HELMHOLTZ) launch_gal_ops<R, Out, FAM_HELMHOLTZ>(a, grid, s);
    else launch_gal_ops<R, Out, FAM_LAPLACE>(a, grid, s);
}

cudaError_t launch_galerkin_regular(const GalArgs &a, cudaStream_t s)
{
    const int ncols = a.j1 - a.j0;
    if (a.test.n == 0 || ncols <= 0) return cudaSuccess;
    dim3 grid((a.test.n + GAL_THREADS - 1) / GAL_THREADS, (ncols + GAL_COLS - 1) / GAL_COLS);
    if (a.precision == 0) {
        if (a.dtype == 0) launch_gal_fam<float, float2>(a, grid, s);
        else launch_gal_fam<float, double2>(a, grid, s);
    } else {
        if (a.dtype == 0) launch_gal_fam<double, float2>(a, grid, s);
        else launch_gal_fam<double, double2>(a, grid, s);
    }
    return cudaGetLastError();
}

cudaError_t launch_galerkin_near(const GalArgs &a, const NearList &near, int extra, int64_t max_items, cudaStream_t s)
{
    if (max_items <= 0) return cudaSuccess;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // two 4-warp blocks per SM: the kernel runs beside the regular one and
    // must leave it most of the register file
    const int64_t want = (max_items + GAL_WARPS - 1) / GAL_WARPS;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, 2 * (int64_t)sms));
    if (a.family == FAM_HELMHOLTZ && a.k_im != 0.0) {
        if (a.dtype == 0) k_galerkin_near<float2, true><<<blocks, GAL_WARPS * 32, 0, s>>>(a, near, extra);
        else k_galerkin_near<double2, true><<<blocks, GAL_WARPS * 32, 0, s>>>(a, near, extra);
    } else {
        if (a.dtype == 0) k_galerkin_near<float2, false><<<blocks, GAL_WARPS * 32, 0, s>>>(a, near, extra);
        else k_galerkin_near<double2, false><<<blocks, GAL_WARPS * 32, 0, s>>>(a, near, extra);
    }
    return cudaGetLastError();
}

template <typename Out>
__global__ void k_add_mass(int n, const double *pts64, double are, double aim, Out *out, int64_t ld)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // w J of the element's one-point rule (parity 0, level 0): its area,
    // exact for flat triangles and bilinear quads
    const double area = pts64[8 * ((int64_t)i * 2 * SLOTS) + 3];
    Out o = out[(int64_t)i * ld + i];
    o.x += are * area;
    o.y += aim * area;
    out[(int64_t)i * ld + i] = o;
}

cudaError_t launch_add_mass(int n, const double *pts64, double are, double aim, int dtype, void *out, int64_t ld,
                            cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const int t = 256, b = (n + t - 1) / t;
    if (dtype == 0) k_add_mass<float2><<<b, t, 0, s>>>(n, pts64, are, aim, (float2 *)out, ld);
    else k_add_mass<double2><<<b, t, 0, s>>>(n, pts64, are, aim, (double2 *)out, ld);
    return cudaGetLastError();
}

}  // namespace nihu
