// Per-pair dispatch of the collocational assembly: self, nearly singular, or
// regular with the quadrature levels of SLP and DLP.
//
// The reference decides in FP64 (nihu/core/double_integral.hpp:543-639):
//   self   : same mesh and same element id (nihu/core/element_match.hpp:84-112)
//   near   : d / D_j < 1.5, d = |c_i - c_j|, D_j = trial mean edge length
//            (nihu/library/helmholtz_nearly_singular_integrals.hpp:234-246)
//   regular: degree = C + interval(d / D_j), strict '<' thresholds
//            (nihu/core/complexity_estimator.hpp:69-75, nihu/tmp/interval.hpp:173-185)
// Here the ratio is first classified in FP32 from hi/lo split centres; a pair
// whose squared ratio lies within a relative band of 1e-5 of any threshold is
// re-classified in FP64 exactly as the reference does, so the outcome is the
// FP64 outcome for every pair.
#pragma once

#include "common.cuh"

namespace nihu {

constexpr int KIND_REGULAR = 0;
constexpr int KIND_NEAR = 1;
constexpr int KIND_SELF = 2;

__device__ __forceinline__ int class_code32(float q)
{
    if (q < 2.25f) return -1;
    int ls = q >= 82.81f ? 0 : (q >= 3.24f ? 1 : 2);
    int ld = q >= 249.64f ? 0 : (q >= 7.84f ? 1 : 2);
    return ls * 3 + ld;
}

__device__ __forceinline__ int class_code64(double ratio)
{
    if (ratio < T_NEAR) return -1;
    int ls = ratio < T_S1 ? 2 : (ratio < T_S0 ? 1 : 0);
    int ld = ratio < T_D1 ? 2 : (ratio < T_D0 ? 1 : 0);
    return ls * 3 + ld;
}

// Returns the kind; for regular pairs ls / ld receive the SLP / DLP level.
// dx receives c_j - c_i in FP32 (hi/lo accurate).
__device__ __forceinline__ int classify_pair(float4 ih, float4 il, float4 jh, float4 jl, int i, int j,
                                             const double *__restrict__ test_center,
                                             const double *__restrict__ trial_center,
                                             const double *__restrict__ trial_size, int same_mesh,
                                             int &ls, int &ld, float &dx, float &dy, float &dz)
{
    dx = (jh.x - ih.x) + (jl.x - il.x);
    dy = (jh.y - ih.y) + (jl.y - il.y);
    dz = (jh.z - ih.z) + (jl.z - il.z);
    if (same_mesh && i == j) { ls = ld = 0; return KIND_SELF; }
    float q = (dx * dx + dy * dy + dz * dz) * jh.w;
    int lo = class_code32(q * (1.0f - 1e-5f));
    int hi = class_code32(q * (1.0f + 1e-5f));
    int code = lo;
    if (lo != hi) {
        double ex = trial_center[3 * (int64_t)j] - test_center[3 * (int64_t)i];
        double ey = trial_center[3 * (int64_t)j + 1] - test_center[3 * (int64_t)i + 1];
        double ez = trial_center[3 * (int64_t)j + 2] - test_center[3 * (int64_t)i + 2];
        code = class_code64(sqrt(ex * ex + ey * ey + ez * ez) / trial_size[j]);
    }
    if (code < 0) { ls = ld = 0; return KIND_NEAR; }
    ls = code / 3;
    ld = code % 3;
    return KIND_REGULAR;
}

// Burton-Miller dispatch: the SLP, DLP (= DLPt) and HSP levels of a regular
// pair, HSP level 3 being the degree-6 rule of 1.5 <= d/D < 1.9
// (nihu/library/distance_kernel_intervals.hpp:143-154).  Code (ls*3+ld)*4+lh.
__device__ __forceinline__ int bm_code32(float q)
{
    if (q < 2.25f) return -1;
    int ls = q >= 82.81f ? 0 : (q >= 3.24f ? 1 : 2);
    int ld = q >= 249.64f ? 0 : (q >= 7.84f ? 1 : 2);
    int lh = q >= 497.29f ? 0 : (q >= 12.96f ? 1 : (q >= 3.61f ? 2 : 3));
    return (ls * 3 + ld) * 4 + lh;
}

__device__ __forceinline__ int bm_code64(double ratio)
{
    if (ratio < T_NEAR) return -1;
    int ls = ratio < T_S1 ? 2 : (ratio < T_S0 ? 1 : 0);
    int ld = ratio < T_D1 ? 2 : (ratio < T_D0 ? 1 : 0);
    int lh = ratio < T_H2 ? 3 : (ratio < T_H1 ? 2 : (ratio < T_H0 ? 1 : 0));
    return (ls * 3 + ld) * 4 + lh;
}

// classify_pair with the HSP level as well (same FP64 guard band)
__device__ __forceinline__ int classify_bm(float4 ih, float4 il, float4 jh, float4 jl, int i, int j,
                                           const double *__restrict__ test_center,
                                           const double *__restrict__ trial_center,
                                           const double *__restrict__ trial_size, int same_mesh, int &ls, int &ld,
                                           int &lh, float &dx, float &dy, float &dz)
{
    dx = (jh.x - ih.x) + (jl.x - il.x);
    dy = (jh.y - ih.y) + (jl.y - il.y);
    dz = (jh.z - ih.z) + (jl.z - il.z);
    ls = ld = lh = 0;
    if (same_mesh && i == j) return KIND_SELF;
    float q = (dx * dx + dy * dy + dz * dz) * jh.w;
    int lo = bm_code32(q * (1.0f - 1e-5f));
    int hi = bm_code32(q * (1.0f + 1e-5f));
    int code = lo;
    if (lo != hi) {
        double ex = trial_center[3 * (int64_t)j] - test_center[3 * (int64_t)i];
        double ey = trial_center[3 * (int64_t)j + 1] - test_center[3 * (int64_t)i + 1];
        double ez = trial_center[3 * (int64_t)j + 2] - test_center[3 * (int64_t)i + 2];
        code = bm_code64(sqrt(ex * ex + ey * ey + ez * ez) / trial_size[j]);
    }
    if (code < 0) return KIND_NEAR;
    lh = code % 4;
    ls = code / 12;
    ld = (code / 4) % 3;
    return KIND_REGULAR;
}

}  // namespace nihu
