// Shared device definitions of the GB300 collocation BEM library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "quad_rules.h"

namespace nihu {

constexpr double PI = 3.14159265358979323846264338327950288;
constexpr double FOUR_PI = 4.0 * PI;
constexpr int TRIA_1_ID = 32303;
constexpr int QUAD_1_ID = 32404;
constexpr int FAM_HELMHOLTZ = 0;
constexpr int FAM_LAPLACE = 1;
constexpr int OP_SLP = 1;
constexpr int OP_DLP = 2;
constexpr int OP_DLPT = 4;  // transposed DLP (normal derivative at the collocation point)
constexpr int OP_HSP = 8;   // hypersingular operator

// Quadrature levels of the regular path.  Level l of a trial element uses the
// rule of degree C + 2l' where C is the field complexity and 2l' the distance
// interval (nihu/library/distance_kernel_intervals.hpp:117-139): level 0 =
// interval 0, level 1 = interval 2, level 2 = interval 4.  Intervals 6 and 8
// only occur for d/D < 1.5, which is always the nearly singular path.
constexpr int NUM_LEVELS = 3;
constexpr int SLOTS = 14;            // 1 + 4 + 9 points at most
__host__ __device__ constexpr int level_slot0(int l) { return l == 0 ? 0 : (l == 1 ? 1 : 5); }

// squared distance-ratio thresholds (x = d/D, strict '<'), reference doubles
// 1.5 (nearly singular), SLP 1.8 / 9.1, DLP 2.8 / 15.8
constexpr double T_NEAR = 1.5;
constexpr double T_S1 = 18.0 / 10.0, T_S0 = 91.0 / 10.0;
constexpr double T_D1 = 28.0 / 10.0, T_D0 = 158.0 / 10.0;
// HSP (1/r^3 far field): degree 6 / 4 / 2 below 1.9 / 3.6 / 22.3, else 0
// (nihu/library/distance_kernel_intervals.hpp:117-154 for the 1/r^3 kernels)
constexpr double T_H2 = 19.0 / 10.0, T_H1 = 36.0 / 10.0, T_H0 = 223.0 / 10.0;

// Per-element device records of a mesh (structure of arrays).
struct DevMesh {
    int n = 0;              // elements
    int has_tria = 0, has_quad = 0;
    // FP64 geometry
    double *corners = nullptr;  // [n][12] (x,y,z) x 4 corners; 4th unused for trias
    double *center = nullptr;   // [n][3]
    double *size = nullptr;     // [n] mean edge length
    int8_t *nc = nullptr;       // [n] 3 or 4
    // FP32 geometry for the regular kernel
    float4 *chi = nullptr;      // [n] (hi(cx), hi(cy), hi(cz), 1/D^2)
    float4 *clo = nullptr;      // [n] (lo(cx), lo(cy), lo(cz), field complexity)
    float4 *p0 = nullptr;       // [n] level-0 point: (w*J, unit normal)
    // regular quadrature points per element and test-complexity parity:
    // [n][2][SLOTS][2] float4 : (y, w*J), (unit normal, 0) -- FP32
    float4 *pts32 = nullptr;
    // the same in FP64: [n][2][SLOTS][8] doubles (y, w*J, unit normal, 0)
    double *pts64 = nullptr;
    // triangles: the 42 points of the degree-14 rule used by the nearly
    // singular dynamic part, (y, w*J) in FP64; [n][42] (unused for quads)
    struct Pt4 *dyn42 = nullptr;
    // corner node indices (-1 for the 4th of a triangle): element adjacency
    // of the Galerkin singular quadratures
    int4 *nid = nullptr;
    // triangles: the plane frame of the nearly singular static part (rows
    // T0, T1, T2: first side, in-plane normal to it, unit normal) and the
    // corners' in-plane coordinates relative to corner 0, [n][16] doubles
    // (T row-major, then (u, v) of corners 0..2, one unused)
    double *frame = nullptr;
};

// number of points of a regular level for (trial corners, test complexity)
__host__ __device__ inline int level_npts(int trial_nc, int test_c, int level)
{
    if (trial_nc == 4) return level == 0 ? 1 : (level == 1 ? 4 : 9);
    if (test_c == 0) return level == 0 ? 1 : (level == 1 ? 3 : 6);
    return level == 0 ? 1 : (level == 1 ? 4 : 7);
}

// sin and cos of x (radians) in FP32: x less the nearest multiple n of 2 pi,
// formed with one fused multiply-add (Cody-Waite reduction with a one-term
// constant: the FP32 rounding of 2 pi adds |n| x 1.75e-7 rad), leaves about
// [-pi, pi] for the hardware approximation (absolute error about 4e-7 there)
__device__ __forceinline__ void sincos_reduced(float x, float &s, float &c)
{
    const float n = rintf(x * 0.159154943091895335769f);
    __sincosf(fmaf(-6.28318530717958647692f, n, x), &s, &c);
}

// one quadrature point of the SLP (weight ws) and DLP (weight wd) kernels at
// r_vec = (rx, ry, rz) with trial weight w J and unit normal n, sharing 1/r and
// one sincos (Helmholtz: e^{-ikr} convention)
template <int FAM, typename R>
__device__ __forceinline__ void eval_point(R rx, R ry, R rz, R wj, R nx, R ny, R nz, R k, R ws, R wd, R &sr,
                                           R &si, R &dr, R &di)
{
    constexpr R INV4PI = R(1.0 / (4.0 * 3.14159265358979323846));
    R r2 = rx * rx + ry * ry + rz * rz;
    R rinv;
    if constexpr (sizeof(R) == 4) rinv = rsqrtf(r2);
    else rinv = rsqrt(r2);
    R g = wj * rinv * INV4PI;
    R rdn = (rx * nx + ry * ny + rz * nz) * rinv;
    if constexpr (FAM == FAM_HELMHOLTZ) {
        R kr = k * (r2 * rinv);
        R s, c;
        if constexpr (sizeof(R) == 4) sincos_reduced(kr, s, c);
        else sincos(kr, &s, &c);
        // SLP: G = e^{-ikr}/(4 pi r) = (c - i s)/(4 pi r)
        R gs = g * ws;
        sr += gs * c;
        si -= gs * s;
        // DLP: dG/dr (r.n)/r = -(1 + ikr) e^{-ikr} / (4 pi r^2) * (r.n)/r
        R f = -g * rinv * rdn * wd;
        dr += f * (c + kr * s);
        di += f * (kr * c - s);
    } else {
        sr += g * ws;
        dr -= g * rinv * rdn * wd;
    }
}

// eval_point for a complex (lossy) wave number k + i ki:
// e^{-i(k + i ki) r} = e^{ki r} (cos kr - i sin kr) and 1 + i(k + i ki) r =
// (1 - ki r) + i kr, so the SLP is damped by e^{ki r} and the DLP factor
// -(1 + ikr) e^{-ikr} takes 1 - ki r in place of 1
// (nihu/library/helmholtz_kernel.hpp:42-54,180-195 with a complex wave number)
template <typename R>
__device__ __forceinline__ void eval_point_ck(R rx, R ry, R rz, R wj, R nx, R ny, R nz, R k, R ki, R ws, R wd, R &sr,
                                              R &si, R &dr, R &di)
{
    constexpr R INV4PI = R(1.0 / (4.0 * 3.14159265358979323846));
    R r2 = rx * rx + ry * ry + rz * rz;
    R rinv;
    if constexpr (sizeof(R) == 4) rinv = rsqrtf(r2);
    else rinv = rsqrt(r2);
    const R g = wj * rinv * INV4PI;
    const R rdn = (rx * nx + ry * ny + rz * nz) * rinv;
    const R r = r2 * rinv;
    const R kr = k * r;
    R s, c, damp;
    if constexpr (sizeof(R) == 4) {
        sincos_reduced(kr, s, c);
        damp = expf(ki * r);
    } else {
        sincos(kr, &s, &c);
        damp = exp(ki * r);
    }
    c *= damp;
    s *= damp;
    const R gs = g * ws;
    sr += gs * c;
    si -= gs * s;
    const R f = -g * rinv * rdn * wd;
    const R a1 = R(1) - ki * r;
    dr += f * (a1 * c + kr * s);
    di += f * (kr * c - a1 * s);
}

struct cd { double re, im; };

// four doubles in one 32-byte aligned record (point + weight)
struct __align__(32) Pt4 {
    double x, y, z, w;
};

__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd cscale(cd a, double s) { return {a.re * s, a.im * s}; }

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace nihu
