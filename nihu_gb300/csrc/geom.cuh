// FP64 element geometry and quadrature tables on the device.
#pragma once

#include "common.cuh"

namespace nihu {

// Quadrature tables in global memory (lanes of a warp read different points,
// which constant memory would serialise).  One copy per translation unit.
static __device__ const double g_gauss[NIHU_GAUSS_DATA_LEN] = NIHU_GAUSS_DATA;
static __device__ const int g_gauss_off[NIHU_GAUSS_MAX_N] = NIHU_GAUSS_OFFSETS;
static __device__ const double g_tri[NIHU_TRI_DATA_LEN] = NIHU_TRI_DATA;
static __device__ const int g_tri_npts[15] = NIHU_TRI_NPTS;
static __device__ const int g_tri_off[15] = NIHU_TRI_OFFSETS;

// node and weight of point a of the n-point Gauss-Legendre rule
__device__ __forceinline__ void gauss_pt(int n, int a, double &x, double &w)
{
    const double *g = g_gauss + 2 * (g_gauss_off[n - 1] + a);
    x = g[0];
    w = g[1];
}

// point p of the Dunavant rule of the given degree (weights sum to 1/2)
__device__ __forceinline__ void tri_pt(int degree, int p, double &xi, double &eta, double &w)
{
    const double *q = g_tri + 3 * (g_tri_off[degree] + p);
    xi = q[0];
    eta = q[1];
    w = q[2];
}

struct Elem64 {
    int nc;
    double c[4][3];
};

__device__ __forceinline__ void load_elem(const DevMesh &m, int e, Elem64 &el)
{
    el.nc = m.nc[e];
    const double *src = m.corners + 12 * (int64_t)e;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) el.c[a][d] = src[3 * a + d];
}

// shape functions: linear triangle on (0,0),(1,0),(0,1); bilinear quad on
// (-1,-1),(1,-1),(1,1),(-1,1) (nihu/library/lib_shape.hpp, lib_domain.cpp:59-94)
__device__ __forceinline__ void shape(int nc, double xi, double eta, double N[4])
{
    if (nc == 3) {
        N[0] = 1.0 - xi - eta; N[1] = xi; N[2] = eta; N[3] = 0.0;
    } else {
        N[0] = (1.0 - xi) * (1.0 - eta) * 0.25;
        N[1] = (1.0 + xi) * (1.0 - eta) * 0.25;
        N[2] = (1.0 + xi) * (1.0 + eta) * 0.25;
        N[3] = (1.0 - xi) * (1.0 + eta) * 0.25;
    }
}

__device__ __forceinline__ void dshape(int nc, double xi, double eta, double dN[4][2])
{
    if (nc == 3) {
        dN[0][0] = -1.0; dN[0][1] = -1.0; dN[1][0] = 1.0; dN[1][1] = 0.0;
        dN[2][0] = 0.0;  dN[2][1] = 1.0;  dN[3][0] = 0.0; dN[3][1] = 0.0;
    } else {
        dN[0][0] = -(1.0 - eta) * 0.25; dN[0][1] = -(1.0 - xi) * 0.25;
        dN[1][0] = (1.0 - eta) * 0.25;  dN[1][1] = -(1.0 + xi) * 0.25;
        dN[2][0] = (1.0 + eta) * 0.25;  dN[2][1] = (1.0 + xi) * 0.25;
        dN[3][0] = -(1.0 + eta) * 0.25; dN[3][1] = (1.0 - xi) * 0.25;
    }
}

__device__ __forceinline__ void ex(const Elem64 &e, double xi, double eta, double x[3])
{
    double N[4];
    shape(e.nc, xi, eta, N);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int a = 0; a < e.nc; ++a) s += N[a] * e.c[a][d];
        x[d] = s;
    }
}

__device__ __forceinline__ void edx(const Elem64 &e, double xi, double eta, double a[3], double b[3])
{
    double dN[4][2];
    dshape(e.nc, xi, eta, dN);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double s0 = 0.0, s1 = 0.0;
        for (int c = 0; c < e.nc; ++c) { s0 += dN[c][0] * e.c[c][d]; s1 += dN[c][1] * e.c[c][d]; }
        a[d] = s0; b[d] = s1;
    }
}

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ double norm3(const double a[3]) { return sqrt(dot3(a, a)); }

// unnormalised normal dx/dxi x dx/deta (nihu/core/element.hpp:503-515)
__device__ __forceinline__ void enormal(const Elem64 &e, double xi, double eta, double n[3])
{
    double a[3], b[3];
    edx(e, xi, eta, a, b);
    cross3(a, b, n);
}

__device__ __forceinline__ void domain_corner(int nc, int i, double &xi, double &eta)
{
    if (nc == 3) {
        xi = (i == 1) ? 1.0 : 0.0;
        eta = (i == 2) ? 1.0 : 0.0;
    } else {
        xi = (i == 1 || i == 2) ? 1.0 : -1.0;
        eta = (i >= 2) ? 1.0 : -1.0;
    }
}

__device__ __forceinline__ void domain_center(int nc, double &xi, double &eta)
{
    if (nc == 3) { xi = 1.0 / 3.0; eta = 1.0 / 3.0; }
    else { xi = 0.0; eta = 0.0; }
}

}  // namespace nihu
