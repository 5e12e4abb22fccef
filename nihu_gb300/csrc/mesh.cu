// Element geometry on the GPU: centres, sizes, normals and the regular
// quadrature points of every element, computed once per mesh.
#include "kernels.h"
#include "planar.cuh"

namespace nihu {

// one thread per element
__global__ void k_mesh_geometry(const double *__restrict__ nodes, int64_t n_nodes, const int32_t *__restrict__ elems,
                                int n, int cols, DevMesh m, int *bad, unsigned long long *size_max)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int32_t *row = elems + (int64_t)e * cols;
    int nc = row[0] == TRIA_1_ID ? 3 : (row[0] == QUAD_1_ID ? 4 : 0);
    if (nc == 0 || cols < 1 + nc) { atomicCAS(bad, 0, e + 1); return; }
    Elem64 el;
    el.nc = nc;
    for (int a = 0; a < 4; ++a) {
        int nd = a < nc ? row[1 + a] : row[nc];  // 4th corner of a triangle repeats the 3rd
        if (nd < 0 || nd >= n_nodes) { atomicCAS(bad, 0, e + 1); return; }
        for (int d = 0; d < 3; ++d) el.c[a][d] = nodes[3 * (int64_t)nd + d];
    }
    m.nc[e] = (int8_t)nc;
    m.nid[e] = make_int4(row[1], row[2], row[3], nc == 4 ? row[4] : -1);
    double *cdst = m.corners + 12 * (int64_t)e;
    for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) cdst[3 * a + d] = el.c[a][d];

    // centre = x(domain centre), size = mean edge length (nihu/core/element.hpp:271-292)
    double xi, eta, cen[3];
    domain_center(nc, xi, eta);
    ex(el, xi, eta, cen);
    double s = 0.0;
    for (int ed = 0; ed < nc; ++ed) {
        double a0, a1, b0, b1, x0[3], x1[3];
        domain_corner(nc, ed, a0, a1);
        domain_corner(nc, (ed + 1) % nc, b0, b1);
        ex(el, a0, a1, x0);
        ex(el, b0, b1, x1);
        double dv[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
        s += norm3(dv);
    }
    double size = s / nc;
    for (int d = 0; d < 3; ++d) m.center[3 * (int64_t)e + d] = cen[d];
    m.size[e] = size;
    atomicMax(size_max, (unsigned long long)__double_as_longlong(size));  // positive doubles order as integers

    // FP32 centre split into hi + lo parts so that centre differences keep
    // ~FP32 relative accuracy however close two elements are
    float hx = (float)cen[0], hy = (float)cen[1], hz = (float)cen[2];
    m.chi[e] = make_float4(hx, hy, hz, (float)(1.0 / (size * size)));
    m.clo[e] = make_float4((float)(cen[0] - (double)hx), (float)(cen[1] - (double)hy), (float)(cen[2] - (double)hz),
                           nc == 4 ? 1.0f : 0.0f);

    // plane frame of the nearly singular static part (triangles): the
    // frame of plane_local_frame, which depends on the element only, and the
    // corners' in-plane coordinates relative to corner 0
    if (nc == 3) {
        double loc[4][2], z, T[3][3];
        plane_local_frame(el, el.c[0], loc, z, T);
        double *fr = m.frame + 16 * (int64_t)e;
        for (int r = 0; r < 3; ++r)
            for (int d = 0; d < 3; ++d) fr[3 * r + d] = T[r][d];
        for (int a = 0; a < 3; ++a) {
            fr[9 + 2 * a] = loc[a][0];
            fr[10 + 2 * a] = loc[a][1];
        }
        fr[15] = 0.0;
    }

    // degree-14 points of the nearly singular dynamic part (triangles)
    if (nc == 3) {
        double nv[3];
        enormal(el, 1.0 / 3.0, 1.0 / 3.0, nv);
        const double J = norm3(nv);
        for (int p = 0; p < 42; ++p) {
            double qx, qe, w, y[3];
            tri_pt(14, p, qx, qe, w);
            ex(el, qx, qe, y);
            m.dyn42[42 * (int64_t)e + p] = Pt4{y[0], y[1], y[2], w * J};
        }
    }

    // regular quadrature points for both test-complexity parities
    for (int par = 0; par < 2; ++par) {
        for (int lev = 0; lev < NUM_LEVELS; ++lev) {
            int np = level_npts(nc, par, lev);
            for (int p = 0; p < np; ++p) {
                double qx, qe, w;
                if (nc == 3) {
                    tri_pt(par + 2 * lev, p, qx, qe, w);
                } else {
                    int ng = lev + 1;  // degree 1 + 2 lev -> (1 + 2 lev)/2 + 1 points
                    double w0, w1;
                    gauss_pt(ng, p / ng, qx, w0);
                    gauss_pt(ng, p % ng, qe, w1);
                    w = w0 * w1;
                }
                double y[3], nv[3];
                ex(el, qx, qe, y);
                enormal(el, qx, qe, nv);
                double J = norm3(nv);
                double wj = w * J;
                int slot = level_slot0(lev) + p;
                int64_t base = ((int64_t)e * 2 + par) * SLOTS + slot;
                // FP32 points relative to the element centre: r = (c_j - x) + (y - c_j)
                // keeps FP32 relative accuracy of r however far the mesh is from the origin
                m.pts32[2 * base] = make_float4((float)(y[0] - cen[0]), (float)(y[1] - cen[1]), (float)(y[2] - cen[2]),
                                                (float)wj);
                m.pts32[2 * base + 1] = make_float4((float)(nv[0] / J), (float)(nv[1] / J), (float)(nv[2] / J), 0.0f);
                double *d64 = m.pts64 + 8 * base;
                d64[0] = y[0]; d64[1] = y[1]; d64[2] = y[2]; d64[3] = wj;
                d64[4] = nv[0] / J; d64[5] = nv[1] / J; d64[6] = nv[2] / J; d64[7] = 0.0;
                if (par == 0 && lev == 0)
                    m.p0[e] = make_float4((float)wj, (float)(nv[0] / J), (float)(nv[1] / J), (float)(nv[2] / J));
            }
        }
    }
}

cudaError_t launch_mesh_geometry(const double *nodes, int64_t n_nodes, const int32_t *elems, int n, int cols,
                                 DevMesh m, int *bad, unsigned long long *size_max, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    int threads = 128;
    k_mesh_geometry<<<(n + threads - 1) / threads, threads, 0, s>>>(nodes, n_nodes, elems, n, cols, m, bad, size_max);
    return cudaGetLastError();
}

}  // namespace nihu
