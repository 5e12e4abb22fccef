// C++ front-end check (driven by tests/test_gpu_cpp_shim.py): the collocation
// sequence of nihu/test/matlab/acoustic_bem.mex.cpp:30-50 written against
// include/nihu_gb300/nihu.hpp, plus the pulsating-sphere solve of
// nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:28-76.
//
// usage: test_shim <mesh.bin> <k> <out.bin>
//   mesh.bin: int64 n_nodes, int64 n_elems, n_nodes*3 doubles, n_elems*5 int32
//   out.bin : Ls, Ms (n*n complex128 each, column-major), p (n complex128),
//             then the Burton-Miller matrices Gs, Hs and pressure p_bm of
//             nihu/applications/helmholtz/helmholtz_3d_coll.cpp:36-120 (BM defined),
//             then the Galerkin L, M, I and pressure of
//             nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:40-70
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>

#include "nihu_gb300/nihu.hpp"

using namespace nihu_gb300;
typedef std::complex<double> C;

struct host_mat {
    std::vector<double> d;
    int64_t r, c;
    int64_t rows() const { return r; }
    int64_t cols() const { return c; }
    double operator()(int64_t i, int64_t j) const { return d[(size_t)(i * c + j)]; }
};

int main(int argc, char **argv)
{
    if (argc < 4) {
        std::fprintf(stderr, "usage: test_shim mesh.bin k out.bin\n");
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int64_t nn = 0, ne = 0;
    in.read((char *)&nn, 8);
    in.read((char *)&ne, 8);
    host_mat nodes{std::vector<double>((size_t)nn * 3), nn, 3};
    in.read((char *)nodes.d.data(), nn * 3 * 8);
    std::vector<int32_t> el((size_t)ne * 5);
    in.read((char *)el.data(), ne * 5 * 4);
    host_mat elems{std::vector<double>(el.begin(), el.end()), ne, 5};
    if (!in) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    const double k = std::atof(argv[2]);

    try {
        auto surf_mesh = create_mesh(nodes, elems, tria_1_tag(), quad_1_tag());
        auto const &surf_sp = constant_view(surf_mesh);
        const int64_t n = surf_sp.get_num_dofs();
        dense_matrix<C> Ls(n, n), Ms(n, n);
        auto I = identity_integral_operator();
        auto Lop = create_integral_operator(helmholtz_3d_SLP_kernel<double>(k));
        auto Mop = create_integral_operator(helmholtz_3d_DLP_kernel<double>(k));
        Ls << dirac(surf_sp) * Lop[surf_sp];
        Ms << dirac(surf_sp) * Mop[surf_sp];
        Ms << dirac(surf_sp) * (-.5 * I)[surf_sp];

        // (M - I/2) p = L q with q = 1 (pulsating sphere)
        std::vector<C> q((size_t)n, C(1.0, 0.0)), rhs((size_t)n, 0.0);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < n; ++i) rhs[(size_t)i] += Ls(i, j) * q[(size_t)j];
        std::vector<C> p = lu_solve(Ms, rhs);

        // error behaviour: a result of the wrong size is rejected
        bool threw = false;
        try {
            dense_matrix<C> bad(n, n + 1);
            bad << dirac(surf_sp) * Lop[surf_sp];
        } catch (std::invalid_argument const &) {
            threw = true;
        }
        if (!threw) {
            std::fprintf(stderr, "size mismatch not rejected\n");
            return 1;
        }

        // Burton-Miller: Gs << G + alpha Ht + alpha/2 I, Hs << alpha D - I/2 + H, alpha = -i/k
        const C alpha(0.0, -1.0 / k);
        auto Htop = create_integral_operator(helmholtz_3d_DLPt_kernel<double>(k));
        auto Dop = create_integral_operator(helmholtz_3d_HSP_kernel<double>(k));
        dense_matrix<C> Gs(n, n), Hs(n, n);
        Gs << dirac(surf_sp) * Lop[surf_sp];
        Gs << dirac(surf_sp) * (alpha * Htop)[surf_sp];
        Gs << dirac(surf_sp) * (alpha / 2. * I)[surf_sp];
        Hs << dirac(surf_sp) * (alpha * Dop)[surf_sp];
        Hs << dirac(surf_sp) * (-.5 * I)[surf_sp];
        Hs << dirac(surf_sp) * Mop[surf_sp];
        std::vector<C> rhs_bm((size_t)n, 0.0);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < n; ++i) rhs_bm[(size_t)i] += Gs(i, j) * q[(size_t)j];
        std::vector<C> p_bm = gmres(Hs, rhs_bm, 1e-10, 50, 1000);

        // Galerkin: I, L, M << test_space * Op[trial_space] with the function space as test space
        dense_matrix<C> Lg(n, n), Mg(n, n), Ig(n, n);
        Ig << surf_sp * I[surf_sp];
        Lg << surf_sp * Lop[surf_sp];
        Mg << surf_sp * Mop[surf_sp];
        dense_matrix<C> Ag(n, n);
        std::vector<C> rhs_g((size_t)n, 0.0);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < n; ++i) {
                Ag(i, j) = Mg(i, j) - 0.5 * Ig(i, j);
                rhs_g[(size_t)i] += Lg(i, j) * q[(size_t)j];
            }
        std::vector<C> p_g = lu_solve(Ag, rhs_g);

        std::ofstream out(argv[3], std::ios::binary);
        out.write((const char *)Ls.data(), n * n * 16);
        out.write((const char *)Ms.data(), n * n * 16);
        out.write((const char *)p.data(), n * 16);
        out.write((const char *)Gs.data(), n * n * 16);
        out.write((const char *)Hs.data(), n * n * 16);
        out.write((const char *)p_bm.data(), n * 16);
        out.write((const char *)Lg.data(), n * n * 16);
        out.write((const char *)Mg.data(), n * n * 16);
        out.write((const char *)Ig.data(), n * n * 16);
        out.write((const char *)p_g.data(), n * 16);
        C pa = -1.0 / (1.0 + C(0.0, k));
        double err = 0.0;
        for (auto v : p) err = std::max(err, std::abs(v - pa) / std::abs(pa));
        std::printf("n=%lld k=%g max|p - p_analytic|/|p_analytic| = %.3e\n", (long long)n, k, err);
    } catch (std::exception const &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
