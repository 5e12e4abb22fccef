// nihu_gb300/nihu.hpp -- C++ front end shaped like NiHu's integral-operator API
// for the GB300 collocation BEM library (header only, over include/nihu_gb300.h).
//
// NiHu user code for the collocational path, e.g.
// (nihu/test/matlab/acoustic_bem.mex.cpp:30-50)
//
//     auto mesh = create_mesh(nodes, elements, tria_1_tag());
//     auto const &sp = constant_view(mesh);
//     auto Lop = create_integral_operator(helmholtz_3d_SLP_kernel<double>(k));
//     Ls << dirac(sp) * Lop[sp];
//     Ms << dirac(sp) * (-.5 * I)[sp];
//
// compiles against this header with `using namespace nihu_gb300;` and runs on
// the GPU.  Semantics kept from the reference:
//  * `<<` adds into the caller's (zeroed) matrix (nihu/core/weighted_residual.hpp:197-206,
//    block "+=" nihu/util/matrix_block.hpp)
//  * row = test DOF = test element id, column = trial DOF, column-major storage
//  * the same mesh object for test and trial enables the singular self terms
//    (nihu/core/integral_transform.hpp:156)
//  * scaled operators multiply the block (nihu/core/integral_operator.hpp:159-167)
//  * errors: std::out_of_range / std::runtime_error / std::invalid_argument
// A result type is any matrix with data(), rows(), cols() and column-major
// complex (or, for Laplace, real) storage: Eigen dynamic matrices qualify, as
// does nihu_gb300::dense_matrix below.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../nihu_gb300.h"

namespace nihu_gb300 {

// ------------------------------------------------------------------ errors

inline void check(nihu_gb_ctx *ctx, nihu_gb_status st)
{
    if (st == NIHU_GB_OK) return;
    std::string msg = ctx ? nihu_gb_last_error(ctx) : "nihu_gb300: no context";
    switch (st) {
    case NIHU_GB_ERR_OUT_OF_RANGE: throw std::out_of_range(msg);
    case NIHU_GB_ERR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
    default: throw std::runtime_error(msg);
    }
}

// ------------------------------------------------------------------ context

class context {
public:
    explicit context(int device = 0, size_t hbm_budget_bytes = 0)
    {
        nihu_gb_ctx *c = nullptr;
        nihu_gb_status st = nihu_gb_ctx_create(device, nullptr, hbm_budget_bytes, &c);
        if (st != NIHU_GB_OK) throw std::runtime_error("nihu_gb300: cannot create a GPU context");
        h_.reset(c, nihu_gb_ctx_destroy);
    }
    nihu_gb_ctx *handle() const { return h_.get(); }

    // process-wide default context on device 0
    static context &get_default()
    {
        static context c(0);
        return c;
    }

private:
    std::shared_ptr<nihu_gb_ctx> h_;
};

// --------------------------------------------------------------- matrices

// column-major dense matrix, the in-repo stand-in for Eigen's MatrixX<T>
template <class T>
class dense_matrix {
public:
    dense_matrix(int64_t rows = 0, int64_t cols = 0) : r_(rows), c_(cols), d_((size_t)(rows * cols), T(0)) {}
    T &operator()(int64_t i, int64_t j) { return d_[(size_t)(i + j * r_)]; }
    T const &operator()(int64_t i, int64_t j) const { return d_[(size_t)(i + j * r_)]; }
    T *data() { return d_.data(); }
    T const *data() const { return d_.data(); }
    int64_t rows() const { return r_; }
    int64_t cols() const { return c_; }
    void setZero() { std::fill(d_.begin(), d_.end(), T(0)); }

private:
    int64_t r_, c_;
    std::vector<T> d_;
};

// ------------------------------------------------------------------ mesh

struct tria_1_tag {};
struct quad_1_tag {};

// create_mesh(nodes, elements, tags...) (nihu/core/mesh.hpp:175-193,285-290):
// nodes n x 3, elements m x (1 + corners) with the type id in column 0.
// The mesh keeps host copies and uploads itself to a context on first use.
class mesh {
public:
    mesh(std::vector<double> nodes, std::vector<int32_t> elems, int64_t elem_cols)
        : nodes_(std::move(nodes)), elems_(std::move(elems)), cols_(elem_cols)
    {
        if (nodes_.size() % 3 || cols_ < 4 || elems_.size() % (size_t)cols_)
            throw std::invalid_argument("create_mesh: nodes must be n x 3, elements m x cols (cols >= 4)");
    }
    int64_t num_elements() const { return (int64_t)(elems_.size() / (size_t)cols_); }

    // element areas with the one-point rule of the Galerkin identity
    // (nihu/core/single_integral.hpp:97-140): |e1 x e2| / 2 on triangles,
    // 4 |x_xi x x_eta| at the centre on quads
    std::vector<double> areas() const
    {
        std::vector<double> a((size_t)num_elements());
        for (int64_t e = 0; e < num_elements(); ++e) {
            const int32_t *row = elems_.data() + (size_t)(e * cols_);
            const bool quad = row[0] == NIHU_GB_QUAD_1;
            double c[4][3];
            for (int k = 0; k < (quad ? 4 : 3); ++k)
                for (int d = 0; d < 3; ++d) c[k][d] = nodes_[(size_t)(3 * row[1 + k] + d)];
            double t1[3], t2[3];
            for (int d = 0; d < 3; ++d) {
                t1[d] = quad ? (c[1][d] + c[2][d] - c[0][d] - c[3][d]) / 4 : c[1][d] - c[0][d];
                t2[d] = quad ? (c[2][d] + c[3][d] - c[0][d] - c[1][d]) / 4 : c[2][d] - c[0][d];
            }
            const double n0 = t1[1] * t2[2] - t1[2] * t2[1], n1 = t1[2] * t2[0] - t1[0] * t2[2],
                         n2 = t1[0] * t2[1] - t1[1] * t2[0];
            a[(size_t)e] = std::sqrt(n0 * n0 + n1 * n1 + n2 * n2) * (quad ? 4.0 : 0.5);
        }
        return a;
    }

    nihu_gb_mesh *on(context &ctx) const
    {
        if (!dev_ || ctx_ != ctx.handle()) {
            nihu_gb_mesh *m = nullptr;
            check(ctx.handle(), nihu_gb_mesh_create(ctx.handle(), nodes_.data(), (int64_t)(nodes_.size() / 3),
                                                    elems_.data(), num_elements(), cols_, &m));
            dev_.reset(m, nihu_gb_mesh_destroy);
            ctx_ = ctx.handle();
        }
        return dev_.get();
    }

private:
    std::vector<double> nodes_;
    std::vector<int32_t> elems_;
    int64_t cols_;
    mutable std::shared_ptr<nihu_gb_mesh> dev_;
    mutable nihu_gb_ctx *ctx_ = nullptr;
};

// from any row-major-indexable matrices with rows(), cols() and operator()(i, j)
template <class NodeMat, class ElemMat, class... Tags>
mesh create_mesh(NodeMat const &nodes, ElemMat const &elements, Tags...)
{
    std::vector<double> nd((size_t)nodes.rows() * 3);
    for (int64_t i = 0; i < (int64_t)nodes.rows(); ++i)
        for (int d = 0; d < 3; ++d) nd[(size_t)(3 * i + d)] = (double)nodes(i, d);
    int64_t cols = std::max<int64_t>((int64_t)elements.cols(), 5);
    std::vector<int32_t> el((size_t)(elements.rows() * cols), -1);
    for (int64_t i = 0; i < (int64_t)elements.rows(); ++i)
        for (int64_t j = 0; j < (int64_t)elements.cols(); ++j)
            el[(size_t)(i * cols + j)] = (int32_t)elements(i, j);
    return mesh(std::move(nd), std::move(el), cols);
}

// ------------------------------------------------------------- spaces

class function_space {
public:
    explicit function_space(mesh const &m) : m_(&m) {}
    mesh const &get_mesh() const { return *m_; }
    int64_t get_num_dofs() const { return m_->num_elements(); }

private:
    mesh const *m_;
};

class dirac_space {
public:
    explicit dirac_space(function_space const &s) : s_(s) {}
    mesh const &get_mesh() const { return s_.get_mesh(); }
    int64_t get_num_dofs() const { return s_.get_num_dofs(); }

private:
    function_space s_;
};

inline function_space constant_view(mesh const &m) { return function_space(m); }
inline dirac_space dirac(function_space const &s) { return dirac_space(s); }

// ------------------------------------------------------------- kernels

struct kernel_desc {
    int family, op;
    double k;
    double k_im = 0.0;  // imaginary part of a complex (lossy) wave number
};

namespace detail {
// the wave number as (k, k_im): double, or std::complex<double> as the
// reference's WaveNumber template parameter allows (nihu/library/helmholtz_kernel.hpp:42-54)
inline kernel_desc with_k(int family, int op, double k) { return {family, op, k, 0.0}; }
inline kernel_desc with_k(int family, int op, std::complex<double> k) { return {family, op, k.real(), k.imag()}; }
}  // namespace detail

template <class WaveNumber = double>
inline kernel_desc helmholtz_3d_SLP_kernel(WaveNumber k) { return detail::with_k(NIHU_GB_HELMHOLTZ_3D, NIHU_GB_SLP, k); }
template <class WaveNumber = double>
inline kernel_desc helmholtz_3d_DLP_kernel(WaveNumber k) { return detail::with_k(NIHU_GB_HELMHOLTZ_3D, NIHU_GB_DLP, k); }
inline kernel_desc laplace_3d_SLP_kernel() { return {NIHU_GB_LAPLACE_3D, NIHU_GB_SLP, 0.0}; }
inline kernel_desc laplace_3d_DLP_kernel() { return {NIHU_GB_LAPLACE_3D, NIHU_GB_DLP, 0.0}; }
// Burton-Miller kernels (nihu/library/helmholtz_kernel.hpp:326-334): constant
// triangle trial elements only
template <class WaveNumber = double>
inline kernel_desc helmholtz_3d_DLPt_kernel(WaveNumber k) { return detail::with_k(NIHU_GB_HELMHOLTZ_3D, NIHU_GB_DLPT, k); }
template <class WaveNumber = double>
inline kernel_desc helmholtz_3d_HSP_kernel(WaveNumber k) { return detail::with_k(NIHU_GB_HELMHOLTZ_3D, NIHU_GB_HSP, k); }
inline kernel_desc laplace_3d_DLPt_kernel() { return {NIHU_GB_LAPLACE_3D, NIHU_GB_DLPT, 0.0}; }
inline kernel_desc laplace_3d_HSP_kernel() { return {NIHU_GB_LAPLACE_3D, NIHU_GB_HSP, 0.0}; }

// ------------------------------------------------------------- operators

struct integral_transform;

struct integral_operator {
    kernel_desc kernel;
    std::complex<double> scale{1.0, 0.0};
    bool identity = false;
    integral_transform operator[](function_space const &trial) const;
};

inline integral_operator create_integral_operator(kernel_desc k) { return integral_operator{k, {1.0, 0.0}, false}; }
inline integral_operator identity_integral_operator() { return integral_operator{{0, 0, 0.0}, {1.0, 0.0}, true}; }

template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline integral_operator operator*(S alpha, integral_operator op)
{
    op.scale *= (double)alpha;
    return op;
}
inline integral_operator operator*(std::complex<double> alpha, integral_operator op)
{
    op.scale *= alpha;
    return op;
}

struct integral_transform {
    integral_operator op;
    function_space trial;
};

inline integral_transform integral_operator::operator[](function_space const &trial) const { return {*this, trial}; }

template <class TestSpace>
struct weighted_residual {
    TestSpace test;
    integral_transform tr;
    context *ctx;
    int precision;
};

// test_space * Op[trial_space] (nihu/core/weighted_residual.hpp:176-186)
inline weighted_residual<dirac_space> operator*(dirac_space const &t, integral_transform const &tr)
{
    return {t, tr, &context::get_default(), NIHU_GB_REGULAR_FP32};
}
inline weighted_residual<function_space> operator*(function_space const &t, integral_transform const &tr)
{
    return {t, tr, &context::get_default(), NIHU_GB_REGULAR_FP32};
}

// select the context / the regular-quadrature precision of one evaluation
template <class TS>
weighted_residual<TS> on(weighted_residual<TS> wr, context &ctx, int precision = NIHU_GB_REGULAR_FP32)
{
    wr.ctx = &ctx;
    wr.precision = precision;
    return wr;
}

namespace detail {
template <class T> inline void add_scalar(T &dst, std::complex<double> v) { dst += T(v.real()); }
template <class R> inline void add_scalar(std::complex<R> &dst, std::complex<double> v)
{
    dst += std::complex<R>((R)v.real(), (R)v.imag());
}
template <class T> struct storage;
template <> struct storage<std::complex<float>> { static constexpr int dtype = NIHU_GB_C64; };
template <> struct storage<std::complex<double>> { static constexpr int dtype = NIHU_GB_C128; };
}  // namespace detail

// result << test_space * Op[trial_space]: adds the operator matrix into result
template <class Res, class TS>
Res &operator<<(Res &result, weighted_residual<TS> const &wr)
{
    typedef typename std::remove_cv<typename std::remove_reference<decltype(*result.data())>::type>::type T;
    mesh const &tm = wr.test.get_mesh();
    mesh const &rm = wr.tr.trial.get_mesh();
    const int64_t m = tm.num_elements(), n = rm.num_elements();
    if ((int64_t)result.rows() != m || (int64_t)result.cols() != n)
        throw std::invalid_argument("result matrix size does not match the operator");
    integral_operator const &op = wr.tr.op;
    // a function-space test space is the Galerkin formalism, dirac() collocation
    constexpr bool galerkin = std::is_same<TS, function_space>::value;
    if (op.identity) {  // (alpha I)[sp] on coinciding elements: 1 (collocation) or the area (Galerkin)
        if (&tm == &rm) {
            const std::vector<double> area = galerkin ? tm.areas() : std::vector<double>();
            for (int64_t i = 0; i < m; ++i)
                detail::add_scalar(result.data()[i + i * m], op.scale * (galerkin ? area[(size_t)i] : 1.0));
        }
        return result;
    }
    context &ctx = *wr.ctx;
    nihu_gb_mesh *tmh = tm.on(ctx);
    nihu_gb_mesh *rmh = (&tm == &rm) ? tmh : rm.on(ctx);
    const int kop = op.kernel.op;
    if (kop == NIHU_GB_SLP || kop == NIHU_GB_DLP) {
        void *out_s = kop == NIHU_GB_SLP ? (void *)result.data() : nullptr;
        void *out_d = kop == NIHU_GB_DLP ? (void *)result.data() : nullptr;
        if (op.kernel.k_im != 0.0) {
            auto fn = galerkin ? nihu_gb_assemble_galerkin_c : nihu_gb_assemble_c;
            check(ctx.handle(), fn(ctx.handle(), tmh, rmh, op.kernel.family, kop, op.kernel.k, op.kernel.k_im,
                                   op.scale.real(), op.scale.imag(), wr.precision, detail::storage<T>::dtype, out_s,
                                   out_d, m, 1, NIHU_GB_HOST));
        } else {
            auto fn = galerkin ? nihu_gb_assemble_galerkin : nihu_gb_assemble;
            check(ctx.handle(), fn(ctx.handle(), tmh, rmh, op.kernel.family, kop, op.kernel.k, op.scale.real(),
                                   op.scale.imag(), wr.precision, detail::storage<T>::dtype, out_s, out_d, m, 1,
                                   NIHU_GB_HOST));
        }
    } else if (galerkin) {
        throw std::invalid_argument("Galerkin formalism: SLP and DLP kernels only");
    } else {
        void *out_t = kop == NIHU_GB_DLPT ? (void *)result.data() : nullptr;
        void *out_h = kop == NIHU_GB_HSP ? (void *)result.data() : nullptr;
        check(ctx.handle(), nihu_gb_assemble_bm_c(ctx.handle(), tmh, rmh, op.kernel.family, kop, op.kernel.k,
                                                  op.kernel.k_im, op.scale.real(), op.scale.imag(), wr.precision,
                                                  detail::storage<T>::dtype, out_t, out_h, m, 1, NIHU_GB_HOST));
    }
    return result;
}

// ------------------------------------------------------------- solvers

// x = A^{-1} b on the GPU (FP64 LU), A complex<double> column-major
inline std::vector<std::complex<double>> lu_solve(dense_matrix<std::complex<double>> const &A,
                                                  std::vector<std::complex<double>> const &b,
                                                  context &ctx = context::get_default())
{
    std::vector<std::complex<double>> x(b.size());
    check(ctx.handle(), nihu_gb_lu_solve(ctx.handle(), (void *)A.data(), A.rows(), A.rows(), b.data(), x.data(),
                                         NIHU_GB_HOST));
    return x;
}

// restarted GMRES on the GPU (FP32 matvec for complex<float> A, FP64 Arnoldi)
template <class T>
std::vector<std::complex<double>> gmres(dense_matrix<T> const &A, std::vector<std::complex<double>> const &b,
                                        double tol = 1e-6, int restart = 50, int max_iters = 1000,
                                        int *iters = nullptr, context &ctx = context::get_default())
{
    std::vector<std::complex<double>> x(b.size(), 0.0);
    int it = 0;
    double res = 0.0;
    check(ctx.handle(), nihu_gb_gmres(ctx.handle(), detail::storage<T>::dtype, A.data(), A.rows(), A.rows(), b.data(),
                                      x.data(), restart, max_iters, tol, &it, &res, NIHU_GB_HOST));
    if (iters) *iters = it;
    return x;
}

}  // namespace nihu_gb300
