// C-ABI shim over the UNMODIFIED reference nearfield construction
// (tbenthompson/3bem: cpp/nearfield_operator.h, cpp/integral_term.cpp,
// cpp/limit_direction.cpp, cpp/intersect_balls.cpp, cpp/sinh_quad.cpp,
// cpp/gauss_quad.cpp), compiled with oracle/ref/gte_restated.cpp standing in
// for the absent GTEngine.  Test infrastructure only: it generates the
// nearfield fixtures under tests/golden/ and pins the product's GPU
// construction; the product never links it.
//
// Meshes cross this interface as vertices [n][3] (z ignored in 2D) and
// facets [n][dim] (vertex indices).  Kernel ids follow include/tbem_gpu.h.
#include <cstring>
#include <memory>
#include <vector>
#include <omp.h>

#include "elastic_kernels.h"
#include "galerkin_operator.h"
#include "interpolation_operator.h"
#include "mass_operator.h"
#include "integral_operator.h"
#include "identity_kernels.h"
#include "integral_term.h"
#include "laplace_kernels.h"
#include "mesh.h"
#include "nearfield_operator.h"

using namespace tbem;

namespace {

template <size_t dim>
Mesh<dim> make_mesh(const double* verts, long n_verts, const long* facets, long n_facets)
{
    std::vector<Vec<double, dim>> v(n_verts);
    for (long i = 0; i < n_verts; i++)
        for (size_t d = 0; d < dim; d++) v[i][d] = verts[3 * i + d];
    std::vector<std::array<size_t, dim>> f(n_facets);
    for (long i = 0; i < n_facets; i++)
        for (size_t d = 0; d < dim; d++) f[i][d] = (size_t)facets[dim * i + d];
    return Mesh<dim>::from_vertices_faces(v, f);
}

struct Strategy {
    int strategy;  // 0 adaptive, 1 sinh
    double near_tol;
    long sinh_order, obs_near_order, obs_far_order, src_far_order, n_singular_steps;
    double far_threshold;
};

template <size_t dim, size_t R, size_t C>
IntegrationStrategy<dim, R, C> make_strategy(const Strategy& s, const Kernel<dim, R, C>& K)
{
    if (s.strategy == 0)
        return make_adaptive_integrator(s.near_tol, s.obs_near_order, s.obs_far_order,
                                        s.src_far_order, s.n_singular_steps, s.far_threshold, K);
    return make_sinh_integrator(s.sinh_order, s.obs_near_order, s.obs_far_order, s.src_far_order,
                                s.n_singular_steps, s.far_threshold, K);
}

struct Csr {
    long n_rows = 0, n_cols = 0;
    std::vector<double> values;
    std::vector<long> cols, rowptr;
};

template <size_t dim, size_t R, size_t C>
Csr build(const Kernel<dim, R, C>& K, const Mesh<dim>& m, const Strategy& s, int which)
{
    auto mthd = make_strategy(s, K);
    auto obs = galerkin_obs_pts(m, which == 0 ? mthd.obs_near_quad : mthd.obs_far_quad, m);
    SparseOperator op = which == 0 ? make_nearfield_operator(obs, m, mthd)
                                   : make_farfield_correction_operator(obs, m, mthd);
    Csr c;
    c.n_rows = (long)op.n_rows();
    c.n_cols = (long)op.n_cols();
    c.values = op.values;
    c.cols.assign(op.column_indices.begin(), op.column_indices.end());
    c.rowptr.assign(op.row_ptrs.begin(), op.row_ptrs.end());
    return c;
}

// the same for given points (interior_obs_pts) against the mesh
template <size_t dim, size_t R, size_t C>
Csr build_points(const Kernel<dim, R, C>& K, const Mesh<dim>& m, const Strategy& s, int which,
                 const double* locs, const double* nrms, long n)
{
    auto mthd = make_strategy(s, K);
    std::vector<Vec<double, dim>> l(n), nn(n);
    for (long i = 0; i < n; i++)
        for (size_t d = 0; d < dim; d++) { l[i][d] = locs[3 * i + d]; nn[i][d] = nrms[3 * i + d]; }
    auto obs = interior_obs_pts(l, nn, m);
    SparseOperator op = which == 0 ? make_nearfield_operator(obs, m, mthd)
                                   : make_farfield_correction_operator(obs, m, mthd);
    Csr c;
    c.n_rows = (long)op.n_rows();
    c.n_cols = (long)op.n_cols();
    c.values = op.values;
    c.cols.assign(op.column_indices.begin(), op.column_indices.end());
    c.rowptr.assign(op.row_ptrs.begin(), op.row_ptrs.end());
    return c;
}

template <size_t dim>
Csr dispatch(int kernel, double mu, double nu, const Mesh<dim>& m, const Strategy& s, int which);

template <>
Csr dispatch<3>(int kernel, double mu, double nu, const Mesh<3>& m, const Strategy& s, int which)
{
    switch (kernel) {
    case 0: return build(LaplaceSingle<3>(), m, s, which);
    case 1: return build(LaplaceDouble<3>(), m, s, which);
    case 2: return build(ElasticDisplacement<3>(mu, nu), m, s, which);
    case 3: return build(ElasticTraction<3>(mu, nu), m, s, which);
    case 4: return build(ElasticAdjointTraction<3>(mu, nu), m, s, which);
    case 5: return build(IdentityScalar<3>(), m, s, which);
    case 6: return build(ElasticHypersingular<3>(mu, nu), m, s, which);
    }
    return Csr{-1};
}

template <>
Csr dispatch<2>(int kernel, double mu, double nu, const Mesh<2>& m, const Strategy& s, int which)
{
    switch (kernel) {
    case 16: return build(LaplaceSingle<2>(), m, s, which);
    case 17: return build(LaplaceDouble<2>(), m, s, which);
    case 18: return build(LaplaceHypersingular<2>(), m, s, which);
    case 19: return build(ElasticDisplacement<2>(mu, nu), m, s, which);
    case 20: return build(ElasticTraction<2>(mu, nu), m, s, which);
    case 21: return build(ElasticAdjointTraction<2>(mu, nu), m, s, which);
    case 22: return build(ElasticHypersingular<2>(mu, nu), m, s, which);
    case 23: return build(IdentityScalar<2>(), m, s, which);
    }
    return Csr{-1};
}

template <size_t dim, size_t R, size_t C>
long term(const Kernel<dim, R, C>& K, const Strategy& s, const double* loc, const double* nrm,
          const double* dir, const double* facet, double* out)
{
    auto mthd = make_strategy(s, K);
    Vec<double, dim> l, n, r;
    for (size_t d = 0; d < dim; d++) { l[d] = loc[d]; n[d] = nrm[d]; r[d] = dir[d]; }
    Facet<dim> f;
    for (size_t v = 0; v < dim; v++)
        for (size_t d = 0; d < dim; d++) f[v][d] = facet[3 * v + d];
    ObsPt<dim> obs{l, n, r};
    auto info = FacetInfo<dim>::build(f);
    IntegralTerm<dim, R, C> t{obs, info};
    auto res = mthd.compute_term(t);
    for (size_t b = 0; b < dim; b++)
        for (size_t i = 0; i < R; i++)
            for (size_t j = 0; j < C; j++) out[(b * R + i) * C + j] = res[b][i][j];
    return (long)(dim * R * C);
}

template <size_t dim>
long obs_points(const Mesh<dim>& m, long order, double* locs, double* normals, double* dirs)
{
    auto pts = galerkin_obs_pts(m, gauss_facet<dim>((size_t)order), m);
    if (locs)
        for (size_t i = 0; i < pts.size(); i++)
            for (size_t d = 0; d < 3; d++) {
                locs[3 * i + d] = d < dim ? pts[i].loc[d] : 0.0;
                normals[3 * i + d] = d < dim ? pts[i].normal[d] : 0.0;
                dirs[3 * i + d] = d < dim ? pts[i].richardson_dir[d] : 0.0;
            }
    return (long)pts.size();
}

}  // namespace

extern "C" {

// The nearfield operator (which 0, cpp/nearfield_operator.h:97-106) or the
// farfield correction (which 1, :108-117) of a mesh against itself, Galerkin
// observation points from the mesh (cpp/nearfield_operator.h:12-25).
// strategy 0: make_adaptive_integrator(near_tol, ...), 1:
// make_sinh_integrator(sinh_order, ...) (cpp/integral_term.h:100-150).
// Writes the CSR when cap >= nnz; returns nnz (or -1).  One thread: the
// reference collects entries inside an omp critical section.
long ref_nearfield(int kernel, double mu, double nu, int dim, const double* verts, long n_verts,
                   const long* facets, long n_facets, int strategy, double near_tol,
                   long sinh_order, long obs_near_order, long obs_far_order, long src_far_order,
                   long n_singular_steps, double far_threshold, int which, long* shape,
                   double* values, long* cols, long* rowptr, long cap)
{
    Strategy s{strategy, near_tol, sinh_order, obs_near_order, obs_far_order, src_far_order,
               n_singular_steps, far_threshold};
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    Csr c = dim == 2 ? dispatch<2>(kernel, mu, nu, make_mesh<2>(verts, n_verts, facets, n_facets), s, which)
                     : dispatch<3>(kernel, mu, nu, make_mesh<3>(verts, n_verts, facets, n_facets), s, which);
    omp_set_num_threads(saved);
    if (c.n_rows < 0) return -1;
    const long nnz = (long)c.values.size();
    if (shape) { shape[0] = c.n_rows; shape[1] = c.n_cols; }
    if (cap >= nnz && values) {
        std::memcpy(values, c.values.data(), nnz * sizeof(double));
        std::memcpy(cols, c.cols.data(), nnz * sizeof(long));
        std::memcpy(rowptr, c.rowptr.data(), (c.n_rows + 1) * sizeof(long));
    }
    return nnz;
}

// Galerkin observation points with their Richardson directions
// (galerkin_obs_pts, cpp/nearfield_operator.h:12-40); outputs [n][3].
long ref_obs_points(int dim, const double* verts, long n_verts, const long* facets, long n_facets,
                    long order, double* locs, double* normals, double* dirs)
{
    return dim == 2 ? obs_points(make_mesh<2>(verts, n_verts, facets, n_facets), order, locs, normals, dirs)
                    : obs_points(make_mesh<3>(verts, n_verts, facets, n_facets), order, locs, normals, dirs);
}

// The nearfield / correction operator for given points [n][3] (the
// interior_obs_pts path of dense_interior_operator,
// cpp/integral_operator.h:132-158); CSR when cap >= nnz; returns nnz.
long ref_nearfield_points(int kernel, double mu, double nu, int dim, const double* verts,
                          long n_verts, const long* facets, long n_facets, const double* locs,
                          const double* nrms, long n, long sinh_order, long obs_near_order,
                          long obs_far_order, long src_far_order, long n_singular_steps,
                          double far_threshold, int which, long* shape, double* values,
                          long* cols, long* rowptr, long cap)
{
    Strategy s{1, 0.0, sinh_order, obs_near_order, obs_far_order, src_far_order, n_singular_steps,
               far_threshold};
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    Csr c{-1};
    if (dim == 3) {
        auto m = make_mesh<3>(verts, n_verts, facets, n_facets);
        switch (kernel) {
        case 0: c = build_points(LaplaceSingle<3>(), m, s, which, locs, nrms, n); break;
        case 1: c = build_points(LaplaceDouble<3>(), m, s, which, locs, nrms, n); break;
        case 2: c = build_points(ElasticDisplacement<3>(mu, nu), m, s, which, locs, nrms, n); break;
        case 3: c = build_points(ElasticTraction<3>(mu, nu), m, s, which, locs, nrms, n); break;
        }
    } else {
        auto m = make_mesh<2>(verts, n_verts, facets, n_facets);
        switch (kernel) {
        case 16: c = build_points(LaplaceSingle<2>(), m, s, which, locs, nrms, n); break;
        case 17: c = build_points(LaplaceDouble<2>(), m, s, which, locs, nrms, n); break;
        case 19: c = build_points(ElasticDisplacement<2>(mu, nu), m, s, which, locs, nrms, n); break;
        }
    }
    omp_set_num_threads(saved);
    if (c.n_rows < 0) return -1;
    const long nnz = (long)c.values.size();
    if (shape) { shape[0] = c.n_rows; shape[1] = c.n_cols; }
    if (cap >= nnz && values) {
        std::memcpy(values, c.values.data(), nnz * sizeof(double));
        std::memcpy(cols, c.cols.data(), nnz * sizeof(long));
        std::memcpy(rowptr, c.rowptr.data(), (c.n_rows + 1) * sizeof(long));
    }
    return nnz;
}

// dense_boundary_operator (cpp/integral_operator.h:100-130) of a mesh against
// itself with the sinh strategy: the dense (R n_dofs) x (C n_dofs) matrix,
// row-major, written when out != NULL; returns the number of entries.
long ref_dense_boundary(int kernel, double mu, double nu, int dim, const double* verts,
                        long n_verts, const long* facets, long n_facets, long sinh_order,
                        long obs_near_order, long obs_far_order, long src_far_order,
                        long n_singular_steps, double far_threshold, double* out)
{
    Strategy s{1, 0.0, sinh_order, obs_near_order, obs_far_order, src_far_order, n_singular_steps,
               far_threshold};
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    std::vector<double> data;
    auto run = [&](const auto& K, const auto& m) {
        auto mthd = make_strategy(s, K);
        auto op = dense_boundary_operator(m, m, mthd, m);
        data = op.data();
    };
    if (dim == 3) {
        auto m = make_mesh<3>(verts, n_verts, facets, n_facets);
        if (kernel == 0) run(LaplaceSingle<3>(), m);
        else if (kernel == 1) run(LaplaceDouble<3>(), m);
        else if (kernel == 2) run(ElasticDisplacement<3>(mu, nu), m);
        else if (kernel == 3) run(ElasticTraction<3>(mu, nu), m);
    } else {
        auto m = make_mesh<2>(verts, n_verts, facets, n_facets);
        if (kernel == 16) run(LaplaceSingle<2>(), m);
        else if (kernel == 17) run(LaplaceDouble<2>(), m);
        else if (kernel == 19) run(ElasticDisplacement<2>(mu, nu), m);
        else if (kernel == 20) run(ElasticTraction<2>(mu, nu), m);
    }
    omp_set_num_threads(saved);
    if (out) std::memcpy(out, data.data(), data.size() * sizeof(double));
    return (long)data.size();
}

// dense_interior_operator (cpp/integral_operator.h:133-158) for given points
// [n][3] against a mesh (also the all-mesh) with the sinh strategy: the dense
// (R n) x (C n_dofs) matrix, row-major, written when out != NULL; returns the
// number of entries (or -1).
long ref_dense_interior(int kernel, double mu, double nu, int dim, const double* verts,
                        long n_verts, const long* facets, long n_facets, const double* locs,
                        const double* nrms, long n, long sinh_order, long obs_near_order,
                        long obs_far_order, long src_far_order, long n_singular_steps,
                        double far_threshold, double* out)
{
    Strategy s{1, 0.0, sinh_order, obs_near_order, obs_far_order, src_far_order, n_singular_steps,
               far_threshold};
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    std::vector<double> data;
    bool done = false;
    auto run = [&](const auto& K, const auto& m, auto dimc) {
        constexpr size_t D = decltype(dimc)::value;
        auto mthd = make_strategy(s, K);
        std::vector<Vec<double, D>> l(n), nn(n);
        for (long i = 0; i < n; i++)
            for (size_t d = 0; d < D; d++) { l[i][d] = locs[3 * i + d]; nn[i][d] = nrms[3 * i + d]; }
        auto op = dense_interior_operator(l, nn, m, mthd, m);
        data = op.data();
        done = true;
    };
    if (dim == 3) {
        auto m = make_mesh<3>(verts, n_verts, facets, n_facets);
        std::integral_constant<size_t, 3> d3;
        if (kernel == 0) run(LaplaceSingle<3>(), m, d3);
        else if (kernel == 1) run(LaplaceDouble<3>(), m, d3);
        else if (kernel == 2) run(ElasticDisplacement<3>(mu, nu), m, d3);
        else if (kernel == 3) run(ElasticTraction<3>(mu, nu), m, d3);
    } else {
        auto m = make_mesh<2>(verts, n_verts, facets, n_facets);
        std::integral_constant<size_t, 2> d2;
        if (kernel == 16) run(LaplaceSingle<2>(), m, d2);
        else if (kernel == 17) run(LaplaceDouble<2>(), m, d2);
        else if (kernel == 19) run(ElasticDisplacement<2>(mu, nu), m, d2);
    }
    omp_set_num_threads(saved);
    if (!done) return -1;
    if (out) std::memcpy(out, data.data(), data.size() * sizeof(double));
    return (long)data.size();
}

// One IntegrationStrategy::compute_term (cpp/integral_term.cpp:33-53) for an
// observation point (loc, normal, Richardson direction, 3-vectors) against
// one facet ([dim][3]); out [dim basis][R][C].  Returns dim * R * C or -1.
long ref_term(int kernel, double mu, double nu, int strategy, double near_tol, long sinh_order,
              long obs_near_order, long obs_far_order, long src_far_order, long n_singular_steps,
              double far_threshold, const double* loc, const double* nrm, const double* dir,
              const double* facet, double* out)
{
    Strategy s{strategy, near_tol, sinh_order, obs_near_order, obs_far_order, src_far_order,
               n_singular_steps, far_threshold};
    switch (kernel) {
    case 0: return term(LaplaceSingle<3>(), s, loc, nrm, dir, facet, out);
    case 1: return term(LaplaceDouble<3>(), s, loc, nrm, dir, facet, out);
    case 2: return term(ElasticDisplacement<3>(mu, nu), s, loc, nrm, dir, facet, out);
    case 3: return term(ElasticTraction<3>(mu, nu), s, loc, nrm, dir, facet, out);
    case 4: return term(ElasticAdjointTraction<3>(mu, nu), s, loc, nrm, dir, facet, out);
    case 5: return term(IdentityScalar<3>(), s, loc, nrm, dir, facet, out);
    case 6: return term(ElasticHypersingular<3>(mu, nu), s, loc, nrm, dir, facet, out);
    case 16: return term(LaplaceSingle<2>(), s, loc, nrm, dir, facet, out);
    case 17: return term(LaplaceDouble<2>(), s, loc, nrm, dir, facet, out);
    case 18: return term(LaplaceHypersingular<2>(), s, loc, nrm, dir, facet, out);
    case 19: return term(ElasticDisplacement<2>(mu, nu), s, loc, nrm, dir, facet, out);
    case 20: return term(ElasticTraction<2>(mu, nu), s, loc, nrm, dir, facet, out);
    case 21: return term(ElasticAdjointTraction<2>(mu, nu), s, loc, nrm, dir, facet, out);
    case 22: return term(ElasticHypersingular<2>(mu, nu), s, loc, nrm, dir, facet, out);
    case 23: return term(IdentityScalar<2>(), s, loc, nrm, dir, facet, out);
    }
    return -1;
}

// make_galerkin_operator (which 0, cpp/galerkin_operator.cpp:9-44) or
// make_interpolation_operator (which 1, cpp/interpolation_operator.cpp:9-39)
// with gauss_facet(order); CSR written when cap >= nnz; returns nnz.
long ref_galerkin_interp(int which, int dim, long n_components, const double* verts, long n_verts,
                         const long* facets, long n_facets, long order, long* shape,
                         double* values, long* cols, long* rowptr, long cap)
{
    auto build = [&](auto m, auto q) {
        return which == 0 ? make_galerkin_operator(n_components, m, q)
                          : make_interpolation_operator(n_components, m, q);
    };
    SparseOperator op = dim == 2
        ? build(make_mesh<2>(verts, n_verts, facets, n_facets), gauss_facet<2>((size_t)order))
        : build(make_mesh<3>(verts, n_verts, facets, n_facets), gauss_facet<3>((size_t)order));
    const long nnz = (long)op.values.size();
    if (shape) { shape[0] = (long)op.n_rows(); shape[1] = (long)op.n_cols(); }
    if (cap >= nnz && values) {
        std::memcpy(values, op.values.data(), nnz * sizeof(double));
        for (long k = 0; k < nnz; k++) cols[k] = (long)op.column_indices[k];
        for (size_t r = 0; r < op.row_ptrs.size(); r++) rowptr[r] = (long)op.row_ptrs[r];
    }
    return nnz;
}

// interior_obs_pts' limit directions (cpp/nearfield_operator.h:27-40) for
// given points [n][3] against a mesh; dirs [n][3].
long ref_interior_dirs(int dim, const double* locs, long n, const double* verts, long n_verts,
                       const long* facets, long n_facets, double* dirs)
{
    auto run = [&](auto m, auto tag) {
        constexpr size_t D = decltype(tag)::value;
        std::vector<Vec<double, D>> l(n), nn(n);
        for (long i = 0; i < n; i++)
            for (size_t d = 0; d < D; d++) { l[i][d] = locs[3 * i + d]; nn[i][d] = 0.0; }
        auto pts = interior_obs_pts(l, nn, m);
        for (long i = 0; i < n; i++)
            for (size_t d = 0; d < 3; d++) dirs[3 * i + d] = d < D ? pts[i].richardson_dir[d] : 0.0;
    };
    if (dim == 2) run(make_mesh<2>(verts, n_verts, facets, n_facets), std::integral_constant<size_t, 2>());
    else run(make_mesh<3>(verts, n_verts, facets, n_facets), std::integral_constant<size_t, 3>());
    return n;
}

// mass_operator<dim,R,R> (cpp/mass_operator.h:10-19); CSR when cap >= nnz.
long ref_mass(int dim, long R, const double* verts, long n_verts, const long* facets,
              long n_facets, long n_q, long* shape, double* values, long* cols, long* rowptr,
              long cap)
{
    SparseOperator op = dim == 2
        ? (R == 1 ? mass_operator<2, 1, 1>(make_mesh<2>(verts, n_verts, facets, n_facets), n_q)
                  : mass_operator<2, 2, 2>(make_mesh<2>(verts, n_verts, facets, n_facets), n_q))
        : (R == 1 ? mass_operator<3, 1, 1>(make_mesh<3>(verts, n_verts, facets, n_facets), n_q)
                  : mass_operator<3, 3, 3>(make_mesh<3>(verts, n_verts, facets, n_facets), n_q));
    const long nnz = (long)op.values.size();
    if (shape) { shape[0] = (long)op.n_rows(); shape[1] = (long)op.n_cols(); }
    if (cap >= nnz && values) {
        std::memcpy(values, op.values.data(), nnz * sizeof(double));
        for (long k = 0; k < nnz; k++) cols[k] = (long)op.column_indices[k];
        for (size_t r = 0; r < op.row_ptrs.size(); r++) rowptr[r] = (long)op.row_ptrs[r];
    }
    return nnz;
}

// Gauss rule on the reference facet (gauss_facet, cpp/gauss_quad.cpp:155-165):
// [n][dim - 1] points and weights.
long ref_gauss_facet(int dim, long n, double* x, double* w)
{
    if (dim == 2) {
        auto q = gauss_facet<2>((size_t)n);
        if (x)
            for (size_t i = 0; i < q.size(); i++) { x[i] = q[i].x_hat[0]; w[i] = q[i].w; }
        return (long)q.size();
    }
    auto q = gauss_facet<3>((size_t)n);
    if (x)
        for (size_t i = 0; i < q.size(); i++) {
            x[2 * i] = q[i].x_hat[0];
            x[2 * i + 1] = q[i].x_hat[1];
            w[i] = q[i].w;
        }
    return (long)q.size();
}

// One closest-point query (the restated GTE query the reference calls):
// ref_pt [dim - 1], pt [3], returns the distance.
double ref_closest_pt(int dim, const double* p, const double* facet, double* ref_pt, double* pt)
{
    if (dim == 2) {
        Vec<double, 2> q{p[0], p[1]};
        Vec<Vec<double, 2>, 2> f{{{facet[0], facet[1]}, {facet[3], facet[4]}}};
        auto r = closest_pt_facet(q, f);
        ref_pt[0] = r.ref_pt[0];
        pt[0] = r.pt[0]; pt[1] = r.pt[1]; pt[2] = 0.0;
        return r.distance;
    }
    Vec<double, 3> q{p[0], p[1], p[2]};
    Vec<Vec<double, 3>, 3> f{{{facet[0], facet[1], facet[2]}, {facet[3], facet[4], facet[5]},
                              {facet[6], facet[7], facet[8]}}};
    auto r = closest_pt_facet(q, f);
    ref_pt[0] = r.ref_pt[0]; ref_pt[1] = r.ref_pt[1];
    for (int d = 0; d < 3; d++) pt[d] = r.pt[d];
    return r.distance;
}

}  // extern "C"
