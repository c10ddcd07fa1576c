// C-ABI shim over the UNMODIFIED reference FMM (tbenthompson/3bem, cpp/).
//
// Test infrastructure only: this file is compiled together with the
// reference's own sources (cpp/fmm.cpp, cpp/octree.cpp, ...) into
// oracle/_ref/libtbem_ref.so by oracle/ref/Makefile.  It is used to pin the
// oracle restatement (oracle/fmm_oracle.cpp) and to generate the golden
// fixtures under tests/golden/.  The product never links or loads it.
//
// Kernel ids follow include/tbem_gpu.h:
//   0 LaplaceSingle<3>, 1 LaplaceDouble<3>, 2 ElasticDisplacement<3>,
//   3 ElasticTraction<3>, 4 ElasticAdjointTraction<3>, 5 IdentityScalar<3>,
//   6 ElasticHypersingular<3>;
//   16 LaplaceSingle<2>, 17 LaplaceDouble<2>, 18 LaplaceHypersingular<2>,
//   19 ElasticDisplacement<2>, 20 ElasticTraction<2>,
//   21 ElasticAdjointTraction<2>, 22 ElasticHypersingular<2>,
//   23 IdentityScalar<2>.
// Points cross this interface as [n][3]; the 2D operators read x and y.
#include <memory>
#include <vector>
#include <cstring>
#include <omp.h>

#include "fmm.h"
#include "nbody_operator.h"
#include "laplace_kernels.h"
#include "elastic_kernels.h"
#include "identity_kernels.h"

using namespace tbem;

namespace {

template <size_t dim>
Vec<double, dim> vec_at(const double* p, long i)
{
    Vec<double, dim> v;
    for (size_t k = 0; k < dim; k++) v[k] = p[3 * i + k];
    return v;
}

template <size_t dim>
NBodyData<dim> make_data(const double* obs_locs, const double* obs_normals, long n_obs,
                         const double* src_locs, const double* src_normals,
                         const double* src_weights, long n_src)
{
    NBodyData<dim> d;
    d.obs_locs.resize(n_obs);
    d.obs_normals.resize(n_obs);
    d.src_locs.resize(n_src);
    d.src_normals.resize(n_src);
    d.src_weights.resize(n_src);
    for (long i = 0; i < n_obs; i++) {
        d.obs_locs[i] = vec_at<dim>(obs_locs, i);
        d.obs_normals[i] = vec_at<dim>(obs_normals, i);
    }
    for (long i = 0; i < n_src; i++) {
        d.src_locs[i] = vec_at<dim>(src_locs, i);
        d.src_normals[i] = vec_at<dim>(src_normals, i);
        d.src_weights[i] = src_weights[i];
    }
    return d;
}

std::unique_ptr<Kernel<3, 1, 1>> scalar_kernel3(int id)
{
    if (id == 0) return std::unique_ptr<Kernel<3, 1, 1>>(new LaplaceSingle<3>());
    if (id == 1) return std::unique_ptr<Kernel<3, 1, 1>>(new LaplaceDouble<3>());
    if (id == 5) return std::unique_ptr<Kernel<3, 1, 1>>(new IdentityScalar<3>());
    return nullptr;
}

std::unique_ptr<Kernel<3, 3, 3>> tensor_kernel3(int id, double mu, double nu)
{
    if (id == 2) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticDisplacement<3>(mu, nu));
    if (id == 3) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticTraction<3>(mu, nu));
    if (id == 4) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticAdjointTraction<3>(mu, nu));
    if (id == 6) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticHypersingular<3>(mu, nu));
    return nullptr;
}

std::unique_ptr<Kernel<2, 1, 1>> scalar_kernel2(int id)
{
    if (id == 16) return std::unique_ptr<Kernel<2, 1, 1>>(new LaplaceSingle<2>());
    if (id == 17) return std::unique_ptr<Kernel<2, 1, 1>>(new LaplaceDouble<2>());
    if (id == 18) return std::unique_ptr<Kernel<2, 1, 1>>(new LaplaceHypersingular<2>());
    if (id == 23) return std::unique_ptr<Kernel<2, 1, 1>>(new IdentityScalar<2>());
    return nullptr;
}

std::unique_ptr<Kernel<2, 2, 2>> tensor_kernel2(int id, double mu, double nu)
{
    if (id == 19) return std::unique_ptr<Kernel<2, 2, 2>>(new ElasticDisplacement<2>(mu, nu));
    if (id == 20) return std::unique_ptr<Kernel<2, 2, 2>>(new ElasticTraction<2>(mu, nu));
    if (id == 21) return std::unique_ptr<Kernel<2, 2, 2>>(new ElasticAdjointTraction<2>(mu, nu));
    if (id == 22) return std::unique_ptr<Kernel<2, 2, 2>>(new ElasticHypersingular<2>(mu, nu));
    return nullptr;
}

struct Handle {
    int kernel;
    std::unique_ptr<FMMOperator<3, 1, 1>> op31;
    std::unique_ptr<FMMOperator<3, 3, 3>> op33;
    std::unique_ptr<FMMOperator<2, 1, 1>> op21;
    std::unique_ptr<FMMOperator<2, 2, 2>> op22;
};

// Calls f on whichever operator the handle holds.
template <typename F>
auto visit(const Handle& h, F f) -> decltype(f(*h.op31))
{
    if (h.op31) return f(*h.op31);
    if (h.op33) return f(*h.op33);
    if (h.op21) return f(*h.op21);
    return f(*h.op22);
}

template <size_t dim>
void collect_cells(const Octree<dim>& c, std::vector<const Octree<dim>*>& out)
{
    out.push_back(&c);
    for (auto& ch : c.children) {
        if (ch != nullptr) collect_cells<dim>(*ch, out);
    }
}

template <size_t dim, size_t R, size_t C>
long tree_cells(const FMMOperator<dim, R, C>& op, int which, long* level, long* index,
                double* center, double* hw, long* n_idx, long* n_children)
{
    std::vector<const Octree<dim>*> cells;
    collect_cells<dim>(which == 0 ? op.src_oct : op.obs_oct, cells);
    for (size_t i = 0; i < cells.size(); i++) {
        auto c = cells[i];
        if (level) level[i] = (long)c->level;
        if (index) index[i] = (long)c->index;
        for (size_t k = 0; k < 3; k++) {
            if (center) center[3 * i + k] = k < dim ? c->bounds.center[k] : 0.0;
            if (hw) hw[3 * i + k] = k < dim ? c->bounds.half_width[k] : 0.0;
        }
        if (n_idx) n_idx[i] = (long)c->indices.size();
        if (n_children) n_children[i] = (long)c->n_immediate_children();
    }
    return (long)cells.size();
}

template <size_t dim, size_t R, size_t C>
long tree_indices(const FMMOperator<dim, R, C>& op, int which, long* out)
{
    std::vector<const Octree<dim>*> cells;
    collect_cells<dim>(which == 0 ? op.src_oct : op.obs_oct, cells);
    long k = 0;
    for (auto c : cells) {
        for (auto idx : c->indices) {
            if (out) out[k] = (long)idx;
            k++;
        }
    }
    return k;
}

template <size_t dim, size_t R, size_t C>
long task_list(const FMMOperator<dim, R, C>& op, int kind, long* a, long* b)
{
    const auto& t = op.tasks;
    auto cell_list = [&](const std::vector<typename FMMTasks<dim>::CellTask>& v) {
        for (size_t i = 0; i < v.size(); i++) {
            if (a) a[i] = (long)v[i].cell.index;
            if (b) b[i] = -1;
        }
        return (long)v.size();
    };
    auto pair_list = [&](const std::vector<typename FMMTasks<dim>::CellPairTask>& v) {
        for (size_t i = 0; i < v.size(); i++) {
            if (a) a[i] = (long)v[i].obs_cell.index;
            if (b) b[i] = (long)v[i].src_cell.index;
        }
        return (long)v.size();
    };
    switch (kind) {
        case 0: return cell_list(t.p2ms);
        case 1: return cell_list(t.m2ms);
        case 2: return pair_list(t.p2ps);
        case 3: return pair_list(t.m2ps);
        case 4: return pair_list(t.p2ls);
        case 5: return pair_list(t.m2ls);
        case 6: return cell_list(t.l2ls);
        case 7: return cell_list(t.l2ps);
    }
    return -1;
}

// Run the reference's execute_tasks on the subset of task lists selected by
// `mask` (bit k selects list k in the numbering of task_list above).
template <size_t dim, size_t R, size_t C>
void apply_masked(const FMMOperator<dim, R, C>& op, int mask, const double* x, double* y)
{
    std::vector<double> xv(x, x + op.n_cols());
    std::vector<double> out;
    if (mask == 0xff) {
        out = op.apply(xv);
    } else {
        // Task entries hold references (not assignable): copy-construct them.
        FMMTasks<dim> sub;
        auto take = [](auto& dst, const auto& src) {
            for (const auto& t : src) dst.push_back(t);
        };
        if (mask & 1) take(sub.p2ms, op.tasks.p2ms);
        if (mask & 2) take(sub.m2ms, op.tasks.m2ms);
        if (mask & 4) take(sub.p2ps, op.tasks.p2ps);
        if (mask & 8) take(sub.m2ps, op.tasks.m2ps);
        if (mask & 16) take(sub.p2ls, op.tasks.p2ls);
        if (mask & 32) take(sub.m2ls, op.tasks.m2ls);
        if (mask & 64) take(sub.l2ls, op.tasks.l2ls);
        if (mask & 128) take(sub.l2ps, op.tasks.l2ps);
        out = op.execute_tasks(sub, xv, op.up_check_to_equiv, op.down_check_to_equiv);
    }
    std::memcpy(y, out.data(), out.size() * sizeof(double));
}

template <size_t dim, size_t R, size_t C>
int kernel_tensor(const Kernel<dim, R, C>& K, const double* obs, const double* src,
                  const double* nobs, const double* nsrc, double* out)
{
    auto v = K(vec_at<dim>(obs, 0), vec_at<dim>(src, 0), vec_at<dim>(nobs, 0),
               vec_at<dim>(nsrc, 0));
    for (size_t a = 0; a < R; a++)
        for (size_t b = 0; b < C; b++) out[C * a + b] = v[a][b];
    return (int)(R * C);
}

}  // namespace

extern "C" {

void* ref_fmm_create(int kernel, double mu, double nu,
                     const double* obs_locs, const double* obs_normals, long n_obs,
                     const double* src_locs, const double* src_normals,
                     const double* src_weights, long n_src,
                     double mac, long order, long min_pts, double d, int small_cells)
{
    FMMConfig cfg(mac, (size_t)order, (size_t)min_pts, d, small_cells != 0);
    // Cell indices are assigned inside an omp critical section during the
    // parallel level-0 loop; one thread makes them deterministic (post-order).
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    auto h = new Handle();
    h->kernel = kernel;
    if (kernel >= 16) {
        auto data = make_data<2>(obs_locs, obs_normals, n_obs, src_locs, src_normals,
                                 src_weights, n_src);
        if (auto k1 = scalar_kernel2(kernel)) h->op21.reset(new FMMOperator<2, 1, 1>(*k1, data, cfg));
        else if (auto k2 = tensor_kernel2(kernel, mu, nu))
            h->op22.reset(new FMMOperator<2, 2, 2>(*k2, data, cfg));
    } else {
        auto data = make_data<3>(obs_locs, obs_normals, n_obs, src_locs, src_normals,
                                 src_weights, n_src);
        if (auto k1 = scalar_kernel3(kernel)) h->op31.reset(new FMMOperator<3, 1, 1>(*k1, data, cfg));
        else if (auto k3 = tensor_kernel3(kernel, mu, nu))
            h->op33.reset(new FMMOperator<3, 3, 3>(*k3, data, cfg));
    }
    omp_set_num_threads(saved);
    if (!h->op31 && !h->op33 && !h->op21 && !h->op22) {
        delete h;
        h = nullptr;
    }
    return h;
}

void ref_fmm_destroy(void* p) { delete static_cast<Handle*>(p); }

void ref_fmm_apply_masked(void* p, int mask, const double* x, double* y)
{
    visit(*static_cast<Handle*>(p), [&](const auto& op) { apply_masked(op, mask, x, y); });
}

void ref_fmm_apply(void* p, const double* x, double* y) { ref_fmm_apply_masked(p, 0xff, x, y); }

long ref_fmm_n_surf(void* p)
{
    return visit(*static_cast<Handle*>(p),
                 [](const auto& op) { return (long)op.up_equiv_surface.pts.size(); });
}

long ref_fmm_tree_cells(void* p, int which, long* level, long* index, double* center,
                        double* hw, long* n_idx, long* n_children)
{
    return visit(*static_cast<Handle*>(p), [&](const auto& op) {
        return tree_cells(op, which, level, index, center, hw, n_idx, n_children);
    });
}

long ref_fmm_tree_indices(void* p, int which, long* out)
{
    return visit(*static_cast<Handle*>(p),
                 [&](const auto& op) { return tree_indices(op, which, out); });
}

long ref_fmm_list(void* p, int kind, long* a, long* b)
{
    return visit(*static_cast<Handle*>(p),
                 [&](const auto& op) { return task_list(op, kind, a, b); });
}

// which: 0 = up (source tree), 1 = down (observation tree).
long ref_fmm_c2e(void* p, int which, long level, double* out)
{
    return visit(*static_cast<Handle*>(p), [&](const auto& op) -> long {
        const CheckToEquiv& ops = which == 0 ? op.up_check_to_equiv : op.down_check_to_equiv;
        if (level < 0) return (long)ops.size();
        if ((size_t)level >= ops.size()) return -1;
        if (out) std::memcpy(out, ops[level].data(), ops[level].size() * sizeof(double));
        return (long)ops[level].size();
    });
}

// Matrix-free direct sum through the reference's nbody_eval.
int ref_direct_apply(int kernel, double mu, double nu,
                     const double* obs_locs, const double* obs_normals, long n_obs,
                     const double* src_locs, const double* src_normals,
                     const double* src_weights, long n_src, const double* x, double* y)
{
    std::vector<double> out;
    if (kernel >= 16) {
        auto data = make_data<2>(obs_locs, obs_normals, n_obs, src_locs, src_normals,
                                 src_weights, n_src);
        if (auto k1 = scalar_kernel2(kernel)) out = nbody_eval(*k1, data, x);
        else if (auto k2 = tensor_kernel2(kernel, mu, nu)) out = nbody_eval(*k2, data, x);
        else return -1;
    } else {
        auto data = make_data<3>(obs_locs, obs_normals, n_obs, src_locs, src_normals,
                                 src_weights, n_src);
        if (auto k1 = scalar_kernel3(kernel)) out = nbody_eval(*k1, data, x);
        else if (auto k3 = tensor_kernel3(kernel, mu, nu)) out = nbody_eval(*k3, data, x);
        else return -1;
    }
    std::memcpy(y, out.data(), out.size() * sizeof(double));
    return 0;
}

// One kernel tensor K(obs, src, nobs, nsrc) (row-major R x C); the four
// vectors are 3-vectors (z ignored by the 2D kernels).  Returns R * C.
int ref_kernel(int kernel, double mu, double nu, const double* obs, const double* src,
               const double* nobs, const double* nsrc, double* out)
{
    if (auto k = scalar_kernel3(kernel)) return kernel_tensor(*k, obs, src, nobs, nsrc, out);
    if (auto k = tensor_kernel3(kernel, mu, nu)) return kernel_tensor(*k, obs, src, nobs, nsrc, out);
    if (auto k = scalar_kernel2(kernel)) return kernel_tensor(*k, obs, src, nobs, nsrc, out);
    if (auto k = tensor_kernel2(kernel, mu, nu)) return kernel_tensor(*k, obs, src, nobs, nsrc, out);
    return -1;
}

// Unit translation-surface points for a requested order ([n][3], z = 0 in 2D).
long ref_surface(long order, int dim, double* pts)
{
    if (dim == 2) {
        auto s = TranslationSurface<2>::make_surrounding_surface((size_t)order);
        if (pts)
            for (size_t i = 0; i < s.pts.size(); i++)
                for (int k = 0; k < 3; k++) pts[3 * i + k] = k < 2 ? s.pts[i][k] : 0.0;
        return (long)s.pts.size();
    }
    auto s = TranslationSurface<3>::make_surrounding_surface((size_t)order);
    if (pts)
        for (size_t i = 0; i < s.pts.size(); i++)
            for (int k = 0; k < 3; k++) pts[3 * i + k] = s.pts[i][k];
    return (long)s.pts.size();
}

}  // extern "C"
