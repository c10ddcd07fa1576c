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
//   6 ElasticHypersingular<3>.
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

struct Handle {
    int kernel;
    size_t R;
    std::unique_ptr<FMMOperator<3, 1, 1>> op1;
    std::unique_ptr<FMMOperator<3, 3, 3>> op3;
};

NBodyData<3> make_data(const double* obs_locs, const double* obs_normals, long n_obs,
                       const double* src_locs, const double* src_normals,
                       const double* src_weights, long n_src)
{
    NBodyData<3> d;
    d.obs_locs.resize(n_obs);
    d.obs_normals.resize(n_obs);
    d.src_locs.resize(n_src);
    d.src_normals.resize(n_src);
    d.src_weights.resize(n_src);
    for (long i = 0; i < n_obs; i++) {
        for (int k = 0; k < 3; k++) {
            d.obs_locs[i][k] = obs_locs[3 * i + k];
            d.obs_normals[i][k] = obs_normals[3 * i + k];
        }
    }
    for (long i = 0; i < n_src; i++) {
        for (int k = 0; k < 3; k++) {
            d.src_locs[i][k] = src_locs[3 * i + k];
            d.src_normals[i][k] = src_normals[3 * i + k];
        }
        d.src_weights[i] = src_weights[i];
    }
    return d;
}

std::unique_ptr<Kernel<3, 1, 1>> scalar_kernel(int id)
{
    if (id == 0) return std::unique_ptr<Kernel<3, 1, 1>>(new LaplaceSingle<3>());
    if (id == 1) return std::unique_ptr<Kernel<3, 1, 1>>(new LaplaceDouble<3>());
    if (id == 5) return std::unique_ptr<Kernel<3, 1, 1>>(new IdentityScalar<3>());
    return nullptr;
}

std::unique_ptr<Kernel<3, 3, 3>> tensor_kernel(int id, double mu, double nu)
{
    if (id == 2) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticDisplacement<3>(mu, nu));
    if (id == 3) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticTraction<3>(mu, nu));
    if (id == 4) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticAdjointTraction<3>(mu, nu));
    if (id == 6) return std::unique_ptr<Kernel<3, 3, 3>>(new ElasticHypersingular<3>(mu, nu));
    return nullptr;
}

template <typename Op>
void collect_cells(const Octree<3>& c, std::vector<const Octree<3>*>& out)
{
    out.push_back(&c);
    for (auto& ch : c.children) {
        if (ch != nullptr) collect_cells<Op>(*ch, out);
    }
}

template <typename Op>
const Octree<3>& tree_of(const Op& op, int which)
{
    return which == 0 ? op.src_oct : op.obs_oct;
}

template <typename Op>
long tree_cells(const Op& op, int which, long* level, long* index, double* center,
                double* hw, long* n_idx, long* n_children)
{
    std::vector<const Octree<3>*> cells;
    collect_cells<Op>(tree_of(op, which), cells);
    for (size_t i = 0; i < cells.size(); i++) {
        auto c = cells[i];
        if (level) level[i] = (long)c->level;
        if (index) index[i] = (long)c->index;
        if (center) for (int k = 0; k < 3; k++) center[3 * i + k] = c->bounds.center[k];
        if (hw) for (int k = 0; k < 3; k++) hw[3 * i + k] = c->bounds.half_width[k];
        if (n_idx) n_idx[i] = (long)c->indices.size();
        if (n_children) n_children[i] = (long)c->n_immediate_children();
    }
    return (long)cells.size();
}

template <typename Op>
long tree_indices(const Op& op, int which, long* out)
{
    std::vector<const Octree<3>*> cells;
    collect_cells<Op>(tree_of(op, which), cells);
    long k = 0;
    for (auto c : cells) {
        for (auto idx : c->indices) {
            if (out) out[k] = (long)idx;
            k++;
        }
    }
    return k;
}

template <typename Op>
long task_list(const Op& op, int kind, long* a, long* b)
{
    const auto& t = op.tasks;
    auto cell_list = [&](const std::vector<FMMTasks<3>::CellTask>& v) {
        for (size_t i = 0; i < v.size(); i++) {
            if (a) a[i] = (long)v[i].cell.index;
            if (b) b[i] = -1;
        }
        return (long)v.size();
    };
    auto pair_list = [&](const std::vector<FMMTasks<3>::CellPairTask>& v) {
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
template <typename Op>
void apply_masked(const Op& op, int mask, const double* x, double* y)
{
    std::vector<double> xv(x, x + op.n_cols());
    std::vector<double> out;
    if (mask == 0xff) {
        out = op.apply(xv);
    } else {
        // Task entries hold references (not assignable): copy-construct them.
        FMMTasks<3> sub;
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

}  // namespace

extern "C" {

void* ref_fmm_create(int kernel, double mu, double nu,
                     const double* obs_locs, const double* obs_normals, long n_obs,
                     const double* src_locs, const double* src_normals,
                     const double* src_weights, long n_src,
                     double mac, long order, long min_pts, double d, int small_cells)
{
    auto data = make_data(obs_locs, obs_normals, n_obs, src_locs, src_normals,
                          src_weights, n_src);
    FMMConfig cfg(mac, (size_t)order, (size_t)min_pts, d, small_cells != 0);
    // Cell indices are assigned inside an omp critical section during the
    // parallel level-0 loop; one thread makes them deterministic (post-order).
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    auto h = new Handle();
    h->kernel = kernel;
    if (auto k1 = scalar_kernel(kernel)) {
        h->R = 1;
        h->op1.reset(new FMMOperator<3, 1, 1>(*k1, data, cfg));
    } else if (auto k3 = tensor_kernel(kernel, mu, nu)) {
        h->R = 3;
        h->op3.reset(new FMMOperator<3, 3, 3>(*k3, data, cfg));
    } else {
        delete h;
        h = nullptr;
    }
    omp_set_num_threads(saved);
    return h;
}

void ref_fmm_destroy(void* p) { delete static_cast<Handle*>(p); }

void ref_fmm_apply_masked(void* p, int mask, const double* x, double* y)
{
    auto h = static_cast<Handle*>(p);
    if (h->op1) apply_masked(*h->op1, mask, x, y);
    else apply_masked(*h->op3, mask, x, y);
}

void ref_fmm_apply(void* p, const double* x, double* y) { ref_fmm_apply_masked(p, 0xff, x, y); }

long ref_fmm_n_surf(void* p)
{
    auto h = static_cast<Handle*>(p);
    return h->op1 ? (long)h->op1->up_equiv_surface.pts.size()
                  : (long)h->op3->up_equiv_surface.pts.size();
}

long ref_fmm_tree_cells(void* p, int which, long* level, long* index, double* center,
                        double* hw, long* n_idx, long* n_children)
{
    auto h = static_cast<Handle*>(p);
    return h->op1 ? tree_cells(*h->op1, which, level, index, center, hw, n_idx, n_children)
                  : tree_cells(*h->op3, which, level, index, center, hw, n_idx, n_children);
}

long ref_fmm_tree_indices(void* p, int which, long* out)
{
    auto h = static_cast<Handle*>(p);
    return h->op1 ? tree_indices(*h->op1, which, out) : tree_indices(*h->op3, which, out);
}

long ref_fmm_list(void* p, int kind, long* a, long* b)
{
    auto h = static_cast<Handle*>(p);
    return h->op1 ? task_list(*h->op1, kind, a, b) : task_list(*h->op3, kind, a, b);
}

// which: 0 = up (source tree), 1 = down (observation tree).
long ref_fmm_c2e(void* p, int which, long level, double* out)
{
    auto h = static_cast<Handle*>(p);
    const CheckToEquiv& ops = h->op1
        ? (which == 0 ? h->op1->up_check_to_equiv : h->op1->down_check_to_equiv)
        : (which == 0 ? h->op3->up_check_to_equiv : h->op3->down_check_to_equiv);
    if (level < 0) return (long)ops.size();
    if ((size_t)level >= ops.size()) return -1;
    if (out) std::memcpy(out, ops[level].data(), ops[level].size() * sizeof(double));
    return (long)ops[level].size();
}

// Matrix-free direct sum through the reference's nbody_eval.
int ref_direct_apply(int kernel, double mu, double nu,
                     const double* obs_locs, const double* obs_normals, long n_obs,
                     const double* src_locs, const double* src_normals,
                     const double* src_weights, long n_src, const double* x, double* y)
{
    auto data = make_data(obs_locs, obs_normals, n_obs, src_locs, src_normals,
                          src_weights, n_src);
    std::vector<double> out;
    if (auto k1 = scalar_kernel(kernel)) {
        out = nbody_eval(*k1, data, x);
    } else if (auto k3 = tensor_kernel(kernel, mu, nu)) {
        out = nbody_eval(*k3, data, x);
    } else {
        return -1;
    }
    std::memcpy(y, out.data(), out.size() * sizeof(double));
    return 0;
}

// One kernel tensor K(obs, src, nobs, nsrc) (row-major R x C).
int ref_kernel(int kernel, double mu, double nu, const double* obs, const double* src,
               const double* nobs, const double* nsrc, double* out)
{
    Vec<double, 3> o{obs[0], obs[1], obs[2]}, s{src[0], src[1], src[2]};
    Vec<double, 3> no{nobs[0], nobs[1], nobs[2]}, ns{nsrc[0], nsrc[1], nsrc[2]};
    if (auto k1 = scalar_kernel(kernel)) {
        out[0] = (*k1)(o, s, no, ns)[0][0];
        return 1;
    }
    if (auto k3 = tensor_kernel(kernel, mu, nu)) {
        auto v = (*k3)(o, s, no, ns);
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) out[3 * a + b] = v[a][b];
        return 9;
    }
    return -1;
}

// Unit translation-surface points for a requested order (n x 3).
long ref_surface(long order, double* pts)
{
    auto s = TranslationSurface<3>::make_surrounding_surface((size_t)order);
    if (pts) {
        for (size_t i = 0; i < s.pts.size(); i++)
            for (int k = 0; k < 3; k++) pts[3 * i + k] = s.pts[i][k];
    }
    return (long)s.pts.size();
}

}  // extern "C"
