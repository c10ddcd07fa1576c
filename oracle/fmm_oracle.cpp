// ORACLE -- test infrastructure, not product code.
//
// A CPU restatement of the reference KIFMM operator apply (tbenthompson/3bem,
// cpp/fmm.{h,cpp}, cpp/octree.cpp, cpp/geometry.cpp, cpp/kernel.h,
// cpp/laplace_kernels.h, cpp/elastic_kernels.h, cpp/nbody_operator.h), used
// only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline /
// reference arm, to check results.  The product (3bem_gb300/) never links it.
//
// Floating-point operations are written in the reference's evaluation order
// (and this file is compiled with -ffp-contract=off) so that with one thread
// the restatement reproduces the reference bit for bit; it is pinned against
// the reference compiled from its own sources (oracle/_ref) and against the
// fixtures in tests/golden.  The check-to-equivalent pseudo-inverses are
// supplied by the Python side (oracle/oracle.py) through LAPACK dgesvd, like
// the reference's svd_pseudoinverse (cpp/blas_wrapper.cpp:67-127).
//
// Kernel ids: 0 LaplaceSingle, 1 LaplaceDouble, 2 ElasticDisplacement,
// 3 ElasticTraction, 4 ElasticAdjointTraction, 5 IdentityScalar,
// 6 ElasticHypersingular (3D); 16 LaplaceSingle, 17 LaplaceDouble,
// 18 LaplaceHypersingular, 19 ElasticDisplacement, 20 ElasticTraction,
// 21 ElasticAdjointTraction, 22 ElasticHypersingular, 23 IdentityScalar (2D:
// FMMOperator<2,1,1> and <2,2,2>, cpp/fmm.cpp:651-652).  Points are passed as
// [n][3] for both; a 2D operator reads x and y and keeps z = 0, which leaves
// every sum, product and square root of the 2D arithmetic unchanged.
#include <cmath>
#include <cstring>
#include <cstdint>
#include <vector>
#include <memory>
#include <array>
#include <algorithm>
#include <omp.h>

namespace {

typedef std::array<double, 3> V3;

inline double dot3(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline double dot2(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1]; }

inline bool valid_kernel(int id) { return (id >= 0 && id <= 6) || (id >= 16 && id <= 23); }
inline int space_dim(int id) { return id >= 16 ? 2 : 3; }

// ---------------------------------------------------------------- kernels
// cpp/kernel.h:19-33: delta = src - obs, zero tensor when r2 < 1e-12.
struct KernelSpec {
    int id;
    int R;
    double mu, nu;
    // constants precomputed like the reference's constructors
    double c1, c2, c3 = 0.0, c4 = 0.0;
};

KernelSpec make_kernel(int id, double mu, double nu)
{
    const int R = (id == 2 || id == 3 || id == 4 || id == 6) ? 3 : (id >= 19 && id <= 22) ? 2 : 1;
    KernelSpec k{id, R, mu, nu, 0.0, 0.0};
    if (id == 19) {  // cpp/elastic_kernels.h:29-34
        k.c1 = 1.0 / (8 * M_PI * mu * (1 - nu));
        k.c2 = 3 - 4 * nu;
    } else if (id == 20 || id == 21) {  // cpp/elastic_kernels.h:67-72, 109-114
        k.c1 = 1.0 / (4 * M_PI * (1 - nu));
        k.c2 = 1 - 2 * nu;
    } else if (id == 22) {  // cpp/elastic_kernels.h:150-155
        k.c2 = 1 - 2 * nu;
    }
    if (id == 2) {  // cpp/elastic_kernels.h:198-203
        k.c1 = 1.0 / (16 * M_PI * mu * (1 - nu));
        k.c2 = 3 - 4 * nu;
    } else if (id == 3 || id == 4) {  // cpp/elastic_kernels.h:236-241, 278-283
        k.c1 = 1.0 / (8 * M_PI * (1 - nu));
        k.c2 = 1 - 2 * nu;
    } else if (id == 6) {  // cpp/elastic_kernels.h:323-331
        k.c1 = mu / (4 * M_PI * (1 - nu));
        k.c2 = 1 - 2 * nu;
        k.c3 = 3 * nu;
        k.c4 = -1 + 4 * nu;
    }
    return k;
}

// Writes the R x C tensor (row-major) into out.
inline void kernel_eval(const KernelSpec& K, const V3& obs, const V3& src, const V3& nobs,
                        const V3& nsrc, double* out)
{
    const V3 d{src[0] - obs[0], src[1] - obs[1], src[2] - obs[2]};
    const double r2 = dot3(d, d);
    const int n = K.R * K.R;
    if (r2 < 1e-12) {
        for (int i = 0; i < n; i++) out[i] = 0.0;
        return;
    }
    switch (K.id) {
    case 0:  // cpp/laplace_kernels.h:25
        out[0] = 1.0 / (4.0 * M_PI * std::sqrt(r2));
        return;
    case 1:  // cpp/laplace_kernels.h:41
        out[0] = dot3(nsrc, d) / (4 * M_PI * r2 * std::sqrt(r2));
        return;
    case 2: {  // cpp/elastic_kernels.h:206-217
        for (int k = 0; k < 3; k++) {
            for (int j = 0; j < 3; j++) {
                double r = std::sqrt(r2);
                out[3 * k + j] = (K.c1 / r) * (K.c2 * (k == j ? 1.0 : 0.0) + d[k] * d[j] / r2);
            }
        }
        return;
    }
    case 3: {  // cpp/elastic_kernels.h:244-259
        const double r = std::sqrt(r2);
        const double drdn = dot3(d, nsrc) / r;
        for (int k = 0; k < 3; k++) {
            for (int j = 0; j < 3; j++) {
                const double term1 = (K.c2 * (k == j ? 1.0 : 0.0) + 3 * d[k] * d[j] / r2);
                const double term2 = K.c2 * (nsrc[j] * d[k] - nsrc[k] * d[j]) / r;
                out[3 * k + j] = -(K.c1 / r2) * (term1 * drdn - term2);
            }
        }
        return;
    }
    case 4: {  // cpp/elastic_kernels.h:286-301
        double r = std::sqrt(r2);
        const double drdm = dot3(d, nobs) / r;
        for (int k = 0; k < 3; k++) {
            for (int j = 0; j < 3; j++) {
                const double term1 = (K.c2 * (k == j ? 1.0 : 0.0) + 3 * d[k] * d[j] / r2);
                const double term2 = K.c2 * (nobs[j] * d[k] - nobs[k] * d[j]) / r;
                out[3 * k + j] = (K.c1 / r2) * (term1 * drdm + term2);
            }
        }
        return;
    }
    case 6: {  // cpp/elastic_kernels.h:333-357: traction (observation normal m) of the
               // displacement of a dislocation (source normal n)
        const double r = std::sqrt(r2);
        // Vec / scalar multiplies by the reciprocal (cpp/vec_ops.h:151-155)
        const double ir = 1 / r;
        const V3 e{d[0] * ir, d[1] * ir, d[2] * ir};
        const double em = dot3(d, nobs) / r;
        const double en = dot3(e, nsrc);
        const double nm = dot3(nsrc, nobs);
        const double C = K.c1 / (r2 * r);
        for (int k = 0; k < 3; k++) {
            for (int j = 0; j < 3; j++) {
                const double dkj = k == j ? 1.0 : 0.0;
                const double t1 = 3 * en * (K.c2 * nobs[k] * e[j] + K.nu * (nobs[j] * e[k] + dkj * em) -
                                            5 * e[k] * e[j] * em);
                const double t2 = K.c2 * (3 * nsrc[j] * e[k] * em + dkj * nm + nsrc[k] * nobs[j]);
                const double t3 = K.c3 * (nsrc[k] * e[j] * em + nm * e[k] * e[j]);
                const double t4 = K.c4 * nsrc[j] * nobs[k];
                out[3 * k + j] = C * (t1 + t2 + t3 + t4);
            }
        }
        return;
    }
    case 16:  // cpp/laplace_kernels.h:70
        out[0] = std::log(std::sqrt(r2)) / (2 * M_PI);
        return;
    case 17:  // cpp/laplace_kernels.h:89
        out[0] = dot2(nsrc, d) / (2 * M_PI * r2);
        return;
    case 18:  // cpp/laplace_kernels.h:104-106
        out[0] = ((-dot2(nobs, nsrc) / r2) + ((2 * dot2(nsrc, d) * dot2(nobs, d)) / (r2 * r2))) /
                 (2 * M_PI);
        return;
    case 19: {  // cpp/elastic_kernels.h:36-49
        const double r = std::sqrt(r2);
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                out[2 * k + j] =
                    K.c1 * (-K.c2 * (k == j ? 1.0 : 0.0) * std::log(r) + d[k] * d[j] / r2);
        return;
    }
    case 20: {  // cpp/elastic_kernels.h:74-91
        const double r = std::sqrt(r2);
        const double drdn = dot2(d, nsrc) / r;
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++) {
                const double term1 = (K.c2 * (k == j ? 1.0 : 0.0) + 2 * d[k] * d[j] / r2);
                const double term2 = K.c2 * (nsrc[j] * d[k] - nsrc[k] * d[j]) / r;
                out[2 * k + j] = -(K.c1 / r) * (term1 * drdn - term2);
            }
        return;
    }
    case 21: {  // cpp/elastic_kernels.h:116-133
        const double r = std::sqrt(r2);
        const double drdm = dot2(d, nobs) / r;
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++) {
                const double term1 = (K.c2 * (k == j ? 1.0 : 0.0) + 2 * d[k] * d[j] / r2);
                const double term2 = K.c2 * (nobs[j] * d[k] - nobs[k] * d[j]) / r;
                out[2 * k + j] = (K.c1 / r) * (term1 * drdm + term2);
            }
        return;
    }
    case 22: {  // cpp/elastic_kernels.h:157-181
        const double r = std::sqrt(r2);
        const double ir = 1 / r;  // Vec / scalar, cpp/vec_ops.h:151-155
        const V3 e{d[0] * ir, d[1] * ir, 0.0};
        const double drdn = dot2(e, nsrc);
        const double drdm = dot2(e, nobs);
        const double nm = dot2(nsrc, nobs);
        const double nu = K.nu;
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++) {
                const double dkj = k == j ? 1.0 : 0.0;
                const double line1 = 2 * drdn * (K.c2 * nobs[k] * e[j] +
                                                 nu * (nobs[j] * e[k] + dkj * drdm) -
                                                 4 * e[k] * e[j] * drdm);
                const double line2 = K.c2 * (2 * nsrc[j] * e[k] * drdm + dkj * nm + nsrc[k] * nobs[j]);
                const double line3 = 2 * nu * (nsrc[k] * e[j] * drdm + nm * e[k] * e[j]);
                const double line4 = -(1 - 4 * nu) * nsrc[j] * nobs[k];
                const double C = (K.mu / (2 * M_PI * (1 - nu) * r2));
                out[2 * k + j] = C * (line1 + line2 + line3 + line4);
            }
        return;
    }
    default:  // IdentityScalar, cpp/identity_kernels.h:13-30 (ids 5 and 23)
        out[0] = 1.0;
        return;
    }
}

// Point set with the reference NBodyData layout (cpp/nbody_operator.h:29-36).
struct Pts {
    std::vector<V3> locs, normals;
    std::vector<double> weights;  // sources only
};

// nbody_eval (cpp/nbody_operator.h:117-141): out[d1*n_obs+i] += (w_j K)[d1][d2] x[d2*n_src+j]
std::vector<double> nbody_eval(const KernelSpec& K, const std::vector<V3>& obs_locs,
                               const std::vector<V3>& obs_normals,
                               const std::vector<V3>& src_locs,
                               const std::vector<V3>& src_normals,
                               const std::vector<double>& src_weights, const double* x)
{
    const size_t no = obs_locs.size(), ns = src_locs.size();
    const int R = K.R;
    std::vector<double> out(R * no, 0.0);
    double kv[9];
    for (size_t i = 0; i < no; i++) {
        for (size_t j = 0; j < ns; j++) {
            kernel_eval(K, obs_locs[i], src_locs[j], obs_normals[i], src_normals[j], kv);
            for (int e = 0; e < R * R; e++) kv[e] = src_weights[j] * kv[e];
            for (int d1 = 0; d1 < R; d1++) {
                size_t row = d1 * no + i;
                for (int d2 = 0; d2 < R; d2++) {
                    size_t col = d2 * ns + j;
                    out[row] += kv[d1 * R + d2] * x[col];
                }
            }
        }
    }
    return out;
}

// nbody_matrix (cpp/nbody_operator.h:87-115), row-major (R*no) x (C*ns).
std::vector<double> nbody_matrix(const KernelSpec& K, const std::vector<V3>& obs_locs,
                                 const std::vector<V3>& obs_normals,
                                 const std::vector<V3>& src_locs,
                                 const std::vector<V3>& src_normals,
                                 const std::vector<double>& src_weights)
{
    const size_t no = obs_locs.size(), ns = src_locs.size();
    const int R = K.R;
    std::vector<double> op(no * ns * R * R);
    double kv[9];
    for (size_t i = 0; i < no; i++) {
        for (size_t j = 0; j < ns; j++) {
            kernel_eval(K, obs_locs[i], src_locs[j], obs_normals[i], src_normals[j], kv);
            for (int d1 = 0; d1 < R; d1++) {
                size_t row = d1 * no + i;
                for (int d2 = 0; d2 < R; d2++) {
                    size_t col = d2 * ns + j;
                    op[row * R * ns + col] = src_weights[j] * kv[d1 * R + d2];
                }
            }
        }
    }
    return op;
}

// mat_vec (cpp/fmm.cpp:58-70): naive square product.
std::vector<double> mat_vec(const std::vector<double>& A, const std::vector<double>& x)
{
    const size_t n = x.size();
    std::vector<double> out(n, 0.0);
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < n; j++) out[i] += A[i * n + j] * x[j];
    return out;
}

// ---------------------------------------------------------------- geometry
struct Box {
    V3 center, hw;
};

// Box::bounding_box for zero-radius balls (cpp/geometry.cpp:61-80).
Box bounding_box(const std::vector<V3>& pts, const std::vector<size_t>& idx)
{
    if (idx.empty()) return Box{{0, 0, 0}, {0, 0, 0}};
    V3 mn = pts[idx[0]], mx = pts[idx[0]];
    for (size_t i = 1; i < idx.size(); i++) {
        const V3& c = pts[idx[i]];
        for (int d = 0; d < 3; d++) {
            mn[d] = std::min(mn[d], c[d] - 0.0);
            mx[d] = std::max(mx[d], c[d] + 0.0);
        }
    }
    Box b;
    for (int d = 0; d < 3; d++) {
        b.center[d] = (mx[d] + mn[d]) / 2.0;
        b.hw[d] = (mx[d] - mn[d]) / 2.0;
    }
    return b;
}

// expand_by_max_axis_multiple (cpp/geometry.cpp:13-17) over the first dim axes.
Box expand(const Box& b, double factor, int dim)
{
    double m = b.hw[0];
    for (int d = 1; d < dim; d++) m = std::max(m, b.hw[d]);
    double e = factor * m;
    Box out = b;
    for (int d = 0; d < dim; d++) out.hw[d] = b.hw[d] + e;
    return out;
}

// get_subcell with make_child_idx bit order: the last axis is bit 0, the
// first axis bit dim - 1 (cpp/geometry.cpp:20-28, cpp/octree.cpp:65-75).
Box subcell(const Box& b, int i, int dim)
{
    Box out = b;
    for (int d = 0; d < dim; d++) {
        const int idx = (i >> (dim - 1 - d)) & 1;
        out.hw[d] = b.hw[d] / 2.0;
        out.center[d] = b.center[d] + ((static_cast<double>(idx) * 2) - 1) * out.hw[d];
    }
    return out;
}

// find_containing_subcell (cpp/geometry.cpp:83-95): '>' sends ties to the low child.
int containing_subcell(const Box& b, const V3& p, int dim)
{
    int c = 0;
    for (int d = 0; d < dim; d++) {
        if (p[d] > b.center[d]) c++;
        if (d < dim - 1) c <<= 1;
    }
    return c;
}

inline double hypot3(const V3& v) { return std::sqrt(dot3(v, v)); }

// ---------------------------------------------------------------- octree
struct Cell {
    Box bounds;
    std::vector<size_t> indices;
    size_t level;
    size_t index;
    std::array<std::unique_ptr<Cell>, 8> children;
    bool is_leaf() const
    {
        for (auto& c : children)
            if (c) return false;
        return true;
    }
    size_t n_immediate_children() const
    {
        size_t n = 0;
        for (auto& c : children)
            if (c) n++;
        return n;
    }
};

// build_children (cpp/octree.cpp:97-153), sequential: indices are handed out
// after a child's subtree is built, i.e. in post-order.
std::array<std::unique_ptr<Cell>, 8> build_children(const Box& bounds, const std::vector<V3>& pts,
                                                    const std::vector<size_t>& indices,
                                                    size_t level, size_t min_pts,
                                                    size_t& next_index, int dim)
{
    std::array<std::unique_ptr<Cell>, 8> children;
    if (indices.size() <= min_pts) return children;
    std::array<std::vector<size_t>, 8> child_idx;
    for (size_t i = 0; i < indices.size(); i++)
        child_idx[containing_subcell(bounds, pts[indices[i]], dim)].push_back(indices[i]);
    for (int i = 0; i < (1 << dim); i++) {
        if (child_idx[i].empty()) continue;
        Box cb = subcell(bounds, i, dim);
        Box tight = bounding_box(pts, child_idx[i]);
        std::array<std::unique_ptr<Cell>, 8> sub;
        // recurse unless every point coincides (all half widths equal the zero
        // radius; a 2D operator's z half width is always zero)
        if (tight.hw[0] != 0.0 || tight.hw[1] != 0.0 || tight.hw[2] != 0.0)
            sub = build_children(cb, pts, child_idx[i], level + 1, min_pts, next_index, dim);
        size_t my_index = next_index++;
        children[i].reset(new Cell{cb, child_idx[i], level + 1, my_index, {}});
        children[i]->children = std::move(sub);
    }
    return children;
}

// make_octree (cpp/octree.cpp:156-171): root bounds are the expanded box, the
// children are cut from the unexpanded one.
std::unique_ptr<Cell> make_octree(const std::vector<V3>& pts, size_t min_pts, int dim)
{
    std::vector<size_t> all(pts.size());
    for (size_t i = 0; i < all.size(); i++) all[i] = i;
    Box box = bounding_box(pts, all);
    Box ebox = expand(box, 1e-5, dim);
    size_t next_index = 1;
    auto ch = build_children(box, pts, all, 0, min_pts, next_index, dim);
    std::unique_ptr<Cell> root(new Cell{ebox, all, 0, 0, {}});
    root->children = std::move(ch);
    return root;
}

size_t count_cells(const Cell& c)
{
    size_t n = 1;
    for (auto& ch : c.children)
        if (ch) n += count_cells(*ch);
    return n;
}

void preorder(const Cell& c, std::vector<const Cell*>& out)
{
    out.push_back(&c);
    for (auto& ch : c.children)
        if (ch) preorder(*ch, out);
}

// ---------------------------------------------------------------- surfaces
// surrounding_surface_sphere (cpp/fmm.cpp:22-45).
std::vector<V3> sphere_surface(size_t order)
{
    std::vector<V3> pts;
    double a = 4 * M_PI / order;
    double d = std::sqrt(a);
    auto M_theta = static_cast<size_t>(std::round(M_PI / d));
    double d_theta = M_PI / M_theta;
    double d_phi = a / d_theta;
    for (size_t m = 0; m < M_theta; m++) {
        double theta = M_PI * (m + 0.5) / M_theta;
        auto M_phi = static_cast<size_t>(std::round(2 * M_PI * std::sin(theta) / d_phi));
        for (size_t n = 0; n < M_phi; n++) {
            double phi = 2 * M_PI * n / M_phi;
            pts.push_back({std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi),
                           std::cos(theta)});
        }
    }
    return pts;
}

// TranslationSurface<2>::make_surrounding_surface (cpp/fmm.cpp:7-20): order
// points on the unit circle at theta_i = linspace(0, 2 pi, order + 1)[i]
// (cpp/numbers.cpp:5-12).
std::vector<V3> circle_surface(size_t order)
{
    std::vector<V3> pts;
    const double a = 0, b = 2 * M_PI;
    const size_t count = order + 1;
    for (size_t i = 0; i < order; i++) {
        const double theta = a + i * (b - a) / ((double)count - 1);
        pts.push_back({std::cos(theta), std::sin(theta), 0.0});
    }
    return pts;
}

std::vector<V3> unit_surface(size_t order, int dim)
{
    return dim == 2 ? circle_surface(order) : sphere_surface(order);
}

struct Surface {
    std::vector<V3> pts;      // scaled by r_ref (TranslationSurface::scale)
    std::vector<V3> normals;  // the unscaled unit points
    // TranslationSurface::move (cpp/fmm.h:19-31)
    std::vector<V3> move(const Box& b) const
    {
        double r = hypot3(b.hw);
        std::vector<V3> out(pts.size());
        for (size_t i = 0; i < pts.size(); i++)
            for (int d = 0; d < 3; d++) out[i][d] = r * pts[i][d] + b.center[d];
        return out;
    }
};

Surface make_surface(size_t order, double r_ref, int dim)
{
    Surface s;
    s.normals = unit_surface(order, dim);
    s.pts.resize(s.normals.size());
    for (size_t i = 0; i < s.pts.size(); i++)
        for (int d = 0; d < 3; d++) s.pts[i][d] = r_ref * s.normals[i][d];
    return s;
}

// ---------------------------------------------------------------- operator
struct Task {
    const Cell* obs;
    const Cell* src;
};

struct Oracle {
    KernelSpec K;
    Pts obs, src;  // obs.weights unused
    double mac;
    size_t order, min_pts;
    double dd;
    bool small_cells;
    Surface up_equiv, up_check, down_equiv, down_check;
    std::unique_ptr<Cell> src_oct, obs_oct;
    std::vector<std::vector<double>> up_c2e, down_c2e;
    std::vector<const Cell*> src_first_at_level, obs_first_at_level;
    std::vector<Task> p2ms, m2ms, p2ps, m2ps, p2ls, m2ls, l2ls, l2ps;
    std::vector<double> ones;

    size_t ns() const { return up_equiv.pts.size(); }

    // upward_traversal (cpp/fmm.cpp:561-575)
    void upward(const Cell& c)
    {
        if (c.is_leaf()) {
            p2ms.push_back({&c, nullptr});
        } else {
            for (auto& ch : c.children)
                if (ch) upward(*ch);
            m2ms.push_back({&c, nullptr});
        }
    }

    // dual_tree (cpp/fmm.cpp:578-630)
    void dual(const Cell& o, const Cell& s)
    {
        double r_src = hypot3(s.bounds.hw);
        double r_obs = hypot3(o.bounds.hw);
        double r_max = std::max(r_src, r_obs);
        double r_min = std::min(r_src, r_obs);
        V3 dc{o.bounds.center[0] - s.bounds.center[0], o.bounds.center[1] - s.bounds.center[1],
              o.bounds.center[2] - s.bounds.center[2]};
        double sep = hypot3(dc);
        if (r_max + mac * r_min <= mac * sep) {
            bool small_src = s.indices.size() <= down_equiv.pts.size();
            bool small_obs = o.indices.size() <= up_equiv.pts.size();
            if (small_cells) {
                if (small_obs && small_src) p2ps.push_back({&o, &s});
                else if (small_obs) m2ps.push_back({&o, &s});
                else if (small_src) p2ls.push_back({&o, &s});
                else m2ls.push_back({&o, &s});
            } else {
                m2ls.push_back({&o, &s});
            }
            return;
        }
        if (o.is_leaf() && s.is_leaf()) {
            p2ps.push_back({&o, &s});
            return;
        }
        bool src_is_shallower = o.level > s.level;
        bool split_src = (src_is_shallower && !s.is_leaf()) || o.is_leaf();
        if (split_src) {
            for (auto& ch : s.children)
                if (ch) dual(o, *ch);
        } else {
            for (auto& ch : o.children)
                if (ch) dual(*ch, s);
        }
    }

    // downward_traversal (cpp/fmm.cpp:633-648)
    void downward(const Cell& c)
    {
        if (c.is_leaf()) {
            l2ps.push_back({&c, nullptr});
        } else {
            l2ls.push_back({&c, nullptr});
            for (auto& ch : c.children)
                if (ch) downward(*ch);
        }
    }

    // build_check_to_equiv's choice of cell per level (cpp/fmm.cpp:130-160):
    // the first cell of each level in pre-order.
    static void first_at_level(const Cell& root, std::vector<const Cell*>& out)
    {
        std::vector<const Cell*> cells;
        preorder(root, cells);
        for (auto c : cells) {
            if (c->level >= out.size()) out.resize(c->level + 1, nullptr);
            if (!out[c->level]) out[c->level] = c;
        }
    }

    // The (R n_s) x (C n_s) system whose thresholded pseudo-inverse is the
    // check-to-equivalent operator (svd_inverse_nbody, cpp/fmm.cpp:113-127).
    std::vector<double> c2e_system(int which, size_t level) const
    {
        const Cell* c = which == 0 ? src_first_at_level[level] : obs_first_at_level[level];
        const Surface& eq = which == 0 ? up_equiv : down_equiv;
        const Surface& ck = which == 0 ? up_check : down_check;
        std::vector<double> w(eq.pts.size(), 1.0);
        return nbody_matrix(K, ck.move(c->bounds), ck.normals, eq.move(c->bounds), eq.normals, w);
    }

    void gather_src(const Cell& c, const std::vector<double>& x, std::vector<V3>& l,
                    std::vector<V3>& n, std::vector<double>& w, std::vector<double>& str) const
    {
        const size_t m = c.indices.size(), N = src.locs.size();
        l.resize(m);
        n.resize(m);
        w.resize(m);
        str.resize(K.R * m);
        for (size_t i = 0; i < m; i++) {
            l[i] = src.locs[c.indices[i]];
            n[i] = src.normals[c.indices[i]];
            w[i] = src.weights[c.indices[i]];
            for (int d = 0; d < K.R; d++) str[d * m + i] = x[d * N + c.indices[i]];
        }
    }

    void gather_obs(const Cell& c, std::vector<V3>& l, std::vector<V3>& n) const
    {
        const size_t m = c.indices.size();
        l.resize(m);
        n.resize(m);
        for (size_t i = 0; i < m; i++) {
            l[i] = obs.locs[c.indices[i]];
            n[i] = obs.normals[c.indices[i]];
        }
    }

    void scatter_out(const Cell& c, const std::vector<double>& res, std::vector<double>& out) const
    {
        const size_t m = c.indices.size(), N = obs.locs.size();
        for (size_t i = 0; i < m; i++)
            for (int d = 0; d < K.R; d++) {
#pragma omp atomic
                out[d * N + c.indices[i]] += res[d * m + i];
            }
    }

    // execute_tasks (cpp/fmm.cpp:445-548) restricted to the lists in `mask`
    // (bit order p2m, m2m, p2p, m2p, p2l, m2l, l2l, l2p).
    std::vector<double> apply(const double* xp, int mask, double list_fraction = 1.0) const
    {
        const size_t R = K.R, n = ns();
        const size_t n_src_cells = count_cells(*src_oct), n_obs_cells = count_cells(*obs_oct);
        std::vector<double> x(xp, xp + R * src.locs.size());
        std::vector<double> mult(n_src_cells * n * R, 0.0);
        std::vector<double> out(R * obs.locs.size(), 0.0);
        auto lim = [&](const std::vector<Task>& v) {
            return (long)std::llround(list_fraction * (double)v.size());
        };

        if (mask & 1) {  // P2M (cpp/fmm.cpp:163-202)
            long nt = lim(p2ms);
#pragma omp parallel for schedule(dynamic)
            for (long t = 0; t < nt; t++) {
                const Cell& c = *p2ms[t].obs;
                std::vector<V3> l, nn;
                std::vector<double> w, str;
                gather_src(c, x, l, nn, w, str);
                auto ce = nbody_eval(K, up_check.move(c.bounds), up_check.normals, l, nn, w,
                                     str.data());
                auto eq = mat_vec(up_c2e[c.level], ce);
                std::memcpy(&mult[c.index * n * R], eq.data(), R * n * sizeof(double));
            }
        }
        if (mask & 2) {  // M2M (cpp/fmm.cpp:205-251), serial post-order
            long nt = lim(m2ms);
            for (long t = 0; t < nt; t++) {
                const Cell& c = *m2ms[t].obs;
                size_t nc = c.n_immediate_children(), nsrc = nc * n;
                std::vector<V3> sl(nsrc), sn(nsrc);
                std::vector<double> sw(nsrc, 1.0), str(nsrc * R);
                size_t ci = 0;
                for (auto& ch : c.children) {
                    if (!ch) continue;
                    auto ep = up_equiv.move(ch->bounds);
                    for (size_t i = 0; i < n; i++) {
                        size_t idx = ci * n + i;
                        sl[idx] = ep[i];
                        sn[idx] = up_equiv.normals[i];
                        for (size_t d = 0; d < R; d++)
                            str[d * nsrc + idx] = mult[ch->index * n * R + d * n + i];
                    }
                    ci++;
                }
                auto ce = nbody_eval(K, up_check.move(c.bounds), up_check.normals, sl, sn, sw,
                                     str.data());
                auto eq = mat_vec(up_c2e[c.level], ce);
                std::memcpy(&mult[c.index * n * R], eq.data(), R * n * sizeof(double));
            }
        }
        if (mask & 4) {  // P2P (cpp/fmm.cpp:255-294)
            long nt = lim(p2ps);
#pragma omp parallel for schedule(dynamic)
            for (long t = 0; t < nt; t++) {
                std::vector<V3> sl, sn, ol, on;
                std::vector<double> sw, str;
                gather_src(*p2ps[t].src, x, sl, sn, sw, str);
                gather_obs(*p2ps[t].obs, ol, on);
                auto res = nbody_eval(K, ol, on, sl, sn, sw, str.data());
                scatter_out(*p2ps[t].obs, res, out);
            }
        }
        if (mask & 8) {  // M2P (cpp/fmm.cpp:333-360)
            long nt = lim(m2ps);
#pragma omp parallel for schedule(dynamic)
            for (long t = 0; t < nt; t++) {
                std::vector<V3> ol, on;
                gather_obs(*m2ps[t].obs, ol, on);
                auto res = nbody_eval(K, ol, on, up_equiv.move(m2ps[t].src->bounds),
                                      up_equiv.normals, ones,
                                      &mult[m2ps[t].src->index * n * R]);
                scatter_out(*m2ps[t].obs, res, out);
            }
        }
        std::vector<double> loc(n_obs_cells * n * R, 0.0);
        if (mask & 16) {  // P2L (cpp/fmm.cpp:297-330)
            long nt = lim(p2ls);
#pragma omp parallel for schedule(dynamic)
            for (long t = 0; t < nt; t++) {
                const Cell& oc = *p2ls[t].obs;
                std::vector<V3> l, nn;
                std::vector<double> w, str;
                gather_src(*p2ls[t].src, x, l, nn, w, str);
                auto ce = nbody_eval(K, down_check.move(oc.bounds), down_check.normals, l, nn, w,
                                     str.data());
                auto eq = mat_vec(down_c2e[oc.level], ce);
                for (size_t i = 0; i < eq.size(); i++) {
#pragma omp atomic
                    loc[oc.index * n * R + i] += eq[i];
                }
            }
        }
        if (mask & 32) {  // M2L (cpp/fmm.cpp:363-382)
            long nt = lim(m2ls);
#pragma omp parallel for schedule(dynamic)
            for (long t = 0; t < nt; t++) {
                const Cell& oc = *m2ls[t].obs;
                const Cell& sc = *m2ls[t].src;
                auto ce = nbody_eval(K, down_check.move(oc.bounds), down_check.normals,
                                     up_equiv.move(sc.bounds), up_equiv.normals, ones,
                                     &mult[sc.index * n * R]);
                auto eq = mat_vec(down_c2e[oc.level], ce);
                for (size_t i = 0; i < eq.size(); i++) {
#pragma omp atomic
                    loc[oc.index * n * R + i] += eq[i];
                }
            }
        }
        if (mask & 64) {  // L2L (cpp/fmm.cpp:385-413), serial pre-order
            long nt = lim(l2ls);
            for (long t = 0; t < nt; t++) {
                const Cell& c = *l2ls[t].obs;
                auto ep = down_equiv.move(c.bounds);
                for (auto& ch : c.children) {
                    if (!ch) continue;
                    auto ce = nbody_eval(K, down_check.move(ch->bounds), down_check.normals, ep,
                                         down_equiv.normals, ones, &loc[c.index * n * R]);
                    auto eq = mat_vec(down_c2e[c.level + 1], ce);
                    for (size_t i = 0; i < eq.size(); i++) loc[ch->index * n * R + i] += eq[i];
                }
            }
        }
        if (mask & 128) {  // L2P (cpp/fmm.cpp:416-441)
            long nt = lim(l2ps);
#pragma omp parallel for schedule(dynamic)
            for (long t = 0; t < nt; t++) {
                const Cell& c = *l2ps[t].obs;
                std::vector<V3> ol, on;
                gather_obs(c, ol, on);
                auto res = nbody_eval(K, ol, on, down_equiv.move(c.bounds), down_equiv.normals,
                                      ones, &loc[c.index * n * R]);
                scatter_out(c, res, out);
            }
        }
        return out;
    }
};

void read_pts(Pts& p, const double* locs, const double* normals, const double* weights, long n)
{
    p.locs.resize(n);
    p.normals.resize(n);
    if (weights) p.weights.assign(weights, weights + n);
    for (long i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            p.locs[i][d] = locs[3 * i + d];
            p.normals[i][d] = normals[3 * i + d];
        }
}

const std::vector<Task>& list_of(const Oracle& o, int kind)
{
    switch (kind) {
    case 0: return o.p2ms;
    case 1: return o.m2ms;
    case 2: return o.p2ps;
    case 3: return o.m2ps;
    case 4: return o.p2ls;
    case 5: return o.m2ls;
    case 6: return o.l2ls;
    default: return o.l2ps;
    }
}

}  // namespace

extern "C" {

// Build trees, surfaces and task lists (FMMOperator ctor, cpp/fmm.cpp:72-101).
// The check-to-equivalent operators are installed afterwards with
// oracle_set_c2e.  Returns nullptr on a bad kernel id or min_pts == 0.
void* oracle_create(int kernel, double mu, double nu, const double* obs_locs,
                    const double* obs_normals, long n_obs, const double* src_locs,
                    const double* src_normals, const double* src_weights, long n_src,
                    double mac, long order, long min_pts, double d, int small_cells)
{
    if (!valid_kernel(kernel) || min_pts <= 0 || order <= 0) return nullptr;
    const int dim = space_dim(kernel);
    auto o = new Oracle();
    o->K = make_kernel(kernel, mu, nu);
    read_pts(o->obs, obs_locs, obs_normals, nullptr, n_obs);
    read_pts(o->src, src_locs, src_normals, src_weights, n_src);
    o->mac = mac;
    o->order = order;
    o->min_pts = min_pts;
    o->dd = d;
    o->small_cells = small_cells != 0;
    double r_far = 4.0 - std::sqrt(2) - 2 * d;  // cpp/fmm.h:44,64
    o->up_check = make_surface(order, r_far, dim);
    o->up_equiv = make_surface(order, 0.3, dim);     // cpp/fmm.h:51
    o->down_check = make_surface(order, 0.3, dim);   // cpp/fmm.h:58
    o->down_equiv = make_surface(order, r_far, dim);
    o->src_oct = make_octree(o->src.locs, min_pts, dim);
    o->obs_oct = make_octree(o->obs.locs, min_pts, dim);
    Oracle::first_at_level(*o->src_oct, o->src_first_at_level);
    Oracle::first_at_level(*o->obs_oct, o->obs_first_at_level);
    o->up_c2e.resize(o->src_first_at_level.size());
    o->down_c2e.resize(o->obs_first_at_level.size());
    o->ones.assign(o->ns(), 1.0);
    o->upward(*o->src_oct);
    o->dual(*o->obs_oct, *o->src_oct);
    o->downward(*o->obs_oct);
    return o;
}

void oracle_destroy(void* p) { delete static_cast<Oracle*>(p); }

long oracle_n_surf(void* p) { return (long)static_cast<Oracle*>(p)->ns(); }

// which: 0 = up (source tree), 1 = down (observation tree)
long oracle_n_levels(void* p, int which)
{
    auto o = static_cast<Oracle*>(p);
    return (long)(which == 0 ? o->src_first_at_level.size() : o->obs_first_at_level.size());
}

long oracle_c2e_system(void* p, int which, long level, double* out)
{
    auto o = static_cast<Oracle*>(p);
    if (level < 0 || level >= oracle_n_levels(p, which)) return -1;
    auto m = o->c2e_system(which, (size_t)level);
    if (out) std::memcpy(out, m.data(), m.size() * sizeof(double));
    return (long)m.size();
}

long oracle_set_c2e(void* p, int which, long level, const double* mat)
{
    auto o = static_cast<Oracle*>(p);
    if (level < 0 || level >= oracle_n_levels(p, which)) return -1;
    size_t n = o->ns() * o->K.R;
    auto& v = which == 0 ? o->up_c2e : o->down_c2e;
    v[level].assign(mat, mat + n * n);
    return 0;
}

// Apply the FMM (or the lists in `mask`); `list_fraction` < 1 runs only that
// leading fraction of every list (a bounded CPU timing sample).
void oracle_apply(void* p, const double* x, double* y, int mask, double list_fraction)
{
    auto o = static_cast<Oracle*>(p);
    auto out = o->apply(x, mask, list_fraction);
    std::memcpy(y, out.data(), out.size() * sizeof(double));
}

// Cells in pre-order: level, post-order index, center, half width, #points, #children.
long oracle_tree_cells(void* p, int which, long* level, long* index, double* center,
                       double* hw, long* n_idx, long* n_children)
{
    auto o = static_cast<Oracle*>(p);
    std::vector<const Cell*> cells;
    preorder(which == 0 ? *o->src_oct : *o->obs_oct, cells);
    for (size_t i = 0; i < cells.size(); i++) {
        const Cell* c = cells[i];
        if (level) level[i] = (long)c->level;
        if (index) index[i] = (long)c->index;
        if (center) for (int d = 0; d < 3; d++) center[3 * i + d] = c->bounds.center[d];
        if (hw) for (int d = 0; d < 3; d++) hw[3 * i + d] = c->bounds.hw[d];
        if (n_idx) n_idx[i] = (long)c->indices.size();
        if (n_children) n_children[i] = (long)c->n_immediate_children();
    }
    return (long)cells.size();
}

long oracle_tree_indices(void* p, int which, long* out)
{
    auto o = static_cast<Oracle*>(p);
    std::vector<const Cell*> cells;
    preorder(which == 0 ? *o->src_oct : *o->obs_oct, cells);
    long k = 0;
    for (auto c : cells)
        for (auto i : c->indices) {
            if (out) out[k] = (long)i;
            k++;
        }
    return k;
}

long oracle_list(void* p, int kind, long* a, long* b)
{
    auto o = static_cast<Oracle*>(p);
    if (kind < 0 || kind > 7) return -1;
    const auto& v = list_of(*o, kind);
    for (size_t i = 0; i < v.size(); i++) {
        if (a) a[i] = (long)v[i].obs->index;
        if (b) b[i] = v[i].src ? (long)v[i].src->index : -1;
    }
    return (long)v.size();
}

// Unit translation-surface points ([n][3]; z = 0 for dim 2).
long oracle_surface(long order, int dim, double* pts)
{
    auto s = unit_surface((size_t)order, dim);
    if (pts)
        for (size_t i = 0; i < s.size(); i++)
            for (int d = 0; d < 3; d++) pts[3 * i + d] = s[i][d];
    return (long)s.size();
}

int oracle_kernel(int kernel, double mu, double nu, const double* obs, const double* src,
                  const double* nobs, const double* nsrc, double* out)
{
    if (!valid_kernel(kernel)) return -1;
    auto K = make_kernel(kernel, mu, nu);
    kernel_eval(K, {obs[0], obs[1], obs[2]}, {src[0], src[1], src[2]},
                {nobs[0], nobs[1], nobs[2]}, {nsrc[0], nsrc[1], nsrc[2]}, out);
    return K.R * K.R;
}

// Direct FP64 sum (nbody_eval over all pairs, cpp/nbody_operator.h:117-141),
// parallel over observation points; the densities are component-major.
int oracle_direct(int kernel, double mu, double nu, const double* obs_locs,
                  const double* obs_normals, long n_obs, const double* src_locs,
                  const double* src_normals, const double* src_weights, long n_src,
                  const double* x, double* y)
{
    if (!valid_kernel(kernel)) return -1;
    auto K = make_kernel(kernel, mu, nu);
    const int R = K.R;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n_obs; i++) {
        V3 o{obs_locs[3 * i], obs_locs[3 * i + 1], obs_locs[3 * i + 2]};
        V3 on{obs_normals[3 * i], obs_normals[3 * i + 1], obs_normals[3 * i + 2]};
        double acc[3] = {0, 0, 0};
        double kv[9];
        for (long j = 0; j < n_src; j++) {
            V3 s{src_locs[3 * j], src_locs[3 * j + 1], src_locs[3 * j + 2]};
            V3 sn{src_normals[3 * j], src_normals[3 * j + 1], src_normals[3 * j + 2]};
            kernel_eval(K, o, s, on, sn, kv);
            for (int e = 0; e < R * R; e++) kv[e] = src_weights[j] * kv[e];
            for (int d1 = 0; d1 < R; d1++)
                for (int d2 = 0; d2 < R; d2++) acc[d1] += kv[d1 * R + d2] * x[d2 * n_src + j];
        }
        for (int d1 = 0; d1 < R; d1++) y[d1 * n_obs + i] = acc[d1];
    }
    return 0;
}

int oracle_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
