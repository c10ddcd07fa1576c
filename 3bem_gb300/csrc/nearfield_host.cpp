// Host side of the nearfield construction: facet geometry, Gauss rules, the
// ball-octree facet search, Richardson (limit) directions and the Galerkin
// observation points.  Compiled without FMA contraction, like tree.cpp, so the
// geometry rounds as the reference's does on any host.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <exception>
#include <mutex>
#include <thread>

#include "nearfield.h"

namespace tbem {
namespace nf {

namespace {

inline V3 sub(const V3& a, const V3& b) { return V3{{a[0] - b[0], a[1] - b[1], a[2] - b[2]}}; }
inline V3 add(const V3& a, const V3& b) { return V3{{a[0] + b[0], a[1] + b[1], a[2] + b[2]}}; }
inline V3 scale(const V3& a, double s) { return V3{{a[0] * s, a[1] * s, a[2] * s}}; }
inline double dot(const V3& a, const V3& b, int dim)
{
    double s = a[0] * b[0] + a[1] * b[1];
    return dim == 3 ? s + a[2] * b[2] : s;
}
inline double norm(const V3& a, int dim) { return std::sqrt(dot(a, a, dim)); }
inline V3 cross(const V3& a, const V3& b)
{
    return V3{{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}};
}

// cpp/geometry.h:113-126
V3 unscaled_normal(const Facet& f, int dim)
{
    if (dim == 2) return V3{{-(f.c[1][1] - f.c[0][1]), f.c[1][0] - f.c[0][0], 0.0}};
    return cross(sub(f.c[2], f.c[0]), sub(f.c[2], f.c[1]));
}

// Vec / scalar multiplies by the reciprocal (cpp/vec_ops.h:151-155)
V3 normalized(const V3& v, int dim) { return scale(v, 1 / norm(v, dim)); }

double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// ---- segment / facet intersections (the queries decide_limit_dir makes;
// the same published methods as the oracle's restatement of GTEngine)

// 2D segments A, B: 0, 1 or 2 points (collinear overlaps give both ends).
int seg_seg(const V3& a0, const V3& a1, const V3& b0, const V3& b1, V3* out)
{
    const double rx = a1[0] - a0[0], ry = a1[1] - a0[1];
    const double sx = b1[0] - b0[0], sy = b1[1] - b0[1];
    const double qx = b0[0] - a0[0], qy = b0[1] - a0[1];
    const double den = cross2(rx, ry, sx, sy);
    auto at = [&](double t) { return V3{{a0[0] + t * rx, a0[1] + t * ry, 0.0}}; };
    if (den != 0.0) {
        const double t = cross2(qx, qy, sx, sy) / den, u = cross2(qx, qy, rx, ry) / den;
        if (t >= 0.0 && t <= 1.0 && u >= 0.0 && u <= 1.0) {
            out[0] = at(t);
            return 1;
        }
        return 0;
    }
    if (cross2(qx, qy, rx, ry) != 0.0) return 0;
    const double rr = rx * rx + ry * ry;
    if (rr == 0.0) {
        const double ss = sx * sx + sy * sy;
        if (ss == 0.0) {
            if (a0[0] == b0[0] && a0[1] == b0[1]) { out[0] = a0; return 1; }
            return 0;
        }
        const double u = ((a0[0] - b0[0]) * sx + (a0[1] - b0[1]) * sy) / ss;
        if (u >= 0.0 && u <= 1.0) { out[0] = a0; return 1; }
        return 0;
    }
    double t0 = (qx * rx + qy * ry) / rr;
    double t1 = ((b1[0] - a0[0]) * rx + (b1[1] - a0[1]) * ry) / rr;
    if (t0 > t1) std::swap(t0, t1);
    const double lo = std::max(0.0, t0), hi = std::min(1.0, t1);
    if (lo > hi) return 0;
    out[0] = at(lo);
    if (lo == hi) return 1;
    out[1] = at(hi);
    return 2;
}

// Moller-Trumbore with the segment parameter in [0, 1]; false when parallel.
bool seg_tri_hit(const Facet& T, const V3& s0, const V3& s1, V3& out)
{
    const V3 dir = sub(s1, s0), e1 = sub(T.c[1], T.c[0]), e2 = sub(T.c[2], T.c[0]);
    const V3 h = cross(dir, e2);
    const double a = dot(e1, h, 3);
    if (a == 0.0) return false;
    const double f = 1.0 / a;
    const V3 s = sub(s0, T.c[0]);
    const double u = f * dot(s, h, 3);
    if (u < 0.0 || u > 1.0) return false;
    const V3 q = cross(s, e1);
    const double v = f * dot(dir, q, 3);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = f * dot(e2, q, 3);
    if (t < 0.0 || t > 1.0) return false;
    out = add(s0, scale(dir, t));
    return true;
}

bool near_any(const std::vector<V3>& set, const V3& p, double thr)
{
    for (const V3& q : set)
        if (norm(sub(q, p), 3) < thr) return true;
    return false;
}

// Segment-triangle intersection with the coplanar case done in the
// triangle's plane: the segment against the three edges plus the segment
// ends lying on the triangle, duplicates within 1e-14 radii merged.
std::vector<V3> seg_tri(const Facet& T, const V3& s0, const V3& s1)
{
    V3 hit;
    if (seg_tri_hit(T, s0, s1, hit)) return {hit};
    const V3 n = normalized(cross(sub(T.c[2], T.c[0]), sub(T.c[1], T.c[0])), 3);
    const FacetInfo ti = facet_info(T, 3);
    const double thr = 1e-14 * ti.radius;
    if (std::fabs(dot(n, sub(s0, T.c[0]), 3)) > thr || std::fabs(dot(n, sub(s1, T.c[0]), 3)) > thr)
        return {};
    V3 ax0{{1, 0, 0}};
    double fd = dot(n, ax0, 3);
    if (fd > 0.95) {
        ax0 = V3{{0, 1, 0}};
        fd = dot(n, ax0, 3);
    }
    ax0 = normalized(sub(ax0, scale(n, fd)), 3);
    const V3 ax1 = cross(n, ax0);
    const V3& o = T.c[0];
    auto plane = [&](const V3& p) {
        const V3 d = sub(p, o);
        return V3{{dot(d, ax0, 3), dot(d, ax1, 3), 0.0}};
    };
    const V3 a0 = plane(s0), a1 = plane(s1);
    const V3 t2[3] = {plane(T.c[0]), plane(T.c[1]), plane(T.c[2])};
    std::vector<V3> out;
    for (int e = 0; e < 3; e++) {
        const V3& e0 = t2[e];
        const V3& e1 = t2[(e + 1) % 3];
        const V3 mid = scale(add(e0, e1), 0.5);
        const double ethr = 1e-14 * norm(sub(e0, mid), 2);
        V3 pts[2];
        const int k = seg_seg(a0, a1, e0, e1, pts);
        for (int i = 0; i < k; i++) {
            const V3 p3 = add(add(scale(ax0, pts[i][0]), scale(ax1, pts[i][1])), o);
            if (!near_any(out, p3, ethr)) out.push_back(p3);
        }
    }
    const V3 ends[2] = {s0, s1};
    for (const V3& e : ends)
        if (closest_point(e, T, 3).dist < thr && !near_any(out, e, thr)) out.push_back(e);
    return out;
}

std::vector<V3> seg_facet(const Facet& f, const V3& s0, const V3& s1, int dim)
{
    if (dim == 3) return seg_tri(f, s0, s1);
    V3 pts[2];
    const int k = seg_seg(f.c[0], f.c[1], s0, s1, pts);
    return std::vector<V3>(pts, pts + k);
}

// backup_halfway_from_intersection (cpp/limit_direction.cpp:57-84)
V3 backup_halfway(V3 end_pt, double len_scale, const V3& pt, const std::vector<size_t>& near,
                  size_t nearest, const FacetSet& all, int dim)
{
    for (size_t f : near) {
        if (f == nearest) continue;
        const std::vector<V3> hits = seg_facet(all.facet(f), end_pt, pt, dim);
        if (hits.size() == 1 && !(hits[0][0] == pt[0] && hits[0][1] == pt[1] && hits[0][2] == pt[2])) {
            const V3 to = sub(hits[0], pt);
            if (norm(to, dim) < 1e-12 * len_scale) continue;
            end_pt = add(pt, scale(to, 1 / 2.0));
        }
    }
    return end_pt;
}

// ref_to_real with the linear basis (cpp/numerics.h:61-100)
V3 ref_to_real(const double* xh, const Facet& f, int dim)
{
    V3 p{{0, 0, 0}};
    if (dim == 2) {
        const double b0 = 0.5 - 0.5 * xh[0], b1 = 0.5 + 0.5 * xh[0];
        for (int d = 0; d < 2; d++) p[d] = b0 * f.c[0][d] + b1 * f.c[1][d];
    } else {
        const double b0 = 1 - xh[0] - xh[1], b1 = xh[0], b2 = xh[1];
        for (int d = 0; d < 3; d++) p[d] = b0 * f.c[0][d] + b1 * f.c[1][d] + b2 * f.c[2][d];
    }
    return p;
}

}  // namespace

FacetInfo facet_info(const Facet& f, int dim)
{
    FacetInfo fi;
    V3 c{{0, 0, 0}};
    for (int v = 0; v < dim; v++) c = add(c, f.c[v]);
    c = scale(c, 1 / static_cast<double>(dim));
    double r2 = dot(sub(c, f.c[0]), sub(c, f.c[0]), dim);
    for (int v = 1; v < dim; v++) r2 = std::max(r2, dot(sub(c, f.c[v]), sub(c, f.c[v]), dim));
    fi.centroid = c;
    fi.radius = std::sqrt(r2);
    fi.length_scale = 2 * fi.radius;
    const V3 un = unscaled_normal(f, dim);
    fi.jacobian = dim == 2 ? 0.5 * norm(un, 2) : 2.0 * (0.5 * norm(un, 3));
    fi.normal = normalized(un, dim);
    return fi;
}

Closest closest_point(const V3& p, const Facet& f, int dim)
{
    Closest r;
    r.ref[0] = r.ref[1] = 0.0;
    if (dim == 2) {
        const V3 d = sub(f.c[1], f.c[0]);
        const double L2 = dot(d, d, 2);
        double t = 0.0;
        if (L2 > 0.0) {
            t = dot(sub(p, f.c[0]), d, 2) / L2;
            t = std::min(1.0, std::max(0.0, t));
        }
        r.pt = t == 1.0 ? f.c[1] : t == 0.0 ? f.c[0] : add(f.c[0], scale(d, t));
        r.pt[2] = 0.0;
        r.ref[0] = 2 * t - 1;
        r.dist = norm(sub(p, r.pt), 2);
        return r;
    }
    const V3 &a = f.c[0], &b = f.c[1], &c = f.c[2];
    const V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const double d1 = dot(ab, ap, 3), d2 = dot(ac, ap, 3);
    const V3 bp = sub(p, b);
    const double d3 = dot(ab, bp, 3), d4 = dot(ac, bp, 3);
    const V3 cp = sub(p, c);
    const double d5 = dot(ab, cp, 3), d6 = dot(ac, cp, 3);
    const double vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
    double v = 0.0, w = 0.0;
    V3 q;
    if (d1 <= 0.0 && d2 <= 0.0) {
        q = a;
    } else if (d3 >= 0.0 && d4 <= d3) {
        v = 1.0;
        q = b;
    } else if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        v = d1 / (d1 - d3);
        q = add(a, scale(ab, v));
    } else if (d6 >= 0.0 && d5 <= d6) {
        w = 1.0;
        q = c;
    } else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        w = d2 / (d2 - d6);
        q = add(a, scale(ac, w));
    } else if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        v = 1.0 - w;
        q = add(b, scale(sub(c, b), w));
    } else {
        const double inv = 1.0 / (va + vb + vc);
        v = vb * inv;
        w = vc * inv;
        q = add(add(a, scale(ab, v)), scale(ac, w));
    }
    r.ref[0] = v;
    r.ref[1] = w;
    r.pt = q;
    r.dist = norm(sub(p, q), 3);
    return r;
}

void gauss_rule(int n, std::vector<double>& x, std::vector<double>& w)
{
    // Newton on the Legendre recurrence from cos(pi (i + 3/4) / (n + 1/2)),
    // mirrored about 0 (the method of cpp/gauss_quad.cpp:9-52)
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const size_t N = (size_t)n;
    const size_t m = (N + 1) / 2;
    for (size_t i = 0; i < m; i++) {
        double xi = std::cos(M_PI * (i + (3.0 / 4.0)) / (N + 0.5));
        double dp = 0, dx = 10;
        while (std::fabs(dx) > 1e-14) {
            double p_cur = 1., p_last = 0.;
            for (size_t j = 0; j < N; ++j) {
                const double p_temp = p_last;
                p_last = p_cur;
                p_cur = ((2. * j + 1.) * xi * p_last - j * p_temp) / (j + 1);
            }
            dp = (N + 1) * (xi * p_cur - p_last) / (xi * xi - 1);
            dx = p_cur / dp;
            xi = xi - dx;
        }
        const double wi = 2 * (N + 1) * (N + 1) / (N * N * (1 - xi * xi) * dp * dp);
        x[i] = -xi;
        w[i] = wi;
        x[N - i - 1] = xi;
        w[N - i - 1] = wi;
    }
}

void gauss_facet(int dim, int n, std::vector<double>& x, std::vector<double>& w)
{
    std::vector<double> g, gw;
    gauss_rule(n, g, gw);
    x.clear();
    w.clear();
    if (dim == 2) {
        for (int i = 0; i < n; i++) {
            x.push_back(g[i]);
            x.push_back(0.0);
            w.push_back(gw[i]);
        }
        return;
    }
    // tensor product mapped to the triangle (0,0)-(1,0)-(0,1)
    // (tri_gauss, cpp/gauss_quad.cpp:118-153)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const double x01 = 0.5 * g[i] + 0.5, y01 = 0.5 * g[j] + 0.5;
            const double ww = gw[i] * gw[j];
            x.push_back(x01 * (1 - y01));
            x.push_back(y01);
            w.push_back((ww / 4.0) * (1 - y01));
        }
}

// ---- facet set with the reference's ball octree

FacetSet::FacetSet(const std::vector<Facet>& facets, int dim) : dim_(dim), facets_(facets)
{
    info_.reserve(facets.size());
    for (const Facet& f : facets_) info_.push_back(facet_info(f, dim_));
    build();
}

namespace {
struct BallBox {
    double c[3], h[3];
};

// Box::bounding_box over balls (cpp/geometry.cpp:61-80)
BallBox ball_bounds(const std::vector<FacetInfo>& b, const std::vector<size_t>& idx, int dim)
{
    BallBox o{{0, 0, 0}, {0, 0, 0}};
    if (idx.empty()) return o;
    double mn[3], mx[3];
    for (int d = 0; d < dim; d++) {
        mn[d] = b[idx[0]].centroid[d] - b[idx[0]].radius;
        mx[d] = b[idx[0]].centroid[d] + b[idx[0]].radius;
    }
    for (size_t i = 1; i < idx.size(); i++)
        for (int d = 0; d < dim; d++) {
            mn[d] = std::min(mn[d], b[idx[i]].centroid[d] - b[idx[i]].radius);
            mx[d] = std::max(mx[d], b[idx[i]].centroid[d] + b[idx[i]].radius);
        }
    for (int d = 0; d < dim; d++) {
        o.c[d] = (mx[d] + mn[d]) / 2.0;
        o.h[d] = (mx[d] - mn[d]) / 2.0;
    }
    return o;
}

struct BallNode {
    BallBox bounds;     // geometric cell (children are cut from it)
    BallBox tight;      // expanded tight box of the member balls
    std::vector<size_t> idx;
    int child[8];
};
}  // namespace

void FacetSet::build()
{
    // make_octree over balls with 20 per leaf (cpp/octree.cpp:95-176):
    // children split by ball centre, recursion stops when every half width of
    // a child's tight box equals its largest radius
    const size_t n = facets_.size();
    std::vector<BallNode> nodes;
    std::vector<size_t> all(n);
    for (size_t i = 0; i < n; i++) all[i] = i;
    auto expand = [&](BallBox b) {
        double m = b.h[0];
        for (int d = 1; d < dim_; d++) m = std::max(m, b.h[d]);
        const double e = 1e-5 * m;
        for (int d = 0; d < dim_; d++) b.h[d] = b.h[d] + e;
        return b;
    };
    BallNode root;
    const BallBox box = ball_bounds(info_, all, dim_);
    root.bounds = expand(box);
    root.tight = root.bounds;
    root.idx = all;
    for (int k = 0; k < 8; k++) root.child[k] = -1;
    nodes.push_back(root);
    struct Job { int node; BallBox cut; };
    std::vector<Job> stack{{0, box}};
    while (!stack.empty()) {
        Job jb = stack.back();
        stack.pop_back();
        const std::vector<size_t> idx = nodes[jb.node].idx;
        if (idx.size() <= 20) continue;
        std::vector<size_t> part[8];
        for (size_t i : idx) {
            int c = 0;
            for (int d = 0; d < dim_; d++) {
                if (info_[i].centroid[d] > jb.cut.c[d]) c++;
                if (d < dim_ - 1) c <<= 1;
            }
            part[c].push_back(i);
        }
        for (int o = 0; o < (1 << dim_); o++) {
            if (part[o].empty()) continue;
            BallNode ch;
            ch.bounds = jb.cut;
            for (int d = 0; d < dim_; d++) {
                const int bit = (o >> (dim_ - 1 - d)) & 1;
                ch.bounds.h[d] = jb.cut.h[d] / 2.0;
                ch.bounds.c[d] = jb.cut.c[d] + ((static_cast<double>(bit) * 2) - 1) * ch.bounds.h[d];
            }
            const BallBox tight = ball_bounds(info_, part[o], dim_);
            double largest = info_[part[o][0]].radius;
            for (size_t i : part[o]) largest = std::max(largest, info_[i].radius);
            bool split = false;
            for (int d = 0; d < dim_; d++) split = split || tight.h[d] != largest;
            ch.tight = expand(tight);
            ch.idx = std::move(part[o]);
            for (int k = 0; k < 8; k++) ch.child[k] = -1;
            nodes.push_back(std::move(ch));
            const int id = (int)nodes.size() - 1;
            nodes[jb.node].child[o] = id;
            if (split) stack.push_back({id, nodes[id].bounds});
        }
    }
    // flatten: children contiguous in child order, leaves' facets in pre-order
    cells_.clear();
    order_.clear();
    std::vector<int> q{0};
    std::vector<int> flat(nodes.size(), -1);
    for (size_t k = 0; k < q.size(); k++) {
        flat[q[k]] = (int)k;
        for (int o = 0; o < 8; o++)
            if (nodes[q[k]].child[o] >= 0) q.push_back(nodes[q[k]].child[o]);
    }
    cells_.resize(q.size());
    for (size_t k = 0; k < q.size(); k++) {
        const BallNode& nd = nodes[q[k]];
        Cell& c = cells_[k];
        for (int d = 0; d < 3; d++) {
            c.lo[d] = nd.tight.c[d] - nd.tight.h[d];
            c.hi[d] = nd.tight.c[d] + nd.tight.h[d];
            c.gc[d] = nd.bounds.c[d];
        }
        c.first_child = -1;
        c.n_children = 0;
        for (int o = 0; o < 8; o++)
            if (nd.child[o] >= 0) {
                if (c.first_child < 0) c.first_child = flat[nd.child[o]];
                c.n_children++;
            }
    }
    // pre-order ranges
    struct Fr { int node; int state; };
    std::vector<Fr> st{{0, 0}};
    while (!st.empty()) {
        Fr fr = st.back();
        st.pop_back();
        Cell& c = cells_[flat[fr.node]];
        if (fr.state == 0) {
            c.begin = (long)order_.size();
            bool leaf = true;
            for (int o = 0; o < 8; o++) leaf = leaf && nodes[fr.node].child[o] < 0;
            if (leaf) {
                for (size_t i : nodes[fr.node].idx) order_.push_back(i);
                c.end = (long)order_.size();
            } else {
                st.push_back({fr.node, 1});
                for (int o = 7; o >= 0; o--)
                    if (nodes[fr.node].child[o] >= 0) st.push_back({nodes[fr.node].child[o], 0});
            }
        } else {
            c.end = (long)order_.size();
        }
    }
}

// nearest_facet (cpp/nearest_neighbors.h:62-104): the closest child (by
// geometric centre) first, the others only when their ball box is within the
// best distance; strict '<' keeps the first of equal distances.
void FacetSet::nearest(int ci, const V3& p, size_t& best, double& best_d) const
{
    const Cell& c = cells_[ci];
    if (c.n_children == 0) {
        for (long k = c.begin; k < c.end; k++) {
            const size_t i = order_[k];
            if (norm(sub(info_[i].centroid, p), dim_) > best_d + info_[i].radius) continue;
            const double d = closest_point(p, facets_[i], dim_).dist;
            if (d < best_d) {
                best_d = d;
                best = i;
            }
        }
        return;
    }
    auto box_dist2 = [&](const Cell& cc) {
        double s = 0.0;
        for (int d = 0; d < dim_; d++) {
            const double mid = 0.5 * (cc.lo[d] + cc.hi[d]), hw = 0.5 * (cc.hi[d] - cc.lo[d]);
            const double e = std::fabs(p[d] - mid) - hw;
            if (e > 0.0) s += e * e;
        }
        return s;
    };
    // find_closest_nonempty_child (cpp/octree.cpp:44-60): the child whose
    // geometric centre is closest goes first
    int first = c.first_child;
    double fd = DBL_MAX;
    for (int k = 0; k < c.n_children; k++) {
        const Cell& cc = cells_[c.first_child + k];
        double s = 0.0;
        for (int d = 0; d < dim_; d++) s += (p[d] - cc.gc[d]) * (p[d] - cc.gc[d]);
        if (s < fd) {
            fd = s;
            first = c.first_child + k;
        }
    }
    nearest(first, p, best, best_d);
    for (int k = 0; k < c.n_children; k++) {
        const int cc = c.first_child + k;
        if (cc == first) continue;
        if (best_d < DBL_MAX && box_dist2(cells_[cc]) > best_d * best_d) continue;
        nearest(cc, p, best, best_d);
    }
}

void FacetSet::range(int ci, const V3& ctr, double r, std::vector<size_t>& out) const
{
    const Cell& c = cells_[ci];
    for (int d = 0; d < dim_; d++)
        if (ctr[d] + r < c.lo[d] || ctr[d] - r > c.hi[d]) return;
    if (c.n_children == 0) {
        for (long k = c.begin; k < c.end; k++) {
            const size_t i = order_[k];
            bool hit = true;  // balls_intersect (cpp/geometry.h:247-251): per axis
            for (int d = 0; d < dim_; d++)
                hit = hit && std::fabs(info_[i].centroid[d] - ctr[d]) <= info_[i].radius + r;
            if (hit) out.push_back(i);
        }
        return;
    }
    for (int k = 0; k < c.n_children; k++) range(c.first_child + k, ctr, r, out);
}

void FacetSet::find(const V3& p, double far_threshold, std::vector<size_t>& near, size_t& nearest_i,
                    double& dist) const
{
    near.clear();
    nearest_i = 0;
    dist = 0.0;
    if (facets_.empty()) return;
    double best_d = DBL_MAX;
    size_t best = 0;
    nearest(0, p, best, best_d);
    nearest_i = best;
    dist = best_d;
    const FacetInfo& nb = info_[best];
    const double R = nb.radius * far_threshold;
    std::vector<size_t> cand;
    range(0, nb.centroid, R, cand);
    for (size_t i : cand)
        if (closest_point(p, facets_[i], dim_).dist <= R) near.push_back(i);
}

V3 limit_direction(const V3& p, const FacetSet& all, int dim)
{
    std::vector<size_t> near;
    size_t nearest = 0;
    double dist = 0.0;
    all.find(p, 1.0, near, nearest, dist);
    const V3 zero{{0, 0, 0}};
    if (near.empty()) return zero;
    const FacetInfo& ci = all.info(nearest);
    const double len_scale = ci.radius * 2;
    if (dist > len_scale * 1e-2) return zero;
    const V3 end_pt = add(ci.centroid, scale(ci.normal, len_scale));
    const V3 interior = backup_halfway(end_pt, len_scale, ci.centroid, near, nearest, all, dim);
    const V3 backup = backup_halfway(interior, len_scale, p, near, nearest, all, dim);
    V3 d = scale(sub(backup, p), 0.4);
    if (dim == 2) d[2] = 0.0;
    return d;
}

void parallel_for(long n, const std::function<void(long)>& body, long grain)
{
    const long hw = (long)std::max(1u, std::thread::hardware_concurrency());
    const long nt = std::min(hw, std::max(1L, n / std::max(1L, grain)));
    if (nt <= 1) {
        for (long i = 0; i < n; i++) body(i);
        return;
    }
    std::vector<std::thread> th;
    std::exception_ptr failure;
    std::mutex m;
    for (long t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            try {
                for (long i = n * t / nt; i < n * (t + 1) / nt; i++) body(i);
            } catch (...) {  // handed to the caller after the join
                std::lock_guard<std::mutex> lock(m);
                if (!failure) failure = std::current_exception();
            }
        });
    for (auto& x : th) x.join();
    if (failure) std::rethrow_exception(failure);
}

ObsPoints galerkin_obs_points(const std::vector<Facet>& obs, const FacetSet& all, int order, int dim)
{
    std::vector<double> qx, qw;
    gauss_facet(dim, order, qx, qw);
    ObsPoints o;
    for (const Facet& f : obs) {
        const FacetInfo fi = facet_info(f, dim);
        for (size_t q = 0; q < qw.size(); q++) {
            o.loc.push_back(ref_to_real(&qx[2 * q], f, dim));
            o.normal.push_back(fi.normal);
        }
    }
    // the limit directions, point by point (the reference's interior_obs_pts loop)
    o.dir.resize(o.loc.size());
    parallel_for((long)o.loc.size(), [&](long i) { o.dir[i] = limit_direction(o.loc[i], all, dim); });
    return o;
}

TermPlan plan_terms(const ObsPoints& pts, const std::vector<Facet>& src, const FacetSet& src_set,
                    double far_threshold, int n_steps, int dim, bool farfield_only)
{
    TermPlan tp;
    const long n_pts = (long)pts.loc.size();
    // the nearfield facets of every point (NearfieldFacetFinder), then the
    // terms point by point
    std::vector<std::vector<size_t>> near_of(n_pts);
    parallel_for(n_pts, [&](long i) {
        size_t nearest = 0;
        double dist = 0.0;
        src_set.find(pts.loc[i], far_threshold, near_of[i], nearest, dist);
    });
    std::vector<long> tb(n_pts + 1, 0);
    for (long i = 0; i < n_pts; i++) tb[i + 1] = tb[i] + (long)near_of[i].size();
    const long n_terms = tb[n_pts];
    tp.t_obs.resize(n_terms);
    tp.t_fac.resize(n_terms);
    parallel_for(n_pts, [&](long i) {
        long t = tb[i];
        for (size_t f : near_of[i]) {
            tp.t_obs[t] = (int)i;
            tp.t_fac[t++] = (int)f;
        }
        std::vector<size_t>().swap(near_of[i]);
    });
    // each term's category as compute_term decides it (cpp/integral_term.cpp:
    // 33-53): 0 far, 1 near, 2 singular (near the facet with a limit direction)
    std::vector<char> cat(n_terms, 0), on_facet(n_terms, 0);
    if (!farfield_only)
        parallel_for(n_terms, [&](long t) {
            const long o = tp.t_obs[t], f = tp.t_fac[t];
            const double dist = closest_point(pts.loc[o], src[f], dim).dist;
            const double ls = src_set.info(f).length_scale;
            if (!(dist < far_threshold * ls)) return;
            double d2 = 0.0;
            for (int d = 0; d < dim; d++) d2 += pts.dir[o][d] * pts.dir[o][d];
            if (dist < 1.0 * ls && d2 > 1e-10 * ls) {
                cat[t] = 2;
            } else {
                cat[t] = 1;
                on_facet[t] = !(dist > 0.0);
            }
        });
    tp.on_facet = std::find(on_facet.begin(), on_facet.end(), 1) != on_facet.end();
    tp.first.resize(n_terms + 1);
    tp.first[0] = 0;
    for (long t = 0; t < n_terms; t++) tp.first[t + 1] = tp.first[t] + (cat[t] == 2 ? n_steps : 1);
    const long n_items = tp.first[n_terms];
    tp.sing.assign(n_terms, 0);
    tp.i_obs.resize(n_items);
    tp.i_fac.resize(n_items);
    tp.i_near.resize(n_items);
    tp.iloc.resize(3 * n_items);
    parallel_for(n_terms, [&](long t) {
        const long o = tp.t_obs[t], f = tp.t_fac[t];
        const V3& p = pts.loc[o];
        long i = tp.first[t];
        auto put = [&](int nearflag, const V3& at) {
            tp.i_obs[i] = (int)o;
            tp.i_fac[i] = (int)f;
            tp.i_near[i] = nearflag;
            for (int d = 0; d < 3; d++) tp.iloc[3 * i + d] = at[d];
            i++;
        };
        if (cat[t] != 2) {
            put(cat[t], p);
            return;
        }
        tp.sing[t] = 1;
        for (int k = 0; k < n_steps; k++) {  // get_step_loc (cpp/integral_term.cpp:55-60)
            const double step = 1.0 / std::pow(2.0, (double)k);
            const double sd = 1.0 * step;
            V3 q;
            for (int d = 0; d < 3; d++) q[d] = p[d] + sd * pts.dir[o][d];
            put(1, q);
        }
    });
    return tp;
}

void assemble_csr(const TermPlan& tp, const std::vector<double>& ivals, long n_pts, long n_src, int dim,
                  int R, int n_steps, bool negate, std::vector<double>& vals, std::vector<long>& cols,
                  std::vector<long>& row_ptr)
{
    const int E = dim * R * R;
    const long n_terms = (long)tp.t_obs.size();
    // the terms of point o are [tb[o], tb[o + 1]) (planned point by point)
    std::vector<long> tb(n_pts + 1, 0);
    for (long t = 0; t < n_terms; t++) tb[tp.t_obs[t] + 1]++;
    for (long o = 0; o < n_pts; o++) tb[o + 1] += tb[o];
    // row d1 * n_pts + o: the dim * R entries (basis b, component d2) of each
    // of o's terms, term after term -- where the reference's COO loop
    // (cpp/nearfield_operator.h:59-84) and csr_from_coo's stable order put them
    const long n_rows = R * n_pts, n_dofs = n_src * dim;
    row_ptr.assign(n_rows + 1, 0);
    for (long r = 0; r < n_rows; r++) {
        const long o = r % n_pts;
        row_ptr[r + 1] = row_ptr[r] + (tb[o + 1] - tb[o]) * dim * R;
    }
    vals.resize(row_ptr[n_rows]);
    cols.resize(row_ptr[n_rows]);
    parallel_for(n_pts, [&](long o) {
        std::vector<double> tab(n_steps), v(E);
        for (long t = tb[o]; t < tb[o + 1]; t++) {
            const double* x = &ivals[(size_t)tp.first[t] * E];
            for (int e = 0; e < E; e++) {
                double r = x[e];
                if (tp.sing[t]) {  // richardson_limit (cpp/richardson.h:10-34), step ratio 2
                    for (int k = 0; k < n_steps; k++) tab[k] = x[k * E + e];
                    for (int m = 1; m < n_steps; m++) {
                        const double mult = std::pow(2.0, m);
                        const double factor = 1.0 / (mult - 1.0);
                        for (int i = 0; i < n_steps - m; i++) tab[i] = factor * (mult * tab[i + 1] - tab[i]);
                    }
                    r = tab[0];
                }
                v[e] = negate ? -r : r;
            }
            for (int b = 0; b < dim; b++)
                for (int d1 = 0; d1 < R; d1++)
                    for (int d2 = 0; d2 < R; d2++) {
                        const long k = row_ptr[d1 * n_pts + o] + (t - tb[o]) * dim * R + b * R + d2;
                        cols[k] = d2 * n_dofs + (long)tp.t_fac[t] * dim + b;
                        vals[k] = v[(b * R + d1) * R + d2];
                    }
        }
    });
}

}  // namespace nf
}  // namespace tbem
