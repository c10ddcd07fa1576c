// Test infrastructure: a restatement of the geometry queries that the
// reference (tbenthompson/3bem, cpp/gte_wrapper.h) takes from the
// third-party Geometric Tools Engine (GTEngine 1.14, downloaded by
// tbempy/download.py:65 and absent from the reference checkout).  With it the
// reference's own nearfield construction (cpp/integral_term.cpp,
// cpp/limit_direction.cpp, cpp/nearfield_operator.h, ...) compiles into
// oracle/_ref.  The product never links this file.
//
// Published methods restated here (not GTEngine code):
//   * point-segment distance: projection parameter clamped to [0, 1];
//   * point-triangle distance: the barycentric Voronoi-region walk of
//     C. Ericson, Real-Time Collision Detection (2005), section 5.1.5;
//   * segment-triangle intersection: Moller-Trumbore (1997) with the
//     segment parameter in [0, 1], no hit for a segment parallel to the
//     plane; the coplanar case is then handled the way cpp/gte_wrapper.cpp
//     documents it (project into the triangle's plane, intersect with the
//     three edges, add endpoints lying on the triangle);
//   * 2D segment-segment intersection: parametric solve, collinear overlaps
//     give the two ends of the overlap;
//   * box-ball test: squared distance from the centre to the box <= r^2;
//   * point in polygon: the even-odd crossing rule.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <vector>

#include "geometry.h"
#include "gte_wrapper.h"
#include "vec_ops.h"

namespace tbem {

namespace {

NearestPoint<2> closest_pt_seg(const Vec<double, 2>& p, const Vec<Vec<double, 2>, 2>& s)
{
    const Vec<double, 2> d = s[1] - s[0];
    const double L2 = dot_product(d, d);
    double t = 0.0;
    if (L2 > 0.0) {
        t = dot_product(p - s[0], d) / L2;
        t = std::min(1.0, std::max(0.0, t));
    }
    const Vec<double, 2> q = t == 1.0 ? s[1] : t == 0.0 ? s[0] : s[0] + t * d;
    return {{2 * t - 1}, q, hypot(p - q)};
}

// Ericson's closest point on triangle abc; (v, w) such that q = a + v (b - a) + w (c - a).
NearestPoint<3> closest_pt_tri(const Vec<double, 3>& p, const Vec<Vec<double, 3>, 3>& T)
{
    const auto& a = T[0];
    const auto& b = T[1];
    const auto& c = T[2];
    const Vec<double, 3> ab = b - a, ac = c - a, ap = p - a;
    double v = 0.0, w = 0.0;
    Vec<double, 3> q;
    const double d1 = dot_product(ab, ap), d2 = dot_product(ac, ap);
    const Vec<double, 3> bp = p - b;
    const double d3 = dot_product(ab, bp), d4 = dot_product(ac, bp);
    const Vec<double, 3> cp = p - c;
    const double d5 = dot_product(ab, cp), d6 = dot_product(ac, cp);
    const double vc = d1 * d4 - d3 * d2;
    const double vb = d5 * d2 - d1 * d6;
    const double va = d3 * d6 - d5 * d4;
    if (d1 <= 0.0 && d2 <= 0.0) {
        q = a;
    } else if (d3 >= 0.0 && d4 <= d3) {
        v = 1.0;
        q = b;
    } else if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        v = d1 / (d1 - d3);
        q = a + v * ab;
    } else if (d6 >= 0.0 && d5 <= d6) {
        w = 1.0;
        q = c;
    } else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        w = d2 / (d2 - d6);
        q = a + w * ac;
    } else if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        v = 1.0 - w;
        q = b + w * (c - b);
    } else {
        const double inv = 1.0 / (va + vb + vc);
        v = vb * inv;
        w = vc * inv;
        q = a + v * ab + w * ac;
    }
    return {{v, w}, q, hypot(p - q)};
}

double cross2(const Vec<double, 2>& a, const Vec<double, 2>& b) { return a[0] * b[1] - a[1] * b[0]; }

std::vector<Vec<double, 2>> seg_seg_intersection(const Vec<Vec<double, 2>, 2>& A,
                                                 const Vec<Vec<double, 2>, 2>& B)
{
    const Vec<double, 2> r = A[1] - A[0], s = B[1] - B[0], qp = B[0] - A[0];
    const double den = cross2(r, s);
    if (den != 0.0) {
        const double t = cross2(qp, s) / den, u = cross2(qp, r) / den;
        if (t >= 0.0 && t <= 1.0 && u >= 0.0 && u <= 1.0) return {A[0] + t * r};
        return {};
    }
    if (cross2(qp, r) != 0.0) return {};  // parallel, not collinear
    const double rr = dot_product(r, r);
    if (rr == 0.0) {  // A is a point
        const double ss = dot_product(s, s);
        if (ss == 0.0) return A[0] == B[0] ? std::vector<Vec<double, 2>>{A[0]} : std::vector<Vec<double, 2>>{};
        const double u = dot_product(A[0] - B[0], s) / ss;
        if (u >= 0.0 && u <= 1.0) return {A[0]};
        return {};
    }
    double t0 = dot_product(B[0] - A[0], r) / rr, t1 = dot_product(B[1] - A[0], r) / rr;
    if (t0 > t1) std::swap(t0, t1);
    const double lo = std::max(0.0, t0), hi = std::min(1.0, t1);
    if (lo > hi) return {};
    if (lo == hi) return {A[0] + lo * r};
    return {A[0] + lo * r, A[0] + hi * r};
}

// Moller-Trumbore with the segment parameter in [0, 1]; false when parallel.
bool seg_tri_hit(const Vec<Vec<double, 3>, 3>& T, const Vec<Vec<double, 3>, 2>& S, Vec<double, 3>& out)
{
    const Vec<double, 3> dir = S[1] - S[0];
    const Vec<double, 3> e1 = T[1] - T[0], e2 = T[2] - T[0];
    const Vec<double, 3> h = cross(dir, e2);
    const double a = dot_product(e1, h);
    if (a == 0.0) return false;
    const double f = 1.0 / a;
    const Vec<double, 3> s = S[0] - T[0];
    const double u = f * dot_product(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const Vec<double, 3> q = cross(s, e1);
    const double v = f * dot_product(dir, q);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = f * dot_product(e2, q);
    if (t < 0.0 || t > 1.0) return false;
    out = S[0] + t * dir;
    return true;
}

Vec<Vec<double, 3>, 2> planar_axes(const Vec<double, 3>& n)
{
    Vec<double, 3> first{1, 0, 0};
    double fd = dot_product(n, first);
    if (fd > 0.95) {
        first = {0, 1, 0};
        fd = dot_product(n, first);
    }
    first = normalized(first - fd * n);
    return {first, cross(n, first)};
}

Vec<double, 2> to_plane(const Vec<double, 3>& o, const Vec<Vec<double, 3>, 2>& ax, const Vec<double, 3>& p)
{
    return {dot_product(p - o, ax[0]), dot_product(p - o, ax[1])};
}

bool already_in(const std::vector<Vec<double, 3>>& set, const Vec<double, 3>& p, double thr)
{
    for (auto& q : set)
        if (dist(q, p) < thr) return true;
    return false;
}

std::vector<Vec<double, 3>> seg_tri_intersection(const Vec<Vec<double, 3>, 3>& T,
                                                 const Vec<Vec<double, 3>, 2>& S)
{
    Vec<double, 3> hit;
    if (seg_tri_hit(T, S, hit)) return {hit};
    // a segment in the triangle's plane: intersect in plane coordinates
    const Vec<double, 3> n = normalized(cross(T[2] - T[0], T[1] - T[0]));
    const double thr = 1e-14 * facet_ball(T).radius;
    if (std::fabs(dot_product(n, S[0] - T[0])) > thr || std::fabs(dot_product(n, S[1] - T[0])) > thr)
        return {};
    const auto ax = planar_axes(n);
    const auto& o = T[0];
    const Vec<Vec<double, 2>, 2> seg{to_plane(o, ax, S[0]), to_plane(o, ax, S[1])};
    const Vec<double, 2> t2[3] = {to_plane(o, ax, T[0]), to_plane(o, ax, T[1]), to_plane(o, ax, T[2])};
    std::vector<Vec<double, 3>> out;
    for (int e = 0; e < 3; e++) {
        const Vec<Vec<double, 2>, 2> edge{t2[e], t2[(e + 1) % 3]};
        const double ethr = 1e-14 * facet_ball(edge).radius;
        for (auto& p2 : seg_seg_intersection(seg, edge)) {
            const Vec<double, 3> p3 = p2[0] * ax[0] + p2[1] * ax[1] + o;
            if (!already_in(out, p3, ethr)) out.push_back(p3);
        }
    }
    for (int k = 0; k < 2; k++)
        if (closest_pt_tri(S[k], T).distance < thr && !already_in(out, S[k], thr)) out.push_back(S[k]);
    return out;
}

void add_hits(const Vec<Vec<double, 3>, 3>& T, const Vec<Vec<double, 3>, 2>& S,
              std::vector<Vec<double, 3>>& out)
{
    const double thr = 1e-14 * facet_ball(T).radius;
    for (auto& p : seg_tri_intersection(T, S))
        if (!already_in(out, p, thr)) out.push_back(p);
}

}  // namespace

template <>
NearestPoint<2> closest_pt_facet(const Vec<double, 2>& pt, const Vec<Vec<double, 2>, 2> f)
{
    return closest_pt_seg(pt, f);
}

template <>
NearestPoint<3> closest_pt_facet(const Vec<double, 3>& pt, const Vec<Vec<double, 3>, 3> f)
{
    return closest_pt_tri(pt, f);
}

template <>
std::vector<Vec<double, 2>> seg_facet_intersection(const Vec<Vec<double, 2>, 2>& f,
                                                   const Vec<Vec<double, 2>, 2>& seg)
{
    return seg_seg_intersection(f, seg);
}

template <>
std::vector<Vec<double, 3>> seg_facet_intersection(const Vec<Vec<double, 3>, 3>& f,
                                                   const Vec<Vec<double, 3>, 2>& seg)
{
    return seg_tri_intersection(f, seg);
}

template <>
std::vector<Vec<double, 2>> facet_facet_intersection(const Vec<Vec<double, 2>, 2>& a,
                                                     const Vec<Vec<double, 2>, 2>& b)
{
    return seg_seg_intersection(a, b);
}

template <>
std::vector<Vec<double, 3>> facet_facet_intersection(const Vec<Vec<double, 3>, 3>& A,
                                                     const Vec<Vec<double, 3>, 3>& B)
{
    std::vector<Vec<double, 3>> out;
    for (int k = 0; k < 3; k++) add_hits(A, {B[k], B[(k + 1) % 3]}, out);
    for (int k = 0; k < 3; k++) add_hits(B, {A[k], A[(k + 1) % 3]}, out);
    return out;
}

bool is_point_in_polygon(const Vec<double, 2>& pt, const std::vector<Vec<double, 2>>& poly)
{
    bool inside = false;
    for (size_t i = 0, j = poly.size() - 1; i < poly.size(); j = i++) {
        const auto& a = poly[i];
        const auto& b = poly[j];
        if ((a[1] > pt[1]) != (b[1] > pt[1]) &&
            pt[0] < (b[0] - a[0]) * (pt[1] - a[1]) / (b[1] - a[1]) + a[0])
            inside = !inside;
    }
    return inside;
}

template <size_t dim>
bool is_intersection_box_ball(const Box<dim>& box, const Ball<dim>& ball)
{
    double s = 0.0;
    for (size_t d = 0; d < dim; d++) {
        const double e = std::fabs(ball.center[d] - box.center[d]) - box.half_width[d];
        if (e > 0.0) s += e * e;
    }
    return s <= ball.radius * ball.radius;
}
template bool is_intersection_box_ball(const Box<2>&, const Ball<2>&);
template bool is_intersection_box_ball(const Box<3>&, const Ball<3>&);

template <size_t dim>
bool is_point_in_ball(const Vec<double, dim>& pt, const Ball<dim>& ball)
{
    Box<dim> b{pt, zeros<Vec<double, dim>>::make()};
    return is_intersection_box_ball(b, ball);
}
template bool is_point_in_ball(const Vec<double, 2>&, const Ball<2>&);
template bool is_point_in_ball(const Vec<double, 3>&, const Ball<3>&);

bool is_point_in_triangle(const Vec<double, 2>& pt, const Vec<Vec<double, 2>, 3>& tri)
{
    return is_point_in_polygon(pt, {tri[0], tri[1], tri[2]});
}

}  // namespace tbem
