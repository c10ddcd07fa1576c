// Nearfield and farfield-correction matrix construction (the reference's
// make_nearfield_operator / make_farfield_correction_operator,
// cpp/nearfield_operator.h:12-117, with IntegrationStrategy::compute_term,
// cpp/integral_term.cpp:33-92, and the sinh nearfield integrator,
// cpp/integral_term.cpp:155-203).
//
// Host side (nearfield_host.cpp): facet geometry, the Galerkin observation
// points and their Richardson (limit) directions, the nearfield facet search
// and the list of (observation point, source facet) terms.  Device side
// (nearfield.cu): every term's quadrature on the GPU, one warp per term.
// Points and facets are stored as 3-vectors (z = 0 in 2D).
#pragma once
#include <functional>
#include <vector>

namespace tbem {
namespace nf {

struct V3 {
    double x[3];
    double operator[](int i) const { return x[i]; }
    double& operator[](int i) { return x[i]; }
};

// A facet: dim corners (a segment in 2D, a triangle in 3D).
struct Facet {
    V3 c[3];
};

struct FacetInfo {
    V3 centroid;
    double radius;        // facet_ball radius (cpp/geometry.h:271-279)
    double length_scale;  // 2 * radius (cpp/facet_info.h:24-33)
    double jacobian;      // facet_jacobian (cpp/numerics.h:27-36)
    V3 normal;            // facet_normal (cpp/geometry.h:113-133)
};

FacetInfo facet_info(const Facet& f, int dim);

struct Closest {
    double ref[2];  // reference coordinates of the closest point
    V3 pt;
    double dist;
};

// The closest point of a facet to p (segment: clamped projection, ref in
// [-1, 1]; triangle: Ericson's region walk, ref = (s, t) of c0 + s(c1 - c0) +
// t(c2 - c0)).  Shared with the device (nearfield.cu) formula for formula.
Closest closest_point(const V3& p, const Facet& f, int dim);

// Observation points with their Richardson directions (galerkin_obs_pts /
// interior_obs_pts, cpp/nearfield_operator.h:12-40).
struct ObsPoints {
    std::vector<V3> loc, normal, dir;
};

// Gauss rule on the reference facet (gauss_facet, cpp/gauss_quad.cpp:155-165):
// points [n][2] (second coordinate 0 in 2D) and weights.
void gauss_facet(int dim, int n, std::vector<double>& x, std::vector<double>& w);
// Legendre-Gauss rule on [-1, 1] (gauss, cpp/gauss_quad.cpp:9-52).
void gauss_rule(int n, std::vector<double>& x, std::vector<double>& w);

// A set of facets with its ball octree (the reference's NearestNeighborData,
// cpp/nearest_neighbors.h:22-34: leaves of at most 20 balls).
class FacetSet {
public:
    FacetSet(const std::vector<Facet>& facets, int dim);
    size_t size() const { return facets_.size(); }
    const Facet& facet(size_t i) const { return facets_[i]; }
    const FacetInfo& info(size_t i) const { return info_[i]; }
    // NearfieldFacetFinder::find (cpp/limit_direction.cpp:17-53): the nearest
    // facet and the facets within far_threshold * its ball radius, in the
    // reference's order (its ball octree, leaves in pre-order).
    void find(const V3& p, double far_threshold, std::vector<size_t>& near, size_t& nearest,
              double& dist) const;

private:
    struct Cell {
        double lo[3], hi[3];  // expanded tight box of the member balls (centre +- radius)
        double gc[3];         // centre of the geometric cell (children are cut from it)
        int first_child, n_children;
        long begin, end;      // range of order_
    };
    int dim_;
    std::vector<Facet> facets_;
    std::vector<FacetInfo> info_;
    std::vector<Cell> cells_;
    std::vector<size_t> order_;  // facet ids, leaves in pre-order
    void build();
    void nearest(int cell, const V3& p, size_t& best, double& best_d) const;
    void range(int cell, const V3& c, double r, std::vector<size_t>& out) const;
};

// decide_limit_dir (cpp/limit_direction.cpp:87-147) with the constants
// interior_obs_pts passes (safety factor 0.4, epsilon 1e-2).
V3 limit_direction(const V3& p, const FacetSet& all, int dim);

ObsPoints galerkin_obs_points(const std::vector<Facet>& obs, const FacetSet& all, int order,
                              int dim);

// body(i) for i in [0, n) over the host's cores (contiguous chunks of at
// least `grain` indices per thread; each i writes only its own outputs, so
// the results do not depend on the split).
void parallel_for(long n, const std::function<void(long)>& body, long grain = 256);

// The terms of one nearfield (or farfield-correction) matrix and the
// evaluations they need (IntegrationStrategy::compute_term's split,
// cpp/integral_term.cpp:33-60): every (observation point, source facet) pair
// the facet search returns, point by point in the reference's loop order
// (cpp/nearfield_operator.h:59-84); a far term is one evaluation of the
// source facet's Gauss rule at the point, a near term one sinh-rule
// evaluation, a singular term n_steps sinh-rule evaluations at the points
// stepped back along the limit direction (get_step_loc).
struct TermPlan {
    std::vector<int> t_obs, t_fac;          // per term
    std::vector<long> first;                // per term (+1): its first evaluation
    std::vector<char> sing;                 // per term: 1 = Richardson over its steps
    std::vector<int> i_obs, i_fac, i_near;  // per evaluation (i_near: 1 sinh, 0 far)
    std::vector<double> iloc;               // per evaluation: its point [3]
    bool on_facet = false;  // a near (not singular) term's point lies on its facet
};

// Builds the plan on all host cores (farfield_only: the correction matrix,
// every term one far evaluation at its point).
TermPlan plan_terms(const ObsPoints& pts, const std::vector<Facet>& src, const FacetSet& src_set,
                    double far_threshold, int n_steps, int dim, bool farfield_only);

// The matrix from the evaluations' values ([n_evaluations][dim][R][R]):
// per term its value, its Richardson limit (richardson_limit,
// cpp/richardson.h:10-34) or (negate) its negation, laid out as the
// reference's COO entries compressed to CSR (csr_from_coo's stable row
// order): rows d1 * n_pts + point, columns d2 * dim * n_src + facet * dim +
// basis.
void assemble_csr(const TermPlan& tp, const std::vector<double>& ivals, long n_pts, long n_src, int dim,
                  int R, int n_steps, bool negate, std::vector<double>& vals, std::vector<long>& cols,
                  std::vector<long>& row_ptr);

// Batched evaluation of the functions being integrated: for point k, the
// value (E numbers) of job[k]'s function at t[k], written to out[k * E ...].
using AdaptiveEval = std::function<void(const std::vector<long>& job, const std::vector<double>& t,
                                        std::vector<double>& out)>;

// Adaptive Gauss-Lobatto integrals of job j's function over [a[j], b[j]]
// (adaptive_integrate, cpp/adaptive_quad.h:128-174), all jobs level by level;
// returns [n][E] (nearfield_adaptive.cpp).
std::vector<double> adaptive_batch(int E, const std::vector<double>& a, const std::vector<double>& b,
                                   double p_tol, const AdaptiveEval& eval);

// Batched point influences of the terms being integrated: for point k, term
// item[k]'s basis x kernel x jacobian at the reference point (x0[k], x1[k]).
using InfluenceEval = std::function<void(const std::vector<long>& item, const std::vector<double>& x0,
                                         const std::vector<double>& x1, std::vector<double>& out)>;

// The facet integral of every item by the adaptive rule
// (UnitFacetAdaptiveIntegrator, cpp/integral_term.cpp:96-128): over
// x_hat in [-1, 1] in 2D; over x in [0, 1] of the integral over y in
// [0, 1 - x] in 3D (zero at x = 1).  Returns [n_items][E].  At most
// slice_jobs terms (and inner integrals) share one breadth-first batch,
// which bounds the frontier's memory; the values do not depend on it.
std::vector<double> adaptive_facet_integrals(int dim, int E, long n_items, double tol,
                                             const InfluenceEval& eval, long slice_jobs = 1L << 18);

}  // namespace nf
}  // namespace tbem
