// Adaptive Gauss-Lobatto quadrature of nearfield terms, driven level by level.
//
// The reference integrates a near term over the whole source facet with the
// adaptive Gauss-Lobatto rule of Gander and Gautschi ("Adaptive quadrature --
// revisited", BIT 40, 2000), recursively (cpp/adaptive_quad.h:31-174): in 2D
// over x_hat in [-1, 1]; in 3D over x in [0, 1] of the inner integral over
// y in [0, 1 - x] (cpp/integral_term.cpp:111-128).  Here every term's
// recursion runs at once, breadth first: each level asks the evaluator for
// all new points of all open intervals in one batch (the GPU, in the
// product), then every interval either stops or splits in six, exactly as
// the recursive rule decides; at the end every tree is summed in the
// recursion's order.  In 3D the outer rule's function values are inner
// integrals, computed the same way in one batch per outer level.
#include <cmath>
#include <limits>

#include "nearfield.h"

namespace tbem {
namespace nf {

namespace {

// the rule's abscissae and the Kronrod weights of the 13-point estimate
const double kAlpha = std::sqrt(2. / 3.);
const double kBeta = 1. / std::sqrt(5.);
const double kX1 = .94288241569547971905635175843185720232;
const double kX2 = .64185334234578130578123554132903188354;
const double kX3 = .23638319966214988028222377349205292599;
const double kW[7] = {0.0158271919734802, 0.0942738402188500, 0.155071987336585, 0.188821573960182,
                      0.199773405226859, 0.224926465333340, 0.242611071901408};

// get_error_is (cpp/adaptive_quad.h:88-100), one component
double error_is(double p_tol, double erri1, double erri2, double is, double a, double b)
{
    const double eps = std::numeric_limits<double>::epsilon();
    const double R = (erri2 == 0.0) ? 1.0 : (erri1 / erri2);
    const double tol = (R > 0.0 && R < 1.0) ? (p_tol / R) : p_tol;
    double r = std::fabs(is) * tol / eps;
    if (std::fabs(r) < p_tol) r = b - a;
    return r;
}

struct Node {
    double a, b;
    long fa, fb;      // value slots of f(a), f(b)
    long first = -1;  // first of six children, -1 for a leaf
    long value = -1;  // slot of the leaf's estimate i1
};

struct Job {
    long root = -1;
    long err = -1;  // slot of the error target is (E values)
};

}  // namespace

// Integrates g_j over [a_j, b_j] for every job j, g_j(t) = f(j, t) with
// f evaluated in batches by eval(jobs, ts, out) (out: E values per point).
// Returns the integrals ([n][E]).
std::vector<double> adaptive_batch(int E, const std::vector<double>& a, const std::vector<double>& b,
                                   double p_tol, const AdaptiveEval& eval)
{
    const long n = (long)a.size();
    std::vector<double> pool;  // E values per slot
    auto slot = [&](const double* v) {
        const long s = (long)(pool.size() / E);
        pool.insert(pool.end(), v, v + E);
        return s;
    };
    std::vector<Node> nodes;
    std::vector<Job> jobs(n);
    // the initial 13-point stage (adaptive_integrate, cpp/adaptive_quad.h:128-171)
    {
        std::vector<long> pj;
        std::vector<double> pt;
        for (long j = 0; j < n; j++) {
            const double m = (a[j] + b[j]) / 2., h = (b[j] - a[j]) / 2.;
            const double xs[13] = {a[j], m - kX1 * h, m - kAlpha * h, m - kX2 * h, m - kBeta * h,
                                   m - kX3 * h, m, m + kX3 * h, m + kBeta * h, m + kX2 * h,
                                   m + kAlpha * h, m + kX1 * h, b[j]};
            for (double x : xs) {
                pj.push_back(j);
                pt.push_back(x);
            }
        }
        std::vector<double> y;
        if (!pj.empty()) eval(pj, pt, y);
        std::vector<double> i1(E), i2(E), is(E), err(E);
        for (long j = 0; j < n; j++) {
            const double* Y = &y[(size_t)j * 13 * E];
            const double h = (b[j] - a[j]) / 2.;
            for (int e = 0; e < E; e++) {
                auto v = [&](int k) { return Y[k * E + e]; };
                i2[e] = (h / 6.0) * (v(0) + v(12) + 5.0 * (v(4) + v(8)));
                i1[e] = (h / 1470.0) *
                        (77.0 * (v(0) + v(12)) + 432.0 * (v(2) + v(10)) + 625.0 * (v(4) + v(8)) + 672.0 * v(6));
                is[e] = h * (kW[0] * (v(0) + v(12)) + kW[1] * (v(1) + v(11)) + kW[2] * (v(2) + v(10)) +
                             kW[3] * (v(3) + v(9)) + kW[4] * (v(4) + v(8)) + kW[5] * (v(5) + v(7)) +
                             kW[6] * v(6));
                err[e] = error_is(p_tol, std::fabs(i1[e] - is[e]), std::fabs(i2[e] - is[e]), is[e], a[j], b[j]);
            }
            jobs[j].err = slot(err.data());
            Node root;
            root.a = a[j];
            root.b = b[j];
            root.fa = slot(Y);
            root.fb = slot(Y + 12 * E);
            jobs[j].root = (long)nodes.size();
            nodes.push_back(root);
        }
    }
    // breadth-first adaptlobstp (cpp/adaptive_quad.h:40-79)
    std::vector<long> open, open_job;
    for (long j = 0; j < n; j++) {
        open.push_back(jobs[j].root);
        open_job.push_back(j);
    }
    std::vector<double> i1(E), i2(E);
    while (!open.empty()) {
        std::vector<long> pj;
        std::vector<double> pt;
        for (size_t k = 0; k < open.size(); k++) {
            const Node& nd = nodes[open[k]];
            const double m = (nd.a + nd.b) / 2., h = (nd.b - nd.a) / 2.;
            const double xs[5] = {m - kAlpha * h, m - kBeta * h, m, m + kBeta * h, m + kAlpha * h};
            for (double x : xs) {
                pj.push_back(open_job[k]);
                pt.push_back(x);
            }
        }
        std::vector<double> y;
        eval(pj, pt, y);
        std::vector<long> next, next_job;
        for (size_t k = 0; k < open.size(); k++) {
            const long id = open[k];
            const long j = open_job[k];
            const double na = nodes[id].a, nb = nodes[id].b;
            const double m = (na + nb) / 2., h = (nb - na) / 2.;
            const double mll = m - kAlpha * h, ml = m - kBeta * h, mr = m + kBeta * h, mrr = m + kAlpha * h;
            const double* Y = &y[k * 5 * E];  // fmll, fml, fm, fmr, fmrr
            const double* fa = &pool[(size_t)nodes[id].fa * E];
            const double* fb = &pool[(size_t)nodes[id].fb * E];
            const double* target = &pool[(size_t)jobs[j].err * E];
            bool converged = true;
            for (int e = 0; e < E; e++) {
                i2[e] = (h / 6.) * (fa[e] + fb[e] + 5.0 * (Y[E + e] + Y[3 * E + e]));
                i1[e] = (h / 1470.) * (77.0 * (fa[e] + fb[e]) + 432.0 * (Y[e] + Y[4 * E + e]) +
                                       625.0 * (Y[E + e] + Y[3 * E + e]) + 672.0 * Y[2 * E + e]);
                converged = converged && (target[e] + (i1[e] - i2[e]) == target[e]);
            }
            if (converged || mll <= na || nb <= mrr) {
                nodes[id].value = slot(i1.data());
                continue;
            }
            long s[5];
            for (int q = 0; q < 5; q++) s[q] = slot(Y + q * E);
            const double cut[7] = {na, mll, ml, m, mr, mrr, nb};
            const long fs[7] = {nodes[id].fa, s[0], s[1], s[2], s[3], s[4], nodes[id].fb};
            const long first = (long)nodes.size();
            for (int c = 0; c < 6; c++) {
                Node ch;
                ch.a = cut[c];
                ch.b = cut[c + 1];
                ch.fa = fs[c];
                ch.fb = fs[c + 1];
                nodes.push_back(ch);
                next.push_back(first + c);
                next_job.push_back(j);
            }
            nodes[id].first = first;
        }
        open.swap(next);
        open_job.swap(next_job);
    }
    // sum every tree in the recursion's order: ((((c1 + c2) + c3) + c4) + c5) + c6
    std::vector<double> total((size_t)n * E), acc;
    std::vector<std::pair<long, int>> stack;
    for (long j = 0; j < n; j++) {
        // post-order with an explicit stack; acc holds partial sums per depth
        std::vector<std::vector<double>> partial;
        stack.clear();
        stack.push_back({jobs[j].root, 0});
        partial.push_back(std::vector<double>(E, 0.0));
        std::vector<double> ret(E);
        while (!stack.empty()) {
            auto& top = stack.back();
            const Node& nd = nodes[top.first];
            if (nd.first < 0) {  // leaf: its estimate
                for (int e = 0; e < E; e++) ret[e] = pool[(size_t)nd.value * E + e];
            } else if (top.second < 6) {
                const int c = top.second++;
                stack.push_back({nd.first + c, 0});
                partial.push_back(std::vector<double>(E, 0.0));
                continue;
            } else {
                ret = partial.back();
            }
            stack.pop_back();
            partial.pop_back();
            if (stack.empty()) break;
            // fold ret into the parent: the first child starts the sum
            std::vector<double>& p = partial.back();
            if (stack.back().second == 1) p = ret;
            else
                for (int e = 0; e < E; e++) p[e] = p[e] + ret[e];
        }
        for (int e = 0; e < E; e++) total[(size_t)j * E + e] = ret[e];
    }
    return total;
}

std::vector<double> adaptive_facet_integrals(int dim, int E, long n_items, double tol,
                                             const InfluenceEval& eval)
{
    if (dim == 2) {
        const std::vector<double> a(n_items, -1.0), b(n_items, 1.0);
        return adaptive_batch(E, a, b, tol, [&](const std::vector<long>& job, const std::vector<double>& t,
                                                std::vector<double>& out) {
            eval(job, t, std::vector<double>(t.size(), 0.0), out);
        });
    }
    const std::vector<double> a(n_items, 0.0), b(n_items, 1.0);
    return adaptive_batch(E, a, b, tol, [&](const std::vector<long>& job, const std::vector<double>& xs,
                                            std::vector<double>& out) {
        // the outer function at x: the inner integral over y in [0, 1 - x]
        out.assign(xs.size() * E, 0.0);
        std::vector<long> inner_item, inner_of;
        std::vector<double> ia, ib, ix;
        for (size_t k = 0; k < xs.size(); k++) {
            if (xs[k] == 1.0) continue;  // zero, as the reference's outer lambda returns
            inner_item.push_back(job[k]);
            inner_of.push_back((long)k);
            ia.push_back(0.0);
            ib.push_back(1 - xs[k]);
            ix.push_back(xs[k]);
        }
        if (inner_item.empty()) return;
        const std::vector<double> v =
            adaptive_batch(E, ia, ib, tol, [&](const std::vector<long>& ij, const std::vector<double>& ys,
                                               std::vector<double>& o) {
                std::vector<long> it(ij.size());
                std::vector<double> x0(ij.size());
                for (size_t q = 0; q < ij.size(); q++) {
                    it[q] = inner_item[ij[q]];
                    x0[q] = ix[ij[q]];
                }
                eval(it, x0, ys, o);
            });
        for (size_t q = 0; q < inner_of.size(); q++)
            for (int e = 0; e < E; e++) out[(size_t)inner_of[q] * E + e] = v[q * E + e];
    });
}

}  // namespace nf
}  // namespace tbem
