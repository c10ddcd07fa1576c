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
// the recursive rule decides.  In 3D the outer rule's function values are
// inner integrals, computed the same way in one batch per outer level.
//
// An interval that splits waits for its six children's integrals; once the
// sixth arrives it sums them in the recursion's order,
// ((((c1 + c2) + c3) + c4) + c5) + c6, and passes the sum up in turn.  So the
// results are the recursion's bit for bit, and memory follows the open
// frontier and its pending ancestors, not the whole tree.
//
// The host work between the batches (emitting points, the stop rule, the
// splits and sums) runs on all host cores: the terms are dealt to chunks and
// every term's arithmetic stays in its own chunk.
#include <algorithm>
#include <cmath>
#include <limits>
#include <thread>

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

// An interval that split and waits for its children's integrals (6 E
// values in the chunk's block values).
struct Block {
    long parent;  // the block of the interval it is a child of, -1 for a root
    int child;    // which child of that interval it is
    int done;     // children's integrals received
    long job;     // local job
};

// An interval still open at this level; its f(a) and f(b) are the entry's
// 2 E values in the frontier's value array.
struct Open {
    long parent;  // block waiting for this interval's integral, -1 for a root
    int child;
    long job;  // local job
    double a, b;
};

// The jobs j = c, c + C, c + 2C, ... of chunk c (dealt round robin, so that
// runs of hard terms spread over the chunks) with their pending intervals.
struct Chunk {
    std::vector<long> job;     // job ids
    std::vector<double> err;   // per local job: the error target (E values)
    std::vector<Block> blocks;
    std::vector<double> bvals;       // per block: six children's integrals
    std::vector<long> free_blocks;   // blocks to reuse
    std::vector<Open> open, next;
    std::vector<double> fab, next_fab;  // per open interval: f(a), f(b)
    std::vector<double> sum;            // scratch for a completed block's sum
    long offset = 0;  // this chunk's first point in the current batch
    void reset()  // empty, keeping the memory
    {
        job.clear();
        for (auto* v : {&err, &bvals, &fab, &next_fab}) v->clear();
        blocks.clear();
        free_blocks.clear();
        open.clear();
        next.clear();
    }
    long new_block(const Block& b, int E)
    {
        if (!free_blocks.empty()) {
            const long id = free_blocks.back();
            free_blocks.pop_back();
            blocks[id] = b;
            return id;
        }
        blocks.push_back(b);
        bvals.resize(bvals.size() + 6 * (size_t)E);
        return (long)blocks.size() - 1;
    }
    // Hands the integral v of an interval to the block waiting for it (or,
    // for a root, to the job's result) and completes every block it fills.
    void deliver(long parent, int child, long q, const double* v, int E, std::vector<double>& total)
    {
        sum.assign(v, v + E);
        while (parent >= 0) {
            double* slots = &bvals[(size_t)parent * 6 * E];
            std::copy(sum.begin(), sum.end(), slots + (size_t)child * E);
            Block& bk = blocks[parent];
            if (++bk.done < 6) return;
            // adaptlobstp's return: the six children's integrals in order
            for (int e = 0; e < E; e++) {
                double s = slots[e];
                for (int r = 1; r < 6; r++) s = s + slots[r * E + e];
                sum[e] = s;
            }
            free_blocks.push_back(parent);
            child = bk.child;
            q = bk.job;
            parent = bk.parent;
        }
        std::copy(sum.begin(), sum.end(), &total[(size_t)job[q] * E]);
    }
};

// The buffers of one batch driver, kept between its calls: the 3D inner
// integrals run one batch per outer level, and reusing memory already
// touched spares the page faults of fresh buffers.
struct Work {
    std::vector<Chunk> ch;
    std::vector<long> pj;
    std::vector<double> pt, y;
};

// adaptive_batch over a[0..n), b[0..n) into total ([n][E]), with w's buffers.
void run_batch(int E, const double* a, const double* b, long n, double p_tol, const AdaptiveEval& eval,
               Work& w, std::vector<double>& total)
{
    total.resize((size_t)n * E);
    if (n == 0) return;
    const long hw = (long)std::max(1u, std::thread::hardware_concurrency());
    const long C = std::max(1L, std::min(4 * hw, n / 64));
    if ((long)w.ch.size() < C) w.ch.resize(C);
    std::vector<Chunk>& ch = w.ch;
    for (Chunk& k : ch) k.reset();
    for (long c = 0; c < C; c++)
        for (long j = c; j < n; j += C) ch[c].job.push_back(j);
    std::vector<long>& pj = w.pj;
    std::vector<double>&pt = w.pt, &y = w.y;
    // lays the chunks' points out one after the other: count(chunk) points each
    auto layout = [&](long (*count)(const Chunk&)) {
        long tot = 0;
        for (Chunk& k : ch) {
            k.offset = tot;
            tot += count(k);
        }
        pj.resize(tot);
        pt.resize(tot);
        return tot;
    };

    // the initial 13-point stage (adaptive_integrate, cpp/adaptive_quad.h:128-171)
    layout([](const Chunk& k) { return 13 * (long)k.job.size(); });
    parallel_for(
        C,
        [&](long c) {
            const Chunk& k = ch[c];
            long o = k.offset;
            for (long j : k.job) {
                const double m = (a[j] + b[j]) / 2., h = (b[j] - a[j]) / 2.;
                const double xs[13] = {a[j], m - kX1 * h, m - kAlpha * h, m - kX2 * h, m - kBeta * h,
                                       m - kX3 * h, m, m + kX3 * h, m + kBeta * h, m + kX2 * h,
                                       m + kAlpha * h, m + kX1 * h, b[j]};
                for (double x : xs) {
                    pj[o] = j;
                    pt[o++] = x;
                }
            }
        },
        1);
    eval(pj, pt, y);
    parallel_for(
        C,
        [&](long c) {
            Chunk& k = ch[c];
            std::vector<double> i1(E), i2(E), is(E);
            const long nj = (long)k.job.size();
            k.err.resize((size_t)nj * E);
            for (long q = 0; q < nj; q++) {
                const long j = k.job[q];
                const double* Y = &y[(size_t)(k.offset + 13 * q) * E];
                const double h = (b[j] - a[j]) / 2.;
                for (int e = 0; e < E; e++) {
                    auto v = [&](int i) { return Y[i * E + e]; };
                    i2[e] = (h / 6.0) * (v(0) + v(12) + 5.0 * (v(4) + v(8)));
                    i1[e] = (h / 1470.0) * (77.0 * (v(0) + v(12)) + 432.0 * (v(2) + v(10)) +
                                            625.0 * (v(4) + v(8)) + 672.0 * v(6));
                    is[e] = h * (kW[0] * (v(0) + v(12)) + kW[1] * (v(1) + v(11)) + kW[2] * (v(2) + v(10)) +
                                 kW[3] * (v(3) + v(9)) + kW[4] * (v(4) + v(8)) + kW[5] * (v(5) + v(7)) +
                                 kW[6] * v(6));
                    k.err[q * E + e] = error_is(p_tol, std::fabs(i1[e] - is[e]), std::fabs(i2[e] - is[e]),
                                                is[e], a[j], b[j]);
                }
                k.open.push_back({-1, 0, q, a[j], b[j]});
                k.fab.insert(k.fab.end(), Y, Y + E);                // f(a)
                k.fab.insert(k.fab.end(), Y + 12 * E, Y + 13 * E);  // f(b)
            }
        },
        1);

    // breadth-first adaptlobstp (cpp/adaptive_quad.h:40-79)
    while (layout([](const Chunk& k) { return 5 * (long)k.open.size(); }) > 0) {
        parallel_for(
            C,
            [&](long c) {
                const Chunk& k = ch[c];
                long o = k.offset;
                for (const Open& op : k.open) {
                    const double m = (op.a + op.b) / 2., h = (op.b - op.a) / 2.;
                    const double xs[5] = {m - kAlpha * h, m - kBeta * h, m, m + kBeta * h, m + kAlpha * h};
                    const long j = k.job[op.job];
                    for (double x : xs) {
                        pj[o] = j;
                        pt[o++] = x;
                    }
                }
            },
            1);
        eval(pj, pt, y);
        parallel_for(
            C,
            [&](long c) {
                Chunk& k = ch[c];
                std::vector<double> i1(E), i2(E);
                k.next.clear();
                k.next_fab.clear();
                for (size_t i = 0; i < k.open.size(); i++) {
                    const Open op = k.open[i];
                    const double na = op.a, nb = op.b;
                    const double m = (na + nb) / 2., h = (nb - na) / 2.;
                    const double mll = m - kAlpha * h, ml = m - kBeta * h, mr = m + kBeta * h,
                                 mrr = m + kAlpha * h;
                    const double* Y = &y[(size_t)(k.offset + 5 * (long)i) * E];  // fmll, fml, fm, fmr, fmrr
                    const double* fa = &k.fab[2 * E * i];
                    const double* fb = fa + E;
                    const double* target = &k.err[(size_t)op.job * E];
                    bool converged = true;
                    for (int e = 0; e < E; e++) {
                        i2[e] = (h / 6.) * (fa[e] + fb[e] + 5.0 * (Y[E + e] + Y[3 * E + e]));
                        i1[e] = (h / 1470.) * (77.0 * (fa[e] + fb[e]) + 432.0 * (Y[e] + Y[4 * E + e]) +
                                               625.0 * (Y[E + e] + Y[3 * E + e]) + 672.0 * Y[2 * E + e]);
                        converged = converged && (target[e] + (i1[e] - i2[e]) == target[e]);
                    }
                    if (converged || mll <= na || nb <= mrr) {
                        k.deliver(op.parent, op.child, op.job, i1.data(), E, total);
                        continue;
                    }
                    const long blk = k.new_block({op.parent, op.child, 0, op.job}, E);
                    const double cut[7] = {na, mll, ml, m, mr, mrr, nb};
                    const double* fs[7] = {fa, Y, Y + E, Y + 2 * E, Y + 3 * E, Y + 4 * E, fb};
                    for (int r = 0; r < 6; r++) {
                        k.next.push_back({blk, r, op.job, cut[r], cut[r + 1]});
                        k.next_fab.insert(k.next_fab.end(), fs[r], fs[r] + E);
                        k.next_fab.insert(k.next_fab.end(), fs[r + 1], fs[r + 1] + E);
                    }
                }
                k.open.swap(k.next);
                k.fab.swap(k.next_fab);
            },
            1);
    }
}

}  // namespace

// Integrates g_j over [a_j, b_j] for every job j, g_j(t) = f(j, t) with
// f evaluated in batches by eval(jobs, ts, out) (out: E values per point).
// Returns the integrals ([n][E]).
std::vector<double> adaptive_batch(int E, const std::vector<double>& a, const std::vector<double>& b,
                                   double p_tol, const AdaptiveEval& eval)
{
    Work w;
    std::vector<double> total;
    run_batch(E, a.data(), b.data(), (long)a.size(), p_tol, eval, w, total);
    return total;
}

std::vector<double> adaptive_facet_integrals(int dim, int E, long n_items, double tol,
                                             const InfluenceEval& eval, long slice_jobs)
{
    // A batch's frontier grows with its jobs (near-singular 3D terms reach
    // tens of millions of open points in one level), so the terms -- and
    // each outer level's inner integrals -- go in slices of slice_jobs jobs.
    // The jobs are independent: the slicing changes no value.
    const long S = std::max(1L, slice_jobs);
    std::vector<double> total((size_t)n_items * E), part, zeros, ia, ib, ix, x0, v;
    std::vector<long> jobs, inner_item, inner_of, it;
    Work outer, inner;  // kept across slices and outer levels
    for (long s0 = 0; s0 < n_items; s0 += S) {
        const long m = std::min(S, n_items - s0);
        const std::vector<double> a(m, dim == 2 ? -1.0 : 0.0), b(m, 1.0);
        AdaptiveEval outer_eval;
        if (dim == 2) {
            outer_eval = [&](const std::vector<long>& job, const std::vector<double>& t,
                             std::vector<double>& out) {
                jobs.resize(job.size());
                for (size_t k = 0; k < job.size(); k++) jobs[k] = job[k] + s0;
                zeros.assign(t.size(), 0.0);
                eval(jobs, t, zeros, out);
            };
        } else {
            outer_eval = [&](const std::vector<long>& job, const std::vector<double>& xs,
                             std::vector<double>& out) {
                // the outer function at x: the inner integral over y in [0, 1 - x]
                out.assign(xs.size() * E, 0.0);
                for (auto* u : {&inner_item, &inner_of}) u->clear();
                for (auto* u : {&ia, &ib, &ix}) u->clear();
                for (size_t k = 0; k < xs.size(); k++) {
                    if (xs[k] == 1.0) continue;  // zero, as the reference's outer lambda returns
                    inner_item.push_back(job[k] + s0);
                    inner_of.push_back((long)k);
                    ia.push_back(0.0);
                    ib.push_back(1 - xs[k]);
                    ix.push_back(xs[k]);
                }
                const long n_in = (long)ia.size();
                for (long i0 = 0; i0 < n_in; i0 += S) {
                    const long mi = std::min(S, n_in - i0);
                    run_batch(
                        E, ia.data() + i0, ib.data() + i0, mi, tol,
                        [&](const std::vector<long>& ij, const std::vector<double>& ys, std::vector<double>& o) {
                            it.resize(ij.size());
                            x0.resize(ij.size());
                            parallel_for(
                                (long)ij.size(),
                                [&](long q) {
                                    it[q] = inner_item[i0 + ij[q]];
                                    x0[q] = ix[i0 + ij[q]];
                                },
                                1 << 16);
                            eval(it, x0, ys, o);
                        },
                        inner, v);
                    for (long q = 0; q < mi; q++)
                        for (int e = 0; e < E; e++) out[(size_t)inner_of[i0 + q] * E + e] = v[q * E + e];
                }
            };
        }
        run_batch(E, a.data(), b.data(), m, tol, outer_eval, outer, part);
        std::copy(part.begin(), part.end(), total.begin() + s0 * E);
    }
    return total;
}

}  // namespace nf
}  // namespace tbem
