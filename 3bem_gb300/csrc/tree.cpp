// Host octree + task lists.  Compiled with -ffp-contract=off so that the box
// arithmetic rounds exactly like the reference on every host architecture.
#include "tree.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <memory>
#include <mutex>
#include <thread>

namespace tbem {
namespace {

struct Box {
    double c[3], h[3];
};

// Box::bounding_box over zero-radius balls (cpp/geometry.cpp:61-80).
Box bounding_box(const double* pts, const std::vector<long>& idx)
{
    Box b{{0, 0, 0}, {0, 0, 0}};
    if (idx.empty()) return b;
    double mn[3], mx[3];
    for (int d = 0; d < 3; d++) mn[d] = mx[d] = pts[3 * idx[0] + d];
    for (size_t i = 1; i < idx.size(); i++)
        for (int d = 0; d < 3; d++) {
            double v = pts[3 * idx[i] + d];
            mn[d] = std::min(mn[d], v - 0.0);
            mx[d] = std::max(mx[d], v + 0.0);
        }
    for (int d = 0; d < 3; d++) {
        b.c[d] = (mx[d] + mn[d]) / 2.0;
        b.h[d] = (mx[d] - mn[d]) / 2.0;
    }
    return b;
}

// expand_by_max_axis_multiple (cpp/geometry.cpp:13-17) over the first dim
// axes (a 2D box keeps z = 0)
Box expand(const Box& b, double f, int dim)
{
    double m = b.h[0];
    for (int d = 1; d < dim; d++) m = std::max(m, b.h[d]);
    double e = f * m;
    Box o = b;
    for (int d = 0; d < dim; d++) o.h[d] = b.h[d] + e;
    return o;
}

// get_subcell with make_child_idx's bit order: the first axis is the high bit
// (bit dim - 1), cpp/geometry.cpp:20-28, cpp/octree.cpp:65-75
Box subcell(const Box& b, int oct, int dim)
{
    Box o = b;
    for (int d = 0; d < dim; d++) {
        const int idx = (oct >> (dim - 1 - d)) & 1;
        o.h[d] = b.h[d] / 2.0;
        o.c[d] = b.c[d] + ((static_cast<double>(idx) * 2) - 1) * o.h[d];
    }
    return o;
}

// find_containing_subcell: strict '>' (cpp/geometry.cpp:83-95)
int containing(const Box& b, const double* p, int dim)
{
    int c = 0;
    for (int d = 0; d < dim; d++) {
        if (p[d] > b.c[d]) c++;
        if (d < dim - 1) c <<= 1;
    }
    return c;
}

struct Node {
    Box b;
    std::vector<long> idx;
    int level;
    long ref_index;
    int child[8];
    int octant;
};

struct Builder {
    const double* pts;
    long min_pts;
    int dim;
    std::vector<Node> nodes;
    long next_index = 1;

    // build_children (cpp/octree.cpp:97-153) run sequentially: a child's
    // index is taken after its subtree is built (post-order).
    void build_children(int node, const Box& bounds, int level)
    {
        if ((long)nodes[node].idx.size() <= min_pts) return;
        // an inner cell keeps no point list (only the leaves' are read)
        const std::vector<long> idx = std::move(nodes[node].idx);
        nodes[node].idx.clear();
        std::vector<long> part[8];
        for (long i : idx) part[containing(bounds, &pts[3 * i], dim)].push_back(i);
        for (int o = 0; o < (1 << dim); o++) {
            if (part[o].empty()) continue;
            Box cb = subcell(bounds, o, dim);
            Box tight = bounding_box(pts, part[o]);
            Node n;
            n.b = cb;
            n.idx = std::move(part[o]);
            n.level = level + 1;
            n.ref_index = -1;
            n.octant = o;
            for (int k = 0; k < 8; k++) n.child[k] = -1;
            nodes.push_back(std::move(n));
            int id = (int)nodes.size() - 1;
            nodes[node].child[o] = id;
            if (tight.h[0] != 0.0 || tight.h[1] != 0.0 || tight.h[2] != 0.0)
                build_children(id, cb, level + 1);
            nodes[id].ref_index = next_index++;
        }
    }
};

}  // namespace

namespace {
Tree flatten(const std::vector<Node>& N, long n);

// build_children(0, bounds, 0) with the root's children's subtrees built on
// threads, each in a builder of its own numbered from 1 (the subtree's root
// last, as post-order gives it), then merged with the node ids and the
// reference indices offset: subtree k's indices follow those of subtrees
// 0 .. k-1, exactly the sequential post-order numbering.
constexpr long TREE_THREADS_MIN_POINTS = 1L << 17;

template <typename S>
long n_points_of(const std::vector<S>& sub)
{
    long n = 0;
    for (const S& w : sub) n += (long)w.b.nodes[0].idx.size();
    return n;
}

void build_root_children(Builder& B, const Box& bounds)
{
    if ((long)B.nodes[0].idx.size() <= B.min_pts) return;
    std::vector<long> idx = std::move(B.nodes[0].idx);
    B.nodes[0].idx.clear();
    std::vector<long> part[8];
    for (long i : idx) part[containing(bounds, &B.pts[3 * i], B.dim)].push_back(i);
    std::vector<long>().swap(idx);
    struct Sub {
        Builder b;
        Box cb;
        bool recurse;
        int octant;
    };
    std::vector<Sub> sub;
    for (int o = 0; o < (1 << B.dim); o++) {
        if (part[o].empty()) continue;
        Sub w;
        w.b.pts = B.pts;
        w.b.min_pts = B.min_pts;
        w.b.dim = B.dim;
        w.cb = subcell(bounds, o, B.dim);
        const Box tight = bounding_box(B.pts, part[o]);
        w.recurse = tight.h[0] != 0.0 || tight.h[1] != 0.0 || tight.h[2] != 0.0;
        w.octant = o;
        Node n;
        n.b = w.cb;
        n.idx = std::move(part[o]);
        n.level = 1;
        n.ref_index = -1;
        n.octant = o;
        for (int k = 0; k < 8; k++) n.child[k] = -1;
        w.b.nodes.push_back(std::move(n));
        sub.push_back(std::move(w));
    }
    auto run = [&](size_t k) {
        Sub& w = sub[k];
        if (w.recurse) w.b.build_children(0, w.cb, 1);
        w.b.nodes[0].ref_index = w.b.next_index++;
    };
    // threads only for large trees (small ones are often built many at a
    // time already, one per mesh)
    const bool threaded = n_points_of(sub) >= TREE_THREADS_MIN_POINTS;
    if (threaded && sub.size() > 1 && std::thread::hardware_concurrency() > 1) {
        std::vector<std::thread> th;
        std::exception_ptr failure;
        std::mutex m;
        for (size_t k = 0; k < sub.size(); k++)
            th.emplace_back([&, k] {
                try {
                    run(k);
                } catch (...) {  // handed to the caller after the join
                    std::lock_guard<std::mutex> lock(m);
                    if (!failure) failure = std::current_exception();
                }
            });
        for (auto& t : th) t.join();
        if (failure) std::rethrow_exception(failure);
    } else {
        for (size_t k = 0; k < sub.size(); k++) run(k);
    }
    long offset = 0;
    for (Sub& w : sub) {
        const int base = (int)B.nodes.size();
        B.nodes[0].child[w.octant] = base;
        for (Node& n : w.b.nodes) {
            for (int k = 0; k < 8; k++)
                if (n.child[k] >= 0) n.child[k] += base;
            n.ref_index += offset;
            B.nodes.push_back(std::move(n));
        }
        offset += w.b.next_index - 1;
    }
    B.next_index = offset + 1;
}
}  // namespace

Tree build_tree(const double* pts, long n, long min_pts, int dim)
{
    Builder B;
    B.pts = pts;
    B.min_pts = min_pts;
    B.dim = dim;
    std::vector<long> all(n);
    for (long i = 0; i < n; i++) all[i] = i;
    Box box = bounding_box(pts, all);
    Node root;
    root.b = expand(box, 1e-5, dim);  // the root's bounds are the expanded box ...
    root.idx = all;
    root.level = 0;
    root.ref_index = 0;
    root.octant = -1;
    for (int k = 0; k < 8; k++) root.child[k] = -1;
    B.nodes.reserve(2 * (size_t)(n / std::max<long>(min_pts, 1)) + 16);
    B.nodes.push_back(std::move(root));
    build_root_children(B, box);  // ... but its children are cut from the unexpanded one
    return flatten(B.nodes, n);
}

Tree build_tree_cube(const double* pts, long n, long min_pts, const double center[3], double hw)
{
    Builder B;
    B.pts = pts;
    B.min_pts = min_pts;
    B.dim = 3;
    std::vector<long> all(n);
    for (long i = 0; i < n; i++) all[i] = i;
    Box box{{center[0], center[1], center[2]}, {hw, hw, hw}};
    Node root;
    root.b = box;
    root.idx = all;
    root.level = 0;
    root.ref_index = 0;
    root.octant = -1;
    for (int k = 0; k < 8; k++) root.child[k] = -1;
    B.nodes.reserve(2 * (size_t)(n / std::max<long>(min_pts, 1)) + 16);
    B.nodes.push_back(std::move(root));
    build_root_children(B, box);
    return flatten(B.nodes, n);
}

Tree merge_forest(const std::vector<Tree>& trees, const std::vector<long>& pt_off,
                  std::vector<std::vector<int>>& gid)
{
    Tree F;
    const size_t M = trees.size();
    gid.assign(M, {});
    int max_l = -1;
    size_t total = 0;
    for (size_t m = 0; m < M; m++) {
        max_l = std::max(max_l, trees[m].n_levels() - 1);
        total += trees[m].cells.size();
        gid[m].assign(trees[m].cells.size(), -1);
    }
    F.cells.reserve(total);
    F.level_start.assign(max_l + 2, 0);
    // level-major over the meshes: level l of mesh 0, of mesh 1, ...
    for (int l = 0; l <= max_l; l++) {
        F.level_start[l] = (int)F.cells.size();
        for (size_t m = 0; m < M; m++) {
            const Tree& t = trees[m];
            if (l >= t.n_levels()) continue;
            for (int i = t.level_start[l]; i < t.level_start[l + 1]; i++) {
                gid[m][i] = (int)F.cells.size();
                F.cells.push_back(t.cells[i]);
            }
        }
    }
    F.level_start[max_l + 1] = (int)F.cells.size();
    for (size_t m = 0; m < M; m++) {
        const Tree& t = trees[m];
        for (size_t i = 0; i < t.cells.size(); i++) {
            Cell& c = F.cells[gid[m][i]];
            if (c.parent >= 0) c.parent = gid[m][c.parent];
            if (c.first_child >= 0) c.first_child = gid[m][c.first_child];
            c.pt_begin += pt_off[m];
            c.pt_end += pt_off[m];
        }
        for (long k = 0; k < t.n_points(); k++) F.perm.push_back(pt_off[m] + t.perm[k]);
        for (int p : t.preorder) F.preorder.push_back(gid[m][p]);
    }
    F.first_at_level.assign(max_l + 1, -1);
    for (int p : F.preorder) {
        const int l = F.cells[p].level;
        if (F.first_at_level[l] < 0) F.first_at_level[l] = p;
    }
    return F;
}

TaskLists merge_lists(const std::vector<TaskLists>& lists, const std::vector<std::vector<int>>& gid)
{
    TaskLists L;
    for (size_t m = 0; m < lists.size(); m++) {
        const TaskLists& a = lists[m];
        const std::vector<int>& g = gid[m];
        auto cells = [&](const std::vector<int>& in, std::vector<int>& out) {
            for (int c : in) out.push_back(g[c]);
        };
        auto pairs = [&](const std::vector<CellPair>& in, std::vector<CellPair>& out) {
            for (const CellPair& p : in) out.push_back({g[p.obs], g[p.src]});
        };
        cells(a.p2m, L.p2m);
        cells(a.m2m, L.m2m);
        cells(a.l2l, L.l2l);
        cells(a.l2p, L.l2p);
        pairs(a.p2p, L.p2p);
        pairs(a.m2p, L.m2p);
        pairs(a.p2l, L.p2l);
        pairs(a.m2l, L.m2l);
    }
    return L;
}

namespace {
Tree flatten(const std::vector<Node>& N, long n)
{
    Tree T;
    // level-major flattening: FIFO over the nodes, children pushed in octant order
    std::vector<int> order;
    std::vector<int> flat_of(N.size(), -1);
    order.push_back(0);
    for (size_t q = 0; q < order.size(); q++) {
        const Node& nd = N[order[q]];
        for (int o = 0; o < 8; o++)
            if (nd.child[o] >= 0) order.push_back(nd.child[o]);
    }
    for (size_t i = 0; i < order.size(); i++) flat_of[order[i]] = (int)i;
    T.cells.resize(order.size());
    int max_level = 0;
    for (size_t i = 0; i < order.size(); i++) {
        const Node& nd = N[order[i]];
        Cell& c = T.cells[i];
        for (int d = 0; d < 3; d++) {
            c.center[d] = nd.b.c[d];
            c.hw[d] = nd.b.h[d];
        }
        c.level = nd.level;
        c.octant = nd.octant;
        c.ref_index = nd.ref_index;
        c.parent = -1;
        c.first_child = -1;
        c.n_children = 0;
        for (int o = 0; o < 8; o++) {
            if (nd.child[o] < 0) continue;
            int f = flat_of[nd.child[o]];
            if (c.first_child < 0) c.first_child = f;
            c.n_children++;
        }
        max_level = std::max(max_level, nd.level);
    }
    for (size_t i = 0; i < T.cells.size(); i++) {
        const Cell& c = T.cells[i];
        for (int k = 0; k < c.n_children; k++) T.cells[c.first_child + k].parent = (int)i;
    }
    T.level_start.assign(max_level + 2, 0);
    for (const Cell& c : T.cells) T.level_start[c.level + 1]++;
    for (int l = 0; l <= max_level; l++) T.level_start[l + 1] += T.level_start[l];

    // pre-order and permuted point ranges (leaves in pre-order; inside a
    // leaf the reference's ascending index order)
    T.perm.reserve(n);
    T.first_at_level.assign(max_level + 1, -1);
    std::vector<std::pair<int, int>> stack;  // (node, state)
    stack.push_back({0, 0});
    while (!stack.empty()) {
        auto [node, state] = stack.back();
        stack.pop_back();
        int f = flat_of[node];
        Cell& c = T.cells[f];
        if (state == 0) {
            T.preorder.push_back(f);
            if (T.first_at_level[c.level] < 0) T.first_at_level[c.level] = f;
            c.pt_begin = (long)T.perm.size();
            if (c.n_children == 0) {
                for (long i : N[node].idx) T.perm.push_back(i);
                c.pt_end = (long)T.perm.size();
            } else {
                stack.push_back({node, 1});
                for (int o = 7; o >= 0; o--)
                    if (N[node].child[o] >= 0) stack.push_back({N[node].child[o], 0});
            }
        } else {
            c.pt_end = (long)T.perm.size();
        }
    }
    return T;
}
}  // namespace

namespace {

inline double hyp(const double* v)
{
    return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

struct ListBuilder {
    const Tree& obs;
    const Tree& src;
    double mac;
    long n_surf;
    bool small_cells;
    TaskLists L;

    // upward_traversal (cpp/fmm.cpp:561-575): leaves -> p2m, then the cell -> m2m
    void upward(int c)
    {
        const Cell& cell = src.cells[c];
        if (cell.is_leaf()) {
            L.p2m.push_back(c);
            return;
        }
        for (int k = 0; k < cell.n_children; k++) upward(cell.first_child + k);
        L.m2m.push_back(c);
    }

    // dual_tree (cpp/fmm.cpp:578-630)
    void dual(int o, int s)
    {
        const Cell& oc = obs.cells[o];
        const Cell& sc = src.cells[s];
        double r_src = hyp(sc.hw), r_obs = hyp(oc.hw);
        double r_max = std::max(r_src, r_obs), r_min = std::min(r_src, r_obs);
        double dc[3] = {oc.center[0] - sc.center[0], oc.center[1] - sc.center[1],
                        oc.center[2] - sc.center[2]};
        double sep = hyp(dc);
        if (r_max + mac * r_min <= mac * sep) {
            bool small_src = sc.n_points() <= n_surf;
            bool small_obs = oc.n_points() <= n_surf;
            if (small_cells) {
                if (small_obs && small_src) L.p2p.push_back({o, s});
                else if (small_obs) L.m2p.push_back({o, s});
                else if (small_src) L.p2l.push_back({o, s});
                else L.m2l.push_back({o, s});
            } else {
                L.m2l.push_back({o, s});
            }
            return;
        }
        if (oc.is_leaf() && sc.is_leaf()) {
            L.p2p.push_back({o, s});
            return;
        }
        bool src_is_shallower = oc.level > sc.level;
        bool split_src = (src_is_shallower && !sc.is_leaf()) || oc.is_leaf();
        if (split_src) {
            for (int k = 0; k < sc.n_children; k++) dual(o, sc.first_child + k);
        } else {
            for (int k = 0; k < oc.n_children; k++) dual(oc.first_child + k, s);
        }
    }

    // downward_traversal (cpp/fmm.cpp:633-648): the cell -> l2l, then children
    void downward(int c)
    {
        const Cell& cell = obs.cells[c];
        if (cell.is_leaf()) {
            L.l2p.push_back(c);
            return;
        }
        L.l2l.push_back(c);
        for (int k = 0; k < cell.n_children; k++) downward(cell.first_child + k);
    }
};

}  // namespace

namespace {

// The dual-tree traversal in parallel with the sequential order kept.  The
// recursion is walked to a fixed depth on one thread; what it emits there
// goes into ordered segments, and every call it would make below that depth
// becomes a segment of its own (a subtree of the traversal).  The subtrees
// then run the sequential recursion on worker threads, each into its own
// segment, and the segments are concatenated in order: every list comes out
// exactly as the sequential traversal emits it.
struct DualSegment {
    int o = -1, s = -1;  // a subtree still to traverse, or -1 for emitted pairs
    std::vector<CellPair> p2p, m2p, p2l, m2l;
};

struct DualFrontier {
    const Tree& obs;
    const Tree& src;
    double mac;
    long n_surf;
    bool small_cells;
    int max_depth;
    std::vector<DualSegment> seg;

    DualSegment& open()
    {
        if (seg.empty() || seg.back().o >= 0) seg.emplace_back();
        return seg.back();
    }
    // the branch rules of ListBuilder::dual, one level
    void walk(int o, int s, int depth)
    {
        if (depth >= max_depth) {
            seg.emplace_back();
            seg.back().o = o;
            seg.back().s = s;
            return;
        }
        const Cell& oc = obs.cells[o];
        const Cell& sc = src.cells[s];
        double r_src = hyp(sc.hw), r_obs = hyp(oc.hw);
        double r_max = std::max(r_src, r_obs), r_min = std::min(r_src, r_obs);
        double dc[3] = {oc.center[0] - sc.center[0], oc.center[1] - sc.center[1],
                        oc.center[2] - sc.center[2]};
        double sep = hyp(dc);
        if (r_max + mac * r_min <= mac * sep) {
            bool small_src = sc.n_points() <= n_surf;
            bool small_obs = oc.n_points() <= n_surf;
            DualSegment& g = open();
            if (small_cells) {
                if (small_obs && small_src) g.p2p.push_back({o, s});
                else if (small_obs) g.m2p.push_back({o, s});
                else if (small_src) g.p2l.push_back({o, s});
                else g.m2l.push_back({o, s});
            } else {
                g.m2l.push_back({o, s});
            }
            return;
        }
        if (oc.is_leaf() && sc.is_leaf()) {
            open().p2p.push_back({o, s});
            return;
        }
        bool src_is_shallower = oc.level > sc.level;
        bool split_src = (src_is_shallower && !sc.is_leaf()) || oc.is_leaf();
        if (split_src) {
            for (int k = 0; k < sc.n_children; k++) walk(o, sc.first_child + k, depth + 1);
        } else {
            for (int k = 0; k < oc.n_children; k++) walk(oc.first_child + k, s, depth + 1);
        }
    }
};

void dual_parallel(ListBuilder& B)
{
    // depth 6 of the traversal: up to a few thousand subtrees for the
    // workers, and nothing for small trees (their recursion ends first)
    DualFrontier F{B.obs, B.src, B.mac, B.n_surf, B.small_cells, 6, {}};
    F.walk(0, 0, 0);
    std::vector<long> todo;
    for (size_t i = 0; i < F.seg.size(); i++)
        if (F.seg[i].o >= 0) todo.push_back((long)i);
    const long hw = (long)std::max(1u, std::thread::hardware_concurrency());
    const long nt = std::min<long>(hw, (long)todo.size());
    auto run = [&](long i) {
        DualSegment& g = F.seg[todo[i]];
        ListBuilder W{B.obs, B.src, B.mac, B.n_surf, B.small_cells, {}};
        W.dual(g.o, g.s);
        g.p2p = std::move(W.L.p2p);
        g.m2p = std::move(W.L.m2p);
        g.p2l = std::move(W.L.p2l);
        g.m2l = std::move(W.L.m2l);
    };
    if (nt <= 1) {
        for (long i = 0; i < (long)todo.size(); i++) run(i);
    } else {
        std::atomic<long> next{0};
        std::exception_ptr failure;
        std::mutex m;
        std::vector<std::thread> th;
        for (long t = 0; t < nt; t++)
            th.emplace_back([&] {
                try {
                    for (long i = next++; i < (long)todo.size(); i = next++) run(i);
                } catch (...) {  // handed to the caller after the join
                    std::lock_guard<std::mutex> lock(m);
                    if (!failure) failure = std::current_exception();
                }
            });
        for (auto& x : th) x.join();
        if (failure) std::rethrow_exception(failure);
    }
    auto gather = [&](std::vector<CellPair>& out, std::vector<CellPair> DualSegment::*list) {
        size_t total = out.size();
        for (const DualSegment& g : F.seg) total += (g.*list).size();
        out.reserve(total);
        for (DualSegment& g : F.seg) {
            out.insert(out.end(), (g.*list).begin(), (g.*list).end());
            std::vector<CellPair>().swap(g.*list);
        }
    };
    gather(B.L.p2p, &DualSegment::p2p);
    gather(B.L.m2p, &DualSegment::m2p);
    gather(B.L.p2l, &DualSegment::p2l);
    gather(B.L.m2l, &DualSegment::m2l);
}

}  // namespace

TaskLists build_lists(const Tree& obs, const Tree& src, double mac, long n_surf,
                      bool small_cells)
{
    ListBuilder B{obs, src, mac, n_surf, small_cells, {}};
    if (src.n_points() > 0) B.upward(0);
    // threads only for large trees (small ones are often built many at a
    // time already, one per mesh)
    if (obs.n_points() > 0 && src.n_points() > 0) {
        if (obs.cells.size() + src.cells.size() >= 8192) dual_parallel(B);
        else B.dual(0, 0);
    }
    if (obs.n_points() > 0) B.downward(0);
    return std::move(B.L);
}

// TranslationSurface<2>::make_surrounding_surface (cpp/fmm.cpp:7-20): order
// points on the unit circle at linspace(0, 2 pi, order + 1)'s first order
// angles (cpp/numbers.cpp:5-12), z = 0.
std::vector<double> circle_surface(long order)
{
    std::vector<double> pts;
    const double a = 0, b = 2 * M_PI;
    const size_t count = (size_t)order + 1;
    for (size_t i = 0; i < (size_t)order; i++) {
        const double theta = a + i * (b - a) / ((double)count - 1);
        pts.push_back(std::cos(theta));
        pts.push_back(std::sin(theta));
        pts.push_back(0.0);
    }
    return pts;
}

std::vector<double> sphere_surface(long order)
{
    std::vector<double> pts;
    double a = 4 * M_PI / order;
    double d = std::sqrt(a);
    auto M_theta = static_cast<size_t>(std::round(M_PI / d));
    double d_theta = M_PI / M_theta;
    double d_phi = a / d_theta;
    for (size_t m = 0; m < M_theta; m++) {
        double theta = M_PI * (m + 0.5) / M_theta;
        auto M_phi = static_cast<size_t>(std::round(2 * M_PI * std::sin(theta) / d_phi));
        for (size_t k = 0; k < M_phi; k++) {
            double phi = 2 * M_PI * k / M_phi;
            pts.push_back(std::sin(theta) * std::cos(phi));
            pts.push_back(std::sin(theta) * std::sin(phi));
            pts.push_back(std::cos(theta));
        }
    }
    return pts;
}

}  // namespace tbem
