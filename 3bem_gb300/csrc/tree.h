// Host octree and FMM task lists, flattened for the device.
//
// The tree is built with exactly the reference's arithmetic and rules
// (make_octree / build_children, cpp/octree.cpp:97-180; Box ops,
// cpp/geometry.cpp:13-95) so that cells, bounds, point sets and the
// reference's post-order cell index come out bit-identical; it is then
// flattened level-major (every level contiguous, the children of a cell
// contiguous) with the points permuted so that every cell owns one
// contiguous range of the permuted order.  The task lists follow
// upward_traversal / dual_tree / downward_traversal (cpp/fmm.cpp:561-648).
#pragma once
#include <cstdint>
#include <utility>
#include <vector>

namespace tbem {

struct Cell {
    double center[3];
    double hw[3];
    int level;
    int parent;       // flat id, -1 for the root
    int first_child;  // flat id of the first child, -1 for a leaf
    int n_children;
    int octant;       // child slot within the parent (make_child_idx order), -1 for the root
    long pt_begin;    // permuted point range [pt_begin, pt_end)
    long pt_end;
    long ref_index;   // the reference's post-order index
    long n_points() const { return pt_end - pt_begin; }
    bool is_leaf() const { return n_children == 0; }
};

struct Tree {
    std::vector<Cell> cells;        // level-major
    std::vector<int> level_start;   // cells of level l: [level_start[l], level_start[l+1])
    std::vector<long> perm;         // permuted position -> original point index
    std::vector<int> preorder;      // flat ids in the reference's pre-order
    std::vector<int> first_at_level;  // first pre-order cell of every level
    int n_levels() const { return (int)level_start.size() - 1; }
    long n_points() const { return (long)perm.size(); }
};

// pts: row-major [n][3]; dim 2 builds the reference's quadtree
// (Octree<2>) over x and y, with z = 0 in every point and cell.
Tree build_tree(const double* pts, long n, long min_pts, int dim = 3);

struct CellPair {
    int obs;
    int src;
};

struct TaskLists {
    std::vector<int> p2m, m2m, l2l, l2p;        // flat ids, reference order
    std::vector<CellPair> p2p, m2p, p2l, m2l;   // flat ids, reference order
};

// dual_tree and the two traversals; n_surf is the translation-surface size
// used by the small-cell rules (cpp/fmm.cpp:587-601).
TaskLists build_lists(const Tree& obs, const Tree& src, double mac, long n_surf,
                      bool small_cells);

// The batched form's trees.  build_tree_cube: the same splitting rules with
// the root's bounds, and the box its children are cut from, both the given
// cube -- trees of different point sets in the same cube then have
// bit-identical cells level by level.  merge_forest: several trees as one
// forest, level-major (level l of tree 0, of tree 1, ...), each tree's points
// offset by pt_off[m] in the permuted and the original order; gid[m][i] is
// the forest id of cell i of tree m.  merge_lists: the trees' task lists in
// forest ids, tree after tree.
Tree build_tree_cube(const double* pts, long n, long min_pts, const double center[3], double hw);
Tree merge_forest(const std::vector<Tree>& trees, const std::vector<long>& pt_off,
                  std::vector<std::vector<int>>& gid);
TaskLists merge_lists(const std::vector<TaskLists>& lists, const std::vector<std::vector<int>>& gid);

// Unit points of surrounding_surface_sphere(order) (cpp/fmm.cpp:22-45).
std::vector<double> sphere_surface(long order);
// The 2D surface of order points on the unit circle (cpp/fmm.cpp:7-20), [n][3].
std::vector<double> circle_surface(long order);

}  // namespace tbem
